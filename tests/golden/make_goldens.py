"""Regenerate tests/golden/goldens.json from the reference's own test data.

Run in a checkout that has the reference tree (it is not needed afterwards):
    python tests/golden/make_goldens.py /path/to/cantera
Sources (paths inside the reference project):
  * test_problems/cxx_samples/kin1_blessed.csv - h2o2 constant-pressure ignition trajectory
    (samples/cxx/kinetics1/kinetics1.cpp; compared with tolerance 2e-4, test_problems/SConscript:236-237)
  * test_problems/cxx_samples/opmenmp_ignition_blessed.txt - gri30 ignition delays
    (samples/cxx/openmp_ignition/openmp_ignition.cpp)
  * test/thermo/nasapoly.cpp - NASA7 CO2 coefficients and CHEMKIN-II known answers
  * test/kinetics/pdep.cpp - PLOG and Chebyshev rate constants and rates of progress
    (mechanism test/data/pdep-test.yaml, copied next to this script)
  * test/python/test_kinetics.py (TestChemicallyActivated) - chemically activated rates of
    progress (mechanism test/data/chemically-activated-reaction.yaml, copied)
  * test/data/sri-falloff.yaml, test/data/tsang-falloff.yaml - SRI and Tsang falloff
    mechanisms (copied; no numeric answers in the reference's tests)
"""
import ast
import csv
import json
import math
import os
import re
import shutil
import sys

AVOGADRO = 6.02214076e26                              # 1/kmol (ct_defs.h)
GAS_CONST_CAL = AVOGADRO * 1.380649e-23 / 4184.0      # cal/mol/K (GasConst_cal_mol_K)
HERE = os.path.dirname(os.path.abspath(__file__))
MECH_FILES = ["pdep-test.yaml", "chemically-activated-reaction.yaml", "sri-falloff.yaml",
              "tsang-falloff.yaml"]


def _num(expr, env=None):
    """Evaluate a numeric C++/Python expression of the tests (numbers, + - * /, names in env)."""
    env = dict(env or {})
    tree = ast.parse(expr.strip(), mode="eval")

    def ev(n):
        if isinstance(n, ast.Expression):
            return ev(n.body)
        if isinstance(n, ast.Constant):
            return float(n.value)
        if isinstance(n, ast.UnaryOp) and isinstance(n.op, ast.USub):
            return -ev(n.operand)
        if isinstance(n, ast.BinOp):
            a, b = ev(n.left), ev(n.right)
            return {ast.Add: a + b, ast.Sub: a - b, ast.Mult: a * b, ast.Div: a / b if b else math.inf}[type(n.op)]
        if isinstance(n, ast.Name):
            return env[n.id]
        if isinstance(n, ast.Call) and isinstance(n.func, ast.Name):
            return env[n.func.id](*[ev(a) for a in n.args])
        raise ValueError("unsupported expression: " + expr)
    return ev(tree)


def pdep_cases(src):
    """One case per EXPECT_NEAR of test/kinetics/pdep.cpp: the state (T, P) set before it,
    the compared quantity (kf or ropf, reaction index) and the expected value with its
    absolute tolerance; the molec-vs-mol checks become ratio cases."""
    cases = []
    for name, body in re.findall(r"TEST_F\(PdepTest, (\w+)\)\s*\{(.*?)\n\}", src, re.S):
        T = P = None
        local = {}
        for stmt in re.split(r";", body):
            stmt = " ".join(stmt.split())
            m = re.search(r"set_TP\((.*),(.*)\)", stmt)
            if m:
                T, P = _num(m.group(1)), _num(m.group(2))
                continue
            env = {"Avogadro": AVOGADRO,
                   "k": lambda A, n, Ea, T=T: A * T ** n * math.exp(-Ea / (GAS_CONST_CAL * T))}
            m = re.search(r"double (kf\d) = (.*)", stmt)
            if m:
                local[m.group(1)] = _num(m.group(2), env)
                continue
            m = re.search(r"EXPECT_NEAR\((.*?), (.*?), (.*)\)$", stmt)
            if not m:
                continue
            a, b, tol = m.groups()
            env.update(local)
            q = re.match(r"(kf|ropf)\[(\d)\]$", b)
            if q:
                cases.append({"test": name, "T": T, "P": P, "quantity": q.group(1), "index": int(q.group(2)),
                              "expected": _num(a, env), "tol": _num(tol, env)})
                continue
            r = re.match(r"kf\[(\d)\]/\(Avogadro\*1e-3\)$", b)
            qa = re.match(r"kf\[(\d)\]$", a)
            if r and qa:
                cases.append({"test": name, "T": T, "P": P, "quantity": "kf_ratio", "index": int(qa.group(1)),
                              "other": int(r.group(1)), "factor": AVOGADRO * 1e-3, "tol": _num(tol, env)})
                continue
            raise ValueError("unparsed check in %s: %s" % (name, stmt))
    m = re.search(r'string Xref = "([^"]*)"', src)
    return {"X": m.group(1), "cases": cases}


def chemact_cases(src):
    block = src[src.index("class TestChemicallyActivated"):]
    block = block[:block.index("\nclass ", 10)]
    P = ast.literal_eval(re.search(r"P = (\[[^\]]*\])", block).group(1))
    Rf = ast.literal_eval(re.search(r"Rf = (\[[^\]]*\])", block).group(1))
    m = re.search(r"gas.TPX = ([\d.]+), P\[i\], (\[[^\]]*\])", block)
    rel = float(re.search(r"rel=([\d.e-]+)", block).group(1))
    return {"T": float(m.group(1)), "X": ast.literal_eval(m.group(2)), "P": P, "ropf": Rf, "rel": rel}


def main(ref):
    out = {}
    rows = list(csv.reader(open(os.path.join(ref, "test_problems/cxx_samples/kin1_blessed.csv"))))
    out["kin1"] = {"header": rows[0], "rows": [[float(x) for x in r] for r in rows[1:]],
                   "tolerance": 2e-4, "threshold": 1e-14,
                   "setup": {"mechanism": "h2o2.yaml", "phase": "ohmech", "T0": 1001.0,
                             "P": 101325.0, "X": "H2:2.0, O2:1.0, N2:4.0", "dt": 1e-5, "nsteps": 100}}
    ign = []
    for line in open(os.path.join(ref, "test_problems/cxx_samples/opmenmp_ignition_blessed.txt")):
        f = line.split()
        if len(f) == 2 and re.match(r"^\d", f[0]):
            ign.append([float(f[0]), float(f[1]), f[1]])
    out["ignition"] = {"rows": ign, "setup": {"mechanism": "gri30.yaml", "phase": "gri30",
                                              "X": "CH4:0.5, O2:1.0, N2:3.76", "P": 101325.0, "dT": 500.0},
                       "threshold": 1e-14, "tolerance": 1e-5}
    src = open(os.path.join(ref, "test/thermo/nasapoly.cpp")).read()
    coeffs = [float(x) for x in re.search(r"coeffs\[\] = \{([^}]*)\}", src).group(1).replace("\n", " ").split(",") if x.strip()]
    checks = []
    for block in re.findall(r"set_tpow\(([\d.]+)\);(.*?)(?=set_tpow|\Z)", src, re.S):
        T = float(block[0])
        for val, name, tol in re.findall(r"EXPECT_NEAR\(([-\d.e+]+), (\w+), ([\d.e-]+)\)", block[1]):
            checks.append([T, name, float(val), float(tol)])
    out["nasa7"] = {"coeffs_low": coeffs, "Tmin": 200.0, "Tmax": 1000.0, "checks": checks}
    out["pdep"] = pdep_cases(open(os.path.join(ref, "test/kinetics/pdep.cpp")).read())
    out["chemact"] = chemact_cases(open(os.path.join(ref, "test/python/test_kinetics.py")).read())
    for f in MECH_FILES:
        shutil.copyfile(os.path.join(ref, "test/data", f), os.path.join(HERE, f))
    path = os.path.join(HERE, "goldens.json")
    json.dump(out, open(path, "w"), indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
