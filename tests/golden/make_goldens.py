"""Regenerate tests/golden/goldens.json from the reference's own test data.

Run in a checkout that has the reference tree (it is not needed afterwards):
    python tests/golden/make_goldens.py /path/to/cantera
Sources (paths inside the reference project):
  * test_problems/cxx_samples/kin1_blessed.csv - h2o2 constant-pressure ignition trajectory
    (samples/cxx/kinetics1/kinetics1.cpp; compared with tolerance 2e-4, test_problems/SConscript:236-237)
  * test_problems/cxx_samples/opmenmp_ignition_blessed.txt - gri30 ignition delays
    (samples/cxx/openmp_ignition/openmp_ignition.cpp)
  * test/thermo/nasapoly.cpp - NASA7 CO2 coefficients and CHEMKIN-II known answers
"""
import csv
import json
import os
import re
import sys


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
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "goldens.json")
    json.dump(out, open(path, "w"), indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
