#!/usr/bin/env python3
"""Benchmark: GRI-30 constant-pressure reactors advanced per second on one GB300.

Workload (uneven stiffness): gri30.yaml, 65,536 independent ideal-gas constant-pressure
reactors, T0 ~ U[700, 1800] K, P log-uniform in [1, 40] atm, CH4/air with equivalence
ratio ~ U[0.5, 1.5] (seed 20261203 + 2), each advanced from t = 0 to 1e-2 s at rtol 1e-8,
atol 1e-15 in one persistent launch with a device work queue.  Some reactors ignite, the
cold ones stay nearly inert.  A "step" re-initialises every reactor and advances all of
them to 1e-2 s.  Inputs are synthetic (no dataset is involved).

Usage:  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
Under torchrun each rank takes a contiguous shard of the reactors (no collective on the
data path); the time is the maximum over ranks.
"""
import argparse
import json
import math
import os
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GRI-30 reactors advanced/s on 1 GB300: FP64 BDF vs FP32-LU and NN+fallback @err"
WL = dict(mechanism="gri30.yaml", phase="gri30", n=65536, t_end=1e-2, rtol=1e-8, atol=1e-15,
          T0=(700.0, 1800.0), P_atm=(1.0, 40.0), phi=(0.5, 1.5), fuel="CH4:1",
          oxidizer="O2:1, N2:3.76", seed=20261203 + 2)
CPU_SAMPLE = 8192         # reactors in the bounded CPU sample (a seeded subset of the workload)


def workload_arrays(n, seed, eqr):
    """T0 [n], P [n], Y0 [n, K] (reactor-major); eqr(phi) -> Y."""
    rng = np.random.default_rng(seed)
    T0 = rng.uniform(*WL["T0"], n)
    P = 101325.0 * 10 ** rng.uniform(math.log10(WL["P_atm"][0]), math.log10(WL["P_atm"][1]), n)
    phi = rng.uniform(*WL["phi"], n)
    Y0 = np.array([eqr(p) for p in phi])
    return T0, P, Y0


def cpu_sample_indices(n, size, seed):
    rng = np.random.default_rng(seed + 1000)
    return np.sort(rng.choice(n, min(size, n), replace=False))


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.p = None
        # the raw samples (the JSON line carries their summary)
        self.path = os.environ.get("GBCHEM_CLOCKS_CSV") or os.path.join(tempfile.gettempdir(), "clocks_bench.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()
            self.f.close()

    def summary(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                try:
                    rows.append((float(f[1]), float(f[2]), f[5], f[6], f[7], f[8]))
                except ValueError:
                    pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = sorted(r[0] for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[2 + i].lower().startswith("active")})
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": rows[0][1], "reasons": reasons,
                "samples": len(rows)}


# Declared costs of the transcendental functions in FMA-equivalents, measured once on GB300
# with gb_measure_fp64 (CUDA's double exp: 20.0, log: 35.3); the FLOP count of the algorithm
# uses these constants whatever the engine's own implementation costs.
EXP_FMA, LOG_FMA = 20.0, 35.0


def flop_model(st, N):
    """FP64 operations per evaluation of each integrator component (FMA = 2 flops; exp and
    log at their declared FMA-equivalent cost).  Returns a dict of per-unit FLOPs."""
    E = 2.0 * EXP_FMA
    Lg = 2.0 * LOG_FMA
    Pw = E + Lg
    Dv = 8.0
    K, R = st["K"], st["R"]
    rhs = (3 * K + 20 + 25 * K + 3 * Lg + 2 * st["tb_entries"] + 2 * st["three_body"]
           + R * (4 + E + 6)
           + st["falloff"] * (4 + E + 14 + Dv)
           + st["troe"] * (3 * E + 2 * Lg + Pw + 26)
           + st["reversible"] * (10 + E)
           + 2 * st["gather_entries"] + 4 * K + 10 + Dv)
    jac = 6 * st["jac_col_entries"] + 2 * st["jac_scatter_entries"] + 10 * K * K + 10 * K + 3 * N * N
    lu = (2.0 / 3.0) * N ** 3 + N * Dv
    newton = 2 * N * N + 9 * N
    step = 40 * N + 4 * E
    return {"rhs": rhs, "jac": jac, "lu": lu, "newton": newton, "step": step}


def algorithmic_flops(stats, fm, fp32_lu):
    """Total FP64 FLOPs (and FP32 FLOPs for the mixed form) from per-reactor counters."""
    nrhs = stats["rhs_evals"].sum()
    nset = stats["lin_setups"].sum()
    nni = stats["newton_iters"].sum()
    nst = stats["steps"].sum()
    f64 = nrhs * fm["rhs"] + nset * fm["jac"] + nst * fm["step"]
    f32 = 0.0
    if fp32_lu:
        f32 = nset * fm["lu"] + nni * fm["newton"]
    else:
        f64 += nset * fm["lu"] + nni * fm["newton"]
    return float(f64), float(f32)


def read_traffic():
    """DRAM bytes per launch of the integrator kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "k_bdf_gri30_uneven.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":")[1].split()[0])
            except (IndexError, ValueError):
                return None
    return None


SUR = dict(dt=1e-6, train_reactors=16384, held_reactors=65536, hidden=512, layers=4, epochs=8, batch=4096,
           times=(0.0, 1e-5, 3e-5, 1e-4, 3e-4, 1e-3, 2e-3, 4e-3, 6e-3, 8e-3, 1e-2),
           held_times=(0.0, 2e-5, 5e-5, 2e-4, 5e-4, 1e-3, 1.5e-3, 2.5e-3, 3e-3, 3.5e-3, 4.5e-3, 5e-3, 6.5e-3, 7e-3,
                       9e-3, 1e-2))


def surrogate_leg(sol, dev, torch):
    """The learned arm on the same workload: an MLP trained on integrator pairs (states
    along trajectories of the workload's reactors, each advanced by dt = 1e-6 s), then one
    dt step for 1,048,576 held-out states (65,536 other reactors at 16 times) by the FP64 BDF
    integrator alone and by the surrogate with its gate and BDF fallback."""
    import cantera_gb300 as gb
    from cantera_gb300.surrogate import Surrogate, generate_pairs, trajectory_states
    K = sol.n_species
    eqr = lambda p: sol.equivalence_ratio_mass_fractions(p, WL["fuel"], WL["oxidizer"])

    def initial(n, seed):
        T0, P, Y0 = workload_arrays(n, seed, eqr)
        d = lambda a: torch.tensor(a, device=dev)
        return d(T0), d(P), d(np.ascontiguousarray(Y0.T))

    t0 = time.perf_counter()
    Ts, Ps, Ys, T1, Y1 = generate_pairs(sol, *initial(SUR["train_reactors"], WL["seed"] + 4), SUR["times"], SUR["dt"],
                                        WL["rtol"], WL["atol"])
    t_pairs = time.perf_counter() - t0
    sur = Surrogate(sol, dt=SUR["dt"], hidden=SUR["hidden"], layers=SUR["layers"], seed=0, device=str(dev))
    sur.fit_normalization(Ts, Ps, Ys, T1, Y1)
    X = sur.features(Ts, Ps, Ys)
    Yt = sur.targets(Ts, Ps, Ys, T1, Y1)
    t0 = time.perf_counter()
    losses = sur.train(X, Yt, Ts.shape[0], epochs=SUR["epochs"], batch=SUR["batch"], lr=1e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del X, Yt
    Hs, Hp, Hy = trajectory_states(sol, *initial(SUR["held_reactors"], WL["seed"] + 5), SUR["held_times"],
                                   WL["rtol"], WL["atol"])
    n = Hs.shape[0]
    # the FP64 BDF step alone (the reference result and the method without the network),
    # after one untimed call
    net = gb.ReactorNet(sol, Hs, Hp, Hy, rtol=WL["rtol"], atol=WL["atol"], use_graph=False)
    net.advance(SUR["dt"])
    net.set_state(Hs, Hp, Hy)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    net.advance(SUR["dt"])
    Tb, Yb = torch.empty_like(Hs), torch.empty_like(Hy)
    net.get_state(Tb, Yb)
    torch.cuda.synchronize()
    t_bdf = time.perf_counter() - t0
    del net
    # surrogate + gate + fallback: one untimed call (first-use allocations of the batch's
    # buffers), then the timed one with its phase breakdown
    sur.advance(Hs, Hp, Hy, rtol=WL["rtol"], atol=WL["atol"])
    torch.cuda.synchronize()
    phases = {}
    t0 = time.perf_counter()
    Tsur, Ysur, acc = sur.advance(Hs, Hp, Hy, rtol=WL["rtol"], atol=WL["atol"], timings=phases)
    torch.cuda.synchronize()
    t_sur = time.perf_counter() - t0
    rel_T = ((Tsur - Tb).abs() / Tb)
    major = Yb > 1e-2
    rel_Y = (Ysur - Yb).abs()[major] / Yb[major]
    gflop = 2.0 * n * sum(a * b for a, b in zip(sur.dims[:-1], sur.dims[1:])) / 1e9
    return {"dt": SUR["dt"], "states": n, "unit": "reactor-steps/s",
            "bdf_only": n / t_bdf, "surrogate_with_fallback": n / t_sur, "speedup": t_bdf / t_sur,
            "accepted_fraction": float(acc.float().mean().item()),
            "max_rel_err_T": float(rel_T.max().item()), "max_rel_err_major_species": float(rel_Y.max().item()),
            "network": "%d -> %d x %d (GELU) -> %d, bf16 weights, fp32 accumulation" % (K + 2, SUR["hidden"], SUR["layers"], K + 1),
            "training": {"pairs": int(Ts.shape[0]), "epochs": SUR["epochs"], "loss_first": losses[0],
                         "loss_last": losses[-1], "seconds": t_train, "pair_generation_seconds": t_pairs},
            "inference_gflop": gflop, "phase_seconds": phases,
            "data": "pairs from %d workload reactors at %d trajectory times; held-out %d reactors at %d times"
                    % (SUR["train_reactors"], len(SUR["times"]), SUR["held_reactors"], len(SUR["held_times"]))}


def cpu_baseline(T0, P, Y0, idx, threads, kind="port"):
    """The CPU restatement of the reference path on this host's cores: the reference's
    ReactorNet settings (difference-quotient Jacobian kept between setups) on a bounded,
    seeded sample of the same workload."""
    from oracle import pyoracle as po
    m = po.Mech(os.path.join(ROOT, "cantera_gb300", "data", WL["mechanism"]), WL["phase"])
    o = po.opts(rtol=WL["rtol"], atol=WL["atol"], analytic=False, jac_reuse=True)
    t0 = time.perf_counter()
    T, Y, st, tig = m.advance_batch(T0[idx], P[idx], Y0[idx], WL["t_end"], o, threads=threads)
    dt = time.perf_counter() - t0
    return {"value": len(idx) / dt, "unit": "reactors/s", "cores": threads, "kind": kind,
            "sample": "%d seeded reactors of the workload (subset seed %d), oracle restatement of the "
                      "reference path (not the reference binary), %d host threads, %.1f s"
                      % (len(idx), WL["seed"] + 1000, threads, dt)}, (T, Y, st, tig)


def run_workload(args):
    """The other workloads of the hot path, one JSON line each (not the headline):
    rates - gri30 net production rates and their Jacobian for 1,048,576 random states;
    ndodecane - 16,384 n-dodecane reactors to 5e-3 s, FP64 vs FP32-LU Newton;
    h2o2 - 1,024 hydrogen/air reactors to 1e-3 s against the CPU oracle for every reactor."""
    import torch
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    dev = torch.device("cuda", 0)
    threads = os.cpu_count()
    if args.workload == "rates":
        sol = gb.Solution("gri30.yaml", "gri30")
        K = sol.n_species
        n = args.n if args.n != WL["n"] else 1 << 20
        rng = np.random.default_rng(20261203 + 1)
        T = rng.uniform(300.0, 3000.0, n)
        P = 101325.0 * 10 ** rng.uniform(-1.0, 2.0, n)
        Y = rng.dirichlet(0.5 * np.ones(K), n).T.copy()
        Td, Pd, Yd = (torch.tensor(a, device=dev) for a in (T, P, Y))
        out = {}
        for mode in ("wdot", "wdot+jacobian"):
            fn = (lambda: sol.net_production_rates(Td, Pd, Yd)) if mode == "wdot" else \
                 (lambda: sol.net_production_rates_ddCi(Td, Pd, Yd))
            for _ in range(args.warmup):
                r = fn()
                del r
            torch.cuda.synchronize()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            ev[0].record()
            for _ in range(args.steps):
                r = fn()
                del r
            ev[1].record()
            torch.cuda.synchronize()
            ms = ev[0].elapsed_time(ev[1]) / args.steps
            nnz = len(sol.jac_rowidx)
            bytes_ = n * ((K + 2) * 8 + K * 8 + (nnz * 8 if mode != "wdot" else 0))
            out[mode] = {"states_per_s": n / (ms / 1e3), "ms": ms, "hbm_gbs": bytes_ / (ms / 1e3) / 1e9}
        # CPU: the oracle's rates (and analytic Jacobian) on a sample, all host threads
        m = po.Mech(os.path.join(ROOT, "cantera_gb300", "data", "gri30.yaml"), "gri30")
        ns = 65536
        t0 = time.perf_counter()
        m.rates_batch(T[:ns], P[:ns], np.ascontiguousarray(Y[:, :ns]), threads=threads)
        cpu = ns / (time.perf_counter() - t0)
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
            os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"hbm_gbs": 6800.0}
        line = {"metric": "GRI-30 net production rates (and Jacobian) per second, 1 GB300", "value": out["wdot"]["states_per_s"],
                "unit": "states/s", "workload": "rates", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                "dtype": "f64", "data": "synthetic", "higher_is_better": True,
                "config": {"workload": "gri30, %d states, T U[300,3000] K, P log-U[0.1,100] atm, Y Dirichlet(0.5)" % n},
                "modes": out, "hbm_peak_gbs": peaks.get("hbm_gbs"),
                "cpu_baseline": {"value": cpu, "unit": "states/s (wdot)", "cores": threads, "kind": "port",
                                 "sample": "%d of the states, oracle restatement" % ns}}
        print(json.dumps(line))
        return
    if args.workload == "ndodecane":
        sol = gb.Solution("nDodecane_Reitz.yaml", "nDodecane_IG")
        K = sol.n_species
        n = args.n if args.n != WL["n"] else 16384
        rng = np.random.default_rng(20261203 + 3)
        T0 = rng.uniform(700.0, 1400.0, n)
        P = 101325.0 * 10 ** rng.uniform(1.0, math.log10(60.0), n)
        phi = rng.uniform(0.5, 2.0, n)
        Y0 = np.array([sol.equivalence_ratio_mass_fractions(p, "c12h26:1", "o2:1, n2:3.76") for p in phi])
        Td, Pd, Yd = (torch.tensor(a, device=dev) for a in (T0, P, np.ascontiguousarray(Y0.T)))
        res = {}
        for lu in (64, 32):
            net = gb.ReactorNet(sol, Td, Pd, Yd, rtol=1e-8, atol=1e-15, lu_precision=lu, use_graph=True)
            net.advance(5e-3)
            net.set_state(Td, Pd, Yd)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            net.advance(5e-3)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            Tg, Yg = net.get_state()
            st = net.solver_stats
            res[lu] = {"reactors_per_s": n / dt, "seconds": dt, "launch": net.launch_info,
                       "newton_iters_mean": float(st["newton_iters"].mean()), "steps_mean": float(st["steps"].mean()),
                       "T": Tg, "Y": Yg}
        ns = 64
        m = po.Mech(os.path.join(ROOT, "cantera_gb300", "data", "nDodecane_Reitz.yaml"), "nDodecane_IG")
        t0 = time.perf_counter()
        To, Yo, sto, _ = m.advance_batch(T0[:ns], P[:ns], Y0[:ns], 5e-3, po.opts(rtol=1e-8, atol=1e-15), threads=threads)
        cpu = ns / (time.perf_counter() - t0)
        err = {}
        for lu in (64, 32):
            Tg, Yg = res[lu].pop("T"), res[lu].pop("Y")
            maj = Yo > 1e-2
            err[lu] = {"T_max_rel_vs_oracle": float(np.max(np.abs(Tg[:ns] - To) / To)),
                       "major_species_max_rel_vs_oracle": float(np.max((np.abs(Yg[:, :ns].T - Yo))[maj] / Yo[maj]))}
        line = {"metric": "n-dodecane reactors advanced/s, FP64 vs FP32-LU Newton, 1 GB300",
                "value": res[64]["reactors_per_s"], "unit": "reactors/s", "workload": "ndodecane", "n_gpus": 1,
                "dtype": "f64", "data": "synthetic", "higher_is_better": True,
                "config": {"workload": "nDodecane_IG (K=100, R=553), %d reactors, T0 U[700,1400] K, P log-U[10,60] atm, "
                                       "phi U[0.5,2.0], to 5e-3 s, rtol 1e-8" % n},
                "fp64": res[64], "fp32_lu": res[32], "error": {"fp64": err[64], "fp32_lu": err[32]},
                "cpu_baseline": {"value": cpu, "unit": "reactors/s", "cores": threads, "kind": "port",
                                 "sample": "%d reactors, oracle restatement (difference-quotient Jacobian)" % ns}}
        print(json.dumps(line))
        return
    if args.workload == "h2o2":
        sol = gb.Solution("h2o2.yaml", "ohmech")
        n = 1024
        rng = np.random.default_rng(20261203 + 0)
        T0 = rng.uniform(1000.0, 1600.0, n)
        P = np.full(n, 101325.0)
        phi = rng.uniform(0.5, 2.0, n)
        Y0 = np.array([sol.equivalence_ratio_mass_fractions(p, "H2:1", "O2:1, N2:3.76") for p in phi])
        net = gb.ReactorNet(sol, T0, P, np.ascontiguousarray(Y0.T), rtol=1e-8, atol=1e-15)
        net.advance(1e-3)
        net.set_state(T0, P, np.ascontiguousarray(Y0.T))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        net.advance(1e-3)
        dt = time.perf_counter() - t0
        Tg, Yg = net.get_state()
        tig = net.ignition_times
        m = po.Mech(os.path.join(ROOT, "cantera_gb300", "data", "h2o2.yaml"), "ohmech")
        t0 = time.perf_counter()
        To, Yo, sto, tio = m.advance_batch(T0, P, Y0, 1e-3, po.opts(rtol=1e-8, atol=1e-15), threads=threads)
        cpu = n / (time.perf_counter() - t0)
        maj = Yo > 1e-3
        line = {"metric": "H2/air reactors advanced/s, 1 GB300", "value": n / dt, "unit": "reactors/s",
                "workload": "h2o2", "n_gpus": 1, "dtype": "f64", "data": "synthetic", "higher_is_better": True,
                "config": {"workload": "h2o2, 1024 reactors, T0 U[1000,1600] K, 1 atm, phi U[0.5,2.0], to 1e-3 s, rtol 1e-8"},
                "error_vs_oracle_all_reactors": {"T_max_rel": float(np.max(np.abs(Tg - To) / To)),
                                                 "major_species_max_rel": float(np.max(np.abs(Yg.T - Yo)[maj] / Yo[maj])),
                                                 "ignition_time_max_rel": float(np.max(np.abs(tig - tio) / tio))},
                "cpu_baseline": {"value": cpu, "unit": "reactors/s", "cores": threads, "kind": "port",
                                 "sample": "all 1024 reactors, oracle restatement"}}
        print(json.dumps(line))
        return


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    from oracle import pyoracle as po
    m = po.Mech(os.path.join(ROOT, "cantera_gb300", "data", WL["mechanism"]), WL["phase"])
    T0, P, Y0 = workload_arrays(WL["n"], WL["seed"],
                                lambda p: m.equivalence_ratio(p, WL["fuel"], WL["oxidizer"]))
    threads = os.cpu_count()
    idx = cpu_sample_indices(WL["n"], CPU_SAMPLE, WL["seed"])
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        cb, _ = cpu_baseline(T0, P, Y0, idx, threads)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = len(idx) * len(times) / tot
    line = {"metric": METRIC, "value": value, "unit": "reactors/s", "impl": "reference",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * tot / len(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "gri30 uneven stiffness: %d reactors to %g s (bounded sample of %d per step)"
                       % (WL["n"], WL["t_end"], len(idx)), "rtol": WL["rtol"], "atol": WL["atol"]},
            "cpu_baseline": dict(cb, value=value),
            "e2e": {"value": value, "unit": "reactors/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=WL["n"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="skip the launch-shape autotuner (use the engine's rule)")
    ap.add_argument("--lu-staging", type=int, default=0,
                    help="shared-memory factorisation buffers per block: -1 none, 0 automatic, k at most k")
    ap.add_argument("--workload", default="uneven", choices=["uneven", "rates", "ndodecane", "h2o2"],
                    help="uneven: the headline workload; the others print their own measurement line")
    ap.add_argument("--matrix-placement", type=int, default=0, choices=[0, 1, 2],
                    help="Newton matrix: 0 automatic, 1 shared memory, 2 global slot per warp")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "uneven":
        return run_workload(args)

    import torch
    import cantera_gb300 as gb
    from cantera_gb300.sharding import max_over_ranks, shard_range
    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
        pg = dist
    n_all = args.n
    sol = gb.Solution(WL["mechanism"], WL["phase"])
    K = sol.n_species
    T0, P, Y0 = workload_arrays(n_all, WL["seed"],
                                lambda p: sol.equivalence_ratio_mass_fractions(p, WL["fuel"], WL["oxidizer"]))
    # contiguous shard of this rank
    lo, hi = shard_range(n_all, rank, ws)
    n = hi - lo
    Ts, Ps, Ys = T0[lo:hi].copy(), P[lo:hi].copy(), np.ascontiguousarray(Y0[lo:hi].T)
    dT, dP, dY = (torch.tensor(a, device=dev) for a in (Ts, Ps, Ys))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)   # > L2 (129 MB)

    def barrier():
        torch.cuda.synchronize()
        if pg:
            pg.barrier()

    def maxover(x):
        return max_over_ranks(x, pg, dev)

    fm = flop_model(sol.structure(), K + 1)
    # the launch shape: measured on a strided sample of this rank's reactors (before the
    # timed region)
    tuned = {}
    tune_log = None
    if args.autotune:
        from cantera_gb300.tuning import autotune
        tuned, tune_log = autotune(sol, dT, dP, dY, WL["t_end"] / 10)
    results = {}
    for variant, lu in (("fp64", 64), ("fp32_lu", 32)):
        if variant == "fp32_lu" and args.no_fp32:
            continue
        shape = dict(tuned) if lu == 64 else {}
        shape.setdefault("matrix_placement", args.matrix_placement)
        net = gb.ReactorNet(sol, dT, dP, dY, rtol=WL["rtol"], atol=WL["atol"], lu_precision=lu, use_graph=True,
                            lu_staging=args.lu_staging, **shape)
        launch = net.launch_info
        for _ in range(args.warmup if variant == "fp64" else 1):
            net.set_state(dT, dP, dY)
            net.advance(WL["t_end"])
        barrier()
        steps = args.steps if variant == "fp64" else 1
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        kernel_ms = 0.0
        with Clocks(local) as clk:
            for i in range(steps):
                flush.zero_()
                torch.cuda.synchronize()
                ev[i][0].record()
                net.set_state(dT, dP, dY)
                bad = net.advance(WL["t_end"])
                ev[i][1].record()
                torch.cuda.synchronize()
                kernel_ms += net.last_kernel_ms
        barrier()
        ms = sum(a.elapsed_time(b) for a, b in ev)
        ms_max = maxover(ms)
        stats = net.solver_stats
        f64, f32 = algorithmic_flops(stats, fm, lu == 32)
        Tg, Yg = net.get_state()
        results[variant] = {"ms": ms_max, "steps": steps, "kernel_ms": kernel_ms, "failed": int(bad), "launch": launch,
                            "f64": f64, "f32": f32, "clocks": clk.summary(), "T": Tg, "Y": Yg,
                            "stats": {k: float(v.mean()) for k, v in stats.items()}}
        del net

    # end to end through the public API with host buffers: H2D of the initial state,
    # the advance, D2H of the final state, every step
    shape = dict(tuned)
    shape.setdefault("matrix_placement", args.matrix_placement)
    net = gb.ReactorNet(sol, Ts, Ps, Ys, rtol=WL["rtol"], atol=WL["atol"], lu_precision=64, use_graph=True,
                        lu_staging=args.lu_staging, **shape)
    Th = np.empty(n)
    Yh = np.empty((K, n))
    barrier()
    e2e_ms = 0.0
    e2e_steps = 1
    for i in range(e2e_steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        net.set_state(Ts, Ps, Ys)
        net.advance(WL["t_end"])
        net.get_state(Th, Yh)
        e2e_ms += 1e3 * (time.perf_counter() - t0)
    barrier()
    e2e_ms = maxover(e2e_ms)
    del net

    # FP64 FMA rate of this GPU, measured now that its clocks have settled under load
    fp = gb.measure_fp64()
    if rank != 0:
        if pg:
            pg.destroy_process_group()
        return
    r64 = results["fp64"]
    value = n_all * r64["steps"] / (r64["ms"] / 1e3)
    kernel_s = r64["kernel_ms"] / 1e3 / r64["steps"]
    achieved = r64["f64"] / r64["steps"] / kernel_s / 1e12   # this rank's launches
    peak = fp["gflops"] / 1e3
    line = {"metric": METRIC, "value": value, "unit": "reactors/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r64["ms"] / r64["steps"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "gri30 uneven stiffness: %d reactors, T0 U[700,1800] K, P log-U[1,40] atm, "
                                   "CH4/air phi U[0.5,1.5], to 1e-2 s" % n_all,
                       "rtol": WL["rtol"], "atol": WL["atol"], "seed": WL["seed"],
                       "l2": "flushed (256 MB write) before every timed step",
                       "launch": "persistent kernel, device work queue, CUDA graph", "shards": ws,
                       "launch_shape": r64["launch"],
                       "autotune": tune_log and [{"us_per_reactor": round(t["seconds"] * 1e6, 2), **t["options"]} for t in tune_log]},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": read_traffic(),
                         "peak_source": "FP64 FMA rate measured live by this run (MEASURED_PEAKS.json has no FP64 figure)",
                         "flops_per_reactor": r64["f64"] / r64["steps"] / n_all,
                         "exp_fma_declared": EXP_FMA, "log_fma_declared": LOG_FMA,
                         "exp_fma_measured": fp["exp_fma"], "log_fma_measured": fp["log_fma"]},
            "clocks": r64["clocks"], "gpu_launches": args.steps,
            "solver_stats_mean": r64["stats"], "failed_reactors": r64["failed"],
            "e2e": {"value": n_all * e2e_steps / (e2e_ms / 1e3), "unit": "reactors/s", "steps": e2e_steps,
                    "h2d_bytes_per_step": n * (2 + K) * 8, "d2h_bytes_per_step": n * (1 + K) * 8}}
    if "fp32_lu" in results:
        r32 = results["fp32_lu"]
        line["variants"] = {"fp32_lu": {"value": n_all * r32["steps"] / (r32["ms"] / 1e3), "unit": "reactors/s",
                                        "ms_per_step": r32["ms"] / r32["steps"],
                                        "solver_stats_mean": r32["stats"], "failed_reactors": r32["failed"],
                                        "clocks": r32["clocks"]}}
    if not args.no_surrogate and ws == 1:
        try:
            line.setdefault("variants", {})["surrogate"] = surrogate_leg(sol, dev, torch)
        except Exception as e:   # the learned arm must not cost the FP64 line
            line.setdefault("variants", {})["surrogate"] = {"error": "%s: %s" % (type(e).__name__, e)}
    if not args.no_cpu_baseline and ws == 1:
        idx = cpu_sample_indices(n_all, CPU_SAMPLE, WL["seed"])
        cb, (To, Yo, sto, tio) = cpu_baseline(T0, P, Y0, idx, os.cpu_count())
        line["cpu_baseline"] = cb
        err = {}
        for vname, r in results.items():
            Tg, Yg = r["T"][idx], r["Y"][:, idx].T
            err[vname] = {"T_max_rel": float(np.max(np.abs(Tg - To) / To)),
                          "Y_max_abs": float(np.max(np.abs(Yg - Yo))),
                          "major_species_max_rel": float(np.max(np.abs(Yg - Yo)[Yo > 1e-3] / Yo[Yo > 1e-3]))}
        line["error_vs_cpu_oracle"] = err
    print(json.dumps(line))
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
