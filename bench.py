#!/usr/bin/env python3
"""Benchmark: GRI-30 constant-pressure reactors advanced per second on one GB300.

Workload (uneven stiffness): gri30.yaml, 65,536 independent ideal-gas constant-pressure
reactors, T0 ~ U[700, 1800] K, P log-uniform in [1, 40] atm, CH4/air with equivalence
ratio ~ U[0.5, 1.5] (seed 20261203 + 2), each advanced from t = 0 to 1e-2 s at rtol 1e-8,
atol 1e-15 in one persistent launch with a device work queue.  Some reactors ignite, the
cold ones stay nearly inert.  A "step" re-initialises every reactor and advances all of
them to 1e-2 s.  Inputs are synthetic (no dataset is involved).

The JSON line: `value` (FP64 Newton matrix, state resident in HBM), `e2e` (the same through
the public API with host arrays, copies in the timed region), `roofline` (FP64 operations
of the algorithm per advance over the mean integrator launch, against the FP64 FMA rate
measured live), `variants` (FP32 Newton matrix; the learned surrogate with its fallback),
`workloads` (the other configurations of the hot path: h2o2 1,024 reactors, gri30 rates and
Jacobian for 2^20 states, n-dodecane 16,384 reactors FP64 / FP32), `cpu_baseline` (the
oracle built with the reference's release flags on the host cores), `error_vs_cpu_oracle`
and `error_protocol` (against the oracle configured as the reference's ReactorNet, and
against its tight run at rtol 1e-12, atol 1e-20, with ignition delays).

Usage:  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
        python bench.py --workload rates|ndodecane|h2o2|gemm (one workload's line alone)
Under torchrun each rank advances its own 65,536 reactors, a contiguous shard of the N x 65,536
drawn from the workload's distributions (weak scaling, no collective on the data path); the
time is the maximum over ranks and the value counts the reactors of all ranks.
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
    # the kinetics calls alone: wdot without the reactor's energy and species equations, and
    # d(wdot)/dc (column entries, species scatter, the dense default-efficiency part)
    rates = rhs - (4 * K + 10 + Dv)
    ddci = 6 * st["jac_col_entries"] + 2 * st["jac_scatter_entries"] + 2 * K * K
    return {"rhs": rhs, "jac": jac, "lu": lu, "newton": newton, "step": step, "rates": rates, "ddci": ddci}


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


def integrator_roofline(f64, f32, n, fp32_lu, kernel_ms, fp, sms):
    """Roofline of one integrator launch of n reactors under the operation model: the model's
    FP64 FLOPs of the advance (f64, from that advance's per-reactor counters) over the launch's
    CUDA-event time, against the FP64 FMA rate measured by this run.  With the FP32 Newton
    matrix, the factorisations and solves are FP32 work (f32); the model's time is then
    F64 / peak64 + F32 / peak32, with peak32 the nominal FP32 rate (SMs x 128 lanes x 2 x
    2.07 GHz)."""
    s = kernel_ms / 1e3
    peak = fp["gflops"] / 1e3
    out = {"bound": "fp64", "achieved": f64 / s / 1e12, "peak": peak, "unit": "TFLOP/s",
           "frac": f64 / s / 1e12 / peak, "flops_per_reactor": f64 / n,
           "ceiling_reactors_per_s": peak * 1e12 / (f64 / n),
           "peak_source": "FP64 FMA rate measured live by this run"}
    if fp32_lu:
        peak32 = sms * 128 * 2 * 2.07e9 / 1e12
        t_model = f64 / (peak * 1e12) + f32 / (peak32 * 1e12)
        out.update({"fp32_flops_per_reactor": f32 / n, "fp32_peak_nominal": peak32,
                    "model_time_frac": t_model / s, "ceiling_reactors_per_s": n / t_model})
    return out


def read_profile_value(key, name="k_bdf_gri30_uneven.md"):
    """A `key: value ...` figure of a committed ncu summary (None if absent)."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(key + ":"):
            try:
                return float(line.split(":")[1].split()[0])
            except (IndexError, ValueError):
                return None
    return None


def read_traffic():
    """DRAM bytes per launch of the integrator kernel from the committed ncu summary."""
    return read_profile_value("traffic_bytes_per_launch")


SUR = dict(dt=1e-6, train_reactors=65536, held_reactors=65536, hidden=512, layers=4, epochs=12, batch=16384,
           lr=1e-3, times=tuple([0.0] + [float(t) for t in np.logspace(-6, -2, 63)]),
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
    losses = sur.train(X, Yt, Ts.shape[0], epochs=SUR["epochs"], batch=SUR["batch"], lr=SUR["lr"])
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    gemm = gemm_roofline(sur, torch)
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
    # forward, input-gradient and weight-gradient products of every training row and epoch
    train_flops = 3.0 * 2.0 * Ts.shape[0] * SUR["epochs"] * sum(a * b for a, b in zip(sur.dims[:-1], sur.dims[1:]))
    return {"dt": SUR["dt"], "states": n, "unit": "reactor-steps/s",
            "bdf_only": n / t_bdf, "surrogate_with_fallback": n / t_sur, "speedup": t_bdf / t_sur,
            "accepted_fraction": float(acc.float().mean().item()),
            "max_rel_err_T": float(rel_T.max().item()), "max_rel_err_major_species": float(rel_Y.max().item()),
            "network": "%d -> %d x %d (GELU) -> %d, bf16 weights, fp32 accumulation" % (K + 2, SUR["hidden"], SUR["layers"], K + 1),
            "training": {"pairs": int(Ts.shape[0]), "epochs": SUR["epochs"], "batch": SUR["batch"], "lr": SUR["lr"],
                         "losses": losses, "loss_first": losses[0], "loss_last": losses[-1], "seconds": t_train,
                         "tflops": train_flops / t_train / 1e12, "pair_generation_seconds": t_pairs},
            "gemm_roofline": gemm,
            "inference_gflop": gflop, "phase_seconds": phases,
            "data": "pairs from %d workload reactors at t = 0 and %d log-spaced times to 1e-2 s; held-out %d reactors at %d times"
                    % (SUR["train_reactors"], len(SUR["times"]) - 1, SUR["held_reactors"], len(SUR["held_times"]))}


TIGHT = dict(rtol=1e-12, atol=1e-20)     # the tight reference run of the error protocol
TIGHT_SAMPLE = 512                        # reactors of the headline workload in that protocol


def oracle_opts(po, rtol, atol, tight=False):
    """The reference's ReactorNet configuration (CVODES with its difference-quotient
    Jacobian kept between setups); tight=True: the same method at rtol 1e-12, atol 1e-20."""
    if tight:
        return po.opts(rtol=TIGHT["rtol"], atol=TIGHT["atol"], analytic=False, jac_reuse=True)
    return po.opts(rtol=rtol, atol=atol, analytic=False, jac_reuse=True)


def gemm_roofline(sur, torch, M=65536):
    """The surrogate's dominant product (a hidden layer: M x 512 x 512, bias + GELU epilogue
    keeping the pre-activation) timed alone with CUDA events on the launching stream,
    against the measured dense BF16 peak."""
    hid = sur.dims[1]
    X = torch.randn(M, hid, device=sur.dev).to(torch.bfloat16)
    C = torch.empty(M, hid, dtype=torch.bfloat16, device=sur.dev)
    Z = torch.empty(M, hid, device=sur.dev)
    W, b = sur.Wb[1], sur.b[1]
    for _ in range(3):
        sur._tc(X, W, C, bias=b, act=1, Z=Z)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    reps = 20
    ev[0].record()
    for _ in range(reps):
        sur._tc(X, W, C, bias=b, act=1, Z=Z)
    ev[1].record()
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[1]) / reps
    flops = 2.0 * M * hid * hid
    peaks = measured_peaks()
    peak = peaks.get("bf16_tflops")
    source = "MEASURED_PEAKS.json bf16_tflops (burst)"
    if not peak:
        peak, source = 1900.0, "fallback: 1.9 PFLOP/s dense BF16 burst, an earlier measurement on a GB300"
    tf = flops / (ms / 1e3) / 1e12
    # bytes: X, W in; C (bf16) and Z (fp32) out.  At 2 M N K / bytes ~ 114 FLOP per byte this
    # product sits below the ridge of the BF16 roofline (~280 FLOP per byte): its bound is HBM
    byt = M * hid * 2 + hid * hid * 2 + M * hid * (2 + 4)
    hbm = peaks.get("hbm_gbs") or 6800.0
    gbs = byt / (ms / 1e3) / 1e9
    return {"shape": [M, hid, hid], "ms": ms, "tflops": tf, "peak_tflops": peak,
            "frac": tf / peak, "hbm_gbs": gbs, "hbm_peak_gbs": hbm, "hbm_frac": gbs / hbm,
            "flop_per_byte": flops / byt, "peak_source": source,
            "kernel": "k_umma_gemm (tcgen05.mma kind::f16, TMEM accumulator, TMA 128B-swizzled operands)"}


def cpu_baseline(T0, P, Y0, idx, threads, kind="port"):
    """The CPU restatement of the reference path on this host's cores, built with the
    reference's release flags: the reference's ReactorNet settings (difference-quotient
    Jacobian kept between setups) on a bounded, seeded sample of the same workload."""
    from oracle import pyoracle as po
    m = po.Mech(os.path.join(ROOT, "cantera_gb300", "data", WL["mechanism"]), WL["phase"], fast=True)
    o = oracle_opts(po, WL["rtol"], WL["atol"])
    t0 = time.perf_counter()
    T, Y, st, tig = m.advance_batch(T0[idx], P[idx], Y0[idx], WL["t_end"], o, threads=threads)
    dt = time.perf_counter() - t0
    return {"value": len(idx) / dt, "unit": "reactors/s", "cores": threads, "kind": kind,
            "sample": "%d seeded reactors of the workload (subset seed %d), oracle restatement of the "
                      "reference path (not the reference binary) built with %s, %d host threads, %.1f s"
                      % (len(idx), WL["seed"] + 1000, po.FLAGS[True], threads, dt)}, (T, Y, st, tig)


def state_errors(T, Y, Tr, Yr, major_min=1e-3):
    """T relative, major-species (Y_ref >= 1e-3) relative and Y absolute errors; Y, Yr
    reactor-major."""
    major = Yr >= major_min
    return {"T_max_rel": float(np.max(np.abs(T - Tr) / Tr)),
            "major_species_max_rel": float(np.max(np.abs(Y - Yr)[major] / Yr[major])) if major.any() else 0.0,
            "Y_max_abs": float(np.max(np.abs(Y - Yr)))}


def settled_mask(m, P, Tt, Yt, t_end, rtol):
    """Reactors that are not in mid-ignition at t_end: a relative time shift of 1e-4 moves
    their T by less than 10 x rtol (the tight run's own dT/dt)."""
    dTdt = np.array([m.reactor_rhs(P[s], np.concatenate([[1.0, Tt[s]], Yt[s]]))[1] for s in range(len(P))])
    return np.abs(dTdt) * 1e-4 * t_end < 10 * rtol * Tt


def tight_run(m, po, T0, P, Y0, t_end, threads):
    """The tight solution: the reference's method at rtol 1e-12, atol 1e-20; a reactor whose
    run stops (the difference-quotient Jacobian can stall at the 1000 K midpoint of the NASA7
    fits at this tolerance) is re-run with the analytic Jacobian.  Returns T, Y, stats,
    ignition times, the re-run count and the mask of reactors still without a solution."""
    Tt, Yt, stt, tit = m.advance_batch(T0, P, Y0, t_end, oracle_opts(po, 0, 0, tight=True), threads=threads)
    bad = stt[:, 8] != 0
    rerun = int(bad.sum())
    if rerun:
        o = po.opts(rtol=TIGHT["rtol"], atol=TIGHT["atol"], analytic=True)
        T2, Y2, st2, ti2 = m.advance_batch(T0[bad], P[bad], Y0[bad], t_end, o, threads=threads)
        Tt[bad], Yt[bad], stt[bad], tit[bad] = T2, Y2, st2, ti2
    return Tt, Yt, stt, tit, rerun, stt[:, 8] != 0


def error_protocol(m, po, T0, P, Y0, t_end, rtol, atol, gpu, threads, extra_oracles=None):
    """Error protocol of the integrator workloads on one sample: (i) against the CPU oracle
    configured as the reference's ReactorNet at the same tolerances, (ii) against a tight
    run of it (rtol 1e-12, atol 1e-20), with the oracle's own error against (ii) beside the
    GPU's, and the ignition-delay (time of the largest dT/dt) error of every igniting
    reactor.  gpu: {variant: (T [n], Y [n][K], tign [n])} on the same sample.
    extra_oracles: {name: (oracle options, [variants])}: further configurations of the oracle
    (the reference's other linear solver), each with its own error against (ii) and, for the
    listed GPU variants, the ratio of their error to it."""
    t0 = time.perf_counter()
    To, Yo, sto, tio = m.advance_batch(T0, P, Y0, t_end, oracle_opts(po, rtol, atol), threads=threads)
    Tt, Yt, stt, tit, rerun, tfail = tight_run(m, po, T0, P, Y0, t_end, threads)
    secs = time.perf_counter() - t0
    use = (sto[:, 8] == 0) & ~tfail           # reactors with both oracle solutions
    settled = settled_mask(m, P, Tt, Yt, t_end, rtol) & use
    ign = (Tt > T0 + 400.0) & (tit > 0) & (tit < t_end) & use
    bar = 10 * rtol
    out = {"reactors": int(len(T0)), "compared": int(use.sum()), "igniting": int(ign.sum()),
           "settled": int(settled.sum()), "bar_10rtol": bar, "tight": dict(TIGHT),
           "tight_rerun_with_analytic_jacobian": rerun, "tight_failed": int(tfail.sum()),
           "oracle_failed": int(np.sum(sto[:, 8] != 0)), "oracle_seconds": secs,
           "oracle_vs_tight": {"all": state_errors(To[use], Yo[use], Tt[use], Yt[use]),
                               "settled": state_errors(To[settled], Yo[settled], Tt[settled], Yt[settled])}}
    if ign.any():
        out["oracle_vs_tight"]["ignition_delay_max_rel"] = float(np.max(np.abs(tio[ign] - tit[ign]) / tit[ign]))
    for name, (Tg, Yg, tg) in gpu.items():
        e = {"vs_tight": {"all": state_errors(Tg[use], Yg[use], Tt[use], Yt[use]),
                          "settled": state_errors(Tg[settled], Yg[settled], Tt[settled], Yt[settled])},
             "vs_oracle": state_errors(Tg[use], Yg[use], To[use], Yo[use])}
        if ign.any():
            e["ignition_delay_max_rel_vs_oracle"] = float(np.max(np.abs(tg[ign] - tio[ign]) / tio[ign]))
            e["ignition_delay_max_rel_vs_tight"] = float(np.max(np.abs(tg[ign] - tit[ign]) / tit[ign]))
        a, o_ = e["vs_tight"]["all"], out["oracle_vs_tight"]["all"]
        # two correct integrations at the same tolerance differ in their error by O(1)
        # factors (different Jacobians, different steps): the ratio of the GPU's error to the
        # reference configuration's own, and the 3x bar the tests hold
        e["T_error_ratio_to_oracle"] = a["T_max_rel"] / max(o_["T_max_rel"], 1e-300)
        e["T_within_bar"] = a["T_max_rel"] <= bar
        e["T_within_3x_oracle_error"] = a["T_max_rel"] <= max(bar, 3 * o_["T_max_rel"])
        e["major_species_within_3x_oracle_error"] = a["major_species_max_rel"] <= max(bar, 3 * o_["major_species_max_rel"])
        e["settled_T_within_bar"] = e["vs_tight"]["settled"]["T_max_rel"] <= bar
        if ign.any():
            e["ignition_within_1e-3"] = e["ignition_delay_max_rel_vs_oracle"] <= 1e-3
        out[name] = e
    for oname, (oopts, variants) in (extra_oracles or {}).items():
        Tx, Yx, stx, tix = m.advance_batch(T0, P, Y0, t_end, oopts, threads=threads)
        ok = use & (stx[:, 8] == 0)
        ex = {"failed": int(np.sum(stx[:, 8] != 0)),
              "vs_tight": {"all": state_errors(Tx[ok], Yx[ok], Tt[ok], Yt[ok]),
                           "settled": state_errors(Tx[ok & settled], Yx[ok & settled], Tt[ok & settled],
                                                   Yt[ok & settled])}}
        ig = ign & ok
        if ig.any():
            ex["ignition_delay_max_rel_vs_tight"] = float(np.max(np.abs(tix[ig] - tit[ig]) / tit[ig]))
        out["oracle_" + oname] = ex
        for v in variants:
            if v not in gpu:
                continue
            Tg, Yg, tg = gpu[v]
            a = state_errors(Tg[ok], Yg[ok], Tt[ok], Yt[ok])
            o_ = ex["vs_tight"]["all"]
            out[v]["T_error_ratio_to_oracle_" + oname] = a["T_max_rel"] / max(o_["T_max_rel"], 1e-300)
            out[v]["T_within_3x_oracle_" + oname] = a["T_max_rel"] <= max(bar, 3 * o_["T_max_rel"])
            out[v]["vs_oracle_" + oname] = state_errors(Tg[ok], Yg[ok], Tx[ok], Yx[ok])
            if ig.any():
                out[v]["ignition_delay_max_rel_vs_oracle_" + oname] = float(np.max(np.abs(tg[ig] - tix[ig]) / tix[ig]))
    return out


def time_advance(net, T, P, Y, t_end, flush, torch):
    """One timed advance from the given state (L2 flushed before it): CUDA events on the
    engine's stream around the integrator launch (kernel ms) and on the host (wall ms)."""
    flush.zero_()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    net.set_state(T, P, Y)
    bad = net.advance(t_end)
    torch.cuda.synchronize()
    return bad, net.last_kernel_ms, 1e3 * (time.perf_counter() - t0)


def variant_h2o2(dev, torch, flush, threads, fp):
    """Plain method, small: h2o2, 1,024 reactors, T0 U[1000,1600] K, 1 atm, H2/air phi
    U[0.5,2.0] (seed 20261203), to 1e-3 s at rtol 1e-8, atol 1e-15, every reactor compared
    with the oracle (reference configuration and tight run).  fp: the FP64 rate measured by
    this run (the roofline's peak)."""
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    sol = gb.Solution("h2o2.yaml", "ohmech")
    fm = flop_model(sol.structure(), sol.n_species + 1)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    n, t_end, rtol, atol = 1024, 1e-3, 1e-8, 1e-15
    rng = np.random.default_rng(20261203 + 0)
    T0 = rng.uniform(1000.0, 1600.0, n)
    P = np.full(n, 101325.0)
    phi = rng.uniform(0.5, 2.0, n)
    Y0 = np.array([sol.equivalence_ratio_mass_fractions(p, "H2:1", "O2:1, N2:3.76") for p in phi])
    d = lambda a: torch.tensor(a, device=dev)
    Td, Pd, Yd = d(T0), d(P), d(np.ascontiguousarray(Y0.T))
    res, gpu = {}, {}
    for name, lu in (("fp64", 64), ("fp32_lu", 32)):
        net = gb.ReactorNet(sol, Td, Pd, Yd, rtol=rtol, atol=atol, lu_precision=lu, use_graph=True)
        for _ in range(3):
            time_advance(net, Td, Pd, Yd, t_end, flush, torch)
        runs = [time_advance(net, Td, Pd, Yd, t_end, flush, torch) for _ in range(5)]
        ms = float(np.median([r[1] for r in runs]))
        Tg, Yg = net.get_state()
        st = net.solver_stats           # the last advance's counters (set_state resets them)
        res[name] = {"value": n / (ms / 1e3), "unit": "reactors/s", "kernel_ms": ms,
                     "failed_reactors": int(runs[-1][0]),
                     "solver_stats_mean": {k: float(v.mean()) for k, v in st.items()},
                     "roofline": integrator_roofline(*algorithmic_flops(st, fm, lu == 32), n, lu == 32,
                                                     runs[-1][1], fp, sms)}
        gpu[name] = (Tg, Yg.T, net.ignition_times)
        del net
    m = po.Mech(os.path.join(ROOT, "cantera_gb300", "data", "h2o2.yaml"), "ohmech")
    errs = error_protocol(m, po, T0, P, Y0, t_end, rtol, atol, gpu, threads)
    mf = po.Mech(os.path.join(ROOT, "cantera_gb300", "data", "h2o2.yaml"), "ohmech", fast=True)
    t0 = time.perf_counter()
    mf.advance_batch(T0, P, Y0, t_end, oracle_opts(po, rtol, atol), threads=threads)
    cpu = n / (time.perf_counter() - t0)
    return dict(res["fp64"], variants={"fp32_lu": res["fp32_lu"]},
                config={"workload": "h2o2, 1024 reactors, T0 U[1000,1600] K, 1 atm, H2/air phi U[0.5,2.0], "
                                    "to 1e-3 s", "rtol": rtol, "atol": atol, "seed": 20261203},
                errors=errs,
                cpu_baseline={"value": cpu, "unit": "reactors/s", "cores": threads, "kind": "port",
                              "sample": "all 1024 reactors, oracle restatement built with %s" % po.FLAGS[True]})


def variant_rates(dev, torch, flush, threads, n=1 << 20, peaks=None):
    """Rate evaluation only: gri30, 1,048,576 states, T U[300,3000] K, P log-U[0.1,100] atm,
    Y ~ Dirichlet(0.5) (seed 20261204); wdot and wdot + d(wdot)/dc on the reference's
    pattern, kernel time by CUDA events on the engine's stream, parity of the first 65,536
    states against the oracle (gross-rate-scaled 1e-12 for wdot; 1e-12 of the state's
    largest entry for the Jacobian)."""
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    sol = gb.Solution("gri30.yaml", "gri30")
    K = sol.n_species
    rng = np.random.default_rng(20261203 + 1)
    T = rng.uniform(300.0, 3000.0, n)
    P = 101325.0 * 10 ** rng.uniform(-1.0, 2.0, n)
    Y = rng.dirichlet(0.5 * np.ones(K), n).T.copy()
    Td, Pd, Yd = (torch.tensor(a, device=dev) for a in (T, P, Y))
    fm = flop_model(sol.structure(), K + 1)
    nnz = len(sol.jac_rowidx)
    wdot = torch.empty((K, n), dtype=torch.float64, device=dev)
    jac = torch.empty((nnz, n), dtype=torch.float64, device=dev)
    out = {}
    for mode in ("wdot", "wdot+jacobian"):
        fn = (lambda: sol.net_production_rates(Td, Pd, Yd, out=wdot)) if mode == "wdot" else \
             (lambda: sol.net_production_rates_ddCi(Td, Pd, Yd, vals=jac, wdot=wdot))
        for _ in range(3):
            fn()
        ks = []
        for _ in range(5):
            flush.zero_()
            torch.cuda.synchronize()
            fn()
            ks.append(sol.last_kernel_ms)
        ms = float(np.median(ks))
        bytes_ = n * ((K + 2) * 8 + K * 8 + (nnz * 8 if mode != "wdot" else 0))
        flops = n * (fm["rates"] + (fm["ddci"] if mode != "wdot" else 0.0))
        out[mode] = {"states_per_s": n / (ms / 1e3), "kernel_ms": ms,
                     "algorithmic_bytes_per_state": bytes_ / n, "hbm_gbs": bytes_ / (ms / 1e3) / 1e9,
                     "flops_per_state_model": flops / n, "fp64_tflops_model": flops / (ms / 1e3) / 1e12}
    # parity of the first 65,536 states against the oracle (checker build)
    ns = 65536
    m = po.Mech(os.path.join(ROOT, "cantera_gb300", "data", "gri30.yaml"), "gri30")
    wo, jo, gross = m.rates_batch(T[:ns], P[:ns], np.ascontiguousarray(Y[:, :ns]), mode=1,
                                  pattern=(sol.jac_colptr, sol.jac_rowidx), threads=threads, gross=True)
    wg = wdot[:, :ns].cpu().numpy()
    jg = jac[:, :ns].cpu().numpy()
    w_err = float(np.max(np.abs(wg - wo) / (gross + 1e-300)))
    j_err = float(np.max(np.max(np.abs(jg - jo), axis=0) / np.maximum(np.max(np.abs(jo), axis=0), 1e-300)))
    parity = {"states": ns, "wdot_max_err_over_gross": w_err, "wdot_within_1e-12": w_err <= 1e-12,
              "jac_max_err_over_state_max": j_err, "jac_within_1e-12": j_err <= 1e-12}
    # CPU: the timing build on the same 65,536 states, all host threads
    mf = po.Mech(os.path.join(ROOT, "cantera_gb300", "data", "gri30.yaml"), "gri30", fast=True)
    t0 = time.perf_counter()
    mf.rates_batch(T[:ns], P[:ns], np.ascontiguousarray(Y[:, :ns]), mode=0, threads=threads)
    cpu_w = ns / (time.perf_counter() - t0)
    t0 = time.perf_counter()
    mf.rates_batch(T[:ns], P[:ns], np.ascontiguousarray(Y[:, :ns]), mode=1,
                   pattern=(sol.jac_colptr, sol.jac_rowidx), threads=threads)
    cpu_j = ns / (time.perf_counter() - t0)
    hbm = (peaks or {}).get("hbm_gbs")
    hbm_source = "MEASURED_PEAKS.json hbm_gbs"
    if not hbm:
        hbm, hbm_source = 6800.0, "fallback: 6.8 TB/s, an earlier copy measurement on a GB300"
    return {"value": out["wdot"]["states_per_s"], "unit": "states/s", "modes": out,
            "config": {"workload": "gri30, %d states, T U[300,3000] K, P log-U[0.1,100] atm, Y Dirichlet(0.5)" % n,
                       "seed": 20261204, "l2": "flushed (256 MB write) before every timed call"},
            "hbm_roofline": {"peak_gbs": hbm, "frac_wdot": out["wdot"]["hbm_gbs"] / hbm,
                             "frac_jacobian": out["wdot+jacobian"]["hbm_gbs"] / hbm, "peak_source": hbm_source},
            "parity_vs_oracle": parity,
            "cpu_baseline": {"value": cpu_w, "unit": "states/s (wdot)", "value_jacobian": cpu_j, "cores": threads,
                             "kind": "port", "sample": "%d of the states, oracle restatement built with %s"
                                                       % (ns, po.FLAGS[True])}}


def variant_ndodecane(dev, torch, flush, threads, fp, n=16384, sample=64):
    """Mixed-precision Newton and the Krylov path: nDodecane_IG (K=100, R=553), 16,384 reactors,
    T0 U[700,1400] K, P log-U[10,60] atm, n-dodecane/air phi U[0.5,2.0] (seed 20261206), to
    5e-3 s at rtol 1e-8: the dense path with FP64 and FP32 Newton matrices (each with its
    roofline; fp: the FP64 rate measured by this run), the mole reactor with GMRES and the
    adaptive preconditioner (FP64 and FP32 factors), with Newton counts and the error protocol
    on a sample."""
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    sol = gb.Solution("nDodecane_Reitz.yaml", "nDodecane_IG")
    fm = flop_model(sol.structure(), sol.n_species + 1)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    t_end, rtol, atol = 5e-3, 1e-8, 1e-15
    rng = np.random.default_rng(20261203 + 3)
    T0 = rng.uniform(700.0, 1400.0, n)
    P = 101325.0 * 10 ** rng.uniform(1.0, math.log10(60.0), n)
    phi = rng.uniform(0.5, 2.0, n)
    Y0 = np.array([sol.equivalence_ratio_mass_fractions(p, "c12h26:1", "o2:1, n2:3.76") for p in phi])
    Td, Pd, Yd = (torch.tensor(a, device=dev) for a in (T0, P, np.ascontiguousarray(Y0.T)))
    idx = cpu_sample_indices(n, sample, 20261203 + 3)
    res, gpu = {}, {}
    for name, lu, solver in (("fp64", 64, "DENSE"), ("fp32_lu", 32, "DENSE"), ("gmres", 64, "GMRES"),
                             ("gmres_fp32", 32, "GMRES")):
        net = gb.ReactorNet(sol, Td, Pd, Yd, rtol=rtol, atol=atol, lu_precision=lu, linear_solver=solver)
        net.advance(1e-7)          # untimed first launch (module load, attributes)
        bad, ms, wall = time_advance(net, Td, Pd, Yd, t_end, flush, torch)
        Tg, Yg = net.get_state()
        st = net.solver_stats
        res[name] = {"value": n / (ms / 1e3), "unit": "reactors/s", "kernel_ms": ms, "wall_ms": wall,
                     "failed_reactors": int(bad), "launch": net.launch_info,
                     "newton_iters_mean": float(st["newton_iters"].mean()), "steps_mean": float(st["steps"].mean()),
                     "solver_stats_mean": {k: float(v.mean()) for k, v in st.items()}}
        if solver == "DENSE":
            res[name]["roofline"] = integrator_roofline(*algorithmic_flops(st, fm, lu == 32), n, lu == 32, ms,
                                                        fp, sms)
        if solver == "GMRES":
            res[name]["solver_stats_mean"].update({k: float(v.mean()) for k, v in net.krylov_stats.items()})
            res[name]["method"] = ("IdealGasConstPressureMoleReactor with GMRES and the adaptive preconditioner "
                                   "(ILUT of I - gamma Jp in a minimum-degree order), %s factors and triangular "
                                   "solves, the rest FP64" % ("FP32" if lu == 32 else "FP64"))
        gpu[name] = (Tg[idx], Yg[:, idx].T, net.ignition_times[idx])
        del net
    m = po.Mech(os.path.join(ROOT, "cantera_gb300", "data", "nDodecane_Reitz.yaml"), "nDodecane_IG")
    errs = error_protocol(m, po, T0[idx], P[idx], Y0[idx], t_end, rtol, atol, gpu, threads,
                          extra_oracles={"gmres": (po.opts(rtol=rtol, atol=atol, gmres=True), ["gmres", "gmres_fp32"])})
    mf = po.Mech(os.path.join(ROOT, "cantera_gb300", "data", "nDodecane_Reitz.yaml"), "nDodecane_IG", fast=True)
    t0 = time.perf_counter()
    mf.advance_batch(T0[idx], P[idx], Y0[idx], t_end, oracle_opts(po, rtol, atol), threads=threads)
    cpu = len(idx) / (time.perf_counter() - t0)
    # the Krylov variants' own CPU baseline: the reference's GMRES configuration (mole reactor,
    # adaptive preconditioner) of the timing build on the same sample
    t0 = time.perf_counter()
    mf.advance_batch(T0[idx], P[idx], Y0[idx], t_end, po.opts(rtol=rtol, atol=atol, gmres=True), threads=threads)
    cpu_gm = len(idx) / (time.perf_counter() - t0)
    for k in ("gmres", "gmres_fp32"):
        res[k]["cpu_baseline"] = {"value": cpu_gm, "unit": "reactors/s", "cores": threads, "kind": "port",
                                  "sample": "%d seeded reactors, the oracle's GMRES configuration built with %s"
                                            % (len(idx), po.FLAGS[True])}
    return dict(res["fp64"], variants={k: res[k] for k in ("fp32_lu", "gmres", "gmres_fp32")},
                config={"workload": "nDodecane_IG (K=100, R=553), %d reactors, T0 U[700,1400] K, P log-U[10,60] atm, "
                                    "phi U[0.5,2.0], to 5e-3 s" % n, "rtol": rtol, "atol": atol,
                        "seed": 20261206, "l2": "flushed (256 MB write) before the timed advance"},
                errors=errs,
                cpu_baseline={"value": cpu, "unit": "reactors/s", "cores": threads, "kind": "port",
                              "sample": "%d seeded reactors, oracle restatement built with %s" % (len(idx), po.FLAGS[True])})


def run_workload(args):
    """One secondary workload on its own, one JSON line (the default run carries all of
    them in the headline line's "workloads")."""
    import torch
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    threads = os.cpu_count()
    import cantera_gb300 as gb
    if args.workload == "gemm":
        from cantera_gb300.surrogate import Surrogate
        sur = Surrogate(gb.Solution("gri30.yaml", "gri30"), hidden=SUR["hidden"], layers=SUR["layers"], seed=0,
                        device=str(dev))
        line = dict(workload="gemm", n_gpus=1, dtype="bf16", data="synthetic", higher_is_better=True)
        line.update(gemm_roofline(sur, torch, M=args.n or 65536))
        print(json.dumps(line))
        return
    fn = {"rates": lambda: variant_rates(dev, torch, flush, threads, n=args.n or 1 << 20,
                                         peaks=measured_peaks()),
          "ndodecane": lambda: variant_ndodecane(dev, torch, flush, threads, gb.measure_fp64(), n=args.n or 16384),
          "h2o2": lambda: variant_h2o2(dev, torch, flush, threads, gb.measure_fp64())}[args.workload]
    line = dict(workload=args.workload, n_gpus=1, dtype="f64", data="synthetic", higher_is_better=True)
    line.update(fn())
    print(json.dumps(line))


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    return json.load(open(path)) if os.path.exists(path) else {}


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    from oracle import pyoracle as po
    m = po.Mech(os.path.join(ROOT, "cantera_gb300", "data", WL["mechanism"]), WL["phase"], fast=True)
    n_all = (args.n or WL["n"]) * ws          # the workload of the GPU arm at this world size
    T0, P, Y0 = workload_arrays(n_all, WL["seed"],
                                lambda p: m.equivalence_ratio(p, WL["fuel"], WL["oxidizer"]))
    threads = os.cpu_count()
    idx = cpu_sample_indices(n_all, CPU_SAMPLE, WL["seed"])
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
                       % (n_all, WL["t_end"], len(idx)), "rtol": WL["rtol"], "atol": WL["atol"]},
            "cpu_baseline": dict(cb, value=value),
            "e2e": {"value": value, "unit": "reactors/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=None,
                    help="states or reactors of the workload, per GPU for the headline (default: the "
                         "workload's own size)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--no-gmres", action="store_true",
                    help="skip the Krylov-path variant (mole reactor, GMRES, adaptive preconditioner)")
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--no-workloads", action="store_true",
                    help="skip the other workloads (h2o2, rates, n-dodecane) of the default run")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="skip the launch-shape autotuner (use the engine's rule)")
    ap.add_argument("--lu-staging", type=int, default=0,
                    help="shared-memory factorisation buffers per block: -1 none, 0 automatic, k at most k")
    ap.add_argument("--workload", default="uneven", choices=["uneven", "rates", "ndodecane", "h2o2", "gemm"],
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
    # weak scaling: every rank advances its own n reactors (default 65,536), a contiguous shard
    # of ws x n reactors drawn from the workload's distributions
    n_all = (args.n or WL["n"]) * ws
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
    for variant, lu, solver in (("fp64", 64, "DENSE"), ("fp32_lu", 32, "DENSE"), ("gmres", 64, "GMRES")):
        if (variant == "fp32_lu" and args.no_fp32) or (variant == "gmres" and args.no_gmres):
            continue
        shape = dict(tuned) if variant == "fp64" else {}
        shape.setdefault("matrix_placement", args.matrix_placement)
        net = gb.ReactorNet(sol, dT, dP, dY, rtol=WL["rtol"], atol=WL["atol"], lu_precision=lu, use_graph=True,
                            lu_staging=args.lu_staging, linear_solver=solver, **shape)
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
        # the counters are reset by set_state: they hold the last advance (one step's work)
        stats = net.solver_stats
        f64, f32 = algorithmic_flops(stats, fm, lu == 32)
        Tg, Yg = net.get_state()
        results[variant] = {"ms": ms_max, "steps": steps, "kernel_ms": kernel_ms, "failed": int(bad), "launch": launch,
                            "f64": f64, "f32": f32, "clocks": clk.summary(), "T": Tg, "Y": Yg,
                            "tign": net.ignition_times,
                            "stats": {k: float(v.mean()) for k, v in stats.items()}}
        if solver == "GMRES":
            results[variant]["stats"].update({k: float(v.mean()) for k, v in net.krylov_stats.items()})
        del net

    # end to end through the public API with host buffers: every step the H2D copy of the
    # initial state, the advance and the D2H copy of the final state; one untimed step
    # first (the advance's graph capture), then the mean over the timed steps
    shape = dict(tuned)
    shape.setdefault("matrix_placement", args.matrix_placement)
    net = gb.ReactorNet(sol, Ts, Ps, Ys, rtol=WL["rtol"], atol=WL["atol"], lu_precision=64, use_graph=True,
                        lu_staging=args.lu_staging, **shape)
    Th = np.empty(n)
    Yh = np.empty((K, n))
    net.advance(WL["t_end"])
    net.get_state(Th, Yh)
    barrier()
    e2e_ms = 0.0
    e2e_steps = max(1, min(args.steps, 3))
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
    kernel_s = r64["kernel_ms"] / 1e3 / r64["steps"]       # mean integrator launch
    achieved = r64["f64"] / kernel_s / 1e12                  # FLOPs of one advance / its launch
    peak = fp["gflops"] / 1e3
    fpr = r64["f64"] / n
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
                         "flops_per_reactor": fpr, "kernel_ms_mean": kernel_s * 1e3,
                         "ceiling_reactors_per_s": peak * 1e12 / fpr,
                         # FP64 pipe work counted by ncu (DFMA x 2 + DADD + DMUL thread instructions
                         # per cycle over all SMs) at this run's SM clock: the FP64 arithmetic the
                         # kernel issues, beside the algorithm's operation model above
                         "ncu_fp64_tflops": (read_profile_value("fp64_flops_per_cycle") or 0.0) *
                                            (r64["clocks"].get("sm_mhz") or 0.0) * 1e6 / 1e12 or None,
                         "exp_fma_declared": EXP_FMA, "log_fma_declared": LOG_FMA,
                         "exp_fma_measured": fp["exp_fma"], "log_fma_measured": fp["log_fma"]},
            "clocks": r64["clocks"], "gpu_launches": args.steps,
            "solver_stats_mean": r64["stats"], "failed_reactors": r64["failed"],
            "e2e": {"value": n_all * e2e_steps / (e2e_ms / 1e3), "unit": "reactors/s", "steps": e2e_steps,
                    "h2d_bytes_per_step": n * (2 + K) * 8, "d2h_bytes_per_step": n * (1 + K) * 8}}
    for vname in ("fp32_lu", "gmres"):
        if vname in results:
            rv = results[vname]
            line.setdefault("variants", {})[vname] = {
                "value": n_all * rv["steps"] / (rv["ms"] / 1e3), "unit": "reactors/s",
                "ms_per_step": rv["ms"] / rv["steps"], "solver_stats_mean": rv["stats"],
                "failed_reactors": rv["failed"], "launch": rv["launch"], "clocks": rv["clocks"]}
    if "fp32_lu" in results:
        rv = results["fp32_lu"]
        line["variants"]["fp32_lu"]["roofline"] = integrator_roofline(
            rv["f64"], rv["f32"], n, True, rv["kernel_ms"] / rv["steps"], fp,
            torch.cuda.get_device_properties(dev).multi_processor_count)
    if "gmres" in results:
        line["variants"]["gmres"]["method"] = ("IdealGasConstPressureMoleReactor with GMRES and the adaptive "
                                              "preconditioner (ILUT of I - gamma Jp in a minimum-degree order), FP64")
    threads = os.cpu_count()
    # the other workloads of the hot path (their own configurations), each with its errors
    # and its CPU baseline
    if not args.no_workloads and ws == 1:
        wl = {}
        for name, fn in (("h2o2_1024", lambda: variant_h2o2(dev, torch, flush, threads, fp)),
                         ("rates_gri30_2p20", lambda: variant_rates(dev, torch, flush, threads, peaks=measured_peaks())),
                         ("ndodecane_16384", lambda: variant_ndodecane(dev, torch, flush, threads, fp))):
            try:
                t0 = time.perf_counter()
                wl[name] = fn()
                wl[name]["seconds"] = time.perf_counter() - t0
            except Exception as e:
                wl[name] = {"error": "%s: %s" % (type(e).__name__, e)}
        line["workloads"] = wl
    if not args.no_cpu_baseline and ws == 1:
        idx = cpu_sample_indices(n_all, CPU_SAMPLE, WL["seed"])
        cb, (To, Yo, sto, tio) = cpu_baseline(T0, P, Y0, idx, threads)
        line["cpu_baseline"] = cb
        err = {}
        for vname, r in results.items():
            Tg, Yg = r["T"][idx], r["Y"][:, idx].T
            err[vname] = state_errors(Tg, Yg, To, Yo)
        line["error_vs_cpu_oracle"] = err
        # the error protocol: reference-configured oracle and tight run on a seeded sample
        from oracle import pyoracle as po
        m = po.Mech(os.path.join(ROOT, "cantera_gb300", "data", WL["mechanism"]), WL["phase"])
        tidx = cpu_sample_indices(n_all, TIGHT_SAMPLE, WL["seed"] + 7)
        gpu = {v: (r["T"][tidx], r["Y"][:, tidx].T, r["tign"][tidx]) for v, r in results.items()}
        extra = ({"gmres": (po.opts(rtol=WL["rtol"], atol=WL["atol"], gmres=True), ["gmres"])}
                 if "gmres" in results else None)
        line["error_protocol"] = error_protocol(m, po, T0[tidx], P[tidx], Y0[tidx], WL["t_end"], WL["rtol"],
                                                WL["atol"], gpu, threads, extra_oracles=extra)
    if not args.no_surrogate and ws == 1:
        try:
            line.setdefault("variants", {})["surrogate"] = surrogate_leg(sol, dev, torch)
        except Exception as e:   # the learned arm must not cost the FP64 line
            line.setdefault("variants", {})["surrogate"] = {"error": "%s: %s" % (type(e).__name__, e)}
    print(json.dumps(line))
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
