"""The benchmark's CPU-side arithmetic (no GPU): the error protocol of the integrator
workloads, the FLOP model behind the roofline, and the timing build of the oracle."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

DATA = os.path.join(ROOT, "cantera_gb300", "data")


def h2o2_sample(n=8):
    m = po.Mech(os.path.join(DATA, "h2o2.yaml"), "ohmech")
    rng = np.random.default_rng(7)
    T0 = rng.uniform(1000.0, 1600.0, n)
    P = np.full(n, 101325.0)
    Y0 = np.array([m.equivalence_ratio(p, "H2:1", "O2:1, N2:3.76") for p in rng.uniform(0.5, 2.0, n)])
    return m, T0, P, Y0


def test_error_protocol_fields_and_self_consistency():
    m, T0, P, Y0 = h2o2_sample()
    t_end, rtol, atol = 1e-3, 1e-8, 1e-15
    # the reference-configured oracle stands in for the GPU: its errors against the oracle
    # are zero and against the tight run equal the oracle's own
    To, Yo, _, tio = m.advance_batch(T0, P, Y0, t_end, bench.oracle_opts(po, rtol, atol), threads=2)
    e = bench.error_protocol(m, po, T0, P, Y0, t_end, rtol, atol, {"same": (To, Yo, tio)}, threads=2)
    assert e["reactors"] == len(T0) and e["oracle_failed"] == 0 and e["tight_failed"] == 0
    assert e["igniting"] > 0
    s = e["same"]
    assert s["vs_oracle"]["T_max_rel"] == 0.0 and s["vs_oracle"]["major_species_max_rel"] == 0.0
    assert s["ignition_delay_max_rel_vs_oracle"] == 0.0
    assert s["vs_tight"]["all"] == e["oracle_vs_tight"]["all"]
    assert s["T_within_3x_oracle_error"] and s["major_species_within_3x_oracle_error"]
    # the tight run is closer to the truth than rtol 1e-8: the oracle's own error is small
    assert e["oracle_vs_tight"]["all"]["T_max_rel"] < 1e-5


def test_error_protocol_flags_a_shifted_result():
    m, T0, P, Y0 = h2o2_sample(4)
    t_end, rtol, atol = 1e-3, 1e-8, 1e-15
    To, Yo, _, tio = m.advance_batch(T0, P, Y0, t_end, bench.oracle_opts(po, rtol, atol), threads=2)
    e = bench.error_protocol(m, po, T0, P, Y0, t_end, rtol, atol, {"off": (To * (1 + 1e-4), Yo, tio * 1.01)}, threads=2)
    assert not e["off"]["T_within_bar"] and not e["off"]["T_within_3x_oracle_error"]
    assert e["off"]["ignition_delay_max_rel_vs_oracle"] > 9e-3 and not e["off"]["ignition_within_1e-3"]


def test_error_protocol_extra_oracle_configuration():
    """A further oracle configuration (the Krylov path): its own error against the tight run,
    and for the listed variant the comparison with it - zero when the variant is that
    configuration's own result."""
    m, T0, P, Y0 = h2o2_sample(4)
    t_end, rtol, atol = 1e-3, 1e-8, 1e-15
    og = po.opts(rtol=rtol, atol=atol, gmres=True)
    Tg, Yg, stg, tig = m.advance_batch(T0, P, Y0, t_end, og, threads=2)
    assert np.all(stg[:, 8] == 0)
    e = bench.error_protocol(m, po, T0, P, Y0, t_end, rtol, atol, {"kry": (Tg, Yg, tig)}, threads=2,
                             extra_oracles={"gmres": (og, ["kry"])})
    ex = e["oracle_gmres"]
    assert ex["failed"] == 0 and ex["vs_tight"]["all"] == e["kry"]["vs_tight"]["all"]
    assert e["kry"]["T_error_ratio_to_oracle_gmres"] == 1.0 and e["kry"]["T_within_3x_oracle_gmres"]
    assert e["kry"]["vs_oracle_gmres"]["T_max_rel"] == 0.0
    assert e["kry"]["ignition_delay_max_rel_vs_oracle_gmres"] == 0.0


def test_flop_model_and_roofline_arithmetic():
    st = {"K": 53, "R": 325, "reversible": 309, "falloff": 29, "troe": 26, "three_body": 41,
          "tb_entries": 300, "gather_entries": 1500, "jac_col_entries": 2000, "jac_scatter_entries": 3000}
    fm = bench.flop_model(st, 54)
    assert fm["rates"] < fm["rhs"] and fm["ddci"] > 0
    assert abs(fm["lu"] - (2.0 / 3.0) * 54 ** 3 - 54 * 8.0) < 1e-9
    n = 10
    stats = {"rhs_evals": np.full(n, 100), "lin_setups": np.full(n, 10), "newton_iters": np.full(n, 90),
             "steps": np.full(n, 80)}
    f64, f32 = bench.algorithmic_flops(stats, fm, False)
    expect = n * (100 * fm["rhs"] + 10 * (fm["jac"] + fm["lu"]) + 90 * fm["newton"] + 80 * fm["step"])
    assert abs(f64 - expect) <= 1e-9 * expect and f32 == 0.0
    f64b, f32b = bench.algorithmic_flops(stats, fm, True)
    assert abs(f64b + f32b - f64) <= 1e-9 * f64 and f32b > 0
    # the roofline of one launch: FP64 model FLOPs over the launch time against the measured
    # rate; with the FP32 matrix the model's time adds the FP32 part at the nominal FP32 rate
    fp = {"gflops": 1250.0}
    r = bench.integrator_roofline(f64, f32, n, False, 2.0, fp, 152)
    assert abs(r["achieved"] - f64 / 2e-3 / 1e12) <= 1e-12 * r["achieved"]
    assert abs(r["frac"] - r["achieved"] / 1.25) <= 1e-12 and r["unit"] == "TFLOP/s"
    assert abs(r["ceiling_reactors_per_s"] - 1.25e12 / (f64 / n)) <= 1e-9 * r["ceiling_reactors_per_s"]
    r32 = bench.integrator_roofline(f64b, f32b, n, True, 2.0, fp, 152)
    peak32 = 152 * 128 * 2 * 2.07e9
    t_model = f64b / 1.25e12 + f32b / peak32
    assert abs(r32["model_time_frac"] - t_model / 2e-3) <= 1e-12 * r32["model_time_frac"]
    assert abs(r32["ceiling_reactors_per_s"] - n / t_model) <= 1e-9 * r32["ceiling_reactors_per_s"]
    assert r32["frac"] < r["frac"]          # the FP64 part alone is smaller


def test_timing_build_agrees_with_checker():
    """The timing build (-O3, default contraction) computes the same rates as the checker
    to rounding level, so its time is the time of the same work."""
    m = po.Mech(os.path.join(DATA, "gri30.yaml"), "gri30")
    mf = po.Mech(os.path.join(DATA, "gri30.yaml"), "gri30", fast=True)
    assert mf.L is not m.L
    rng = np.random.default_rng(3)
    n = 64
    T = rng.uniform(300, 3000, n)
    P = 101325.0 * 10 ** rng.uniform(-1, 2, n)
    Y = rng.dirichlet(0.5 * np.ones(m.K), n).T.copy()
    w, _, gross = m.rates_batch(T, P, Y, mode=0, threads=2, gross=True)
    wf, _ = mf.rates_batch(T, P, Y, mode=0, threads=2)
    assert np.all(np.abs(w - wf) <= 1e-12 * gross + 1e-300)


def test_tight_run_recovers_a_stalled_reactor():
    """At rtol 1e-12 / atol 1e-20 the difference-quotient Jacobian stalls on this n-dodecane
    reactor at the 1000 K midpoint of the NASA7 fits (step size too small); the protocol re-runs
    it with the analytic Jacobian, which reaches the same ignited state as a looser tight
    setting."""
    m = po.Mech(os.path.join(DATA, "nDodecane_Reitz.yaml"), "nDodecane_IG")
    T0 = np.array([977.6852944187974])
    P = np.array([2396051.8658179706])
    Y0 = m.equivalence_ratio(0.9402945673491254, "c12h26:1", "o2:1, n2:3.76")[None, :]
    _, _, st, _ = m.advance_batch(T0, P, Y0, 5e-3, bench.oracle_opts(po, 0, 0, tight=True), threads=1)
    assert st[0, 8] == 5
    Tt, Yt, stt, tit, rerun, failed = bench.tight_run(m, po, T0, P, Y0, 5e-3, threads=1)
    assert rerun == 1 and not failed.any()
    To, _, _, _ = m.advance_batch(T0, P, Y0, 5e-3, po.opts(rtol=1e-11, atol=1e-18), threads=1)
    assert abs(Tt[0] - To[0]) / To[0] < 1e-10 and Tt[0] > 2600.0
