"""The integrator and kinetics workloads at their stated sizes against the oracle: the
reference's ReactorNet configuration (difference-quotient Jacobian kept between setups) at
the same tolerances, the same method at rtol 1e-12 / atol 1e-20 as the tight solution,
and the engine's own algorithm (analytic Jacobian) where a tolerance-level comparison
needs the same step sequence.  Also ReactorNet.step on the GPU."""
import numpy as np
import pytest

from conftest import gpu_solution, oracle_mech, random_states

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-8, 1e-15


def ref_opts(po, rtol=RTOL, atol=ATOL):
    return po.opts(rtol=rtol, atol=atol, analytic=False, jac_reuse=True)


def tight(m, T0, P, Y0, t_end):
    """The tight solution of the bench's error protocol (rtol 1e-12, atol 1e-20; a reactor
    whose difference-quotient run stalls is re-run with the analytic Jacobian) and the mask
    of reactors that have one."""
    import bench
    from oracle import pyoracle as po
    Tt, Yt, stt, tit, _, failed = bench.tight_run(m, po, T0, P, Y0, t_end, threads=None)
    return Tt, Yt, tit, ~failed


def major_rel(Y, Yr):
    major = Yr >= 1e-3
    return np.max(np.abs(Y - Yr)[major] / Yr[major])


def settled(m, P, T, Y, t_end, rtol=RTOL):
    """Reactors not in mid-ignition at t_end (a 1e-4 relative time shift moves T by less
    than 10 x rtol)."""
    dTdt = np.array([m.reactor_rhs(P[s], np.concatenate([[1.0, T[s]], Y[s]]))[1] for s in range(len(P))])
    return np.abs(dTdt) * 1e-4 * t_end < 10 * rtol * T


def h2o2_config(n=1024):
    m = oracle_mech("h2o2")
    rng = np.random.default_rng(20261203 + 0)
    T0 = rng.uniform(1000.0, 1600.0, n)
    P = np.full(n, 101325.0)
    phi = rng.uniform(0.5, 2.0, n)
    Y0 = np.array([m.equivalence_ratio(p, "H2:1", "O2:1, N2:3.76") for p in phi])
    return T0, P, Y0


@pytest.mark.parametrize("lu", [64, 32])
def test_h2o2_all_1024_reactors(lu):
    """Plain method, small, as stated: every one of the 1,024 reactors to 1e-3 s."""
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    sol, m = gpu_solution("h2o2"), oracle_mech("h2o2")
    T0, P, Y0 = h2o2_config()
    t_end = 1e-3
    net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=RTOL, atol=ATOL, lu_precision=lu)
    assert net.advance(t_end) == 0
    T, Y = net.get_state()
    Y = Y.T
    tig = net.ignition_times
    # the engine's algorithm on the CPU: the same step sequence to rounding
    Ta, Ya, sta, _ = m.advance_batch(T0, P, Y0, t_end, po.opts(rtol=RTOL, atol=ATOL, analytic=True,
                                                                lu_fp32=(lu == 32)))
    assert np.all(sta[:, 8] == 0)
    assert np.max(np.abs(T - Ta) / Ta) < 10 * RTOL
    assert major_rel(Y, Ya) < 10 * RTOL
    # the reference's configuration and the tight solution
    To, Yo, sto, tio = m.advance_batch(T0, P, Y0, t_end, ref_opts(po))
    Tt, Yt, tit, have = tight(m, T0, P, Y0, t_end)
    assert np.all(sto[:, 8] == 0) and np.all(have)
    ign = (Tt > T0 + 400) & (tit > 0) & (tit < t_end)
    assert ign.sum() > 100
    assert np.max(np.abs(tig[ign] - tio[ign]) / tio[ign]) < 1e-3
    assert np.max(np.abs(tig[ign] - tit[ign]) / tit[ign]) < 1e-3
    gpu_T = np.max(np.abs(T - Tt) / Tt)
    ora_T = np.max(np.abs(To - Tt) / Tt)
    assert gpu_T <= max(10 * RTOL, 3 * ora_T), (gpu_T, ora_T)
    assert major_rel(Y, Yt) <= max(10 * RTOL, 3 * major_rel(Yo, Yt))


def gri30_sample(n, seed_offset=7):
    """A seeded sample of the uneven-stiffness workload (65,536 reactors, seed 20261205)."""
    m = oracle_mech("gri30")
    rng = np.random.default_rng(20261203 + 2)
    N = 65536
    T0 = rng.uniform(700.0, 1800.0, N)
    P = 101325.0 * 10 ** rng.uniform(0.0, np.log10(40.0), N)
    phi = rng.uniform(0.5, 1.5, N)
    idx = np.sort(np.random.default_rng(20261205 + seed_offset + 1000).choice(N, n, replace=False))
    Y0 = np.array([m.equivalence_ratio(p, "CH4:1", "O2:1, N2:3.76") for p in phi[idx]])
    return T0[idx], P[idx], Y0


@pytest.mark.parametrize("lu", [64, 32])
def test_gri30_uneven_sample_against_tight_run(lu):
    """256 reactors of the headline workload to 1e-2 s: the GPU's error against the tight
    solution is within 10 x rtol or within the reference configuration's own error, and
    every igniting reactor's ignition delay is within 0.1 % of the reference configuration."""
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    sol, m = gpu_solution("gri30"), oracle_mech("gri30")
    T0, P, Y0 = gri30_sample(256)
    t_end = 1e-2
    net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=RTOL, atol=ATOL, lu_precision=lu)
    assert net.advance(t_end) == 0
    T, Y = net.get_state()
    Y = Y.T
    tig = net.ignition_times
    To, Yo, sto, tio = m.advance_batch(T0, P, Y0, t_end, ref_opts(po))
    Tt, Yt, tit, have = tight(m, T0, P, Y0, t_end)
    assert np.all(sto[:, 8] == 0) and np.all(have)
    ign = (Tt > T0 + 400) & (tit > 0) & (tit < t_end)
    assert ign.sum() >= 20 and (~ign).sum() >= 20
    assert np.max(np.abs(tig[ign] - tio[ign]) / tio[ign]) < 1e-3
    ok = settled(m, P, Tt, Yt, t_end)
    assert ok.sum() >= len(T0) // 2
    for sel in (ok, np.ones(len(T0), bool)):
        gpu_T = np.max(np.abs(T - Tt)[sel] / Tt[sel])
        ora_T = np.max(np.abs(To - Tt)[sel] / Tt[sel])
        assert gpu_T <= max(10 * RTOL, 3 * ora_T), (gpu_T, ora_T)
        assert major_rel(Y[sel], Yt[sel]) <= max(10 * RTOL, 3 * major_rel(Yo[sel], Yt[sel]))


def ndodecane_config(n=16384):
    m = oracle_mech("nDodecane")
    rng = np.random.default_rng(20261203 + 3)
    T0 = rng.uniform(700.0, 1400.0, n)
    P = 101325.0 * 10 ** rng.uniform(1.0, np.log10(60.0), n)
    phi = rng.uniform(0.5, 2.0, n)
    return m, T0, P, phi


def test_ndodecane_256_reactors_to_5ms():
    """Mixed-precision Newton at its stated horizon: 256 of the 16,384 reactors to 5e-3 s,
    FP64 and FP32 Newton matrices, against the reference configuration (every reactor) and
    the tight solution (32 of them); Newton iteration counts of the two forms compared."""
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    sol = gpu_solution("nDodecane")
    m, T0a, Pa, phia = ndodecane_config()
    idx = np.sort(np.random.default_rng(31).choice(len(T0a), 256, replace=False))
    T0, P = T0a[idx], Pa[idx]
    Y0 = np.array([m.equivalence_ratio(p, "c12h26:1", "o2:1, n2:3.76") for p in phia[idx]])
    t_end = 5e-3
    out = {}
    for lu in (64, 32):
        net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=RTOL, atol=ATOL, lu_precision=lu)
        assert net.advance(t_end) == 0
        T, Y = net.get_state()
        out[lu] = (T, Y.T, net.ignition_times, net.solver_stats)
    To, Yo, sto, tio = m.advance_batch(T0, P, Y0, t_end, ref_opts(po))
    assert np.all(sto[:, 8] == 0)
    ign = (To > T0 + 400) & (tio > 0) & (tio < t_end)
    assert ign.sum() >= 20
    ok = settled(m, P, To, Yo, t_end)
    sub = np.arange(0, 256, 8)
    Tt, Yt, tit, have = tight(m, T0[sub], P[sub], Y0[sub], t_end)
    sub, Tt = sub[have], Tt[have]
    ora_T = np.max(np.abs(To[sub] - Tt) / Tt)
    for lu in (64, 32):
        T, Y, tig, st = out[lu]
        assert np.max(np.abs(tig[ign] - tio[ign]) / tio[ign]) < 1e-3, lu
        # settled reactors: the two methods agree to the tolerance level
        assert np.max(np.abs(T - To)[ok] / To[ok]) < 10 * RTOL * 3, lu
        gpu_T = np.max(np.abs(T[sub] - Tt) / Tt)
        assert gpu_T <= max(10 * RTOL, 3 * ora_T), (lu, gpu_T, ora_T)
    # the FP32 factorisation costs at most a few extra Newton iterations per step
    n64 = out[64][3]["newton_iters"].sum() / out[64][3]["steps"].sum()
    n32 = out[32][3]["newton_iters"].sum() / out[32][3]["steps"].sum()
    assert n32 < 1.5 * n64


def test_rates_and_jacobian_2p16_states():
    """Rate evaluation only: 65,536 gri30 states (T 300-3000 K, P 0.1-100 atm, Dirichlet
    compositions) - wdot to 1e-12 of the gross rates and ddCi to 1e-12 of the state's
    largest entry against the oracle, on the device-pointer path."""
    import torch
    sol, m = gpu_solution("gri30"), oracle_mech("gri30")
    n = 1 << 16
    T, P, Y = random_states(sol.n_species, n, 20261204)
    d = lambda a: torch.tensor(a, device="cuda")
    Td, Pd, Yd = d(T), d(P), d(Y)
    w = sol.net_production_rates(Td, Pd, Yd).cpu().numpy()
    wj = torch.empty((sol.n_species, n), dtype=torch.float64, device="cuda")
    J = sol.net_production_rates_ddCi(Td, Pd, Yd, wdot=wj).cpu().numpy()
    wo, Jo, gross = m.rates_batch(T, P, Y, mode=1, pattern=(sol.jac_colptr, sol.jac_rowidx), gross=True)
    assert np.all(np.abs(w - wo) <= 1e-12 * gross + 1e-300)
    assert np.array_equal(wj.cpu().numpy(), w)
    scale = np.maximum(np.max(np.abs(Jo), axis=0), 1e-300)
    assert np.all(np.max(np.abs(J - Jo), axis=0) <= 1e-12 * scale)


def test_net_step_one_internal_step():
    """ReactorNet.step: each call is one internal step of every reactor, the times grow, the
    states are the integration's at those times, and an advance afterwards continues the
    same integration."""
    import cantera_gb300 as gb
    sol, m = gpu_solution("h2o2"), oracle_mech("h2o2")
    T0, P, Y0 = h2o2_config(16)
    net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=RTOL, atol=ATOL)
    prev = np.zeros(16)
    for k in range(1, 31):
        t = net.step()
        assert net.last_step_failures == 0
        assert np.all(t > prev)
        prev = t.copy()
        assert np.all(net.solver_stats["steps"] == k)
    assert net.time == pytest.approx(t.max())
    # the states after 30 steps are those of the integration at each reactor's own time
    Ts, Ys = net.get_state()
    for s in range(0, 16, 5):
        ref = gb.ReactorNet(sol, T0[s:s + 1], P[s:s + 1], Y0[s:s + 1].T.copy(), rtol=RTOL, atol=ATOL)
        assert ref.advance(t[s]) == 0
        assert abs(ref.T[0] - Ts[s]) / Ts[s] < 10 * RTOL
    # an advance after steps continues the integration
    assert net.advance(1e-3) == 0
    full = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=RTOL, atol=ATOL)
    assert full.advance(1e-3) == 0
    assert np.max(np.abs(net.T - full.T) / full.T) < 10 * RTOL
    with pytest.raises(gb.GBError, match="backwards"):
        net.advance(5e-4)


def test_net_step_device_times_and_facade():
    """Times written to a device array, and the facade's ReactorNet.step."""
    import torch
    import cantera_gb300 as gb
    from cantera_gb300 import compat as ct
    sol = gpu_solution("h2o2")
    T0, P, Y0 = h2o2_config(4)
    net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=RTOL, atol=ATOL)
    td = torch.zeros(4, dtype=torch.float64, device="cuda")
    net.step(td)
    th = net.step()
    assert torch.all(td > 0) and np.all(th > td.cpu().numpy())
    gas = ct.Solution("h2o2.yaml", "ohmech")
    gas.TPX = 1001.0, 101325.0, "H2:2, O2:1, N2:4"
    r = ct.IdealGasConstPressureReactor(gas)
    rn = ct.ReactorNet([r])
    t1 = rn.step()
    t2 = rn.step()
    assert 0 < t1 < t2 == rn.time
    rn.advance(1e-3)
    assert r.T > 2000.0


def test_checkpoint_restore_continues_bit_for_bit():
    """A network checkpointed mid-integration and restored into a new network continues the
    same integration: bit-identical states, counters and ignition times; checkpoints of
    another network size are refused."""
    import cantera_gb300 as gb
    sol = gpu_solution("gri30")
    T0, P, Y0 = gri30_sample(40, seed_offset=11)
    a = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=RTOL, atol=ATOL)
    assert a.advance(2e-3) == 0
    ck = a.checkpoint()
    assert a.advance(1e-2) == 0
    b = gb.ReactorNet(sol, T0 + 100.0, P, Y0.T.copy(), rtol=RTOL, atol=ATOL, use_graph=True)
    b.restore(ck)
    assert b.time == 2e-3
    assert b.advance(1e-2) == 0
    Ta, Ya = a.get_state()
    Tb, Yb = b.get_state()
    assert np.array_equal(Ta, Tb) and np.array_equal(Ya, Yb)
    assert np.array_equal(a.ignition_times, b.ignition_times)
    for k, v in a.solver_stats.items():
        assert np.array_equal(v, b.solver_stats[k]), k
    c = gb.ReactorNet(sol, T0[:20], P[:20], Y0[:20].T.copy())
    with pytest.raises(gb.GBError, match="another size"):
        c.restore(ck)
    with pytest.raises(gb.GBError, match="not a reactor-network checkpoint"):
        b.restore(bytes(len(ck)))
