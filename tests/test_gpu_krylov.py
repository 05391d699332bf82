"""The Krylov path on the GPU (ReactorNet with linear_solver "GMRES": the mole reactor with GMRES
and the adaptive preconditioner) against the oracle's restatement of the same path (oracle.cpp:
MoleReactor, ilutFactor, Bdf::gmresSolve) and against the dense paths, with the bars of the
reference's own test of this solver (test/python/test_reactor.py:1696-1727: Y within 5e-4
relative / 1e-6 absolute, T within 1e-5); the ILUT factors against the oracle's."""
import ctypes

import numpy as np
import pytest

from conftest import gpu_solution, oracle_mech

pytestmark = pytest.mark.gpu

RTOL = 1e-8


def _close_factors(F, Fo, rel):
    """Factors agree entry by entry relative to the largest entry of their row."""
    scale = np.abs(Fo).max(axis=1, keepdims=True) + 1e-300
    return np.max(np.abs(F - Fo) / scale) <= rel


def test_ilut_factors_match_oracle():
    """Random sparse matrices with entries well away from the drop thresholds: the same
    pattern of kept entries and the same values to rounding, through the fill limit (a dense
    row), a zero pivot (row 0 with a zero diagonal) and a batched call."""
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    rng = np.random.default_rng(7)
    for t in range(18):
        N = [10, 33, 54, 70, 101, 130][t % 6]
        # off-diagonal row sums below the diagonal (as in I - gamma J at the steps GMRES takes),
        # so that the elimination has no growth that would amplify rounding differences
        A = rng.standard_normal((N, N)) * (rng.uniform(size=(N, N)) < 0.12)
        A *= 10.0 ** rng.uniform(-4, -1, (N, N))
        A += np.diag(rng.uniform(1, 3, N))
        if t % 3 == 0:
            r = rng.integers(1, N)
            A[r] = 0.01 * (rng.standard_normal(N) + 0.5)   # more entries than the fill limit
            A[r, r] = 2.0
        if t % 4 == 1:
            A[0, 0] = 0.0                                           # a zero pivot
        F, Fo = gb.precond_ilut(A), po.ilut(A)
        assert np.array_equal(F != 0, Fo != 0), t
        assert _close_factors(F, Fo, 1e-9 if t % 4 == 1 else 1e-12), t
    N = 54
    batch = np.stack([np.eye(N) + 0.1 * rng.standard_normal((N, N)) * (rng.uniform(size=(N, N)) < 0.2)
                      for _ in range(40)])
    Fb = gb.precond_ilut(batch)
    for i in (0, 17, 39):
        assert _close_factors(Fb[i], po.ilut(batch[i]), 1e-12)


@pytest.mark.parametrize("name", ["gri30", "nDodecane"])
def test_ilut_of_the_preconditioner_matrices(name):
    """I - gamma Jp of the mechanisms at random states: the GPU and oracle factors give the
    same incomplete LU (entries at the drop thresholds may fall either way under a different
    rounding, so the products are compared)."""
    import cantera_gb300 as gb
    m = oracle_mech(name)
    rng = np.random.default_rng(3)
    R = 6.02214076e26 * 1.380649e-23
    for gamma in (1e-7, 1e-5):
        T = rng.uniform(900, 2200)
        P = 101325.0 * 10 ** rng.uniform(0, 1.5)
        Y = rng.dirichlet(0.5 * np.ones(m.K))
        rho = P / (R * T) / np.sum(Y / m.mw)
        z = np.concatenate([[T], rho * Y / m.mw])
        J, st = m.mole_precond_jacobian(P, z)
        assert st == 0
        A = np.eye(m.K + 1) - gamma * J
        from oracle import pyoracle as po
        F, Fo = gb.precond_ilut(A), po.ilut(A)
        LU = (np.tril(F, -1) + np.eye(m.K + 1)) @ np.triu(F)
        LUo = (np.tril(Fo, -1) + np.eye(m.K + 1)) @ np.triu(Fo)
        assert np.max(np.abs(LU - LUo)) <= 1e-12 * np.max(np.abs(A))
        assert np.count_nonzero((F != 0) != (Fo != 0)) <= 0.001 * F.size


def _ignition_cases():
    m = oracle_mech("gri30")
    Y0 = m.equivalence_ratio(1.0, "CH4:1", "O2:1, N2:3.76")
    T0 = np.array([1200.0, 1150.0, 1300.0, 1450.0])
    P = np.array([101325.0, 3 * 101325.0, 101325.0, 10 * 101325.0])
    return m, T0, P, np.tile(Y0, (4, 1))


@pytest.mark.parametrize("lu", [64, 32])
def test_gmres_ignition_matches_oracle_and_direct_solvers(lu):
    """gri30 ignition at four initial states to 0.1 s: the GPU's GMRES path (FP64 or FP32
    preconditioner factors), the oracle's GMRES path, the oracle's dense mass-fraction reactor
    and the GPU's dense path agree within the reference test's bars; with FP64 factors the GPU
    takes the oracle's step and iteration counts (to the rounding of a different arithmetic
    order); the Krylov counters have the same structure (one J v product per linear
    iteration)."""
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    m, T0, P, Y0 = _ignition_cases()
    sol = gpu_solution("gri30")
    t_end, atol = 0.1, 1e-16
    net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=RTOL, atol=atol, linear_solver="GMRES", lu_precision=lu)
    assert net.advance(t_end) == 0
    Tg, Yg = net.get_state()
    Yg = Yg.T
    tg, stg, kst = net.ignition_times, net.solver_stats, net.krylov_stats
    dense = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=RTOL, atol=atol)
    assert dense.advance(t_end) == 0
    Td, Yd = dense.get_state()
    To, Yo, sto, tio = m.advance_batch(T0, P, Y0, t_end, po.opts(rtol=RTOL, atol=atol, gmres=True), threads=4)
    Tm, Ym, stm, tim = m.advance_batch(T0, P, Y0, t_end, po.opts(rtol=RTOL, atol=atol), threads=4)
    assert np.all(sto[:, 8] == 0) and np.all(stm[:, 8] == 0)
    for Tr, Yr, tr in ((To, Yo, tio), (Tm, Ym, tim), (Td, Yd.T, dense.ignition_times)):
        assert np.all(np.abs(Tg - Tr) <= 1e-5 * Tr)
        assert np.all(np.abs(Yg - Yr) <= 5e-4 * np.abs(Yr) + 1e-6)
        assert np.all(np.abs(tg - tr) <= 1e-3 * tr)
    assert np.all(tg < 0.09)
    # the same algorithm: counts within a few per cent of the oracle's (with FP32 factors the
    # preconditioner differs at the 1e-7 level, and so can the linear iterations)
    tol = 0.1 if lu == 64 else 0.2
    for i, k in ((0, "steps"), (1, "rhs_evals"), (2, "newton_iters")):
        assert np.all(np.abs(stg[k] - sto[:, i]) <= tol * sto[:, i] + 5), (k, stg[k], sto[:, i])
    lin, ps, jtv = kst["lin_iters"], kst["prec_solves"], kst["jt_vec_prod_evals"]
    # one J v product and one preconditioner solve per linear iteration (the engine keeps the
    # preconditioned vectors; the reference solves once more at the end of each GMRES call)
    assert np.all(lin > 0) and np.all(jtv == lin) and np.all(ps == lin)
    assert np.all(sto[:, 10] > sto[:, 9])
    assert np.all(np.abs(lin - sto[:, 9]) <= (0.15 if lu == 64 else 0.3) * sto[:, 9] + 10)


def test_gmres_kin1_blessed_trajectory(goldens):
    """The reference's blessed h2o2 trajectory (kinetics1 sample) through the GPU's GMRES
    path, one advance per output time, with the oracle test's tolerance."""
    import cantera_gb300 as gb
    from test_oracle_goldens import _csv_close
    g = goldens["kin1"]
    m = oracle_mech("h2o2")
    sol = gpu_solution("h2o2")
    data = np.array(g["rows"])
    Y0 = m.mole_to_mass(m.composition(g["setup"]["X"]))
    net = gb.ReactorNet(sol, np.array([1001.0]), np.array([101325.0]), Y0[:, None].copy(), rtol=1e-9,
                        atol=1e-17, linear_solver="GMRES")
    Ts, Ys = [1001.0], [Y0]
    for t in data[1:, 0]:
        assert net.advance(t) == 0
        T, Y = net.get_state()
        Ts.append(T[0])
        Ys.append(Y[:, 0])
    assert net.krylov_stats["lin_iters"][0] > 0
    T, Yt = np.array(Ts), np.array(Ys)
    X = Yt / m.mw
    X /= X.sum(axis=1, keepdims=True)
    idx = [m.species_index(n) for n in g["header"][4:]]
    R = 6.02214076e26 * 1.380649e-23
    rho = 101325.0 / (R * T) / np.sum(Yt / m.mw, axis=1)
    mine = np.column_stack([data[:, 0], T, rho, np.full_like(T, 101325.0), X[:, idx]])
    ok = _csv_close(mine, data, 5e-4, g["threshold"])
    assert ok.all(), np.argwhere(~ok)[:5]


def _ndodecane(n, seed):
    import math
    m = oracle_mech("nDodecane")
    rng = np.random.default_rng(20261203 + 3)
    N = 16384
    T0 = rng.uniform(700.0, 1400.0, N)
    P = 101325.0 * 10 ** rng.uniform(1.0, math.log10(60.0), N)
    phi = rng.uniform(0.5, 2.0, N)
    idx = np.sort(np.random.default_rng(seed).choice(N, n, replace=False))
    Y0 = np.array([m.equivalence_ratio(p, "c12h26:1", "o2:1, n2:3.76") for p in phi[idx]])
    return m, T0[idx], P[idx], Y0


@pytest.mark.parametrize("lu", [64, 32])
def test_gmres_ndodecane_against_oracle_and_dense(lu):
    """256 reactors of the n-dodecane workload to 5e-3 s at its tolerances: the GPU's GMRES path
    (FP64 or FP32 preconditioner factors) against the oracle's GMRES path and the GPU's dense
    path (the reference test's bars on the reactors not in mid-ignition at 5e-3 s, ignition
    delays within 1e-3), with the oracle's step counts."""
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    sol = gpu_solution("nDodecane")
    m, T0, P, Y0 = _ndodecane(256, 41)
    t_end, atol = 5e-3, 1e-15
    net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=RTOL, atol=atol, linear_solver="GMRES", lu_precision=lu)
    assert net.advance(t_end) == 0
    Tg, Yg = net.get_state()
    Yg = Yg.T
    dense = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=RTOL, atol=atol)
    assert dense.advance(t_end) == 0
    Td, Yd = dense.get_state()
    To, Yo, sto, tio = m.advance_batch(T0, P, Y0, t_end, po.opts(rtol=RTOL, atol=atol, gmres=True))
    assert np.all(sto[:, 8] == 0)
    # reactors in mid-ignition at t_end (T moving at up to 1e9 K/s) are compared by their
    # ignition delay; the others by the reference test's bars
    from test_gpu_workloads import settled
    ok = settled(m, P, To, Yo, t_end)
    assert ok.sum() >= 192
    for Tr, Yr in ((To, Yo), (Td, Yd.T)):
        assert np.all(np.abs(Tg - Tr)[ok] <= 1e-5 * Tr[ok])
        assert np.all((np.abs(Yg - Yr) <= 5e-4 * np.abs(Yr) + 1e-6)[ok])
    ign = (To > T0 + 400) & (tio > 0) & (tio < t_end)
    assert ign.sum() >= 20
    assert np.max(np.abs(net.ignition_times[ign] - tio[ign]) / tio[ign]) < 1e-3
    steps = net.solver_stats["steps"]
    assert abs(steps.mean() - sto[:, 0].mean()) <= 0.1 * sto[:, 0].mean()


def test_gmres_step_checkpoint_and_errors():
    """ReactorNet.step and checkpoint / restore on the GMRES path (bit-identical continuation,
    Krylov counters included); a dense network's checkpoint is refused; Krylov counters of a
    dense network and the allocation-free advance with GMRES are errors."""
    import cantera_gb300 as gb
    sol = gpu_solution("gri30")
    m, T0, P, Y0 = _ignition_cases()
    kw = dict(rtol=RTOL, atol=1e-15, linear_solver="GMRES")
    s = gb.ReactorNet(sol, T0, P, Y0.T.copy(), **kw)
    t1 = s.step()
    assert np.all(t1 > 0) and s.last_step_failures == 0
    assert np.all(s.solver_stats["steps"] == 1)
    a = gb.ReactorNet(sol, T0, P, Y0.T.copy(), **kw)
    assert a.advance(2e-3) == 0
    ck = a.checkpoint()
    assert a.advance(2e-2) == 0
    b = gb.ReactorNet(sol, T0 + 50.0, P, Y0.T.copy(), **kw)
    b.restore(ck)
    assert b.advance(2e-2) == 0
    for x, y in zip(a.get_state(), b.get_state()):
        assert np.array_equal(x, y)
    for d1, d2 in ((a.solver_stats, b.solver_stats), (a.krylov_stats, b.krylov_stats)):
        for k, v in d1.items():
            assert np.array_equal(v, d2[k]), k
    dense = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=RTOL, atol=1e-15)
    assert dense.advance(1e-3) == 0
    with pytest.raises(gb.GBError, match="other linear solver"):
        b.restore(dense.checkpoint())
    with pytest.raises(gb.GBError, match="dense linear solver"):
        dense.krylov_stats
    import torch
    L = gb.library()
    o = gb.NetOptions()
    L.gb_net_default_options(ctypes.byref(o))
    o.linear_solver = 1
    Td = torch.tensor(T0, device="cuda")
    Pd = torch.tensor(P, device="cuda")
    Ydv = torch.tensor(Y0.T.copy(), device="cuda")
    st = torch.zeros(4, dtype=torch.int32, device="cuda")
    rc = L.gb_reactors_advance_noalloc(sol._h, 4, 1e-4, gb._ptr(Td), gb._ptr(Pd), gb._ptr(Ydv), gb._ptr(st),
                                       ctypes.byref(o), None)
    assert rc == -999


def test_compat_mole_reactors_with_adaptive_preconditioner():
    """The reference's Python pattern: mole reactors, net.preconditioner =
    AdaptivePreconditioner() switches the network to GMRES (linear_solver_type, Krylov
    counters in solver_stats); mass-fraction reactors with the preconditioner are refused."""
    import cantera_gb300.compat as ct
    gas = ct.Solution("gri30.yaml")
    reactors = []
    for T in (1200.0, 1300.0):
        gas.TPX = T, ct.one_atm, "CH4:1, O2:2, N2:7.52"
        reactors.append(ct.IdealGasConstPressureMoleReactor(gas))
    net = ct.ReactorNet(reactors)
    net.preconditioner = ct.AdaptivePreconditioner()
    assert net.linear_solver_type == "GMRES"
    net.rtol, net.atol = 1e-8, 1e-16
    net.advance(0.05)
    st = net.solver_stats
    assert np.all(st["lin_iters"] > 0) and np.all(st["prec_solves"] > 0)
    assert all(r.T > 2000.0 for r in reactors)
    with pytest.raises(NotImplementedError):
        net.preconditioner.ilut_drop_tol = 1e-10
    gas.TPX = 1200.0, ct.one_atm, "CH4:1, O2:2, N2:7.52"
    bad = ct.ReactorNet([ct.IdealGasConstPressureReactor(gas)])
    bad.preconditioner = ct.AdaptivePreconditioner()
    with pytest.raises(ct.CanteraError, match="IdealGasConstPressureMoleReactor"):
        bad.advance(1e-3)
