"""GPU batched integrator against the oracle (same algorithm, analytic Jacobian) and
against the reference's blessed outputs."""
import numpy as np
import pytest

from conftest import gpu_solution, oracle_mech

pytestmark = pytest.mark.gpu


def check_species(Y, Yo, rtol):
    """Major species (Y >= 1e-3) within 10 x rtol relative.  Minor species carry the global
    error of a tolerance-controlled integration (two correct runs that round differently
    drift apart by O(100) local tolerances over an ignition): 100 x rtol relative down to
    Y = 1e-6 and 1e-12 absolute below (the absolute tolerance is 1e-15)."""
    d = np.abs(Y - Yo)
    a = np.abs(Yo)
    major = a >= 1e-3
    minor = (a >= 1e-6) & ~major
    assert np.max(d[major] / a[major]) < 10 * rtol, ("major species", np.max(d[major] / a[major]))
    assert np.max(d[minor] / a[minor], initial=0.0) < 100 * rtol, ("minor species", np.max(d[minor] / a[minor]))
    assert np.max(d[a < 1e-6], initial=0.0) < 1e-12, ("trace species", np.max(d[a < 1e-6], initial=0.0))


def h2o2_batch(n, seed):
    m = oracle_mech("h2o2")
    rng = np.random.default_rng(seed)
    T0 = rng.uniform(1000, 1600, n)
    phi = rng.uniform(0.5, 2.0, n)
    Y0 = np.array([m.equivalence_ratio(p, "H2:1", "O2:1, N2:3.76") for p in phi])
    return T0, np.full(n, 101325.0), Y0


@pytest.mark.parametrize("lu", [64, 32])
def test_h2o2_batch_matches_oracle(lu):
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    sol, m = gpu_solution("h2o2"), oracle_mech("h2o2")
    rtol, atol = 1e-8, 1e-15
    T0, P, Y0 = h2o2_batch(128, 3)
    net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=rtol, atol=atol, lu_precision=lu)
    assert net.advance(1e-3) == 0
    T, Y = net.get_state()
    To, Yo, sto, tio = m.advance_batch(T0, P, Y0, 1e-3, po.opts(rtol=rtol, atol=atol, analytic=True,
                                                                lu_fp32=(lu == 32)))
    assert np.all(sto[:, 8] == 0) and np.all(net.status == 0)
    # final T and Y within 10 x rtol, ignition within 0.1%
    assert np.max(np.abs(T - To) / To) < 10 * rtol
    check_species(Y.T, Yo, rtol)
    tig = net.ignition_times
    assert np.max(np.abs(tig - tio) / tio) < 1e-3
    st = net.solver_stats
    assert np.all(st["steps"] > 0) and np.all(st["rhs_evals"] >= st["steps"])


def test_kin1_blessed_on_gpu(goldens):
    import cantera_gb300 as gb
    g = goldens["kin1"]
    sol, m = gpu_solution("h2o2"), oracle_mech("h2o2")
    data = np.array(g["rows"])
    Y0 = m.mole_to_mass(m.composition(g["setup"]["X"]))
    net = gb.ReactorNet(sol, np.array([1001.0]), np.array([101325.0]), Y0.reshape(-1, 1).copy())
    rows = [[1001.0] + list(Y0)]
    for t in data[1:, 0]:
        assert net.advance(t) == 0
        T, Y = net.get_state()
        rows.append([T[0]] + list(Y[:, 0]))
    rows = np.array(rows)
    X = rows[:, 1:] / m.mw
    X /= X.sum(axis=1, keepdims=True)
    idx = [m.species_index(n) for n in g["header"][4:]]
    mine = np.column_stack([rows[:, 0], X[:, idx]])
    ref = np.column_stack([data[:, 1], data[:, 4:]])
    ok = np.abs(mine - ref) / (np.maximum(np.abs(mine), np.abs(ref)) + g["threshold"]) < g["tolerance"]
    assert ok.all(), np.argwhere(~ok)[:5]


def test_gri30_uneven_stiffness_matches_oracle():
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    sol, m = gpu_solution("gri30"), oracle_mech("gri30")
    rng = np.random.default_rng(20261203 + 2)
    n = 48
    T0 = rng.uniform(700, 1800, n)
    P = 101325.0 * 10 ** rng.uniform(0, np.log10(40), n)
    phi = rng.uniform(0.5, 1.5, n)
    Y0 = np.array([m.equivalence_ratio(p, "CH4:1", "O2:1, N2:3.76") for p in phi])
    rtol, atol = 1e-8, 1e-15
    net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=rtol, atol=atol)
    assert net.advance(1e-2) == 0
    T, Y = net.get_state()
    To, Yo, sto, tio = m.advance_batch(T0, P, Y0, 1e-2, po.opts(rtol=rtol, atol=atol, analytic=True))
    # reactors still igniting at t_end are compared through their ignition time: a
    # relative time shift of 1e-4 there moves T by more than 10 x rtol
    dTdt = np.array([m.reactor_rhs(P[s], np.concatenate([[1.0, To[s]], Yo[s]]))[1] for s in range(n)])
    steady = np.abs(dTdt) * 1e-4 * 1e-2 < 10 * rtol * To
    assert steady.sum() >= n // 2
    assert np.max(np.abs(T - To)[steady] / To[steady]) < 10 * rtol
    check_species(Y.T[steady], Yo[steady], rtol)
    ign = To > T0 + 400
    assert ign.any() and (~ign).any()   # the batch mixes igniting and inert reactors
    assert np.max(np.abs(net.ignition_times[ign] - tio[ign]) / tio[ign]) < 1e-3


def test_continuation_graph_and_device_state():
    import cantera_gb300 as gb
    sol = gpu_solution("h2o2")
    T0, P, Y0 = h2o2_batch(32, 4)
    a = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=1e-9)
    a.advance(1e-3)
    b = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=1e-9, use_graph=True)
    b.advance(4e-4)
    b.advance(1e-3)
    assert b.time == 1e-3
    Ta, Tb = a.T, b.T
    assert np.max(np.abs(Ta - Tb) / Ta) < 1e-6
    c = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=1e-9, use_graph=True)
    c.advance(1e-3)
    assert np.array_equal(c.T, Ta)   # the captured graph runs the same kernel


def test_failure_status_without_gpu_fault():
    """Integration failures are per-reactor status codes, never a device fault."""
    import cantera_gb300 as gb
    sol = gpu_solution("h2o2")
    T0, P, Y0 = h2o2_batch(8, 5)
    net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), max_steps=5)
    assert net.advance(1e-3) == 8
    assert np.all(net.status == 1)
    T0b = T0.copy()
    T0b[3] = np.nan
    net2 = gb.ReactorNet(sol, T0b, P, Y0.T.copy())
    assert net2.advance(1e-4) == 1
    st = net2.status
    assert st[3] == 4 and np.all(np.delete(st, 3) == 0)
    with pytest.raises(gb.GBError, match="backwards"):
        net2.advance(1e-5)


@pytest.mark.parametrize("placement", [1, 2])
def test_ndodecane_fp32_lu_against_fp64_and_oracle(placement):
    """n-dodecane (K = 100, R = 553): the FP32-LU Newton against the FP64 one and the
    oracle, with the Newton matrix in shared memory (1) or in a global slot per warp (2)."""
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    sol, m = gpu_solution("nDodecane"), oracle_mech("nDodecane")
    rng = np.random.default_rng(20261203 + 3)
    n = 12
    T0 = rng.uniform(700, 1400, n)
    P = 101325.0 * 10 ** rng.uniform(1, np.log10(60), n)
    phi = rng.uniform(0.5, 2.0, n)
    Y0 = np.array([m.equivalence_ratio(p, "c12h26:1", "o2:1, n2:3.76") for p in phi])
    rtol, atol, t_end = 1e-8, 1e-15, 1e-3
    out = {}
    for lu in (64, 32):
        net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=rtol, atol=atol, lu_precision=lu,
                            matrix_placement=placement)
        assert net.advance(t_end) == 0
        out[lu] = net.get_state() + (net.solver_stats,)
    To, Yo, sto, tio = m.advance_batch(T0, P, Y0, t_end, po.opts(rtol=rtol, atol=atol, analytic=True))
    assert np.all(sto[:, 8] == 0)
    dTdt = np.array([m.reactor_rhs(P[s], np.concatenate([[1.0, To[s]], Yo[s]]))[1] for s in range(n)])
    steady = np.abs(dTdt) * 1e-4 * t_end < 10 * rtol * To
    assert steady.sum() >= n // 3
    for lu in (64, 32):
        T, Y, st = out[lu]
        assert np.max(np.abs(T - To)[steady] / To[steady]) < 10 * rtol, lu
        check_species(Y.T[steady], Yo[steady], rtol)
    # the FP32 factorisation changes the Newton iterates, not the accepted solution
    T64, T32 = out[64][0], out[32][0]
    assert np.max(np.abs(T32 - T64)[steady] / T64[steady]) < 10 * rtol


def test_matrix_placement_is_bit_identical():
    """The Newton matrix's location (shared memory or a global slot) does not change a bit."""
    import cantera_gb300 as gb
    sol = gpu_solution("gri30")
    m = oracle_mech("gri30")
    rng = np.random.default_rng(17)
    n = 40
    T0 = rng.uniform(900, 1500, n)
    P = 101325.0 * rng.uniform(1, 20, n)
    Y0 = np.array([m.equivalence_ratio(p, "CH4:1", "O2:1, N2:3.76") for p in rng.uniform(0.6, 1.4, n)])
    res = []
    for placement in (1, 2):
        net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=1e-8, matrix_placement=placement)
        net.advance(2e-3)
        res.append(net.get_state())
    np.testing.assert_array_equal(res[0][0], res[1][0])
    np.testing.assert_array_equal(res[0][1], res[1][1])


def test_jacobian_reuse_option_matches_oracle_policy():
    """With jacobian_reuse the GPU keeps the Jacobian between setups by CVODE's policy, as
    the oracle does with jac_reuse: same tolerance-level agreement, fewer Jacobians."""
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    sol, m = gpu_solution("h2o2"), oracle_mech("h2o2")
    rtol, atol = 1e-8, 1e-15
    T0, P, Y0 = h2o2_batch(64, 13)
    net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=rtol, atol=atol, jacobian_reuse=True)
    assert net.advance(1e-3) == 0
    T, Y = net.get_state()
    To, Yo, sto, tio = m.advance_batch(T0, P, Y0, 1e-3, po.opts(rtol=rtol, atol=atol, analytic=True, jac_reuse=True))
    assert np.max(np.abs(T - To) / To) < 10 * rtol
    # a kept Jacobian lets the two Newton paths (row- vs column-pivoted LU) drift further
    check_species(Y.T, Yo, 3 * rtol)
    st = net.solver_stats
    assert np.all(st["jac_evals"] <= st["lin_setups"]) and st["jac_evals"].sum() < st["lin_setups"].sum()


def test_autotune_picks_a_measured_candidate():
    from cantera_gb300.tuning import autotune, candidates
    sol = gpu_solution("h2o2")
    T0, P, Y0 = h2o2_batch(256, 17)
    best, log = autotune(sol, T0, P, Y0.T.copy(), 1e-4, waves=1, pool=256, use_cache=False)
    assert best in list(candidates())
    assert all(a["seconds"] <= b["seconds"] for a, b in zip(log, log[1:]))
    # the pick is within the margin of the fastest time per reactor, and among those the one
    # with the most resident reactors
    pick = next(e for e in log if e["options"] == best)
    assert pick["seconds"] <= log[0]["seconds"] * 1.03
    cap = lambda e: e["shape"]["blocks"] * e["shape"]["warps_per_block"]
    assert all(cap(e) <= cap(pick) for e in log if e["seconds"] <= log[0]["seconds"] * 1.03)
    # the Krylov path is tuned the same way
    best_k, log_k = autotune(sol, T0, P, Y0.T.copy(), 1e-4, waves=1, pool=256, use_cache=False,
                             linear_solver="GMRES")
    assert best_k in list(candidates()) and len(log_k) >= 2


def test_settings_of_a_network():
    """rtol / atol / max_steps / max_time_step set on a network (ReactorNet's setters) act
    like the same values given at construction; invalid values are errors."""
    import cantera_gb300 as gb
    sol = gpu_solution("h2o2")
    T0, P, Y0 = h2o2_batch(32, 23)
    a = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=1e-7, atol=1e-14, max_time_step=1e-5)
    b = gb.ReactorNet(sol, T0, P, Y0.T.copy())
    b.rtol, b.atol, b.max_time_step = 1e-7, 1e-14, 1e-5
    assert (b.rtol, b.atol, b.max_time_step) == (1e-7, 1e-14, 1e-5)
    assert a.advance(2e-4) == 0 and b.advance(2e-4) == 0
    Ta, Ya = a.get_state()
    Tb, Yb = b.get_state()
    assert np.array_equal(Ta, Tb) and np.array_equal(Ya, Yb)
    c = gb.ReactorNet(sol, T0, P, Y0.T.copy())
    c.max_steps = 3
    assert c.advance(1e-3) > 0 and np.all(c.status == 1)
    with pytest.raises(gb.GBError):
        c.max_steps = 0
    with pytest.raises(gb.GBError):
        c.max_time_step = -1.0


def _rhs_close(d1, T, P, Y, sol, tol):
    """The interpolated first derivative against the reactor right-hand side at the same
    states: within tol of each reactor's largest rate (integration error, not a formula's)."""
    dT, dY = sol.reactor_rhs(T, P, Y)
    sT = np.maximum(np.abs(dT), 1.0)
    assert np.all(np.abs(d1[0] - dT) <= tol * sT), np.max(np.abs(d1[0] - dT) / sT)
    sY = np.maximum(np.max(np.abs(dY), axis=0), 1e-3)
    assert np.all(np.max(np.abs(d1[1:] - dY), axis=0) <= tol * sY), np.max(np.max(np.abs(d1[1:] - dY), axis=0) / sY)


def test_get_derivative_from_the_step_history():
    """ReactorNet.get_derivative: k = 0 is the state gb_net_get_state returns; k = 1 is the
    reactor right-hand side at that state to within the integration error, after an advance
    (interpolated inside the last step) and after one internal step (at the step's end); the
    order range and the not-yet-integrated state are refused."""
    import cantera_gb300 as gb
    sol = gpu_solution("h2o2")
    T0, P, Y0 = h2o2_batch(64, seed=17)
    net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=1e-10, atol=1e-16)
    with pytest.raises(gb.GBError, match="not been integrated"):
        net.get_derivative(1)
    assert net.advance(2e-4) == 0               # some of the reactors mid-ignition
    T, Y = net.get_state()
    d0 = net.get_derivative(0)
    assert np.allclose(d0[0], T, rtol=1e-14, atol=0) and np.allclose(d0[1:], Y, rtol=1e-12, atol=1e-18)
    _rhs_close(net.get_derivative(1), T, P, Y, sol, 1e-4)
    assert np.all(np.isfinite(net.get_derivative(2)))
    with pytest.raises(gb.GBError, match="0..5"):
        net.get_derivative(6)
    times = net.step()
    T, Y = net.get_state()
    assert np.all(times > 2e-4)
    _rhs_close(net.get_derivative(1), T, P, Y, sol, 1e-4)
