"""The oracle's mole-reactor formulation with the preconditioned Krylov linear solver (no GPU):
IdealGasConstPressureMoleReactor (state T and species moles) against the mass-fraction reactor,
the adaptive preconditioner's Jacobian elements, and GMRES-with-preconditioner integrations
against the direct solver with the bars of the reference's own test
(test/python/test_reactor.py:1696-1727: Y within 5e-4 relative / 1e-6 absolute, T within 1e-5)
and against the reference's blessed kin1 trajectory."""
import numpy as np
import pytest

from conftest import oracle_mech

R = 6.02214076e26 * 1.380649e-23


def mole_state(m, T, P, Y, V=1.0):
    rho = P / (R * T) / np.sum(Y / m.mw)
    return np.concatenate([[T], rho * V * Y / m.mw])


@pytest.mark.parametrize("name", ["h2o2", "gri30"])
def test_mole_rhs_matches_mass_fraction_rhs(name):
    """d/dt of the moles, turned into d/dt of the mass fractions (the mass is constant), and
    dT/dt agree with the mass-fraction reactor's right-hand side."""
    m = oracle_mech(name)
    rng = np.random.default_rng(2)
    for _ in range(5):
        T = rng.uniform(900, 2500)
        P = 101325.0 * 10 ** rng.uniform(-0.5, 1.5)
        Y = rng.dirichlet(0.5 * np.ones(m.K))
        z = mole_state(m, T, P, Y)
        zdot, st = m.mole_reactor_rhs(P, z)
        assert st == 0
        ydot = m.reactor_rhs(P, np.concatenate([[1.0, T], Y]))
        mass = np.sum(z[1:] * m.mw)
        dY = zdot[1:] * m.mw / mass
        assert zdot[0] == pytest.approx(ydot[1], rel=1e-12)
        assert np.max(np.abs(dY - ydot[2:])) <= 1e-12 * np.max(np.abs(ydot[2:]))
        # mass conservation of the mole form
        assert abs(np.sum(zdot[1:] * m.mw)) <= 1e-12 * np.sum(np.abs(zdot[1:] * m.mw))


def test_preconditioner_jacobian_elements():
    """Species block = the reference's ddCi, temperature column = a one-sided difference of
    the right-hand side, temperature row from the enthalpy-weighted species block."""
    m = oracle_mech("gri30")
    T, P = 1500.0, 3 * 101325.0
    Y = np.random.default_rng(4).dirichlet(0.5 * np.ones(m.K))
    z = mole_state(m, T, P, Y)
    J, st = m.mole_precond_jacobian(P, z)
    assert st == 0
    D = m.ddci(T, P, Y, mode=0)
    assert np.allclose(J[1:, 1:], D, rtol=1e-12, atol=1e-12 * np.max(np.abs(D)))
    dT = T * np.sqrt(np.finfo(float).eps)
    zp = z.copy()
    zp[0] += dT
    fp, _ = m.mole_reactor_rhs(P, zp)
    f0, _ = m.mole_reactor_rhs(P, z)
    assert np.allclose(J[:, 0], (fp - f0) / dT, rtol=1e-12, atol=0)
    # the T row is the derivative of -sum_k h_k dn_k/dt / (m cp) with d(dn_k/dt)/dn_j from
    # the species block and d(m cp)/dn_j = cp_j: check it against that formula's pieces
    cp, h, _ = m.thermo(T)
    hk, cpj = h * R * T, cp * R
    mcp = np.sum(z[1:] * cpj)
    qdot = np.sum(hk * f0[1:])
    row = (cpj * qdot - mcp * (hk @ D)) / mcp ** 2
    assert np.allclose(J[0, 1:], row, rtol=1e-10, atol=1e-10 * np.max(np.abs(row)))


def test_gmres_matches_direct_solver():
    """gri30 ignition at several initial temperatures: the mole reactor with GMRES and the
    adaptive preconditioner, the mole reactor with the dense solver and the mass-fraction
    reactor agree within the reference test's bars."""
    from oracle import pyoracle as po
    m = oracle_mech("gri30")
    Y0 = m.equivalence_ratio(1.0, "CH4:1", "O2:1, N2:3.76")
    T0 = np.array([1200.0, 1150.0, 1300.0, 1450.0])
    P = np.array([101325.0, 3 * 101325.0, 101325.0, 10 * 101325.0])
    Y = np.tile(Y0, (4, 1))
    runs = {}
    for name, o in [("mass", po.opts(rtol=1e-8, atol=1e-16)),
                    ("mole", po.opts(rtol=1e-8, atol=1e-16, mole_reactor=True)),
                    ("gmres", po.opts(rtol=1e-8, atol=1e-16, gmres=True))]:
        T, Yo, st, tig = m.advance_batch(T0, P, Y, 0.1, o, threads=4)
        assert np.all(st[:, 8] == 0), (name, st[:, 8])
        runs[name] = (T, Yo, st, tig)
    Tg, Yg, stg, tg = runs["gmres"]
    for ref in ("mass", "mole"):
        Tr, Yr, _, tr = runs[ref]
        assert np.all(np.abs(Tg - Tr) <= 1e-5 * Tr)
        assert np.all(np.abs(Yg - Yr) <= 5e-4 * np.abs(Yr) + 1e-6)
        assert np.all(tr < 0.09) and np.all(np.abs(tg - tr) <= 1e-3 * tr)   # ignition inside the run
    # the Krylov path did its work through J v products and preconditioner solves
    lin, ps, jtv = stg[:, 9], stg[:, 10], stg[:, 11]
    assert np.all(lin > 0) and np.all(jtv == lin) and np.all(ps > lin)
    assert np.all(runs["mass"][2][:, 9] == 0)


def test_gmres_kin1_blessed_trajectory(goldens):
    """The reference's blessed h2o2 trajectory (kinetics1 sample) through the mole reactor
    with GMRES and the adaptive preconditioner, with the DQ-Jacobian tolerance of the
    direct-solver oracle test.  The absolute tolerance applies to moles here: 1e-17 kmol in the
    reactor's 1 m^3 (about 0.012 kmol of gas) is the 1e-15 the blessed run put on mass fractions."""
    from oracle import pyoracle as po
    from test_oracle_goldens import _csv_close
    g = goldens["kin1"]
    m = oracle_mech("h2o2")
    data = np.array(g["rows"])
    Y0 = m.mole_to_mass(m.composition(g["setup"]["X"]))
    out, st, rc = m.trajectory(1001.0, 101325.0, Y0, data[1:, 0], po.opts(gmres=True, atol=1e-17))
    assert rc == 0 and st[9] > 0
    T = np.concatenate([[1001.0], out[:, 0]])
    Yt = np.vstack([Y0, out[:, 1:]])
    X = Yt / m.mw
    X /= X.sum(axis=1, keepdims=True)
    idx = [m.species_index(n) for n in g["header"][4:]]
    rho = 101325.0 / (R * T) / np.sum(Yt / m.mw, axis=1)
    mine = np.column_stack([data[:, 0], T, rho, np.full_like(T, 101325.0), X[:, idx]])
    ok = _csv_close(mine, data, 5e-4, g["threshold"])
    assert ok.all(), np.argwhere(~ok)[:5]


def test_gmres_needs_the_mole_reactor():
    from oracle import pyoracle as po
    m = oracle_mech("h2o2")
    o = po.opts(gmres=True)
    o.mole_reactor = 0
    Y0 = m.equivalence_ratio(1.0, "H2:1", "O2:1, N2:3.76")
    _, _, st, _ = m.advance_batch(np.array([1200.0]), np.array([101325.0]), Y0[None, :], 1e-4, o, threads=1)
    assert st[0, 8] != 0
    with pytest.raises(ValueError):
        po.opts(gmres=True, analytic=True)


def test_ilut_rules():
    """The oracle's ILUT (the adaptive preconditioner's factorisation, checked here on the CPU
    and against the GPU's in the GPU tests): a matrix with no entry near the thresholds is
    factored exactly (L U = A); a row with more entries than the fill limit p = 10 nnz / N + 1
    keeps its p largest; a zero pivot becomes sqrt(tau) times the row norm."""
    from oracle import pyoracle as po
    rng = np.random.default_rng(11)
    N = 30
    A = np.eye(N) * 4 + 0.1 * rng.standard_normal((N, N))
    F = po.ilut(A)
    L, U = np.tril(F, -1) + np.eye(N), np.triu(F)
    assert np.allclose(L @ U, A, rtol=0, atol=1e-13)
    # an arrow matrix: diagonal plus one dense last row; nnz = 2N - 1, p = 10 (2N - 1) // N + 1 = 20
    B = np.eye(N) * 2.0
    B[-1, :] = np.arange(1, N + 1, dtype=float)
    Fb = po.ilut(B)
    p = (np.count_nonzero(B) * 10) // N + 1
    kept = np.nonzero(Fb[-1, :-1])[0]
    assert len(kept) == p
    # the multipliers are B[-1, j] / 2, so the largest p are the last p columns of the L part
    assert np.array_equal(kept, np.arange(N - 1 - p, N - 1))
    # a zero pivot in row 0 (no L part): sqrt(1e-12) times the row's 2-norm
    C = np.eye(N) + 0.01 * np.ones((N, N))
    C[0, 0] = 0.0
    Fc = po.ilut(C)
    assert Fc[0, 0] == pytest.approx(1e-6 * np.linalg.norm(C[0]), rel=1e-15)


def _ilut_right_looking(P, tau=1e-12):
    """The GPU kernel's elimination order (devIlut), restated: right-looking, row k finished
    (threshold drops against its original 2-norm, fill limits, zero pivot) when step k reaches
    it, then its kept U entries update the rows below.  Row norms summed in index order and no
    fused multiply-adds, as the oracle's checker build computes."""
    N = P.shape[0]
    a = P.copy()
    fill = np.count_nonzero(a) * 10 // N + 1
    rn = np.zeros(N)
    for i in range(N):
        q = 0.0
        for v in a[i]:
            q += v * v
        rn[i] = np.sqrt(q)
    for k in range(N):
        w = a[k].copy()
        for j in range(N):
            if j != k and not (abs(w[j]) > tau * rn[k]):
                w[j] = 0.0
        for part in (np.arange(N) < k, np.arange(N) > k):
            idx = np.nonzero(part & (w != 0))[0]
            if len(idx) > fill:
                keep = set(sorted(idx, key=lambda j: (-abs(w[j]), j))[:fill])
                for j in idx:
                    if j not in keep:
                        w[j] = 0.0
        if w[k] == 0.0:
            w[k] = np.sqrt(tau) * rn[k]
        a[k] = w
        for i in range(k + 1, N):
            if a[i, k] != 0.0:
                f = a[i, k] / w[k]
                if abs(f) <= tau:
                    f = 0.0
                a[i, k] = f
                if f != 0.0:
                    for j in range(k + 1, N):
                        if w[j] != 0.0:
                            a[i, j] -= f * w[j]
    return a


def test_ilut_right_looking_order_equals_row_by_row():
    """The GPU's right-looking ILUT gives the oracle's row-by-row (IKJ) factors bit for bit:
    each row receives the same updates in the same order before it is finished.  Random sparse
    matrices with entries around the drop thresholds, rows past the fill limit, zero pivots."""
    from oracle import pyoracle as po
    rng = np.random.default_rng(3)
    for trial in range(40):
        N = int(rng.integers(2, 24))
        A = rng.standard_normal((N, N)) * (rng.uniform(size=(N, N)) < rng.uniform(0.05, 0.9))
        A *= 10.0 ** rng.uniform(-14, 2, size=(N, N))
        if trial % 3 == 0:
            A[rng.integers(N)] = rng.standard_normal(N)
        A += np.diag(rng.uniform(0.5, 2, N) * (rng.uniform(size=N) < 0.8))
        with np.errstate(all="ignore"):
            F1, F2 = po.ilut(A), _ilut_right_looking(A)
        assert np.array_equal(F1, F2, equal_nan=True), trial


def _symmetric_structure(K, cp, ri):
    """Adjacency of Jp + Jp^T over z = [T, n_1..n_K]: the species block's pattern and the
    dense T row and column (no diagonal)."""
    N = K + 1
    adj = np.zeros((N, N), dtype=bool)
    adj[0, 1:] = adj[1:, 0] = True
    for c in range(K):
        for r in ri[cp[c]:cp[c + 1]]:
            if r != c:
                adj[1 + r, 1 + c] = adj[1 + c, 1 + r] = True
    return adj


def _elimination_fill(adj, order):
    """Edges the symbolic elimination adds when the nodes are eliminated in `order`."""
    adj = adj.copy()
    alive = np.ones(len(adj), dtype=bool)
    fill = 0
    for v in order:
        nb = np.flatnonzero(alive & adj[v])
        sub = adj[np.ix_(nb, nb)]
        fill += int((~sub).sum()) - len(nb)          # missing off-diagonal pairs
        adj[np.ix_(nb, nb)] = True
        adj[nb, nb] = False
        alive[v] = False
    return fill // 2


@pytest.mark.parametrize("name", ["h2o2", "gri30", "nDodecane"])
def test_preconditioner_order_is_greedy_minimum_degree(name):
    """The Krylov path factors I - gamma Jp in a fill-reducing order that the engine and the
    oracle share.  Restated here: the pattern covers every nonzero of the numeric Jp at a
    generic state; the order eliminates, at every step, a remaining node of least degree in
    the elimination graph (ties to the lowest index); it makes no more fill than the natural
    order (for n-dodecane far less)."""
    m = oracle_mech(name)
    K, N = m.K, m.K + 1
    cp, ri = m.jac_pattern()
    assert cp[0] == 0 and cp[-1] == len(ri) and np.all(np.diff(cp) >= 0)
    # pattern soundness against the numeric preconditioner Jacobian (all species present)
    T, P = 1400.0, 5 * 101325.0
    Y = np.random.default_rng(11).dirichlet(np.ones(K))
    J, st = m.mole_precond_jacobian(P, mole_state(m, T, P, Y))
    assert st == 0
    inpat = np.zeros((K, K), dtype=bool)
    for c in range(K):
        inpat[ri[cp[c]:cp[c + 1]], c] = True
    off = (J[1:, 1:] != 0.0) & ~np.eye(K, dtype=bool)
    assert not np.any(off & ~inpat)
    # greedy minimum degree, restated
    adj0 = _symmetric_structure(K, cp, ri)
    adj = adj0.copy()
    alive = np.ones(N, dtype=bool)
    expect = []
    for _ in range(N):
        deg = np.where(alive, (adj & alive[None, :]).sum(axis=1), N + 1)
        v = int(np.argmin(deg))
        nb = np.flatnonzero(alive & adj[v])
        adj[np.ix_(nb, nb)] = True
        adj[nb, nb] = False
        alive[v] = False
        expect.append(v)
    order = m.prec_order()
    assert sorted(order.tolist()) == list(range(N))
    assert order.tolist() == expect
    f_order, f_natural = _elimination_fill(adj0, order), _elimination_fill(adj0, range(N))
    assert f_order <= f_natural
    if name == "nDodecane":
        assert f_order < 0.5 * f_natural
