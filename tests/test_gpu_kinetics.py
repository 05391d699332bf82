"""GPU kinetics against the oracle: net production rates to 1e-12 of the gross rate
(sum_i |nu_ki| (|ropf_i| + |ropr_i|)), d(wdot)/dc to 1e-12 of max|J| per state (the
reference's own criterion, test/kinetics/rates.cpp:248-279)."""
import numpy as np
import pytest

from conftest import gpu_solution, oracle_mech, random_states

pytestmark = pytest.mark.gpu
WDOT_TOL = 1e-12
JAC_TOL = 1e-12


@pytest.mark.parametrize("name", ["h2o2", "gri30", "nDodecane"])
def test_net_production_rates(name):
    sol, m = gpu_solution(name), oracle_mech(name)
    T, P, Y = random_states(m.K, 3000, seed=11)
    w = sol.net_production_rates(T, P, Y)
    wo, _, gross = m.rates_batch(T, P, Y, gross=True)
    err = np.abs(w - wo)
    assert np.all(err <= WDOT_TOL * gross + 1e-300), np.max(err / (gross + 1e-300))
    # where wdot does not cancel, the plain relative error is tiny too
    big = np.abs(wo) > 1e-6 * gross
    assert np.max(err[big] / np.abs(wo[big])) < 1e-10


@pytest.mark.parametrize("name", ["h2o2", "gri30", "nDodecane"])
def test_ddci_matches_analytic_oracle(name):
    sol, m = gpu_solution(name), oracle_mech(name)
    T, P, Y = random_states(m.K, 500, seed=12)
    J = sol.net_production_rates_ddCi(T, P, Y)
    _, Jo = m.rates_batch(T, P, Y, mode=1, pattern=(sol.jac_colptr, sol.jac_rowidx))
    scale = np.max(np.abs(Jo), axis=0)
    assert np.all(np.max(np.abs(J - Jo), axis=0) <= JAC_TOL * scale)
    # against the reference's own scheme (falloff [M]-derivative by a one-sided difference)
    _, Jr = m.rates_batch(T, P, Y, mode=0, pattern=(sol.jac_colptr, sol.jac_rowidx))
    assert np.all(np.max(np.abs(J - Jr), axis=0) <= 1e-6 * scale)


def test_jacobian_pattern_holds_every_entry():
    sol, m = gpu_solution("gri30"), oracle_mech("gri30")
    T, P, Y = random_states(m.K, 20, seed=13)
    for s in range(20):
        Jd = m.ddci(T[s], P[s], Y[:, s], mode=1)
        mask = np.zeros_like(Jd, dtype=bool)
        for c in range(m.K):
            mask[sol.jac_rowidx[sol.jac_colptr[c]:sol.jac_colptr[c + 1]], c] = True
        assert not np.any((Jd != 0) & ~mask)


def test_edge_cases():
    sol, m = gpu_solution("gri30"), oracle_mech("gri30")
    # n = 0 is a no-op
    out = sol.net_production_rates(np.zeros(0), np.zeros(0), np.zeros((m.K, 0)))
    assert out.shape == (m.K, 0)
    # zeros, tiny and negative mass fractions (the stoichiometry sign rules), T at the
    # polynomial midpoint and at the ends of the data range
    rng = np.random.default_rng(5)
    n = 64
    Y = rng.dirichlet(0.3 * np.ones(m.K), n).T.copy()
    Y[rng.random(Y.shape) < 0.3] = 0.0
    Y[rng.random(Y.shape) < 0.1] *= -1e-3
    Y[rng.random(Y.shape) < 0.1] = 1e-300
    T = np.concatenate([[1000.0, 200.0, 300.0, 3500.0, 5000.0], rng.uniform(300, 3000, n - 5)])
    P = np.full(n, 101325.0)
    w = sol.net_production_rates(T, P, Y)
    wo, _, gross = m.rates_batch(T, P, Y, gross=True)
    assert np.all(np.abs(w - wo) <= WDOT_TOL * gross + 1e-300)
    J = sol.net_production_rates_ddCi(T, P, Y)
    _, Jo = m.rates_batch(T, P, Y, mode=1, pattern=(sol.jac_colptr, sol.jac_rowidx))
    assert np.all(np.max(np.abs(J - Jo), axis=0) <= JAC_TOL * np.max(np.abs(Jo), axis=0))


def test_device_pointers_match_host_path():
    torch = pytest.importorskip("torch")
    sol, m = gpu_solution("h2o2"), oracle_mech("h2o2")
    T, P, Y = random_states(m.K, 1000, seed=14)
    wh = sol.net_production_rates(T, P, Y)
    dev = torch.device("cuda:0")
    wd = sol.net_production_rates(torch.tensor(T, device=dev), torch.tensor(P, device=dev),
                                  torch.tensor(Y, device=dev))
    assert np.array_equal(wd.cpu().numpy(), wh)


def test_bad_buffer_is_an_error():
    import ctypes
    import cantera_gb300 as gb
    sol = gpu_solution("h2o2")
    T = np.full(4, 1000.0)
    Y = np.zeros((10, 4))
    out = np.zeros(40)
    L = gb.library()
    assert L.gb_kin_net_production_rates(sol._h, 4, gb._ptr(T), gb._ptr(T), gb._ptr(Y), 3, gb._ptr(out), 0) == gb.GB_ERR
    buf = ctypes.create_string_buffer(256)
    L.gb_get_error(256, buf)
    assert "too small" in buf.value.decode()


def test_engine_exp_against_library_exp():
    """The engine's table-driven exp stays within 2 ulp of CUDA's exp over the range the
    kinetics uses, and defers to it outside (|x| >= 700, inf, nan)."""
    torch = pytest.importorskip("torch")
    import cantera_gb300 as gb
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(21)
    x = np.concatenate([rng.uniform(-745, 710, 200000), rng.uniform(-5, 5, 200000),
                        np.linspace(-1e-8, 1e-8, 1001), [0.0, -0.0, 699.99, 700.0, -700.0, 709.7, -744.0,
                                                         np.inf, -np.inf, np.nan, 1e-300, -1e-300]])
    xd = torch.tensor(x, device=dev)
    a = torch.empty_like(xd)
    b = torch.empty_like(xd)
    gb._check(gb.library().gb_check_exp(len(x), gb._ptr(xd), gb._ptr(a), gb._ptr(b)))
    a, b = a.cpu().numpy(), b.cpu().numpy()
    both_nan = np.isnan(a) & np.isnan(b)
    with np.errstate(invalid="ignore"):          # inf - inf where both are inf
        assert np.all(both_nan | (a == b) | (np.abs(a - b) <= 2 * np.spacing(np.abs(b))))


def test_engine_log_against_library_log():
    """The engine's integer-pipe log: within one unit in the last place of CUDA's log where
    |ln x| > 1/256, within 2^-60 absolute near x = 1; the library log for x <= 0, subnormal,
    inf and nan."""
    torch = pytest.importorskip("torch")
    import cantera_gb300 as gb
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(22)
    x = np.concatenate([np.exp(rng.uniform(-690, 709, 200000)), rng.uniform(250, 4000, 100000),
                        1 + rng.uniform(-0.01, 0.01, 100000),
                        [1.0, 2.0, 0.5, 1e-300, 1e300, 5e-324, 0.0, -1.0, np.inf, np.nan, 101325.0]])
    xd = torch.tensor(x, device=dev)
    a = torch.empty_like(xd)
    b = torch.empty_like(xd)
    gb._check(gb.library().gb_check_log(len(x), gb._ptr(xd), gb._ptr(a), gb._ptr(b)))
    a, b = a.cpu().numpy(), b.cpu().numpy()
    both_nan = np.isnan(a) & np.isnan(b)
    fin = np.isfinite(b)
    big = fin & (np.abs(b) > 1 / 256)
    with np.errstate(invalid="ignore"):          # inf - inf and nan where the library gives them
        assert np.all(both_nan | ~fin | (a == b) | ~big | (np.abs(a - b) <= 1.01 * np.spacing(np.abs(b))))
    small = fin & ~big
    assert np.max(np.abs(a[small] - b[small])) < 2 ** -60 + np.max(np.spacing(np.abs(b[small])))
    assert np.all((a == b)[~fin] | both_nan[~fin])


@pytest.mark.parametrize("name", ["h2o2", "gri30"])
def test_state_tiles_do_not_change_results(name):
    """The kernel works on tiles of 32 consecutive states: any batch size, and any position
    of a state in its batch, gives the same bits (wdot and ddCi), also through device
    pointers."""
    import torch
    sol, m = gpu_solution(name), oracle_mech(name)
    T, P, Y = random_states(m.K, 100, seed=21)
    w = sol.net_production_rates(T, P, Y)
    J = sol.net_production_rates_ddCi(T, P, Y)
    for a, b in ((0, 1), (5, 38), (31, 64), (67, 100), (3, 35)):
        sl = slice(a, b)
        Ys = np.ascontiguousarray(Y[:, sl])
        assert np.array_equal(sol.net_production_rates(T[sl], P[sl], Ys), w[:, sl])
        assert np.array_equal(sol.net_production_rates_ddCi(T[sl], P[sl], Ys), J[:, sl])
    d = lambda x: torch.tensor(x, device="cuda")
    wd = torch.empty((m.K, 100), dtype=torch.float64, device="cuda")
    Jd = sol.net_production_rates_ddCi(d(T), d(P), d(Y), wdot=wd)
    assert np.array_equal(Jd.cpu().numpy(), J) and np.array_equal(wd.cpu().numpy(), w)
