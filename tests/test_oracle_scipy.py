"""The oracle's integrator against an independent one: scipy's Radau (implicit Runge-Kutta,
order 5) at tight tolerances on the oracle's own reactor right-hand side.  The oracle's BDF
at rtol 1e-12 agrees with it to the level of the tighter of the two (final T and major
species), and at the reference's rtol 1e-8 within 10 x rtol of the tight solution on a
non-igniting and an igniting case."""
import numpy as np
import pytest

from conftest import oracle_mech

scipy_integrate = pytest.importorskip("scipy.integrate")


def radau(m, P, y0, t_end):
    f = lambda t, y: m.reactor_rhs(P, y)
    sol = scipy_integrate.solve_ivp(f, (0.0, t_end), y0, method="Radau", rtol=1e-11,
                                    atol=np.r_[1e-12, 1e-9, np.full(m.K, 1e-20)], dense_output=False)
    assert sol.success, sol.message
    return sol.y[:, -1]


@pytest.mark.parametrize("T0,t_end", [(1001.0, 1e-3), (800.0, 2e-4)])
def test_oracle_bdf_against_scipy_radau(T0, t_end):
    from oracle import pyoracle as po
    m = oracle_mech("h2o2")
    Y0 = m.mole_to_mass(m.composition("H2:2, O2:1, N2:4"))
    P = 101325.0
    y0 = np.concatenate([[1.0, T0], Y0])
    ref = radau(m, P, y0, t_end)
    Tt, Yt, st, _ = m.advance_batch(np.array([T0]), np.array([P]), Y0[None, :], t_end,
                                    po.opts(rtol=1e-12, atol=1e-20, analytic=False, jac_reuse=True), threads=1)
    assert st[0, 8] == 0
    major = ref[2:] > 1e-3
    # measured: 1.1e-12 in T and 1.2e-11 in major species after ignition (1001 K)
    assert abs(Tt[0] - ref[1]) / ref[1] < 1e-10
    assert np.max(np.abs(Yt[0] - ref[2:])[major] / ref[2:][major]) < 1e-9
    To, Yo, so, _ = m.advance_batch(np.array([T0]), np.array([P]), Y0[None, :], t_end,
                                    po.opts(rtol=1e-8, atol=1e-15, analytic=False, jac_reuse=True), threads=1)
    # the reference's configuration: within 10 x rtol (measured 2.7e-9 in T, 3.3e-8 in major species)
    assert abs(To[0] - ref[1]) / ref[1] < 10 * 1e-8
    assert np.max(np.abs(Yo[0] - ref[2:])[major] / ref[2:][major]) < 10 * 1e-8
