"""The oracle's integrator against an independent one: scipy's Radau (implicit Runge-Kutta,
order 5) at tight tolerances on the oracle's own reactor right-hand side, for h2o2, GRI-Mech
3.0 and n-dodecane, igniting and non-igniting.  The oracle's BDF at rtol 1e-12 agrees with it
to the level of the tighter of the two (final T and major species); the reference's
configuration (rtol 1e-8, atol 1e-15) lies within 10 x rtol of it for h2o2 and gri30, and for
n-dodecane within what its absolute tolerance allows."""
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


@pytest.mark.parametrize("T0,P_atm,ignites", [(1500.0, 10.0, True), (1000.0, 1.0, False)])
def test_oracle_bdf_against_scipy_radau_gri30(T0, P_atm, ignites):
    """GRI-Mech 3.0, stoichiometric CH4/air to 1e-3 s: through ignition at 1,500 K and 10 atm,
    and nearly inert at 1,000 K and 1 atm.  Measured (igniting case): the tight oracle 7.6e-14
    in T and 1.7e-11 in major species, the reference's configuration 1.6e-10 and 1.4e-8."""
    from oracle import pyoracle as po
    m = oracle_mech("gri30")
    Y0 = m.equivalence_ratio(1.0, "CH4:1", "O2:1, N2:3.76")
    P, t_end = P_atm * 101325.0, 1e-3
    ref = radau(m, P, np.concatenate([[1.0, T0], Y0]), t_end)
    assert (ref[1] > T0 + 1000.0) == ignites
    major = ref[2:] > 1e-3
    for rtol, atol, bar_T, bar_Y in ((1e-12, 1e-20, 1e-10, 1e-9), (1e-8, 1e-15, 10 * 1e-8, 10 * 1e-8)):
        T, Y, st, _ = m.advance_batch(np.array([T0]), np.array([P]), Y0[None, :], t_end,
                                      po.opts(rtol=rtol, atol=atol, analytic=False, jac_reuse=True), threads=1)
        assert st[0, 8] == 0
        assert abs(T[0] - ref[1]) / ref[1] < bar_T
        assert np.max(np.abs(Y[0] - ref[2:])[major] / ref[2:][major]) < bar_Y


def test_oracle_bdf_against_scipy_radau_ndodecane():
    """nDodecane_IG (100 species), stoichiometric n-dodecane/air at 1,000 K and 20 atm through
    ignition to 1e-3 s: the tight oracle agrees with Radau to 2.7e-11 in T and 2.4e-10 in major
    species.  The reference's own configuration (rtol 1e-8, atol 1e-15) lands 1.7e-7 from it in
    T and 1.6e-6 in major species, 6.6e-8 and 6.1e-7 with atol 1e-18: on this mechanism its
    absolute tolerance, not its relative one, sets its error."""
    from oracle import pyoracle as po
    m = oracle_mech("nDodecane")
    Y0 = m.equivalence_ratio(1.0, "c12h26:1", "o2:1, n2:3.76")
    T0, P, t_end = 1000.0, 20 * 101325.0, 1e-3
    ref = radau(m, P, np.concatenate([[1.0, T0], Y0]), t_end)
    assert ref[1] > T0 + 1000.0
    major = ref[2:] > 1e-3
    for rtol, atol, bar_T, bar_Y in ((1e-12, 1e-20, 1e-10, 1e-9), (1e-8, 1e-15, 1e-6, 1e-5),
                                     (1e-8, 1e-18, 10 * 1e-8, 1e-5)):
        T, Y, st, _ = m.advance_batch(np.array([T0]), np.array([P]), Y0[None, :], t_end,
                                      po.opts(rtol=rtol, atol=atol, analytic=False, jac_reuse=True), threads=1)
        assert st[0, 8] == 0
        assert abs(T[0] - ref[1]) / ref[1] < bar_T
        assert np.max(np.abs(Y[0] - ref[2:])[major] / ref[2:][major]) < bar_Y
