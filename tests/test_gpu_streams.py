"""Device arrays handed to the engine (GB_DEVICE_POINTERS) are read after the work the caller
has already queued on the default stream.  The engine runs on a non-blocking stream of its
own, so without that ordering a call can read an input that the caller's last kernels have
not written yet.  Each test queues a few tens of milliseconds of work on torch's default
stream, writes the input only after it (replacing a sentinel), calls the engine at once and
compares with the same call on host arrays.  (Without the ordering the set_state and reactor
right-hand-side tests read the sentinel; the rates call happened to order itself.)"""
import numpy as np
import pytest

from conftest import gpu_solution, random_states

pytestmark = pytest.mark.gpu


def _queue_kernels_then_write(dst, src):
    """Queue about 25 ms of kernels on the current (default) stream, then write src into dst
    with a kernel that runs after them; returns without waiting."""
    import torch
    big = torch.ones(1 << 26, device=dst.device)
    for _ in range(300):
        big.mul_(1.0000001)
    dst.copy_(src + 0.0 * big[:1].double())


def test_rates_read_inputs_after_the_default_streams_work():
    import torch
    sol = gpu_solution("gri30")
    n = 4096
    T, P, Y = random_states(sol.n_species, n, seed=3)
    ref = sol.net_production_rates(T, P, Y)
    Ts, Pd, Yd = (torch.tensor(a, device="cuda") for a in (T, P, Y))
    Td = torch.full((n,), 5000.0, dtype=torch.float64, device="cuda")     # the sentinel
    # the output allocated up front: an allocation inside the timed window could call
    # cudaMalloc, whose implicit device synchronisation would hide a missing ordering
    w = torch.empty((sol.n_species, n), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    _queue_kernels_then_write(Td, Ts)
    sol.net_production_rates(Td, Pd, Yd, out=w)
    assert np.array_equal(w.cpu().numpy(), ref)


def test_set_state_reads_inputs_after_the_default_streams_work():
    import torch
    import cantera_gb300 as gb
    sol = gpu_solution("h2o2")
    rng = np.random.default_rng(5)
    n = 256
    T0 = rng.uniform(1000.0, 1500.0, n)
    P = np.full(n, 101325.0)
    Y0 = np.array([sol.equivalence_ratio_mass_fractions(p, "H2:1", "O2:1, N2:3.76")
                   for p in rng.uniform(0.5, 2.0, n)]).T.copy()
    host = gb.ReactorNet(sol, T0, P, Y0, rtol=1e-8, atol=1e-15)
    assert host.advance(1e-4) == 0
    Th, Yh = host.get_state()
    Ts, Pd, Yd = (torch.tensor(a, device="cuda") for a in (T0, P, Y0))
    Td = torch.full((n,), 300.0, dtype=torch.float64, device="cuda")      # the sentinel
    net = gb.ReactorNet(sol, Td, Pd, Yd, rtol=1e-8, atol=1e-15)
    torch.cuda.synchronize()
    _queue_kernels_then_write(Td, Ts)
    net.set_state(Td, Pd, Yd)
    assert net.advance(1e-4) == 0
    Tg, Yg = net.get_state()
    assert np.array_equal(Tg, Th) and np.array_equal(Yg, Yh)


def test_reactor_rhs_reads_inputs_after_the_default_streams_work():
    import torch
    import cantera_gb300 as gb
    sol = gpu_solution("gri30")
    n = 2048
    T, P, Y = random_states(sol.n_species, n, seed=9, Tlo=800.0, Thi=2500.0)
    dT_ref, dY_ref = sol.reactor_rhs(T, P, Y)
    Ts, Pd, Yd = (torch.tensor(a, device="cuda") for a in (T, P, Y))
    Td = torch.full((n,), 5000.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    _queue_kernels_then_write(Td, Ts)
    dT, dY = sol.reactor_rhs(Td, Pd, Yd)
    assert np.array_equal(dT.cpu().numpy(), dT_ref) and np.array_equal(dY.cpu().numpy(), dY_ref)
