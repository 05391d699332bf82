"""Allocation-free advance (gb_reactors_advance_noalloc) against the allocating reactor
network entry points, through the C ABI.

Collected last (file name) so that it also runs after every other GPU test in the same
process; it passes alone too.
"""
import ctypes

import numpy as np
import pytest

from conftest import gpu_solution

pytestmark = pytest.mark.gpu


def _errmsg(L):
    buf = ctypes.create_string_buffer(512)
    L.gb_get_error(512, buf)
    return buf.value.decode()


def _workload(sol, n, seed):
    rng = np.random.default_rng(seed)
    T0 = rng.uniform(1000.0, 1400.0, n)
    P = 101325.0 * rng.uniform(1.0, 10.0, n)
    Y0 = np.array([sol.equivalence_ratio_mass_fractions(phi, "H2:1", "O2:1, N2:3.76")
                   for phi in rng.uniform(0.6, 1.4, n)]).T.copy()   # [K, n]
    return T0, P, Y0


def _reference(gb, sol, T0, P, Y0, t_end, opts):
    """The allocating path: gb_net_new / set_state / advance / get_state / get_status, with
    a new Jacobian at every setup as the allocation-free call does."""
    net = gb.ReactorNet(sol, T0, P, Y0, jacobian_reuse=False, **opts)
    net.advance(t_end)
    T, Y = net.get_state()
    return T, Y, net.status


def _noalloc(gb, sol, T0, P, Y0, t_end, opts):
    import torch
    L = gb.library()
    dev = torch.device("cuda:0")
    T = torch.tensor(T0, dtype=torch.float64, device=dev)
    Pd = torch.tensor(P, dtype=torch.float64, device=dev)
    Y = torch.tensor(Y0, dtype=torch.float64, device=dev).contiguous()
    st = torch.full((T0.shape[0],), -1, dtype=torch.int32, device=dev)
    o = gb.NetOptions()
    L.gb_net_default_options(ctypes.byref(o))
    for k, v in opts.items():
        setattr(o, k, v)
    torch.cuda.synchronize()
    rc = L.gb_reactors_advance_noalloc(sol._h, T0.shape[0], t_end, ctypes.c_void_p(T.data_ptr()),
                                       ctypes.c_void_p(Pd.data_ptr()), ctypes.c_void_p(Y.data_ptr()),
                                       ctypes.c_void_p(st.data_ptr()), ctypes.byref(o), None)
    assert rc == 0, _errmsg(L)
    return T.cpu().numpy(), Y.cpu().numpy(), st.cpu().numpy()


@pytest.mark.parametrize("lu", [64, 32])
def test_noalloc_matches_network_two_calls(lu):
    import cantera_gb300 as gb
    sol = gpu_solution("h2o2")
    opts = dict(rtol=1e-9, atol=1e-15, lu_precision=lu)
    T0, P, Y0 = _workload(sol, 300, 7)
    t_end = 1e-3
    Tr, Yr, sr = _reference(gb, sol, T0, P, Y0, t_end, opts)
    assert (sr == 0).all()
    # two calls in a row on the same shared scratch: the second must not see the first
    for _ in range(2):
        Tn, Yn, sn = _noalloc(gb, sol, T0, P, Y0, t_end, opts)
        np.testing.assert_array_equal(sn, sr)
        np.testing.assert_array_equal(Tn, Tr)      # same kernel, same arithmetic: bit-exact
        np.testing.assert_array_equal(Yn, Yr)
    # a different, smaller batch right after
    Tr2, Yr2, _ = _reference(gb, sol, T0[:37], P[:37], Y0[:, :37].copy(), 2e-4, opts)
    Tn2, Yn2, _ = _noalloc(gb, sol, T0[:37], P[:37], Y0[:, :37].copy(), 2e-4, opts)
    np.testing.assert_array_equal(Tn2, Tr2)
    np.testing.assert_array_equal(Yn2, Yr2)


def test_noalloc_gri30_matches_network():
    import cantera_gb300 as gb
    sol = gpu_solution("gri30")
    rng = np.random.default_rng(11)
    n = 64
    T0 = rng.uniform(1000.0, 1500.0, n)
    P = 101325.0 * rng.uniform(1.0, 20.0, n)
    Y0 = np.array([sol.equivalence_ratio_mass_fractions(phi, "CH4:1", "O2:1, N2:3.76")
                   for phi in rng.uniform(0.6, 1.4, n)]).T.copy()
    opts = dict(rtol=1e-8, atol=1e-15)
    Tr, Yr, sr = _reference(gb, sol, T0, P, Y0, 1e-3, opts)
    for _ in range(2):
        Tn, Yn, sn = _noalloc(gb, sol, T0, P, Y0, 1e-3, opts)
        np.testing.assert_array_equal(sn, sr)
        np.testing.assert_array_equal(Tn, Tr)
        np.testing.assert_array_equal(Yn, Yr)


def test_noalloc_rejects_oversize_and_host_pointers():
    import torch
    import cantera_gb300 as gb
    L = gb.library()
    sol = gpu_solution("gri30")
    dev = torch.device("cuda:0")
    T = torch.ones(4, dtype=torch.float64, device=dev)
    Y = torch.ones(4 * sol.n_species, dtype=torch.float64, device=dev)
    st = torch.zeros(4, dtype=torch.int32, device=dev)
    d = lambda t: ctypes.c_void_p(t.data_ptr())
    # checked before anything touches the buffers
    rc = L.gb_reactors_advance_noalloc(sol._h, 1 << 20, 1e-3, d(T), d(T), d(Y), d(st), None, None)
    assert rc == -999
    msg = _errmsg(L)
    assert "exceeds the maximum" in msg and "16 MiB" in msg
    h = np.ones(4)
    rc = L.gb_reactors_advance_noalloc(sol._h, 4, 1e-3, h.ctypes.data_as(ctypes.c_void_p), d(T),
                                       d(Y), d(st), None, None)
    assert rc == -999 and "device pointer" in _errmsg(L)


def test_noalloc_clamps_block_size_and_refuses_capture():
    """More than 8 reactors per block are clamped to the kernel's limit, as the network
    path does; a call on a stream that is being captured is refused with an error (the call
    synchronises its stream), and the stream stays usable."""
    import torch
    import cantera_gb300 as gb
    L = gb.library()
    sol = gpu_solution("h2o2")
    T0, P, Y0 = _workload(sol, 40, 5)
    opts = dict(rtol=1e-9, atol=1e-15, warps_per_block=16)
    Tr, Yr, sr = _reference(gb, sol, T0, P, Y0, 2e-4, dict(opts, warps_per_block=8))
    Tn, Yn, sn = _noalloc(gb, sol, T0, P, Y0, 2e-4, opts)
    np.testing.assert_array_equal(sn, sr)
    np.testing.assert_array_equal(Tn, Tr)
    np.testing.assert_array_equal(Yn, Yr)
    dev = torch.device("cuda:0")
    T = torch.tensor(T0, device=dev)
    Pd = torch.tensor(P, device=dev)
    Y = torch.tensor(Y0, device=dev).contiguous()
    st = torch.zeros(40, dtype=torch.int32, device=dev)
    d = lambda t: ctypes.c_void_p(t.data_ptr())
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        rc = L.gb_reactors_advance_noalloc(sol._h, 40, 2e-4, d(T), d(Pd), d(Y), d(st), None,
                                           ctypes.c_void_p(s.cuda_stream))
        T.add_(0.0)   # a captured node, so that the graph is not empty
    assert rc == -999 and "captured" in _errmsg(L)
    torch.cuda.synchronize()
    Tn2, _, sn2 = _noalloc(gb, sol, T0, P, Y0, 2e-4, opts)
    np.testing.assert_array_equal(Tn2, Tr)
