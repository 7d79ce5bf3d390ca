"""The allocation-free residual entry point (nosh_residual_norm_noalloc).

It serves callers that cannot allocate device memory themselves (a host
framework that owns the whole device pool, a plugin with a fixed budget, a
loop that must not pay cudaMalloc's implicit synchronisation): they pass every
input and output in their own device buffers, and the library keeps the
reduction's scratch in one fixed array of its own.  This test calls it through
the C ABI twice in a row, with different states, and checks F and ||F|| against
the handle-based entry point nosh_nls_compute_f_norm.  The file name sorts
last so that a run stopping at the first failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind(lib):
    fn = lib.nosh_residual_norm_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_int64] + [C.c_void_p] * 6 + [C.c_double] + [C.c_void_p] * 4
    return fn


def _split_graph(rp, ci, vals):
    """complex graph with diagonal -> off-diagonal CSR + real diagonal"""
    N = rp.size - 1
    rows = np.repeat(np.arange(N), np.diff(rp))
    diag = ci == rows
    kdiag = np.zeros(N)
    kdiag[rows[diag]] = vals[diag].real
    keep = ~diag
    counts = np.bincount(rows[keep], minlength=N)
    rp_od = np.zeros(N + 1, np.int32)
    rp_od[1:] = np.cumsum(counts)
    return rp_od, ci[keep].astype(np.int32), np.ascontiguousarray(vals[keep]), kdiag


@pytest.mark.parametrize("m", [12, 41])
def test_noalloc_residual_matches_handle_path(m):
    """m = 12: 2,197 vertices, 18 CTAs; m = 41: 74,088 vertices, 579 CTAs, so
    the finishing CTA sums the partials with its four-accumulator loop."""
    import torch

    import nosh_gb300 as ng
    from nosh_gb300 import meshgen

    fn = _bind(ng.lib())
    dev = torch.device("cuda", 0)
    x, cells, psi0 = meshgen.cube(m, 5)
    A = meshgen.mvp_constant_curl(x)
    gm = ng.mesh(x, cells)
    g, mu = 1.0, 0.37
    model = ng.nls(gm, A, -1.0, g, 1.0, mu=mu)
    model.keo.set_parameters({"mu": mu})
    rp, ci = gm.build_complex_graph()
    rp_od, ci_od, off, kdiag = _split_graph(rp, ci, model.keo.values())
    N = gm.num_vertices
    cvt = gm.control_volumes()  # thickness 1
    V = np.full(N, -1.0)

    def d(a, dtype=torch.float64):
        return torch.as_tensor(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)

    d_rp, d_ci = d(rp_od, torch.int32), d(ci_od, torch.int32)
    d_off = d(np.stack([off.real, off.imag], axis=1).ravel())
    d_kd, d_cvt, d_V = d(kdiag), d(cvt), d(V)
    d_f = torch.empty(2 * N, dtype=torch.float64, device=dev)
    d_norm = torch.empty(1, dtype=torch.float64, device=dev)
    rng = np.random.default_rng(17)
    # both states are on the device before the calls, so nothing else
    # allocates between the free-memory readings below
    states = [psi0, psi0 + 0.3 * rng.standard_normal(psi0.size)]
    d_psi = [d(p) for p in states]
    torch.cuda.synchronize()
    for call in range(2):  # two calls in a row share the scratch array
        free_before = torch.cuda.mem_get_info(dev)[0]
        rc = fn(N, d_rp.data_ptr(), d_ci.data_ptr(), d_off.data_ptr(), d_kd.data_ptr(), d_cvt.data_ptr(),
                d_V.data_ptr(), g, d_psi[call].data_ptr(), d_f.data_ptr(), d_norm.data_ptr(), None)
        assert rc == 0, ng.lib().nosh_last_error()
        torch.cuda.synchronize()
        if call == 1:
            # the first call on a device may load the library's module (and
            # with it the fixed scratch array); later calls allocate nothing
            assert torch.cuda.mem_get_info(dev)[0] == free_before
        f_ref, n_ref = model.compute_f(states[call], {"g": g, "mu": mu}, with_norm=True)
        f = d_f.cpu().numpy()
        assert np.abs(f - f_ref).max() <= 1e-12 * np.abs(f_ref).max()
        assert abs(d_norm.item() - n_ref) <= 1e-12 * n_ref


def test_noalloc_rejects_host_memory():
    import torch

    import nosh_gb300 as ng

    fn = _bind(ng.lib())
    t = torch.zeros(16, dtype=torch.float64, device="cuda")
    h = np.zeros(16)
    p = t.data_ptr()
    rc = fn(2, p, p, p, p, p, p, 1.0, h.ctypes.data, p, p, None)
    assert rc == ng.ERR_INVALID
    assert "current device" in ng.lib().nosh_last_error().decode()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch

    import nosh_gb300 as ng

    fn = _bind(ng.lib())
    t = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = t.data_ptr()
    rc = fn(8_388_609, p, p, p, p, p, p, 1.0, p, p, p, None)
    assert rc == ng.ERR_INVALID
    assert "scratch limit" in ng.lib().nosh_last_error().decode()
