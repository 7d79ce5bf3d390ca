"""Operator parity at the benchmark configurations' full sizes.

Config 1: the jittered 65 x 65 square (4,225 vertices), mu = 0.1.
Config 2: the jittered 64^3 Kuhn cube (274,625 vertices, 1,872,064 edges),
mu = 0.5.  On each, the CUDA path (through the C ABI) against the CPU oracle:

FP64 (relative to the largest reference entry, or to the operator scale for
applies): 1e-12 for the KEO and dK/dmu values, F and ||F||, dF/dmu and dF/dg,
J x, K_reg x and the fine-level Chebyshev smoothing sweep.

FP32 (mixed path), stated separately:
  * J x with the FP32 KEO values and FP32 diagonal blocks: 2e-6 of the
    operator scale max_i sum_j |J_ij| * max |x|;
  * the fine-level Chebyshev sweep (FP32 values, FP32 block inverses, FP32
    Gershgorin bound): 2e-5 of max |reference sweep|.
(The residual F and its norm are FP64 in both paths.)
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

G = 1.0
CONFIGS = {
    "square65_mu0.1": (lambda: O.gen_square(65, 1), 0.1, 30.0),
    "cube64_mu0.5": (lambda: O.gen_cube(64, 2), 0.5, 15.0),
}


@pytest.fixture(scope="module", params=sorted(CONFIGS))
def cfg(request):
    import nosh_gb300 as ng

    gen, mu, ratio = CONFIGS[request.param]
    x, c, psi0 = gen()
    m = O.finish_mesh(x, c)
    A = O.mvp_constant_curl(m.x)
    P = O.Problem(m, A)
    model = ng.nls(ng.mesh(m.x, m.cells), A, -1.0, G, 1.0, mu=mu, precision=ng.PREC_FP64)
    rng = np.random.default_rng(21)
    psi = psi0 + 0.2 * rng.standard_normal(psi0.size)
    return request.param, m, P, model, psi, mu, ratio


def _row_scale(P, mu, d0, d1b):
    """max_i sum_j |A_ij| of the real 2N x 2N operator K + diag blocks."""
    vals = P.keo_values(mu)
    rows = np.repeat(np.arange(P.m.N), np.diff(P.row_ptr))
    off = P.cols != rows
    rs = np.bincount(rows[off], weights=np.abs(vals[off]) * np.sqrt(2.0), minlength=P.m.N)
    kii = np.zeros(P.m.N)
    kii[rows[~off]] = vals[~off].real
    return float(np.max(rs + np.maximum(np.abs(kii + d0[0::2]), np.abs(kii + d0[1::2])) + np.abs(d1b)))


def test_keo_and_dkeo_values_fp64(cfg):
    name, m, P, model, psi, mu, ratio = cfg
    model.keo.set_parameters({"mu": mu})
    ref = P.keo_values(mu)
    assert np.abs(model.keo.values() - ref).max() <= 1e-12 * np.abs(ref).max()
    model.dkeo_dp.set_parameters({"mu": mu})
    ref = P.dkeo_values(mu)
    assert np.abs(model.dkeo_dp.values() - ref).max() <= 1e-12 * np.abs(ref).max()


def test_compute_f_and_dfdp_fp64(cfg):
    name, m, P, model, psi, mu, ratio = cfg
    f, nrm = model.compute_f(psi, {"g": G, "mu": mu}, with_norm=True)
    ref = P.compute_f(psi, G, mu)
    assert np.abs(f - ref).max() <= 1e-12 * np.abs(ref).max()
    assert abs(nrm - np.linalg.norm(ref)) <= 1e-12 * np.linalg.norm(ref)
    d = model.compute_dfdp(psi, {"g": G, "mu": mu})
    for k, par in ((0, "g"), (1, "mu")):
        r = P.dfdp(psi, G, mu, par)
        assert np.abs(d[k] - r).max() <= 1e-12 * np.abs(r).max()


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 2e-6)])
def test_jacobian_apply(cfg, prec, tol):
    name, m, P, model, psi, mu, ratio = cfg
    model.set_precision(prec)
    J = model.create_W_op()
    J.rebuild({"g": G, "mu": mu}, psi)
    x = np.random.default_rng(5).standard_normal(2 * m.N)
    y = J.apply(x)
    ref = P.jac_apply(psi, G, mu, x)
    d0, d1b = P.jac_diags(psi, G)
    scale = _row_scale(P, mu, d0, d1b) * np.abs(x).max()
    assert np.abs(y - ref).max() <= tol * scale
    model.set_precision(0)


def test_keo_regularized_operator_fp64(cfg):
    name, m, P, model, psi, mu, ratio = cfg
    model.set_precision(0)
    Mp = model.create_W_prec()
    Mp.rebuild({"g": G, "mu": mu}, psi)
    x = np.random.default_rng(13).standard_normal(2 * m.N)
    ref = P.kreg_apply(psi, G, mu, x)
    assert np.abs(Mp.operator_apply(x) - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 2e-5)])
def test_fine_level_chebyshev_sweep(cfg, prec, tol):
    name, m, P, model, psi, mu, ratio = cfg
    model.set_precision(prec)
    Mp = model.create_W_prec()
    Mp.rebuild({"g": G, "mu": mu}, psi)
    b = np.random.default_rng(31).standard_normal(2 * m.N)
    y = Mp.smoother_apply(b)
    ref = P.cheb_presmooth(psi, G, mu, b, degree=2, ratio=ratio)
    assert np.abs(y - ref).max() <= tol * np.abs(ref).max()
    model.set_precision(0)


def test_vcycle_is_spd_at_size(cfg):
    name, m, P, model, psi, mu, ratio = cfg
    model.set_precision(0)
    Mp = model.create_W_prec()
    Mp.rebuild({"g": G, "mu": mu}, psi)
    rng = np.random.default_rng(41)
    a, b = rng.standard_normal((2, 2 * m.N))
    Ma, Mb = Mp.apply(a), Mp.apply(b)
    # symmetric up to the V-cycle's roundoff, measured against |a| |Mb| (the
    # dot products cancel by about 1e3 at these sizes)
    assert abs(a @ Mb - b @ Ma) <= 1e-9 * np.linalg.norm(a) * np.linalg.norm(Mb)
    assert a @ Ma > 0 and b @ Mb > 0
