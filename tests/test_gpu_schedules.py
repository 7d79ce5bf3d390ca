"""Both SpMV schedules (staged row blocks and warp-cooperative rows) give the
oracle's results: F and the Jacobian and regularised-KEO applies in FP64
(1e-12 relative) and FP32 (2e-6 of the operator scale), the V-cycle stays a
fixed SPD operator, and mixed-precision Newton converges to the oracle's
state (modulo the global phase)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

MU, G = 0.3, 1.0


def _meshes():
    x, c, _ = O.gen_square(17, 7)
    sq = O.finish_mesh(x, c)
    x, c, _ = O.gen_cube(6, 11)
    cu = O.finish_mesh(x, c)
    return {"square17": sq, "cube6": cu}


MESHES = _meshes()


@pytest.fixture(scope="module", params=[(s, n) for s in ("staged", "warp") for n in sorted(MESHES)],
                ids=lambda p: f"{p[0]}-{p[1]}")
def setup(request):
    import nosh_gb300 as ng

    sched, name = request.param
    m = MESHES[name]
    A = O.mvp_constant_curl(m.x)
    P = O.Problem(m, A)
    gm = ng.mesh(m.x, m.cells)
    model = ng.nls(gm, A, scalar_potential=-1.0, g=G, thickness=1.0, mu=MU, precision=ng.PREC_FP64)
    model.set_spmv_schedule({"staged": ng.SPMV_STAGED, "warp": ng.SPMV_WARP}[sched])
    rng = np.random.default_rng(21)
    psi = np.zeros(2 * m.N)
    psi[0::2] = 1.0
    psi += 0.2 * rng.standard_normal(psi.size)
    return m, P, model, psi


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_compute_f(setup):
    m, P, model, psi = setup
    f, nrm = model.compute_f(psi, {"g": G, "mu": MU}, with_norm=True)
    ref = P.compute_f(psi, G, MU)
    assert rel(f, ref) < 1e-12
    assert abs(nrm - np.linalg.norm(ref)) < 1e-12 * np.linalg.norm(ref)


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 2e-6)])
def test_jacobian_apply(setup, prec, tol):
    m, P, model, psi = setup
    model.set_precision(prec)
    J = model.create_W_op()
    J.rebuild({"g": G, "mu": MU}, psi)
    x = np.random.default_rng(5).standard_normal(2 * m.N)
    ref = P.jac_apply(psi, G, MU, x)
    scale = np.abs(P.jac_csr_real(psi, G, MU)).sum(axis=1).max() * np.abs(x).max()
    assert np.abs(J.apply(x) - ref).max() <= tol * scale
    model.set_precision(0)


def test_regularized_operator_and_vcycle(setup):
    m, P, model, psi = setup
    Mp = model.create_W_prec()
    Mp.rebuild({"g": G, "mu": MU}, psi)
    rng = np.random.default_rng(13)
    x = rng.standard_normal(2 * m.N)
    assert rel(Mp.operator_apply(x), P.kreg_apply(psi, G, MU, x)) < 1e-12
    a, b = rng.standard_normal((2, 2 * m.N))
    Ma, Mb = Mp.apply(a), Mp.apply(b)
    assert abs(a @ Mb - b @ Ma) <= 1e-10 * abs(a @ Mb)
    assert a @ Ma > 0 and b @ Mb > 0


def test_mixed_newton_matches_oracle(setup):
    import nosh_gb300 as ng

    m, P, model, psi = setup
    start = np.zeros(2 * m.N)
    start[0::2] = 1.0
    start += 0.01 * np.random.default_rng(2).standard_normal(start.size)
    ref, _ = O.newton_exact(P, start, G, MU, tol=1e-12)
    x = start.copy()
    st = model.newton(x, {"g": G, "mu": MU}, tol=1e-10, precision=ng.PREC_MIXED)
    assert st["status"] == 0 and st["f_norm"] <= 1e-10
    assert np.linalg.norm(P.compute_f(x, G, MU)) <= 1.5e-10
    assert np.abs(O.align_phase(x, ref) - ref).max() < 1e-8
