"""Phase-fixed Newton (the reference's bordered system [J, i psi; (i psi)^T,
0], src/bordering/ModelEvaluator_Bordered.cpp): every update is orthogonal
to the gauge direction i psi, and the solve still converges to the oracle's
solution modulo the global phase."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

G, MU = 1.0, 0.3


def _setup():
    x, c, _ = O.gen_square(17, 7)
    m = O.finish_mesh(x, c)
    A = O.mvp_constant_curl(m.x)
    P = O.Problem(m, A)
    rng = np.random.default_rng(3)
    z = (1.0 + 0.2 * (rng.standard_normal(m.N) + 1j * rng.standard_normal(m.N))) * np.exp(0.3j)
    start = np.empty(2 * m.N)
    start[0::2], start[1::2] = z.real, z.imag
    return m, A, P, start


def _gauge(psi):
    u = np.empty_like(psi)
    u[0::2], u[1::2] = -psi[1::2], psi[0::2]
    return u


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("mixed", 1e-6)])
def test_phase_fixed_update_and_solution(prec, tol):
    import nosh_gb300 as ng

    m, A, P, start = _setup()
    precision = ng.PREC_FP64 if prec == "fp64" else ng.PREC_MIXED
    model = ng.nls(ng.mesh(m.x, m.cells), A, -1.0, G, 1.0, mu=MU, precision=precision)
    # one Newton step: the update has no component along i psi0
    x1 = start.copy()
    model.newton(x1, {"g": G, "mu": MU}, max_newton=1, phase_fix=True)
    d = x1 - start
    u = _gauge(start)
    assert abs(u @ d) <= tol * np.linalg.norm(u) * np.linalg.norm(d)
    # the full solve matches the oracle's (phase-fixed) solution
    x = start.copy()
    st = model.newton(x, {"g": G, "mu": MU}, tol=1e-10, phase_fix=True)
    assert st["status"] == 0 and st["f_norm"] <= 1e-10
    ref, _ = O.newton_exact(P, start, G, MU, tol=1e-13, phase_fix=True)
    assert np.linalg.norm(P.compute_f(x, G, MU)) <= 1.5e-10
    assert np.abs(O.align_phase(x, ref) - ref).max() < 1e-8
