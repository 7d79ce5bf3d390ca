"""The oracle's pseudo-arclength step (CPU, exact-LU-preconditioned MINRES):
the corrected point solves F = 0 at its mu, satisfies the arclength
constraint, and is the natural-continuation solution at that mu; the
gauge-projected tangent matches a central difference of converged states."""
import numpy as np
import pytest

from oracle import oracle as O

G = 1.0


@pytest.fixture(scope="module")
def branch():
    x, c, p0 = O.gen_square(9, 3)
    m = O.finish_mesh(x, c)
    P = O.Problem(m, O.mvp_constant_curl(m.x))
    psi0, _ = O.newton_exact(P, p0, G, 0.5, tol=1e-13)
    psi1, _ = O.newton_exact(P, psi0, G, 0.45, tol=1e-13)
    return P, psi0, psi1


@pytest.mark.parametrize("predictor", ["tangent", "secant"])
def test_arclength_point_is_on_the_branch(branch, predictor):
    P, psi0, psi1 = branch
    ds, theta = 0.08, 1.0
    prev = (psi1, 0.45)
    psi, mu, tm, its = O.arclength_step(P, psi0, 0.5, ds, G, prev=prev, predictor=predictor, theta=theta)
    assert np.linalg.norm(P.compute_f(psi, G, mu)) <= 1e-12 and its >= 1
    assert mu > 0.5  # continues the direction of travel (0.45 -> 0.5)
    # constraint with the same unit tangent
    n = psi.size
    if predictor == "tangent":
        tx, t = O.tangent(P, psi0, G, 0.5), 1.0
    else:
        tx, t = psi0 - O.align_phase(psi1, psi0), 0.05
    sc = 1.0 / np.sqrt(tx @ tx / n + theta**2 * t * t)
    assert tx @ (psi - psi0) * sc / n + theta**2 * t * sc * (mu - 0.5) == pytest.approx(ds, rel=1e-9)
    assert tm == pytest.approx(t * sc)
    ref, _ = O.newton_exact(P, psi0, G, mu, tol=1e-13)
    assert np.abs(O.align_phase(psi, ref) - ref).max() < 1e-9


def test_tangent_matches_finite_difference(branch):
    P, psi0, _ = branch
    h = 1e-4
    a, _ = O.newton_exact(P, psi0, G, 0.5 + h, tol=1e-14)
    b, _ = O.newton_exact(P, psi0, G, 0.5 - h, tol=1e-14)
    fd = (O.align_phase(a, psi0) - O.align_phase(b, psi0)) / (2 * h)
    t = O.tangent(P, psi0, G, 0.5)
    assert np.abs(t - fd).max() <= 1e-6 * max(np.abs(fd).max(), 1.0)
