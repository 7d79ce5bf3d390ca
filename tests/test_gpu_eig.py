"""Stability eigenvalues on the GPU (LOBPCG on the FP64 Jacobian, AMG
V-cycle preconditioner, gauge mode deflated) against the oracle's
shift-invert Lanczos on the same Jacobian; and the change of stability at
the fold of the vortex-free branch on an 8 x 8 square."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

G = 1.0


@pytest.mark.parametrize("name,mu", [("square17", 0.3), ("cube5", 0.6)])
def test_lowest_eigenvalues_match_oracle(name, mu):
    import nosh_gb300 as ng
    from nosh_gb300 import eig

    if name == "square17":
        x, c, p0 = O.gen_square(17, 5)
    else:
        x, c, p0 = O.gen_cube(5, 9)
    m = O.finish_mesh(x, c)
    A = O.mvp_constant_curl(m.x)
    P = O.Problem(m, A)
    psi, _ = O.newton_exact(P, p0, G, mu, tol=1e-13)
    model = ng.nls(ng.mesh(m.x, m.cells), A, -1.0, G, 1.0, mu=mu)
    lam, X, its = eig.lowest_eigenpairs(model, psi, {"g": G, "mu": mu}, k=4, tol=1e-9)
    ref = O.lowest_eigenvalues(P, psi, G, mu, 4)
    scale = max(1.0, np.abs(ref).max())
    assert np.abs(np.sort(lam) - ref).max() <= 1e-7 * scale, (lam, ref)
    # eigenvectors: unit, orthogonal to the gauge mode, J x = lambda x
    Xh = X.cpu().numpy()
    u = psi.copy()
    u[0::2], u[1::2] = -psi[1::2], psi[0::2]
    u /= np.linalg.norm(u)
    assert np.abs(Xh @ u).max() < 1e-8
    for v, l in zip(Xh, lam):
        assert abs(np.linalg.norm(v) - 1) < 1e-10
        assert np.linalg.norm(P.jac_apply(psi, G, mu, v) - l * v) <= 1e-7 * scale
    assert its < 500


def test_stability_changes_at_the_fold():
    # the vortex-free branch of an 8 x 8 square (97^2 vertices) turns at
    # mu ~ 0.41: stable (lowest eigenvalue > 0) before the fold, unstable on
    # the branch that comes back from it
    import nosh_gb300 as ng
    from nosh_gb300 import eig, stepper

    x, c, _ = O.gen_square(97, 5)
    m = O.finish_mesh(x * 8.0, c)
    A = O.mvp_constant_curl(m.x)
    P = O.Problem(m, A)
    model = ng.nls(ng.mesh(m.x, m.cells), A, -1.0, G, 1.0, mu=0.0)
    psi = np.zeros(2 * m.N)
    psi[0::2] = 1.0
    run = ng.continuation(model, psi, 0.0)
    states = []

    class Keep:
        def __call__(self, index, xs, mu):
            states.append((xs.copy(), mu))

        def close(self):
            pass

    stepper.Stepper(run, method="Arc Length", predictor="Tangent", initial_step=0.02, max_step=0.3, max_steps=10,
                    max_value=1.5, min_value=-0.01, observer=Keep(), tol=1e-10).run()
    mus = [mu for _, mu in states]
    top = int(np.argmax(mus))
    before = max(range(top), key=lambda i: mus[i])  # highest mu before the turn
    after = top + 1  # first state past the fold
    assert after < len(states) and mus[after] < mus[top]
    lows = []
    for i in (before, after):
        xs, mu = states[i]
        lam, _, _ = eig.lowest_eigenpairs(model, xs, {"g": G, "mu": mu}, k=2, tol=1e-8)
        ref = O.lowest_eigenvalues(P, xs, G, mu, 2)
        assert abs(lam.min() - ref.min()) <= 1e-6 * max(1.0, abs(ref).max())
        lows.append(lam.min())
    assert lows[0] > 0 > lows[1], lows
