"""Newton residuals from the kept off-diagonal sums (mixed path).

Close to convergence a Newton step's residual is evaluated as F(psi + dx) =
[off-diagonal sums of K psi, FP64] + K dx (FP32 product of the small update)
+ the per-vertex FP64 terms at psi + dx, with the bound
e = 3 (n_max + 1) 2^-24 R ||dx|| on its deviation from the FP64 evaluation.
Checked here against the oracle's FP64 residual of the returned states:
every reported ||F|| lies within its stated bound (plus the FP64 rounding of
a fresh evaluation) of the oracle's, the states converge, and the steps that
start close to convergence do take the update.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["cube20", "square65"])
def test_update_residuals_match_fp64(name):
    import nosh_gb300 as ng

    if name == "cube20":
        x, c, psi0 = O.gen_cube(20, 3)
        mu0, dmu = 0.5, 0.005
    else:
        x, c, psi0 = O.gen_square(65, 1)
        mu0, dmu = 0.1, 0.005
    m = O.finish_mesh(x, c)
    A = O.mvp_constant_curl(m.x)
    P = O.Problem(m, A)
    model = ng.nls(ng.mesh(m.x, m.cells), A, -1.0, 1.0, 1.0, mu=mu0)
    psi = psi0.copy()
    st = model.newton(psi, {"g": 1.0, "mu": mu0}, tol=1e-10)
    assert st["status"] == 0
    cont = ng.continuation(model, psi, mu0)
    mu, updates = mu0, 0
    for k in range(8):
        mu += dmu
        st = cont.advance(mu, predictor=ng.PREDICT_QUADRATIC if k >= 2 else ng.PREDICT_SECANT)
        assert st["status"] == 0 and st["f_norm"] <= 1e-10, st
        xs, _ = cont.state()
        f = np.linalg.norm(P.compute_f(xs, 1.0, mu))
        assert f <= 1e-10
        # the oracle's FP64 evaluation against the library's, within the
        # stated bound and the FP64 rounding of either evaluation
        assert abs(st["f_norm"] - f) <= st["f_norm_bound"] + 5e-14 + 1e-6 * f, (k, st, f)
        # the bound is that of the final residual (0: evaluated afresh)
        assert st["f_norm_bound"] < 1e-11, st
        assert st["f_norm_bound"] == 0.0 or st["residual_updates"] > 0, st
        updates += st["residual_updates"]
    # the quadratic steps start within 100 tol and end on an update
    assert updates >= 3


def test_fp64_path_evaluates_afresh():
    import nosh_gb300 as ng

    x, c, psi0 = O.gen_cube(12, 5)
    m = O.finish_mesh(x, c)
    A = O.mvp_constant_curl(m.x)
    model = ng.nls(ng.mesh(m.x, m.cells), A, -1.0, 1.0, 1.0, mu=0.5, precision=ng.PREC_FP64)
    psi = psi0.copy()
    st = model.newton(psi, {"g": 1.0, "mu": 0.5}, tol=1e-10)
    assert st["status"] == 0 and st["residual_updates"] == 0 and st["f_norm_bound"] == 0.0
