"""A continuation run writes one state file per step; a new handle built
from the last file alone (mesh, A, psi, mu) finds that state converged."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_saved_state_restarts(tmp_path):
    import nosh_gb300 as ng
    from nosh_gb300 import io as nio
    from nosh_gb300 import stepper

    x, c, p0 = O.gen_square(17, 5)
    m = O.finish_mesh(x, c)
    A = O.mvp_constant_curl(m.x)
    start, _ = O.newton_exact(O.Problem(m, A), p0, 1.0, 0.2, tol=1e-13)
    model = ng.nls(ng.mesh(m.x, m.cells), A, -1.0, 1.0, 1.0, mu=0.2)
    run = ng.continuation(model, start, 0.2)
    saver = nio.DataSaver(m.x, m.cells, directory=str(tmp_path), A=A, observer=stepper.Observer(model))
    out = stepper.Stepper(run, method="Natural", predictor="Secant", initial_step=0.01, max_step=0.05,
                          max_steps=4, observer=saver, tol=1e-10).run()
    assert out["steps"] == 4 and len(saver.paths) == 5
    xs, cs, psi, fields, fd = nio.read_state(saver.paths[-1])
    mu = float(fd["mu"][0])
    assert mu == out["records"][-1]["mu"]
    model2 = ng.nls(ng.mesh(xs, cs), fields["A"], -1.0, 1.0, 1.0, mu=mu)
    st = model2.newton(psi, {"mu": mu}, tol=1e-10)
    assert st["status"] == 0 and st["newton_iters"] == 0 and st["f_norm0"] <= 1e-10
    xr, _ = run.state()
    np.testing.assert_array_equal(psi, xr)
