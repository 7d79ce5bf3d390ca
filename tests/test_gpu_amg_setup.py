"""The preconditioner's hierarchy does not depend on the Newton precision.

The aggregation (a one-time host setup at the first operator rebuild) tests
the strength of each connection against the FP64 regularised diagonal at the
current state.  The mixed path's rebuild writes only FP32 diagonal blocks,
so its first rebuild fills the FP64 diagonal for the setup: a mixed and an
FP64 Newton solve from the same state build the same levels, on a triangle
mesh (strength threshold 0.05, where the diagonal decides which connections
are strong) and on a tetrahedral one (every connection strong).  A handle
created after other handles have come and gone builds the same levels as
the first one did.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _levels(gen, mu, prec, warm=0):
    import nosh_gb300 as ng

    x, c, psi0 = gen()
    m = O.finish_mesh(x, c)
    A = O.mvp_constant_curl(m.x)
    # earlier handles leave freed device memory behind for the next one
    for _ in range(warm):
        other = ng.nls(ng.mesh(m.x, m.cells), A, -1.0, 1.0, 1.0, mu=mu, precision=ng.PREC_FP64)
        psi = psi0.copy()
        assert other.newton(psi, {"g": 1.0, "mu": mu}, tol=1e-10)["status"] == 0
        del other
    model = ng.nls(ng.mesh(m.x, m.cells), A, -1.0, 1.0, 1.0, mu=mu, precision=prec)
    psi = psi0.copy()
    st = model.newton(psi, {"g": 1.0, "mu": mu}, tol=1e-10)
    assert st["status"] == 0, st
    P = O.Problem(m, A)
    assert np.linalg.norm(P.compute_f(psi, 1.0, mu)) <= 2e-10
    return model.amg_levels()


@pytest.mark.parametrize("name", ["square65", "cube20"])
def test_mixed_and_fp64_newton_build_the_same_hierarchy(name):
    import nosh_gb300 as ng

    gen, mu = {"square65": (lambda: O.gen_square(65, 1), 0.1), "cube20": (lambda: O.gen_cube(20, 3), 0.5)}[name]
    ref = _levels(gen, mu, ng.PREC_FP64)
    assert len(ref[0]) >= 2
    assert _levels(gen, mu, ng.PREC_MIXED) == ref
    assert _levels(gen, mu, ng.PREC_MIXED, warm=2) == ref
