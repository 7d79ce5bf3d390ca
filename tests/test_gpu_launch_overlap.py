"""Overlapped launches (programmatic dependent launch) change no result.

The kernels of a MINRES iteration and of the V-cycle are launched so that
each may start while its predecessor finishes, and wait on the device for
the predecessor's results (nosh_nls_set_launch_overlap).  The arithmetic and
its order are the same either way, so a Newton solve, a keo_regularized
V-cycle and a continuation step give bitwise the same states and the same
iteration counts with overlap on and off, for both SpMV schedules and both
precisions, and the states pass the oracle's residual.  The schedules are
set explicitly: the autotuner decides by timing, so two handles could pick
different schedules (and summation orders) for a level.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = {
    "cube20": (lambda: O.gen_cube(20, 3), 0.5),
    "square65": (lambda: O.gen_square(65, 1), 0.1),
}


def _model(name, prec, schedule):
    import nosh_gb300 as ng

    gen, mu = CASES[name]
    x, c, psi0 = gen()
    m = O.finish_mesh(x, c)
    A = O.mvp_constant_curl(m.x)
    P = O.Problem(m, A)
    model = ng.nls(ng.mesh(m.x, m.cells), A, -1.0, 1.0, 1.0, mu=mu, precision=prec)
    model.set_spmv_schedule(schedule)
    return model, P, psi0, mu


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("schedule", [1, 2])
def test_newton_identical_with_and_without_overlap(name, prec, schedule):
    out = {}
    for overlap in (True, False):
        model, P, psi0, mu = _model(name, prec, schedule)
        model.set_launch_overlap(overlap)
        psi = psi0.copy()
        st = model.newton(psi, {"g": 1.0, "mu": mu}, tol=1e-10)
        assert st["status"] == 0, st
        out[overlap] = (psi, st["newton_iters"], st["krylov_iters"])
    (a, na, ka), (b, nb, kb) = out[True], out[False]
    assert (na, ka) == (nb, kb)
    assert np.array_equal(a, b)
    assert np.linalg.norm(P.compute_f(a, 1.0, mu)) <= 2e-10


@pytest.mark.parametrize("prec", [0, 1])
def test_vcycle_identical_with_and_without_overlap(prec):
    res = []
    for overlap in (True, False):
        model, P, psi0, mu = _model("cube20", prec, 1)
        model.set_launch_overlap(overlap)
        Mp = model.create_W_prec()
        Mp.rebuild({"g": 1.0, "mu": mu}, psi0)
        b = np.random.default_rng(3).standard_normal(psi0.size)
        res.append((Mp.apply(b), Mp.smoother_apply(b)))
    assert np.array_equal(res[0][0], res[1][0])
    assert np.array_equal(res[0][1], res[1][1])


def test_continuation_identical_with_and_without_overlap():
    import nosh_gb300 as ng

    states = {}
    for overlap in (True, False):
        model, P, psi0, mu = _model("cube20", 1, 1)
        model.set_launch_overlap(overlap)
        psi = psi0.copy()
        assert model.newton(psi, {"g": 1.0, "mu": mu}, tol=1e-10)["status"] == 0
        run = ng.continuation(model, psi, mu)
        its = []
        for k in range(1, 6):
            st = run.advance(mu + 0.01 * k, ng.PREDICT_QUADRATIC if k > 2 else ng.PREDICT_SECANT)
            assert st["status"] == 0, st
            its.append(st["krylov_iters"])
        states[overlap] = (run.state()[0], its)
    assert states[True][1] == states[False][1]
    assert np.array_equal(states[True][0], states[False][0])
    assert np.linalg.norm(P.compute_f(states[True][0], 1.0, mu + 0.05)) <= 2e-10


def test_learned_continuation_identical_with_and_without_overlap():
    # the learned path adds the inference on a second stream (every second
    # step here) and the operators built while the host waits for the
    # predictor residuals
    import nosh_gb300 as ng

    states = {}
    for overlap in (True, False):
        model, P, psi0, mu = _model("square65", 1, 1)
        model.set_launch_overlap(overlap)
        psi = psi0.copy()
        assert model.newton(psi, {"g": 1.0, "mu": mu}, tol=1e-10)["status"] == 0
        run = ng.continuation(model, psi, mu)
        run.learning(4, 5, 2e-3)
        run.inference_period(2)
        its = []
        for k in range(1, 15):
            st = run.advance(mu + 0.005 * k, ng.PREDICT_LEARNED)
            assert st["status"] == 0, st
            its.append((st["krylov_iters"], run.last_prediction()["used"]))
        states[overlap] = (run.state()[0], its)
    assert states[True][1] == states[False][1]
    assert np.array_equal(states[True][0], states[False][0])
    assert np.linalg.norm(P.compute_f(states[True][0], 1.0, mu + 0.07)) <= 2e-10
