"""Failure paths of the solver, made to fire on purpose on the host side or
with bounded waits (no GPU fault is involved).

The reference asserts that its preconditioner's inner solve converged
(src/keo_regularized.cpp:161) and lets NOX cap or rescue Newton
(examples/conf.xml:82,186-189).  Here each failure is a distinct status code,
and after each one the handle goes on to solve a good problem to the oracle's
residual tolerance:

* a NaN in the host state          -> NOSH_ERR_NAN
* one Newton step / one MINRES step -> NOSH_ERR_NOT_CONVERGED
* a singular regularised KEO       -> NOSH_ERR_BREAKDOWN
  (zero thickness on a patch zeroes the patch's rows of K_reg; the
  preconditioner's refresh finds the diagonal blocks that are not positive
  definite)
* a staged-SpMV wait that runs out -> NOSH_ERR_CUDA (the wait bound is set to
  0 polls, so every staged wait gives up at once and its launch leaves after
  its copies land)
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(prec):
    import nosh_gb300 as ng
    from oracle import oracle as O

    x, c, psi0 = O.gen_square(17, 3)
    m = O.finish_mesh(x, c)
    A = O.mvp_constant_curl(m.x)
    P = O.Problem(m, A)
    model = ng.nls(ng.mesh(m.x, m.cells), A, -1.0, 1.0, 1.0, mu=0.5, precision=prec)
    return model, P, psi0


def _solves_afterwards(model, P, psi0):
    psi = psi0.copy()
    st = model.newton(psi, {"g": 1.0, "mu": 0.5}, tol=1e-10)
    assert st["status"] == 0 and st["f_norm"] <= 1e-10, st
    assert np.linalg.norm(P.compute_f(psi, 1.0, 0.5)) <= 2e-10


@pytest.mark.parametrize("prec", [0, 1])
def test_nan_state_gives_err_nan(prec):
    import nosh_gb300 as ng

    model, P, psi0 = _case(prec)
    bad = psi0.copy()
    bad[7] = np.nan
    with pytest.raises(ng.NoshError) as e:
        model.newton(bad, {"g": 1.0, "mu": 0.5})
    assert e.value.code == ng.ERR_NAN
    _solves_afterwards(model, P, psi0)


@pytest.mark.parametrize("prec", [0, 1])
def test_iteration_caps_give_not_converged(prec):
    import nosh_gb300 as ng

    model, P, psi0 = _case(prec)
    psi = psi0.copy()
    st = model.newton(psi, {"g": 1.0, "mu": 0.5}, max_newton=1)
    assert st["status"] == ng.ERR_NOT_CONVERGED and st["newton_iters"] == 1
    assert st["f_norm"] > 1e-10
    psi = psi0.copy()
    st = model.newton(psi, {"g": 1.0, "mu": 0.5}, max_newton=3, max_krylov=1)
    assert st["status"] == ng.ERR_NOT_CONVERGED
    assert st["newton_iters"] == 3 and st["krylov_iters"] == 3  # one MINRES step per Newton step
    _solves_afterwards(model, P, psi0)


@pytest.mark.parametrize("prec", [0, 1])
def test_singular_preconditioner_gives_breakdown(prec):
    import nosh_gb300 as ng
    from oracle import oracle as O

    # zero thickness on the corner patch x, y < 0.3: the edge coefficients
    # alpha = covolume / length * mean thickness vanish inside it, and so
    # does the regularisation cv t g (...), so the patch's interior rows of
    # K_reg are zero.  The reference's MueLu would divide by those zero
    # diagonals and Belos would fail its Converged assertion
    # (src/keo_regularized.cpp:161).
    x, c, psi0 = O.gen_square(17, 3)
    m = O.finish_mesh(x, c)
    A = O.mvp_constant_curl(m.x)
    t = np.where((m.x[:, 0] < 0.3) & (m.x[:, 1] < 0.3), 0.0, 1.0)
    P = O.Problem(m, A, thickness=t)
    model = ng.nls(ng.mesh(m.x, m.cells), A, -1.0, 1.0, t, mu=0.5, precision=prec)
    with pytest.raises(ng.NoshError) as e:
        model.newton(psi0.copy(), {"g": 1.0, "mu": 0.5})
    assert e.value.code == ng.ERR_BREAKDOWN and "positive definite" in str(e.value)
    # the handle still evaluates the model
    f = model.compute_f(psi0, {"g": 1.0, "mu": 0.5})
    fr = P.compute_f(psi0, 1.0, 0.5)
    assert np.abs(f - fr).max() <= 1e-12 * np.abs(fr).max()


@pytest.mark.parametrize("prec", [0, 1])
def test_stage_wait_timeout_gives_err_cuda(prec):
    import nosh_gb300 as ng
    from oracle import oracle as O

    # 12^3 cube: 2,197 vertices in 18 row blocks, all staged
    x, c, psi0 = O.gen_cube(12, 5)
    m = O.finish_mesh(x, c)
    A = O.mvp_constant_curl(m.x)
    P = O.Problem(m, A)
    model = ng.nls(ng.mesh(m.x, m.cells), A, -1.0, 1.0, 1.0, mu=0.5, precision=prec)
    model.set_spmv_schedule(ng.SPMV_STAGED)
    model.set_stage_wait_limit(0)
    with pytest.raises(ng.NoshError) as e:
        model.newton(psi0.copy(), {"g": 1.0, "mu": 0.5})
    assert e.value.code == ng.ERR_CUDA and "staging copy" in str(e.value)
    # a plain operator apply reports it too
    with pytest.raises(ng.NoshError) as e:
        model.keo.apply(psi0)
    assert e.value.code == ng.ERR_CUDA
    model.set_stage_wait_limit(-1)
    f = model.compute_f(psi0, {"g": 1.0, "mu": 0.5})
    fr = P.compute_f(psi0, 1.0, 0.5)
    assert np.abs(f - fr).max() <= 1e-12 * np.abs(fr).max()
    psi = psi0.copy()
    st = model.newton(psi, {"g": 1.0, "mu": 0.5}, tol=1e-10)
    assert st["status"] == 0 and st["f_norm"] <= 1e-10, st
    assert np.linalg.norm(P.compute_f(psi, 1.0, 0.5)) <= 2e-10
