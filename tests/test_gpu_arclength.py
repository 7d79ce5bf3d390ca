"""Pseudo-arclength continuation on the GPU against the oracle's
restatement: from the same two converged states, one arclength step with
the tangent or the secant predictor reaches the oracle's (psi, mu) (modulo
the global phase), from FP64 and mixed-precision handles (the arclength
solves run in FP64 in both); the natural tangent predictor; a stepper run
with the adaptive step size and the observer's statistics file; and an
arclength run around the fold of the vortex-free branch on an 8 x 8 square."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

G = 1.0
MU0, MU1 = 0.45, 0.5


def _problem(name):
    if name == "square17":
        x, c, p0 = O.gen_square(17, 5)
    else:
        x, c, p0 = O.gen_cube(5, 9)
    m = O.finish_mesh(x, c)
    return m, O.Problem(m, O.mvp_constant_curl(m.x)), p0


@pytest.mark.parametrize("name", ["square17", "cube5"])
@pytest.mark.parametrize("predictor", ["tangent", "secant"])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_arclength_step_matches_oracle(name, predictor, prec):
    import nosh_gb300 as ng

    m, P, p0 = _problem(name)
    start, _ = O.newton_exact(P, p0, G, MU0, tol=1e-13)
    precision = ng.PREC_FP64 if prec == "fp64" else ng.PREC_MIXED
    model = ng.nls(ng.mesh(m.x, m.cells), O.mvp_constant_curl(m.x), -1.0, G, 1.0, mu=MU0, precision=precision)
    run = ng.continuation(model, start, MU0)
    st = run.advance(MU1, ng.PREDICT_SECANT, tol=1e-12 if prec == "fp64" else 1e-10)
    assert st["status"] == 0
    psi0, mu0 = run.state()
    assert mu0 == MU1
    ds, theta = 0.08, 1.0
    pred = ng.PREDICT_TANGENT if predictor == "tangent" else ng.PREDICT_SECANT
    st = run.advance_arclength(ds, pred, theta=theta, tol=1e-10)
    assert st["status"] == 0 and st["f_norm"] <= 1e-10 and st["newton_iters"] >= 1
    psi, mu = run.state()
    assert mu == st["mu"] and mu > MU1
    ref, mu_ref, tm_ref, _ = O.arclength_step(P, psi0, mu0, ds, G, prev=(start, MU0), predictor=predictor,
                                              theta=theta, tol=1e-13)
    tm, th = run.tangent()
    assert th == theta
    # the tangent solve runs at 1e-10 (FP64) or 1e-5 (FP32) relative tolerance
    tol_mu, tol_tm = (1e-8, 1e-7) if prec == "fp64" else (2e-5, 1e-4)
    assert abs(mu - mu_ref) <= tol_mu and abs(tm - tm_ref) <= tol_tm * abs(tm_ref)
    assert np.linalg.norm(P.compute_f(psi, G, mu)) <= 1.5e-10
    # on the branch: the natural solution at the reached mu
    nat, _ = O.newton_exact(P, psi, G, mu, tol=1e-13)
    assert np.abs(O.align_phase(psi, nat) - nat).max() < 1e-8
    assert np.abs(O.align_phase(psi, ref) - ref).max() < (1e-6 if prec == "fp64" else 2e-4)


def test_first_arclength_step_uses_the_tangent_and_ds_sign():
    import nosh_gb300 as ng

    m, P, p0 = _problem("square17")
    start, _ = O.newton_exact(P, p0, G, MU1, tol=1e-13)
    model = ng.nls(ng.mesh(m.x, m.cells), O.mvp_constant_curl(m.x), -1.0, G, 1.0, mu=MU1, precision=ng.PREC_FP64)
    for ds in (0.05, -0.05):
        run = ng.continuation(model, start, MU1)
        st = run.advance_arclength(ds, ng.PREDICT_SECANT, tol=1e-10)  # no secant yet: tangent
        assert st["status"] == 0
        assert np.sign(run.mu - MU1) == np.sign(ds)
        ref, mu_ref, _, _ = O.arclength_step(P, start, MU1, ds, G, predictor="tangent", tol=1e-13)
        assert abs(run.mu - mu_ref) <= 1e-8


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_natural_tangent_predictor(prec):
    import nosh_gb300 as ng

    m, P, p0 = _problem("square17")
    start, _ = O.newton_exact(P, p0, G, MU0, tol=1e-13)
    precision = ng.PREC_FP64 if prec == "fp64" else ng.PREC_MIXED
    model = ng.nls(ng.mesh(m.x, m.cells), O.mvp_constant_curl(m.x), -1.0, G, 1.0, mu=MU0, precision=precision)
    run = ng.continuation(model, start, MU0)
    st = run.advance(MU1, ng.PREDICT_TANGENT, tol=1e-10)
    assert st["status"] == 0 and run.last_prediction()["used"] == ng.PREDICT_TANGENT
    # the tangent prediction is first-order accurate: far better than the
    # previous state
    assert st["f_norm0"] < 0.05 * np.linalg.norm(P.compute_f(start, G, MU1))
    psi, mu = run.state()
    ref, _ = O.newton_exact(P, start, G, MU1, tol=1e-13)
    assert mu == MU1 and np.abs(O.align_phase(psi, ref) - ref).max() < 1e-8


def test_stepper_run_with_observer(tmp_path):
    import nosh_gb300 as ng
    from nosh_gb300 import stepper

    m, P, p0 = _problem("square17")
    start, _ = O.newton_exact(P, p0, G, 0.0, tol=1e-13)
    model = ng.nls(ng.mesh(m.x, m.cells), O.mvp_constant_curl(m.x), -1.0, G, 1.0, mu=0.0)
    run = ng.continuation(model, start, 0.0)
    path = tmp_path / "continuation.dat"
    obs = stepper.Observer(model, str(path))
    out = stepper.Stepper(run, method="Arc Length", predictor="Tangent", initial_step=0.02, max_step=0.2,
                          max_steps=6, max_value=0.6, observer=obs, tol=1e-10).run()
    assert out["status"] == "converged" and out["steps"] >= 3
    mus = [r["mu"] for r in out["records"]]
    assert all(b > a for a, b in zip(mus, mus[1:]))  # no fold below mu 0.6 on this mesh
    # the adaptive step grows while Newton converges in few iterations
    ds = [r["ds"] for r in out["records"][1:]]
    assert ds[1] > ds[0]
    lines = path.read_text().splitlines()
    assert lines[0].startswith("# (0) step") and len(lines) == len(mus) + 1
    x, mu = run.state()
    assert abs(obs.rows[-1]["(1) mu"] - mu) == 0.0
    assert abs(obs.rows[-1]["(2) Gibbs energy"] - P.energy(x)) <= 1e-12 * abs(P.energy(x))
    assert abs(obs.rows[-1]["(2) ||x||_2 scaled"] - np.sqrt(P.inner_product(x, x))) <= 1e-12
    assert np.linalg.norm(P.compute_f(x, G, mu)) <= 1.5e-10


def test_arclength_turns_around_a_fold():
    # 8 x 8 square, 97^2 vertices: the vortex-free branch from mu = 0 has a
    # fold near mu = 0.41; arclength steps follow the branch around it, back
    # to smaller mu
    import nosh_gb300 as ng
    from nosh_gb300 import stepper

    x, c, _ = O.gen_square(97, 5)
    m = O.finish_mesh(x * 8.0, c)
    A = O.mvp_constant_curl(m.x)
    P = O.Problem(m, A)
    model = ng.nls(ng.mesh(m.x, m.cells), A, -1.0, G, 1.0, mu=0.0)
    psi = np.zeros(2 * m.N)
    psi[0::2] = 1.0
    run = ng.continuation(model, psi, 0.0)
    out = stepper.Stepper(run, method="Arc Length", predictor="Tangent", initial_step=0.02, max_step=0.3,
                          max_steps=12, max_value=1.5, min_value=-0.01, tol=1e-10).run()
    mus = [r["mu"] for r in out["records"]]
    top = int(np.argmax(mus))
    assert 0.40 < mus[top] < 0.42 and 0 < top < len(mus) - 1
    assert mus[-1] < mus[top] - 0.1  # came back down past the fold
    assert run.tangent()[0] < 0
    xs, mu = run.state()
    assert np.linalg.norm(P.compute_f(xs, G, mu)) <= 1.5e-10
