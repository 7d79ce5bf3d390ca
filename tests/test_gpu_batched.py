"""Batched independent solves on the GPU: a union of square meshes of uneven
sizes, each with its own mu, solved in one handle (mixed precision) reaches
||F_s|| <= 1e-10 in every system and each system's state matches the
oracle's exact-LU Newton solution of that system alone (modulo its own
global phase)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_batched_squares_match_oracle():
    import nosh_gb300 as ng
    from nosh_gb300 import batch

    sides = [9, 17, 13, 21, 11]
    mus = [0.15, 0.8, 0.45, 0.3, 0.6]
    x, c, off, psi0, A, mu = batch.squares(sides, mus, seed0=40)
    gm = ng.mesh(x, c)
    model = ng.nls(gm, A, -1.0, 1.0, 1.0, mu=0.0)
    model.set_systems(off, mu)
    psi = psi0.copy()
    st = model.newton(psi, {"mu": 0.0}, tol=1e-10)
    assert st["status"] == 0 and st["f_norm"] <= 1e-10
    norms = model.system_norms()
    assert norms.shape == (len(sides),) and np.all(norms <= 1e-10)
    # every system ran its own MINRES recurrences and Newton steps
    nw, kr = model.system_iterations()
    assert nw.shape == kr.shape == (len(sides),)
    assert np.all(nw >= 1) and np.all(kr >= nw) and st["newton_iters"] == nw.max()
    for k, (s, m) in enumerate(zip(sides, mus)):
        xs, cs, p0 = O.gen_square(s, 40 + k)
        mk = O.finish_mesh(xs, cs)
        P = O.Problem(mk, O.mvp_constant_curl(mk.x))
        ref, _ = O.newton_exact(P, p0, 1.0, m, tol=1e-12)
        got = batch.split_state(psi, off)[k]
        assert np.linalg.norm(P.compute_f(got, 1.0, m)) <= 1.5e-10
        assert np.abs(O.align_phase(got, ref) - ref).max() < 1e-8


def test_batched_rejects_cross_system_edges():
    import nosh_gb300 as ng
    from nosh_gb300 import batch

    x, c, off, psi0, A, mu = batch.squares([5, 7], [0.1, 0.2])
    gm = ng.mesh(x, c)
    model = ng.nls(gm, A, -1.0, 1.0, 1.0)
    with pytest.raises(ng.NoshError):
        model.set_systems([0, 20, off[-1]], mu)  # splits the first square


def test_thirty_two_uneven_systems_pass_the_oracle_residual():
    """32 squares with sides drawn from {9..65} and mu from [0, 1] (the
    batched workload's sampling at smaller sides), solved as one batch
    through batch.solve_union: every system's FP64 residual, evaluated by the
    oracle on that system alone, is at most 1.5e-10."""
    from nosh_gb300 import batch

    sides, mus = batch.config_squares(32, lo=9, hi=65, seed=77)
    seeds = [500 + k for k in range(32)]
    norms, st, states = batch.solve_union(sides, mus, seeds)
    assert len(set(int(s) for s in sides)) >= 16  # uneven sizes
    assert np.all(norms <= 1e-10)
    for k in range(32):
        xs, cs, _ = O.gen_square(int(sides[k]), seeds[k])
        mk = O.finish_mesh(xs, cs)
        P = O.Problem(mk, O.mvp_constant_curl(mk.x))
        assert np.linalg.norm(P.compute_f(states[k], 1.0, mus[k])) <= 1.5e-10
