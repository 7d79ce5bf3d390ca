"""The CPU FP64 solver (the timed baseline) against the exact-LU Newton
oracle: same converged state modulo the global phase, and continuation with
the secant predictor stays converged."""
import numpy as np
import pytest

from oracle import oracle as O


@pytest.mark.parametrize("gen,n", [(O.gen_square, 33), (O.gen_cube, 10)])
def test_cpu_newton_matches_exact(gen, n):
    x, c, psi0 = gen(n, 1)
    m = O.finish_mesh(x, c)
    P = O.Problem(m, O.mvp_constant_curl(m.x))
    ref, hist = O.newton_exact(P, psi0, 1.0, 0.5)
    S = O.CpuSolver(P)
    psi = psi0.copy()
    st = S.newton(psi, 0.5, tol=1e-10)
    assert st["status"] == 0 and st["f_norm"] <= 1e-10
    assert np.abs(O.align_phase(psi, ref) - ref).max() < 1e-8
    # both states satisfy ||F|| <= 1e-10; energies agree to that order
    assert abs(P.energy(psi) - P.energy(ref)) < 1e-9


def test_cpu_continuation_secant():
    x, c, psi0 = O.gen_square(33, 2)
    m = O.finish_mesh(x, c)
    P = O.Problem(m, O.mvp_constant_curl(m.x))
    S = O.CpuSolver(P)
    cur = psi0.copy()
    S.newton(cur, 0.2)
    prev = cur.copy()
    st = S.continuation_step(cur, None, 0.21, 0.2, float("nan"))
    assert st["status"] == 0
    mus = [0.2, 0.21]
    for k in range(3):
        mu_new = mus[-1] + 0.01
        st = S.continuation_step(cur, prev, mu_new, mus[-1], mus[-2])
        assert st["status"] == 0 and st["f_norm"] <= 1e-10
        # the secant prediction is much closer than the previous state
        assert st["f_norm0"] < 1e-4
        mus.append(mu_new)
    ref, _ = O.newton_exact(P, cur, 1.0, mus[-1])
    assert np.abs(O.align_phase(cur, ref) - ref).max() < 1e-8
