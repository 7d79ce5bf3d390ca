"""Kernel timing of the fine-level SpMVs (nosh_nls_profile_enable).

Inside the MINRES solve the timed launches run in the captured graphs with
event-record nodes around them; only the launches that did work are counted:
per solve, the prologue's V-cycle and one V-cycle per completed iteration
(4 fine-level SpMV launches each at smoothing degree 2: one pre-smoothing
step, the residual, two post-smoothing steps), and one Jacobian apply per
iteration plus, when convergence fell inside a captured part, the one after
it (that launch applies the last deferred w/x update).  Timing changes no
result.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [0, 1])
def test_timed_solve_counts_working_launches(prec):
    import nosh_gb300 as ng

    x, c, psi0 = O.gen_cube(20, 3)
    m = O.finish_mesh(x, c)
    A = O.mvp_constant_curl(m.x)
    P = O.Problem(m, A)
    out = {}
    for timed in (False, True):
        model = ng.nls(ng.mesh(m.x, m.cells), A, -1.0, 1.0, 1.0, mu=0.5, precision=prec)
        # an explicit schedule: the autotuner decides by timing, and the two
        # handles are compared bitwise
        model.set_spmv_schedule(1)
        model.profile(timed)
        psi = psi0.copy()
        st = model.newton(psi, {"g": 1.0, "mu": 0.5}, tol=1e-10)
        assert st["status"] == 0, st
        jac = model.profile_read(ng.KERNEL_JACOBIAN)
        smo = model.profile_read(ng.KERNEL_SMOOTHER)
        out[timed] = (psi, st, jac, smo)
    psi_a, st_a, _, _ = out[False]
    psi_b, st_b, jac, smo = out[True]
    assert np.array_equal(psi_a, psi_b)
    assert (st_a["newton_iters"], st_a["krylov_iters"]) == (st_b["newton_iters"], st_b["krylov_iters"])
    assert np.linalg.norm(P.compute_f(psi_b, 1.0, 0.5)) <= 2e-10
    n, k = st_b["newton_iters"], st_b["krylov_iters"]
    assert smo[0] == 4 * (n + k)
    assert k <= jac[0] <= k + n
    for launches, ms, nbytes in (jac, smo):
        assert ms > 0.0 and nbytes > 0.0
        assert 0.5e-3 < ms / launches < 1.0  # ms per launch


def test_stream_read_probe_folds_every_word():
    import torch

    import nosh_gb300 as ng

    rng = np.random.default_rng(7)
    words = rng.integers(0, 2**32, size=(3 << 20) // 4 + 12, dtype=np.uint64).astype(np.uint32)
    buf = torch.from_numpy(words.view(np.int32)).cuda()
    out = torch.zeros(1, dtype=torch.int32, device="cuda")
    nb = (words.size * 4) // 16 * 16
    ng.stream_read(buf, nb, out, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    expect = np.bitwise_xor.reduce(words[: nb // 4])
    assert int(out.cpu().numpy().view(np.uint32)[0]) == int(expect)
