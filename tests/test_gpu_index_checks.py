"""Index-check mode: the KEO graph validated on the device, out-of-range
indices recorded in an error word rather than trapped.

* a handle in index-check mode solves as usual (its graph is valid);
* nosh_graph_check accepts the valid off-diagonal graph of a mesh and names
  the first offence of graphs with one planted error each (planted on the
  host, so no kernel ever dereferences a bad index): a column id equal to N,
  a diagonal entry, columns out of order, a decreasing row pointer and a
  wrong entry count.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _graph():
    import nosh_gb300 as ng
    from nosh_gb300 import meshgen

    x, cells, psi0 = meshgen.cube(6, 3)
    gm = ng.mesh(x, cells)
    rp, ci = gm.build_complex_graph()
    N = rp.size - 1
    rows = np.repeat(np.arange(N), np.diff(rp))
    keep = ci != rows
    rp_od = np.zeros(N + 1, np.int32)
    rp_od[1:] = np.cumsum(np.bincount(rows[keep], minlength=N))
    return x, cells, psi0, rp_od, ci[keep].astype(np.int32)


def _check(rp, ci):
    import torch

    import nosh_gb300 as ng

    d_rp = torch.as_tensor(rp).cuda()
    d_ci = torch.as_tensor(ci).cuda()
    ng.graph_check(d_rp, d_ci)


def test_handle_in_index_check_mode_solves():
    import nosh_gb300 as ng
    from nosh_gb300 import meshgen
    from oracle import oracle as O

    x, cells, psi0, _, _ = _graph()
    A = meshgen.mvp_constant_curl(x)
    model = ng.nls(ng.mesh(x, cells), A, -1.0, 1.0, 1.0, mu=0.5)
    model.set_index_checks(True)
    psi = psi0.copy()
    st = model.newton(psi, {"mu": 0.5})
    assert st["status"] == 0 and st["f_norm"] <= 1e-10
    m = O.finish_mesh(x, cells)
    assert np.linalg.norm(O.Problem(m, A).compute_f(psi, 1.0, 0.5)) <= 2e-10


def test_graph_check_names_the_first_offence():
    import nosh_gb300 as ng

    _, _, _, rp, ci = _graph()
    N = rp.size - 1
    _check(rp, ci)  # the mesh's own graph is valid
    k = int(rp[7]) + 2  # an entry of row 7
    cases = []
    bad = ci.copy()
    bad[k] = N
    cases.append((rp, bad, f"entry {k}"))
    bad = ci.copy()
    bad[k] = 7
    cases.append((rp, bad, f"entry {k}"))
    bad = ci.copy()
    bad[k], bad[k + 1] = bad[k + 1], bad[k]  # the second of the pair is out of order
    cases.append((rp, bad, f"entry {k + 1}"))
    brp = rp.copy()
    brp[5] = brp[6] + 1  # row 5 ends before it starts
    cases.append((brp, ci, "row 5"))
    brp = rp.copy()
    brp[N] -= 1  # the last row pointer misses the entry count
    cases.append((brp, ci, f"row {N}"))
    for r, c, where in cases:
        with pytest.raises(ng.NoshError) as e:
            _check(r, c)
        assert e.value.code == ng.ERR_INVALID and where in str(e.value), (where, str(e.value))
