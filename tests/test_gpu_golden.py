"""GPU parity against the committed golden vectors.

tests/golden/small_cases.npz holds inputs and oracle outputs on the
reference's two test meshes, a jittered 17 x 17 square and a jittered 6^3
cube (tests/golden/make_golden.py).  The CUDA path, called through the C
ABI on the stored inputs, must reproduce them: FP64 operator values and
applies within 1e-12 of the operator's scale, the converged Newton state
within 1e-8 modulo the U(1) global phase.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "small_cases.npz"))
MU, MU_LARGE, G = float(GOLD["mu"]), float(GOLD["mu_large"]), float(GOLD["g"])
NAMES = ["rect", "cube", "square17", "cube6"]


def close(a, b, tol, scale=None):
    scale = max(np.abs(b).max(), 1e-300) if scale is None else scale
    return np.abs(a - b).max() <= tol * scale


@pytest.fixture(scope="module", params=NAMES)
def case(request):
    import nosh_gb300 as ng

    n = request.param
    d = {k.split("/", 1)[1]: GOLD[k] for k in GOLD.files if k.startswith(n + "/")}
    gm = ng.mesh(d["x"], d["cells"])
    model = ng.nls(gm, d["A"], scalar_potential=-1.0, g=G, thickness=1.0, mu=MU, precision=ng.PREC_FP64)
    return n, d, gm, model


def test_graph(case):
    n, d, gm, model = case
    rp, ci = gm.build_complex_graph()
    np.testing.assert_array_equal(rp, d["row_ptr"])
    np.testing.assert_array_equal(ci, d["cols"])


def test_keo_values(case):
    n, d, gm, model = case
    model.keo.set_parameters({"mu": MU})
    assert close(model.keo.values(), d["keo"], 1e-12)
    model.keo.set_parameters({"mu": MU_LARGE})
    assert close(model.keo.values(), d["keo_large"], 1e-12)
    model.keo.set_parameters({"mu": MU})
    model.dkeo_dp.set_parameters({"mu": MU})
    assert close(model.dkeo_dp.values(), d["dkeo"], 1e-12)


def test_residual_and_derivatives(case):
    n, d, gm, model = case
    f = model.compute_f(d["psi"], {"g": G, "mu": MU})
    assert close(f, d["f"], 1e-12)
    dfdp = model.compute_dfdp(d["psi"], {"g": G, "mu": MU})
    assert close(dfdp[1], d["dfdmu"], 1e-12)
    assert close(dfdp[0], d["dfdg"], 1e-12)
    e = model.gibbs_energy(d["psi"])
    assert abs(e - float(d["energy"])) <= 1e-13 * abs(float(d["energy"]))


def test_jacobian_apply(case):
    n, d, gm, model = case
    model.set_precision(0)
    J = model.create_W_op()
    J.rebuild({"g": G, "mu": MU}, d["psi"])
    y = J.apply(d["v"])
    assert close(y, d["jv"], 1e-12, float(d["jscale"]) * np.abs(d["v"]).max())


def test_newton_state():
    import nosh_gb300 as ng
    from oracle import oracle as O

    mu = float(GOLD["newton/mu"])
    gm = ng.mesh(GOLD["newton/x"], GOLD["newton/cells"])
    model = ng.nls(gm, O.mvp_constant_curl(GOLD["newton/x"]), -1.0, G, 1.0, mu=mu, precision=ng.PREC_FP64)
    psi = GOLD["newton/psi0"].copy()
    st = model.newton(psi, {"g": G, "mu": mu}, tol=1e-10)
    assert st["status"] == 0 and st["f_norm"] <= 1e-10
    ref = GOLD["newton/psi"]
    assert np.abs(O.align_phase(psi, ref) - ref).max() < 1e-8
