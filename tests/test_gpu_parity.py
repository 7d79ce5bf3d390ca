"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

FP64 results must match within 1e-12 relative (integer work bit-exact);
FP32 (mixed-precision) operator results within 2e-6 relative to the
operator's scale.  Converged states match modulo the U(1) global phase.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

MU, G = 0.01, 1.0


def _cases():
    out = {}
    out["rect"] = O.rectanglesmall()
    out["cube"] = O.cubesmall()
    x, c, _ = O.gen_square(17, 7)
    out["square17"] = O.finish_mesh(x, c)
    x, c, _ = O.gen_cube(6, 11)
    out["cube6"] = O.finish_mesh(x, c)
    return out


CASES = _cases()


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    import nosh_gb300 as ng

    m = CASES[request.param]
    gm = ng.mesh(m.x, m.cells)
    A = O.mvp_constant_curl(m.x)
    P = O.Problem(m, A)
    model = ng.nls(gm, A, scalar_potential=-1.0, g=G, thickness=1.0, mu=MU, precision=ng.PREC_FP64)
    rng = np.random.default_rng(3)
    psi = np.zeros(2 * m.N)
    psi[0::2] = 1.0
    psi += 0.2 * rng.standard_normal(psi.size)
    return request.param, m, P, gm, model, psi


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_mesh_integer_work_bit_exact(case):
    name, m, P, gm, model, psi = case
    assert gm.num_vertices == m.N and gm.num_edges == m.E and gm.nnz_blocks == m.N + 2 * m.E
    np.testing.assert_array_equal(gm.my_edges(), m.edges)
    rp, ci = gm.build_complex_graph()
    np.testing.assert_array_equal(rp, P.row_ptr)
    np.testing.assert_array_equal(ci, P.cols)
    gids = gm.edge_gids_complex
    np.testing.assert_array_equal(gids[:, 0], 2 * (m.edges[:, 0] + 1))
    np.testing.assert_array_equal(gids[:, 3], 2 * (m.edges[:, 1] + 1) + 1)


def test_mesh_geometry(case):
    name, m, P, gm, model, psi = case
    ln, cov = gm.get_edge_data()
    assert rel(ln, m.length) < 1e-14
    assert np.abs(cov - m.covolume).max() < 1e-12 * np.abs(m.covolume).max()
    assert rel(gm.control_volumes(), m.cv) < 1e-12


def test_keo_values_fp64(case):
    name, m, P, gm, model, psi = case
    model.keo.set_parameters({"mu": MU})
    v = model.keo.values()
    ref = P.keo_values(MU)
    assert np.abs(v - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("mu", [0.5, 7.0, 300.0])
def test_keo_values_fp64_large_phases(case, mu):
    # the FP64 assembly evaluates small edge phases by a series and larger
    # ones by sincos: both branches against the oracle
    name, m, P, gm, model, psi = case
    model.keo.set_parameters({"mu": mu})
    v = model.keo.values()
    ref = P.keo_values(mu)
    assert np.abs(v - ref).max() <= 1e-12 * np.abs(ref).max()
    model.dkeo_dp.set_parameters({"mu": mu})
    v = model.dkeo_dp.values()
    ref = P.dkeo_values(mu)
    assert np.abs(v - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1e-300)
    model.keo.set_parameters({"mu": MU})


def test_dkeo_values_fp64(case):
    name, m, P, gm, model, psi = case
    model.dkeo_dp.set_parameters({"mu": MU})
    v = model.dkeo_dp.values()
    ref = P.dkeo_values(MU)
    assert np.abs(v - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1e-300)


def test_keo_apply_and_kat_sums(case):
    name, m, P, gm, model, psi = case
    model.keo.set_parameters({"mu": MU})
    y = model.keo.apply(psi)
    assert rel(y, P.keo_apply(MU, psi)) < 1e-12
    if name in ("rect", "cube"):
        one = np.ones(2 * m.N)
        s = one @ model.keo.apply(one)
        ref = {"rect": 0.01262434246161348, "cube": 1.67083246311428e-4}[name]
        assert abs(s - ref) < 1e-11


def test_compute_f_fp64(case):
    name, m, P, gm, model, psi = case
    f, nrm = model.compute_f(psi, {"g": G, "mu": MU}, with_norm=True)
    ref = P.compute_f(psi, G, MU)
    assert rel(f, ref) < 1e-12
    assert abs(nrm - np.linalg.norm(ref)) < 1e-12 * np.linalg.norm(ref)


def test_compute_f_kat_norms():
    import nosh_gb300 as ng

    for name, mk, refs in [
        ("rect", O.rectanglesmall, (0.50126061034211067, 0.24749434381636057, 0.12373710977782607)),
        ("cube", O.cubesmall, (8.3541623156163313e-05, 2.9536515963905867e-05, 1.0468744547749431e-05)),
    ]:
        m = mk()
        gm = ng.mesh(m.x, m.cells)
        model = ng.nls(gm, O.mvp_constant_curl(m.x), -1.0, 1.0, 1.0, mu=MU)
        psi = np.zeros(2 * m.N)
        psi[0::2] = 1.0
        f = model.compute_f(psi, {"g": 1.0, "mu": MU})
        n1, n2, ni = refs
        assert abs(np.abs(f).sum() - n1) < 1e-10 * n1
        assert abs(np.linalg.norm(f) - n2) < 1e-10 * n2
        assert abs(np.abs(f).max() - ni) < 1e-10 * ni


def test_dfdp(case):
    name, m, P, gm, model, psi = case
    d = model.compute_dfdp(psi, {"g": G, "mu": MU})
    # column 0: "g"; column 1: "mu" (DkeoDP built for "mu")
    assert rel(d[1], P.dfdp(psi, G, MU, "mu")) < 1e-12
    assert rel(d[0], P.dfdp(psi, G, MU, "g", deriv_param="mu")) < 1e-12


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 2e-6)])
def test_jacobian_apply(case, prec, tol):
    import nosh_gb300 as ng

    name, m, P, gm, model, psi = case
    model.set_precision(prec)
    J = model.create_W_op()
    J.rebuild({"g": G, "mu": MU}, psi)
    rng = np.random.default_rng(5)
    X = rng.standard_normal((2, 2 * m.N))
    Y = J.apply(X)
    for k in range(2):
        ref = P.jac_apply(psi, G, MU, X[k])
        scale = np.abs(P.jac_csr_real(psi, G, MU)).sum(axis=1).max() * np.abs(X[k]).max()
        assert np.abs(Y[k] - ref).max() <= tol * scale
    with pytest.raises(ng.NoshError) as e:
        J.apply(X[0], alpha=2.0)
    assert e.value.code == ng.ERR_UNSUPPORTED
    with pytest.raises(ng.NoshError):
        J.apply(X[0], mode=ng.TRANS)
    model.set_precision(0)


def test_energy_and_inner_product(case):
    name, m, P, gm, model, psi = case
    assert abs(model.gibbs_energy(psi) - P.energy(psi)) < 1e-13 * abs(P.energy(psi))
    rng = np.random.default_rng(9)
    phi = rng.standard_normal(psi.size)
    assert abs(model.inner_product(phi, psi) - P.inner_product(phi, psi)) < 1e-12


def test_keo_regularized_operator_and_amg(case):
    name, m, P, gm, model, psi = case
    Mp = model.create_W_prec()
    Mp.rebuild({"g": G, "mu": MU}, psi)
    rng = np.random.default_rng(13)
    x = rng.standard_normal(2 * m.N)
    y = Mp.operator_apply(x)
    assert rel(y, P.kreg_apply(psi, G, MU, x)) < 1e-12
    # the V-cycle is a fixed SPD operator close to K_reg^-1
    a, b = rng.standard_normal((2, 2 * m.N))
    Ma, Mb = Mp.apply(a), Mp.apply(b)
    assert abs(a @ Mb - b @ Ma) <= 1e-10 * (abs(a @ Mb) + 1e-300)
    assert a @ Ma > 0 and b @ Mb > 0
    K = P.kreg_csr_real(psi, G, MU)
    err = np.linalg.norm(K @ Mp.apply(b) - b) / np.linalg.norm(b)
    assert err < 0.9


@pytest.mark.parametrize("prec", [0, 1])
def test_newton_converges_to_oracle_state(prec):
    import nosh_gb300 as ng

    x, c, psi0 = O.gen_square(33, 1)
    m = O.finish_mesh(x, c)
    A = O.mvp_constant_curl(m.x)
    P = O.Problem(m, A)
    mu = 0.5
    ref, hist = O.newton_exact(P, psi0, G, mu, tol=1e-12)
    gm = ng.mesh(m.x, m.cells)
    model = ng.nls(gm, A, -1.0, G, 1.0, mu=mu, precision=prec)
    psi = psi0.copy()
    st = model.newton(psi, {"g": G, "mu": mu}, tol=1e-10)
    assert st["status"] == 0 and st["f_norm"] <= 1e-10
    assert np.linalg.norm(P.compute_f(psi, G, mu)) <= 1.5e-10
    al = O.align_phase(psi, ref)
    assert np.abs(al - ref).max() < 1e-8
    assert abs(model.gibbs_energy(psi) - P.energy(ref)) < 1e-10
