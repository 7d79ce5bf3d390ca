"""Continuation driver and learned predictor on the GPU.

* the device-resident continuation reproduces the oracle's converged states
  (exact-LU Newton, modulo the global phase);
* the message-passing network's readout coefficient and parameter gradient
  match a torch FP32 CPU reference of the same network that rounds the node
  GEMM operands to BF16 and the stored message operands A, B to FP16 as the
  GPU path does (tolerances account for the GPU's FP16 message arithmetic
  and the BF16 operands of the backward GEMMs);
* trained online on the first steps of a continuation, the learned predictor
  starts Newton from a much smaller residual than the secant predictor (the
  plain method), and beats the quadratic extrapolation on the transitions it
  was trained on (training loss < 1).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

H, FX, FE, LAYERS, RH = 64, 10, 4, 3, 32


def _layout():
    o, L = 0, {}

    def take(name, n):
        nonlocal o
        L[name] = (o, n)
        o += n

    take("enc_w", FX * H)
    take("enc_b", H)
    for l in range(LAYERS):
        take(f"wa{l}", H * H)
        take(f"wb{l}", H * H)
        take(f"wc{l}", FE * H)
        take(f"bm{l}", H)
        take(f"wu{l}", 2 * H * H)
        take(f"bu{l}", H)
    take("r1_w", H * RH)
    take("r1_b", RH)
    take("r2_w", RH)
    take("r2_b", 1)
    return L, o


def torch_reference(p, ef, rp, ci, X, gram):
    """The network in torch (CPU, FP32), node GEMM operands rounded to BF16;
    returns the readout coefficient, the loss and the parameter gradient."""
    import torch

    L, total = _layout()
    P = torch.tensor(p, dtype=torch.float32, requires_grad=True)

    def w(name, shape):
        o, n = L[name]
        return P[o : o + n].reshape(shape)

    def bf(t):
        return t.to(torch.bfloat16).float()

    N = X.shape[0]
    rows = torch.tensor(np.repeat(np.arange(N), np.diff(rp)), dtype=torch.long)
    cols = torch.tensor(ci, dtype=torch.long)
    E = torch.tensor(ef, dtype=torch.float32)
    Xt = torch.tensor(X, dtype=torch.float32)
    h = torch.relu(bf(Xt) @ bf(w("enc_w", (FX, H))) + w("enc_b", (H,)))
    for l in range(LAYERS):
        # A, B are stored in FP16 (the GPU also forms the messages in FP16)
        A = (bf(h) @ bf(w(f"wa{l}", (H, H)))).half().float()
        B = (bf(h) @ bf(w(f"wb{l}", (H, H)))).half().float()
        Pij = A[rows] + B[cols] + E @ w(f"wc{l}", (FE, H)) + w(f"bm{l}", (H,))
        M = torch.zeros(N, H).index_add_(0, rows, torch.relu(Pij))
        R = torch.relu(bf(torch.cat([h, M], dim=1)) @ bf(w(f"wu{l}", (2 * H, H))) + w(f"bu{l}", (H,)))
        h = h + R
    z = h.mean(dim=0)
    h1 = torch.relu(z @ w("r1_w", (H, RH)) + w("r1_b", (RH,)))
    wc = (h1 @ w("r2_w", (RH, 1)) + w("r2_b", (1,))).double()[0]
    g = torch.tensor(gram, dtype=torch.float64)
    loss = (wc * wc * g[0] - 2 * wc * g[1] + g[2]) / g[2]
    loss.backward()
    return float(wc.detach()), float(loss.detach()), P.grad.numpy()


@pytest.fixture(scope="module")
def net():
    import nosh_gb300 as ng

    x, c, psi0 = O.gen_cube(6, 3)
    gm = ng.mesh(x, c)
    model = ng.nls(gm, O.mvp_constant_curl(x), -1.0, 1.0, 1.0, mu=0.3)
    return gm, model, ng.mpnn(model)


def test_mpnn_parameter_layout(net):
    gm, model, mp = net
    assert mp.num_params == _layout()[1]


def test_mpnn_forward_and_gradient_match_torch(net):
    pytest.importorskip("torch")
    gm, model, mp = net
    rng = np.random.default_rng(7)
    N = gm.num_vertices
    # a parameter set with well-populated ReLUs and an O(1) readout slope
    # (the readout starts with small weights)
    p = mp.params()
    L, _ = _layout()
    for name, a in (("r1_b", 0.2), ("r2_w", 0.5)):
        o, n = L[name]
        p[o : o + n] = rng.uniform(-a, a, n)
    mp.params(p)
    X = rng.standard_normal((N, FX)).astype(np.float32)
    X[:, FX - 1] = 1.0
    # Gram scalars of two random fields (c, d)
    c, d = rng.standard_normal((2, 2 * N))
    gram = np.array([c @ c, c @ d, d @ d])
    rp, ci = gm.build_complex_graph()
    rows = np.repeat(np.arange(N), np.diff(rp))
    keep = ci != rows
    rp_od = np.concatenate([[0], np.cumsum(np.bincount(rows[keep], minlength=N))]).astype(np.int64)
    ci_od = ci[keep]
    ef = mp.edge_features()
    w_ref, loss_ref, g_ref = torch_reference(p, ef, rp_od, ci_od, X, gram)
    w = mp.forward(X)
    assert abs(w - w_ref) <= 3e-3 * abs(w_ref), (w, w_ref)
    loss, g = mp.loss_grad(X, gram)
    assert abs(loss - loss_ref) <= 1e-3 * loss_ref, (loss, loss_ref)
    cos = float(g @ g_ref / (np.linalg.norm(g) * np.linalg.norm(g_ref)))
    rel = float(np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref))
    assert cos > 0.999 and rel < 3e-2, (cos, rel)
    # the message-passing part on its own (its gradient is much smaller than
    # the readout's and runs through the BF16 backward GEMMs)
    mp_end = L["r1_w"][0]
    gm_, gr_ = g[:mp_end], g_ref[:mp_end]
    cos = float(gm_ @ gr_ / (np.linalg.norm(gm_) * np.linalg.norm(gr_)))
    rel = float(np.linalg.norm(gm_ - gr_) / np.linalg.norm(gr_))
    assert cos > 0.998 and rel < 6e-2, (cos, rel)
    # the loss-gradient query does not change the parameters
    np.testing.assert_array_equal(mp.params(), p)


def _square(s=33, seed=4):
    x, c, psi0 = O.gen_square(s, seed)
    m = O.finish_mesh(x, c)
    return m, O.Problem(m, O.mvp_constant_curl(m.x)), psi0


@pytest.mark.parametrize("predictor", ["secant", "quadratic", "cubic"])
def test_continuation_driver_matches_oracle(predictor):
    import nosh_gb300 as ng

    m, P, psi0 = _square()
    mu0 = 0.2
    x0, _ = O.newton_exact(P, psi0, 1.0, mu0)
    gm = ng.mesh(m.x, m.cells)
    model = ng.nls(gm, P.A, -1.0, 1.0, 1.0, mu=mu0)
    cont = ng.continuation(model, x0, mu0)
    pred = {"secant": ng.PREDICT_SECANT, "quadratic": ng.PREDICT_QUADRATIC, "cubic": ng.PREDICT_CUBIC}[predictor]
    f0 = []
    mu = mu0
    for k in range(5):
        mu += 0.01
        st = cont.advance(mu, predictor=pred)
        assert st["status"] == 0 and st["f_norm"] <= 1e-10
        f0.append(st["f_norm0"])
    x, mu_c = cont.state()
    assert abs(mu_c - mu) < 1e-15
    ref, _ = O.newton_exact(P, x, 1.0, mu)
    assert np.abs(O.align_phase(x, ref) - ref).max() < 1e-8
    assert np.linalg.norm(P.compute_f(x, 1.0, mu)) <= 1.5e-10
    if predictor != "secant":
        # from the third (fourth) step on the 3-point (4-point) predictor is
        # active
        assert f0[-1] < 0.5 * f0[1]


def test_learned_predictor_gains_over_secant():
    import nosh_gb300 as ng

    m, P, psi0 = _square(33, 5)
    mu0 = 0.0
    gm = ng.mesh(m.x, m.cells)
    model = ng.nls(gm, P.A, -1.0, 1.0, 1.0, mu=mu0)
    x0 = psi0.copy()
    model.newton(x0, {"mu": mu0}, refine=1e-12)
    cont = ng.continuation(model, x0, mu0)
    cont.learning(train_steps=16, iters_per_step=20, learning_rate=2e-3)
    mu, gains = mu0, []
    prev = (x0.copy(), mu0)
    for k in range(30):
        mu += 0.01
        cur = cont.state()
        # converged states well below the tolerance serve the 4-point
        # extrapolants the network combines
        st = cont.advance(mu, predictor=ng.PREDICT_LEARNED, refine=1e-12)
        assert st["status"] == 0 and st["f_norm"] <= 1e-10
        lp = cont.last_prediction()
        if k >= 22:  # after the training window (+4 history steps)
            # past the window the coefficient is inferred one step ahead,
            # overlapping the previous step's Newton solve
            assert lp["used"] == ng.PREDICT_LEARNED and np.isfinite(lp["f_learned"]) and np.isfinite(lp["coef"])
            # the secant prediction from the same two states, by the oracle
            xc, mc = cur
            xp = O.align_phase(prev[0], xc)
            sec = xc + (mu - mc) / (mc - prev[1]) * (xc - xp)
            f_sec = np.linalg.norm(P.compute_f(sec, 1.0, mu))
            gains.append(f_sec / max(lp["f_learned"], 1e-16))
            # the fallback's residual, evaluated in the same pass as the
            # learned one, is the oracle's
            assert abs(lp["f_secant"] - f_sec) <= 1e-6 * f_sec, (lp["f_secant"], f_sec)
        prev = cur
    # the trained network beats the quadratic extrapolation on its last
    # training transition, and starts Newton far closer than the secant
    assert 0.0 <= lp["train_loss"] < 1.0, lp
    assert np.median(gains) > 10.0, gains


def test_learned_prediction_between_inferences_matches_oracle():
    """With the coefficient re-inferred on every fourth learned step only,
    the steps in between form the prediction straight from the states (one
    pass, no node features).  On every step past the training window the
    learned prediction's starting residual is the oracle's residual of
    quadratic + w (cubic - quadratic) from the same four phase-aligned
    states, w being the coefficient the step reports."""
    import nosh_gb300 as ng

    m, P, psi0 = _square(33, 5)
    mu0 = 0.0
    model = ng.nls(ng.mesh(m.x, m.cells), P.A, -1.0, 1.0, 1.0, mu=mu0)
    x0 = psi0.copy()
    model.newton(x0, {"mu": mu0}, refine=1e-12)
    cont = ng.continuation(model, x0, mu0)
    cont.learning(train_steps=8, iters_per_step=10, learning_rate=2e-3)
    cont.inference_period(4)
    hist = [(x0.copy(), mu0)]
    mu, checked = mu0, 0
    for k in range(24):
        mu += 0.01
        st = cont.advance(mu, predictor=ng.PREDICT_LEARNED, refine=1e-12)
        assert st["status"] == 0 and st["f_norm"] <= 1e-10
        lp = cont.last_prediction()
        if k >= 14:  # past the 8 training steps and the 4 history steps
            assert lp["used"] == ng.PREDICT_LEARNED
            xs = [h[0] for h in hist[-4:]][::-1]
            ms = [h[1] for h in hist[-4:]][::-1]
            al = [xs[0]] + [O.align_phase(v, xs[0]) for v in xs[1:]]

            def lag(n):
                out = np.zeros_like(xs[0])
                for i in range(n):
                    w = 1.0
                    for j in range(n):
                        if j != i:
                            w *= (mu - ms[j]) / (ms[i] - ms[j])
                    out += w * al[i]
                return out

            q, c = lag(3), lag(4)
            f = np.linalg.norm(P.compute_f(q + lp["coef"] * (c - q), 1.0, mu))
            assert abs(lp["f_learned"] - f) <= 1e-4 * f, (k, lp["f_learned"], f)
            checked += 1
        hist.append(cont.state())
    assert checked == 10


@pytest.mark.parametrize("name", ["cube64", "square65"])
def test_learned_adapts_to_the_better_extrapolation(name):
    """On held-out steps after the training window, the trained network's
    prediction starts Newton within 10 % of the better of the two fixed
    extrapolations it blends (quadratic, cubic) and at least 20 % below the
    worse one.  Which one is better depends on the problem: the quadratic on
    the 64^3 cube (mu 0.5 + k 0.005, where the cubic amplifies the stored
    states' solver noise), the cubic on the 65 x 65 square (mu 0.1 + k
    0.005); a fixed choice loses on one of them.  The residuals come from
    one history per step (nosh_continuation_predictor_residuals)."""
    import torch

    import nosh_gb300 as ng
    from nosh_gb300 import meshgen

    if name == "cube64":
        x, cells, psi0 = meshgen.cube(64, 2)
        mu0 = 0.5
    else:
        x, cells, psi0 = meshgen.square(65, 5)
        mu0 = 0.1
    model = ng.nls(ng.mesh(x, cells), meshgen.mvp_constant_curl(x), -1.0, 1.0, 1.0, mu=mu0)
    x0 = torch.tensor(psi0, dtype=torch.float64, device="cuda")
    assert model.newton(x0, {"mu": mu0})["status"] == 0
    cont = ng.continuation(model, x0, mu0)
    cont.learning(12, 10, 2e-3)
    mu, rows = mu0, []
    for k in range(32):
        mu += 0.005
        if k >= 16:  # past the 12 training steps and the 4 history steps
            rows.append(cont.predictor_residuals(mu))
        st = cont.advance(mu, predictor=ng.PREDICT_LEARNED)
        assert st["status"] == 0 and st["f_norm"] <= 1e-10
    q = np.mean([r["quadratic"] for r in rows])
    c = np.mean([r["cubic"] for r in rows])
    l = np.mean([r["learned"] for r in rows])
    assert l <= 1.10 * min(q, c), (l, q, c)
    assert l <= 0.80 * max(q, c), (l, q, c)
