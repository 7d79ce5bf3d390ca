"""The continuation stepper's host logic (no GPU): LOCA adaptive step size,
failed-step halving and the minimum-step failure, landing on the parameter
bounds, arclength direction handling, and the observer's statistics file in
the reference's csv_writer layout.  A fake continuation run follows the
fold curve mu = 1 - x^2 (natural steps fail past mu = 1)."""
import math

import numpy as np
import pytest

from nosh_gb300 import stepper


class FoldRun:
    """Branch (x, mu) with mu = 1 - x^2 starting at x = 1, mu = 0."""

    def __init__(self, iters=2, fail_above=None):
        self.x, self._mu, self.iters, self.fail_above = 1.0, 0.0, iters, fail_above
        self.prev = None
        self.calls = []
        self._tmu = None

    @property
    def mu(self):
        return self._mu

    def state(self):
        return np.array([self.x, 0.0]), self._mu

    def tangent(self):
        return self._tmu, 1.0

    def _fail(self, step):
        return self.fail_above is not None and abs(step) > self.fail_above

    def advance(self, mu_new, predictor=0, **kw):
        self.calls.append(("natural", mu_new))
        if self._fail(mu_new - self._mu) or mu_new > 1.0:
            return {"status": 3, "newton_iters": kw.get("max_newton", 15), "krylov_iters": 0}
        self.x, self._mu = math.sqrt(1.0 - mu_new), mu_new
        return {"status": 0, "newton_iters": self.iters, "krylov_iters": 10}

    def advance_arclength(self, ds, predictor=2, theta=1.0, **kw):
        # arclength along the curve parametrised by x (unit speed in (x, mu))
        self.calls.append(("arclength", ds))
        if self._fail(ds):
            return {"status": 3, "newton_iters": kw.get("max_newton", 15), "krylov_iters": 0, "mu": self._mu}
        # tangent (dx, dmu) ~ (-1, 2x) normalised, oriented along travel
        d = np.array([-1.0, 2.0 * self.x])
        d /= np.linalg.norm(d)
        if self.prev is not None and d @ (np.array([self.x, self._mu]) - self.prev) < 0:
            d = -d
        self.prev = np.array([self.x, self._mu])
        self.x += ds * d[0]
        self._mu = 1.0 - self.x * self.x
        self._tmu = d[1]
        return {"status": 0, "newton_iters": self.iters, "krylov_iters": 10, "mu": self._mu}


def test_adaptive_step_growth_and_cap():
    s = stepper.Stepper(FoldRun(iters=2), method="Natural", predictor="Secant", initial_step=1e-3, max_step=1e-2,
                        max_steps=6, aggressiveness=2.0, max_nonlinear_iters=15)
    out = s.run()
    ds = [r["ds"] for r in out["records"][1:]]
    grow = 1.0 + 2.0 * (13.0 / 14.0) ** 2
    assert ds[0] == pytest.approx(1e-3)
    assert ds[1] == pytest.approx(1e-3 * grow)
    assert ds[2] == pytest.approx(min(1e-3 * grow**2, 1e-2))
    assert max(ds) == pytest.approx(1e-2) and out["steps"] == 6 and out["status"] == "converged"


def test_constant_step_and_no_growth_at_max_iterations():
    s = stepper.Stepper(FoldRun(iters=2), method="Natural", predictor="Secant", initial_step=2e-3,
                        step_method="Constant", max_steps=4)
    assert [r["ds"] for r in s.run()["records"][1:]] == [2e-3] * 4
    s = stepper.Stepper(FoldRun(iters=15), method="Natural", predictor="Secant", initial_step=2e-3, max_steps=3,
                        max_nonlinear_iters=15)
    assert [r["ds"] for r in s.run()["records"][1:]] == pytest.approx([2e-3] * 3)


def test_failed_steps_halve_then_minimum_step_fails():
    run = FoldRun(iters=2, fail_above=3e-3)
    out = stepper.Stepper(run, method="Natural", predictor="Secant", initial_step=1e-2, max_step=1e-2,
                          max_steps=2).run()
    # 1e-2 and 5e-3 fail, 2.5e-3 succeeds
    assert out["failed_steps"] >= 2 and out["records"][1]["ds"] == pytest.approx(2.5e-3)
    run = FoldRun(iters=2, fail_above=1e-9)
    out = stepper.Stepper(run, method="Natural", predictor="Secant", initial_step=1e-3, min_step=1e-7).run()
    assert out["status"] == "failed" and out["steps"] == 0
    assert out["failed_steps"] == math.ceil(math.log2(1e-3 / 1e-7))


def test_natural_lands_on_max_value():
    out = stepper.Stepper(FoldRun(iters=2), method="Natural", predictor="Secant", initial_step=0.03,
                          max_step=0.03, max_value=0.1).run()
    mus = [r["mu"] for r in out["records"]]
    assert mus[-1] == pytest.approx(0.1, abs=1e-15) and all(m <= 0.1 + 1e-15 for m in mus)
    assert out["status"] == "converged"


def test_arclength_passes_the_fold():
    # natural steps cannot pass mu = 1; arclength steps turn around the fold
    run = FoldRun(iters=3)
    out = stepper.Stepper(run, method="Arc Length", predictor="Tangent", initial_step=0.05, max_step=0.1,
                          max_steps=60, min_value=-0.5, max_value=2.0).run()
    mus = [r["mu"] for r in out["records"]]
    assert max(mus) > 0.99 and mus[-1] < 0.5  # went up to the fold and back down
    assert run.x < 0  # now on the other half of the branch
    assert all(r["ds"] > 0 for r in out["records"][2:])


def test_stepper_rejects_bad_settings():
    with pytest.raises(ValueError):
        stepper.Stepper(FoldRun(), method="Turning Point")
    with pytest.raises(ValueError):
        stepper.Stepper(FoldRun(), method="Arc Length", predictor="Quadratic")
    with pytest.raises(ValueError):
        stepper.Stepper(FoldRun(), initial_step=1.0, max_step=1e-2)


class FakeModel:
    def gibbs_energy(self, x):
        return -float(x @ x) / 4.0

    def inner_product(self, a, b):
        return float(a @ b)


def test_observer_writes_reference_table(tmp_path):
    path = tmp_path / "cont.dat"
    obs = stepper.Observer(FakeModel(), str(path))
    out = stepper.Stepper(FoldRun(iters=2), method="Natural", predictor="Secant", initial_step=0.25,
                          max_step=0.25, max_steps=2, observer=obs).run()
    lines = path.read_text().splitlines()
    assert len(lines) == 4 and out["steps"] == 2
    assert lines[0] == ("# (0) step   " + "(1) mu".ljust(22) + "   " + "(2) Gibbs energy".ljust(22) + "   "
                        + "(2) ||x||_2 scaled".ljust(22))
    # row 1: x = sqrt(0.75), mu = 0.25, energy -0.1875, norm sqrt(0.75)
    want = ("  " + "1".ljust(8) + "   " + "2.500000000000000e-01".ljust(22) + "   "
            + "-1.875000000000000e-01".ljust(22) + "   " + f"{math.sqrt(0.75):.15e}".ljust(22))
    assert lines[2] == want
    assert [r["(0) step"] for r in obs.rows] == [0, 1, 2]
    assert obs.rows[0]["(1) mu"] == 0.0
