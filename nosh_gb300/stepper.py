"""Continuation stepper: the LOCA stepper loop that drives the device-resident
continuation handle, and the per-step statistics observer.

Restated from the reference's configuration and driver (LOCA and NOX are
Trilinos packages, not in the reference tree; their parameters are read from
``examples/conf.xml:35-75`` and ``examples/bratu-continuation/bratu.cpp:
68-86``, the loop from ``executables/nosh-cont/nosh-cont.cpp:226-345``):

* "Continuation Method": ``"Natural"`` (steps in mu) or ``"Arc Length"``
  (pseudo-arclength, bordered Newton corrector on the GPU; the sign of the
  initial step picks the direction, later steps follow the last secant);
* "Predictor" "Method": ``"Tangent"`` or ``"Secant"`` (natural steps also
  take the handle's polynomial and learned predictors);
* "Step Size": ``"Adaptive"`` (after a successful step of N nonlinear
  iterations, ``ds *= 1 + aggressiveness * ((N_max - N) / (N_max - 1))^2``;
  after a failed one ``ds *= 0.5``; ``|ds|`` clipped to the max step, and the
  run fails once it drops below the min step) or ``"Constant"``;
* "Max Steps", "Max Value", "Min Value": the run stops after that many
  successful steps or when mu reaches a bound (the last step is shortened
  to land on it: exactly for natural steps, from the last tangent's dmu/ds
  for arclength steps).

The observer writes the reference's continuation statistics file
(``src/observer.cpp:136-159`` through ``src/csv_writer.cpp``): a ``#`` header
of the labels and one row per converged state with the step index, the
parameter, the Gibbs energy and the scaled norm sqrt(<psi, psi>).
"""
from __future__ import annotations

import math

from . import PREDICT_CUBIC, PREDICT_LEARNED, PREDICT_NONE, PREDICT_QUADRATIC, PREDICT_SECANT, PREDICT_TANGENT

PREDICTORS = {
    "Constant": PREDICT_NONE,
    "Secant": PREDICT_SECANT,
    "Tangent": PREDICT_TANGENT,
    "Quadratic": PREDICT_QUADRATIC,
    "Cubic": PREDICT_CUBIC,
    "Learned": PREDICT_LEARNED,
}


class CsvWriter:
    """Space-delimited statistics table in the layout of the reference's
    csv_writer (src/csv_writer.cpp): "# " then the labels, doubles in
    scientific notation with 15 digits in 22-wide columns, integers in
    columns as wide as their label (at least 5), columns separated by three
    spaces, data rows indented to the header's text."""

    DOUBLE_WIDTH = 22
    INT_WIDTH = 5

    def __init__(self, path):
        self.f = open(path, "w")

    def _cells(self, row, header):
        out = []
        for label, v in row:
            if isinstance(v, int):
                w = max(self.INT_WIDTH, len(label))
                out.append(f"{label if header else v:<{w}}")
            else:
                out.append(f"{label:<{self.DOUBLE_WIDTH}}" if header else f"{v:<{self.DOUBLE_WIDTH}.15e}")
        return "   ".join(out)

    def write_header(self, row):
        self.f.write("# " + self._cells(row, True) + "\n")

    def write_row(self, row):
        self.f.write("  " + self._cells(row, False) + "\n")
        self.f.flush()

    def close(self):
        self.f.close()


class Observer:
    """Continuation statistics per converged state (src/observer.cpp:136-159):
    step index, the parameter, the Gibbs energy and ||psi|| =
    sqrt(inner_product(psi, psi)) (src/model_evaluator_base.hpp).  Rows are
    kept in ``rows`` and, with a path, written as the reference's table."""

    def __init__(self, model, path=None, param_name="mu"):
        self.model = model
        self.param_name = param_name
        self.writer = CsvWriter(path) if path else None
        self.rows = []

    def __call__(self, index, x, param):
        row = [
            ("(0) step", int(index)),
            ("(1) " + self.param_name, float(param)),
            ("(2) Gibbs energy", float(self.model.gibbs_energy(x))),
            ("(2) ||x||_2 scaled", float(math.sqrt(max(self.model.inner_product(x, x), 0.0)))),
        ]
        if self.writer:
            if index == 0:
                self.writer.write_header(row)
            self.writer.write_row(row)
        self.rows.append({k: v for k, v in row})

    def close(self):
        if self.writer:
            self.writer.close()


class Stepper:
    """The LOCA stepper loop over a continuation run (``nosh_gb300.
    continuation`` or any object with ``mu``, ``advance``,
    ``advance_arclength``, ``tangent`` and ``state``).  ``run()`` returns a
    dict with ``status`` ("converged" once a bound or the step limit is
    reached, "failed" when the step size fell below the minimum), the per
    step records and the counts of taken and failed steps."""

    def __init__(self, run, method="Arc Length", predictor="Tangent", initial_step=1e-3, max_step=1e-2,
                 min_step=1e-7, aggressiveness=2.0, step_method="Adaptive", max_steps=1000, max_value=100.0,
                 min_value=-100.0, max_nonlinear_iters=15, theta=1.0, observer=None, **solver):
        if method not in ("Arc Length", "Natural"):
            raise ValueError(f"unknown continuation method {method!r}")
        if predictor not in PREDICTORS:
            raise ValueError(f"unknown predictor {predictor!r}")
        if method == "Arc Length" and predictor not in ("Tangent", "Secant"):
            raise ValueError("arclength steps predict Tangent or Secant")
        if step_method not in ("Adaptive", "Constant"):
            raise ValueError(f"unknown step size method {step_method!r}")
        if not (0 < min_step <= abs(initial_step) <= max_step):
            raise ValueError("need 0 < min step <= |initial step| <= max step")
        if max_nonlinear_iters < 2:
            raise ValueError("max nonlinear iterations must be at least 2")
        self.run_ = run
        self.method, self.predictor = method, predictor
        self.ds, self.max_step, self.min_step = float(initial_step), float(max_step), float(min_step)
        self.aggressiveness, self.step_method = float(aggressiveness), step_method
        self.max_steps, self.max_value, self.min_value = int(max_steps), float(max_value), float(min_value)
        self.max_nl = int(max_nonlinear_iters)
        self.theta = float(theta)
        self.observer = observer
        self.solver = dict(solver)
        self.solver.setdefault("max_newton", self.max_nl)

    # -- step size (LOCA "Adaptive": grows with the Newton iterations saved)
    def next_step(self, ds, newton_iters):
        if self.step_method == "Constant":
            return ds
        ratio = max(0.0, (self.max_nl - newton_iters) / (self.max_nl - 1))
        ds = ds * (1.0 + self.aggressiveness * ratio * ratio)
        return math.copysign(min(abs(ds), self.max_step), ds)

    def _clip(self, ds, mu, dmu_ds):
        """Shorten the step so that the predicted mu lands on the bound it
        would cross; returns (ds, last)."""
        if dmu_ds is None or not math.isfinite(dmu_ds) or dmu_ds == 0.0:
            return ds, False
        target = mu + ds * dmu_ds
        for bound in (self.max_value, self.min_value):
            if (target - bound) * (mu - bound) < 0.0 or target == bound:
                return (bound - mu) / dmu_ds, True
        return ds, False

    def run(self):
        cr = self.run_
        records, failed = [], 0
        x, mu = cr.state()
        if self.observer:
            self.observer(0, x, mu)
        records.append({"step": 0, "mu": mu, "ds": 0.0, "newton_iters": 0, "krylov_iters": 0})
        ds = self.ds
        status = "converged"
        step = 0
        while step < self.max_steps:
            mu = cr.mu
            if mu >= self.max_value or mu <= self.min_value:
                break
            if self.method == "Natural":
                ds_try, last = self._clip(ds, mu, 1.0)
                st = cr.advance(mu + ds_try, predictor=PREDICTORS[self.predictor], **self.solver)
            else:
                dmu_ds = cr.tangent()[0] if step > 0 else None
                ds_try, last = self._clip(ds, mu, dmu_ds)
                st = cr.advance_arclength(ds_try, predictor=PREDICTORS[self.predictor], theta=self.theta,
                                          **self.solver)
            if st["status"] != 0:
                failed += 1
                ds = 0.5 * ds_try
                if abs(ds) < self.min_step:
                    status = "failed"
                    break
                continue
            step += 1
            x, mu_new = cr.state()
            if self.observer:
                self.observer(step, x, mu_new)
            records.append({"step": step, "mu": mu_new, "ds": ds_try, "newton_iters": st["newton_iters"],
                            "krylov_iters": st["krylov_iters"]})
            if last:
                break
            ds = self.next_step(ds_try, st["newton_iters"])
            if self.method == "Arc Length":
                # from the second step on the tangent is oriented along the
                # last secant, so a positive length continues the direction
                # of travel
                ds = abs(ds)
            if abs(ds) < self.min_step:
                ds = math.copysign(self.min_step, ds)
        if self.observer:
            self.observer.close()
        return {"status": status, "records": records, "steps": step, "failed_steps": failed}
