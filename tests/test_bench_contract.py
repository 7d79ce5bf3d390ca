"""The benchmark's reference arm on a small cube, on the CPU (it runs the
FP64 CPU restatement only): one JSON line with the fields the driver reads,
the arm's own cpu_baseline and e2e, and the predictor and precision it
actually runs in its config."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run(
        [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--m", "12", "--steps", "2",
         "--warmup", "1", "--cpu-seconds", "2"],
        capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["unit"] == "steps/s" and d["value"] > 0
    assert d["steps"] == 2 and d["higher_is_better"] is True
    assert d["config"]["predictor"] == "secant" and d["config"]["precision"] == "fp64"
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["e2e"]["d2h_bytes_per_step"] == 0


def test_solve65_reference_arm_prints_one_contract_line():
    """The configuration-1 workload's reference arm: one Newton solve of the
    65 x 65 square on the CPU restatement, in the same JSON contract."""
    r = subprocess.run(
        [sys.executable, os.path.join(ROOT, "bench.py"), "--workload", "solve65", "--impl", "reference",
         "--cpu-seconds", "1"],
        capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "solves/s" and d["value"] > 0
    assert d["config"]["precision"] == "fp64" and d["config"]["mu"] == 0.1
    assert d["cpu_baseline"]["value"] == d["value"] and d["e2e"]["value"] == d["value"]


def test_single_thread_cpu_sample_restores_the_thread_count():
    """The headline's CPU baseline also reports the restatement on one
    OpenMP thread; the sample runs on one thread and leaves the count as it
    found it."""
    import argparse

    sys.path.insert(0, ROOT)
    import bench
    from oracle import oracle as O

    before = O.CpuSolver.threads()
    args = argparse.Namespace(m=8, seed=2, field="constant_curl", mu0=0.5, dmu=0.005)
    out = bench.cpu_single_thread(args, 0.5)
    assert out["cores"] == 1 and out["value"] > 0 and out["unit"] == "steps/s"
    assert out["newton_krylov_per_step"][0] >= 1
    assert O.CpuSolver.threads() == before
