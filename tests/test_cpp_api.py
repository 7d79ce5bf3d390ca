"""The C++ API (include/nosh_gb300.hpp): the reference's own test cases
(mesh, KEO, Jacobian, F, dF/dg) written against it, and the continuation
stepper (host logic on CPU, real runs on the GPU), built by g++ and run."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(name="test_reference_api"):
    import importlib.util

    spec = importlib.util.spec_from_file_location("nosh_gb300_build", os.path.join(ROOT, "nosh_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build()
    return b.build_cpp_tests()[name]


def test_cpp_api_compiles_and_links():
    exe = _build()
    assert os.access(exe, os.X_OK)


@pytest.mark.gpu
def test_cpp_api_reference_cases():
    exe = _build()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all reference-API checks passed" in r.stdout


def test_cpp_stepper_host_logic():
    # the C++ stepper over a fake run and the statistics table: no GPU
    exe = _build("test_stepper")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all stepper checks passed" in r.stdout


@pytest.mark.gpu
def test_cpp_stepper_on_the_gpu():
    exe = _build("test_stepper")
    r = subprocess.run([exe, "--gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all stepper checks passed" in r.stdout


@pytest.mark.gpu
def test_cpp_eigensolver_matches_oracle(tmp_path):
    # the C++ LOBPCG's four lowest eigenvalues of J at its converged state
    # against the oracle's shift-invert Lanczos on the same state
    import numpy as np

    from nosh_gb300 import io as nio
    from oracle import oracle as O

    exe = _build("test_eig")
    path = str(tmp_path / "state.vtu")
    r = subprocess.run([exe, path], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all eig checks passed" in r.stdout
    lam = np.array([float(ln.split()[1]) for ln in r.stdout.splitlines() if ln.startswith("eigenvalue")])
    x, cells, psi, fields, fd = nio.read_state(path)
    m = O.finish_mesh(x, cells)
    P = O.Problem(m, fields["A"])
    mu = float(fd["mu"][0])
    assert np.linalg.norm(P.compute_f(psi, 1.0, mu)) <= 1e-11
    ref = O.lowest_eigenvalues(P, psi, 1.0, mu, 4)
    assert np.abs(lam - ref).max() <= 1e-7 * max(1.0, np.abs(ref).max()), (lam, ref)
