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
