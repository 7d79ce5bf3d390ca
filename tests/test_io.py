"""Mesh and state files (.vtu): bit-exact round trips of meshes, states and
fields, ASCII arrays, the per-step data saver's file names and contents, and
the reader's checks."""
import os

import numpy as np
import pytest

from nosh_gb300 import io as nio
from nosh_gb300 import meshgen


def test_round_trip_triangles_and_tets(tmp_path):
    for x, c, _ in (meshgen.square(9, 3), meshgen.cube(3, 4)):
        rng = np.random.default_rng(1)
        psi = rng.standard_normal(2 * len(x))
        A = meshgen.mvp_constant_curl(x)
        V = rng.standard_normal(len(x))
        p = str(tmp_path / "m.vtu")
        nio.write_vtu(p, x, c, nio.state_point_data(psi, A, V), {"mu": 0.25, "step": 3})
        x2, c2, pd, fd = nio.read_vtu(p)
        np.testing.assert_array_equal(x2[:, : x.shape[1]], x)
        np.testing.assert_array_equal(c2, c)
        np.testing.assert_array_equal(pd["psi"].reshape(-1), psi)
        np.testing.assert_array_equal(pd["A"], A.reshape(-1, 3))
        np.testing.assert_array_equal(pd["V"], V)
        assert fd["mu"][0] == 0.25 and fd["step"][0] == 3
        xs, cs, psi2, fields, _ = nio.read_state(p)
        np.testing.assert_array_equal(psi2, psi)
        assert set(fields) == {"A", "V"}


ASCII = """<?xml version="1.0"?>
<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian">
  <UnstructuredGrid>
    <Piece NumberOfPoints="4" NumberOfCells="2">
      <PointData>
        <DataArray type="Float64" Name="psi" NumberOfComponents="2" format="ascii">1 0 1 0 0.5 0.5 1 -1</DataArray>
      </PointData>
      <Points>
        <DataArray type="Float64" NumberOfComponents="3" format="ascii">0 0 0 1 0 0 0 1 0 1 1 0</DataArray>
      </Points>
      <Cells>
        <DataArray type="Int32" Name="connectivity" format="ascii">0 1 2 1 3 2</DataArray>
        <DataArray type="Int32" Name="offsets" format="ascii">3 6</DataArray>
        <DataArray type="UInt8" Name="types" format="ascii">5 5</DataArray>
      </Cells>
    </Piece>
  </UnstructuredGrid>
</VTKFile>
"""


def test_ascii_arrays(tmp_path):
    p = tmp_path / "a.vtu"
    p.write_text(ASCII)
    x, c, pd, fd = nio.read_vtu(str(p))
    assert x.shape == (4, 3) and c.tolist() == [[0, 1, 2], [1, 3, 2]]
    assert pd["psi"].reshape(-1).tolist() == [1, 0, 1, 0, 0.5, 0.5, 1, -1]
    bad = ASCII.replace(">0 1 2 1 3 2<", ">0 1 2 1 3 7<")
    p.write_text(bad)
    with pytest.raises(ValueError):
        nio.read_vtu(str(p))
    p.write_text(ASCII.replace(">5 5<", ">5 10<"))
    with pytest.raises(ValueError):
        nio.read_vtu(str(p))


def test_point_data_size_checked(tmp_path):
    x, c, _ = meshgen.square(5, 1)
    with pytest.raises(ValueError):
        nio.write_vtu(str(tmp_path / "b.vtu"), x, c, {"V": np.zeros(len(x) + 1)})


def test_data_saver_names_and_contents(tmp_path):
    x, c, _ = meshgen.square(5, 1)
    saver = nio.DataSaver(x, c, directory=str(tmp_path), A=meshgen.mvp_constant_curl(x))
    for k in range(3):
        saver(k, np.full(2 * len(x), k, np.float64), 0.1 * k)
    saver.close()
    assert [os.path.basename(p) for p in saver.paths] == ["out0000.vtu", "out0001.vtu", "out0002.vtu"]
    _, _, psi, fields, fd = nio.read_state(saver.paths[2])
    assert np.all(psi == 2.0) and fd["mu"][0] == pytest.approx(0.2) and "A" in fields and "V" not in fields


def _cpp_io():
    import importlib.util

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("nosh_gb300_build", os.path.join(root, "nosh_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build()
    return b.build_cpp_tests()["test_io"]


def test_cpp_io_self_checks(tmp_path):
    import subprocess

    r = subprocess.run([_cpp_io()], capture_output=True, text=True, timeout=120, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all io checks passed" in r.stdout


def test_cpp_and_python_files_interchange(tmp_path):
    import subprocess

    exe = _cpp_io()
    # C++ writes, Python reads (bit-exact against the same formulas)
    p = str(tmp_path / "cpp.vtu")
    assert subprocess.run([exe, "write", p], timeout=60).returncode == 0
    x, c, pd, fd = nio.read_vtu(p)
    i = np.arange(10)
    np.testing.assert_array_equal(pd["psi"].reshape(-1), np.sin(0.7 * i + 0.1) / 3.0)
    np.testing.assert_array_equal(pd["V"], -1.0 + np.arange(5) / 7.0)
    assert c.tolist() == [[0, 1, 2, 3], [1, 2, 3, 4]] and fd["mu"][0] == 0.25
    # Python writes, C++ reads
    xs, cs, _ = meshgen.cube(2, 1)
    psi = np.random.default_rng(2).standard_normal(2 * len(xs))
    q = str(tmp_path / "py.vtu")
    nio.write_vtu(q, xs, cs, nio.state_point_data(psi, meshgen.mvp_constant_curl(xs)), {"mu": 0.5})
    r = subprocess.run([exe, "read", q], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout
    got = {ln.split()[0] + ("" if len(ln.split()) == 2 else ln.split()[1]): float(ln.split()[-1])
           for ln in r.stdout.splitlines()}
    # plain left-to-right sums, in the reader's order (bit-exact values;
    # Python's sum() compensates, numpy's sums pairwise)
    def seq(a):
        t = 0.0
        for v in np.asarray(a, np.float64).reshape(-1).tolist():
            t += v
        return t

    assert got["points"] == seq(xs)
    assert got["cells"] == seq(cs)
    assert got["psi2"] == seq(psi)
    assert got["fieldmu"] == 0.5 and got["nvc"] == 4


def test_reference_io_case_rectanglesmall(tmp_path):
    # the reference's io test (test/io.cpp:30-44 with the constants of
    # :52-58): the "rectanglesmall" state psi = 1 and A = 1/2(-y, x, 0),
    # written and read back, has ||psi||_1 = 4, ||psi||_inf = 1 and the
    # per-component max norms {0.25, 2.5, 0} of A
    from oracle import oracle as O

    m = O.rectanglesmall()
    psi = np.zeros(2 * m.N)
    psi[0::2] = 1.0
    A = O.mvp_constant_curl(m.x)
    p = str(tmp_path / "rectanglesmall.vtu")
    nio.write_vtu(p, m.x, m.cells, nio.state_point_data(psi, A))
    _, _, psi_r, fields, _ = nio.read_state(p)
    assert np.abs(psi_r).sum() == 4.0 and np.abs(psi_r).max() == 1.0
    np.testing.assert_allclose(np.abs(fields["A"]).max(axis=0), [0.25, 2.5, 0.0], rtol=0, atol=1e-15)
