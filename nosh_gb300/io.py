"""Mesh and state files: VTK XML unstructured grids (.vtu).

The reference reads meshes with their ``psi``, ``A`` and ``V`` vertex tags
through MOAB (``src/mesh_reader.cpp:20-162``) and writes one state file per
continuation step (``src/continuation_data_saver.hpp:26-50``: ``out0000.h5m``,
``out0001.h5m``, ...).  MOAB's .h5m and Exodus need HDF5 / netCDF, which are
not in this image, so the files here are VTK XML unstructured grids, the
format ParaView (the reference's viewer) reads natively:

* points (N x 3 FP64), cells (triangles, VTK type 5, or tetrahedra, type 10);
* point data: ``psi`` as a 2-component FP64 array (Re, Im), ``A`` (3
  components), ``V`` and any other per-vertex array;
* field data: the continuation parameter of the state (``mu``) and the step.

Arrays are written base64-encoded ("binary" format, UInt64 size headers,
little endian) and read back bit for bit; the reader also takes ASCII arrays.
"""
from __future__ import annotations

import base64
import os
import xml.etree.ElementTree as ET

import numpy as np

VTK_TRIANGLE, VTK_TETRA = 5, 10
_TYPES = {np.dtype("float64"): "Float64", np.dtype("float32"): "Float32", np.dtype("int64"): "Int64",
          np.dtype("int32"): "Int32", np.dtype("uint8"): "UInt8"}
_DTYPES = {v: k for k, v in _TYPES.items()}


def _encode(a):
    a = np.ascontiguousarray(a)
    a = a.astype(a.dtype.newbyteorder("<"), copy=False)
    raw = a.tobytes()
    return base64.b64encode(np.uint64(len(raw)).astype("<u8").tobytes() + raw).decode("ascii")


def _decode(text, dtype):
    blob = base64.b64decode("".join(text.split()))
    n = int(np.frombuffer(blob[:8], "<u8")[0])
    return np.frombuffer(blob[8:8 + n], np.dtype(dtype).newbyteorder("<")).astype(dtype)


def _array(parent, name, a, ncomp):
    a = np.asarray(a)
    el = ET.SubElement(parent, "DataArray", type=_TYPES[a.dtype], Name=name, format="binary")
    if ncomp > 1:
        el.set("NumberOfComponents", str(ncomp))
    el.text = _encode(a.reshape(-1))
    return el


def write_vtu(path, x, cells, point_data=None, field_data=None):
    """Write a mesh and its per-vertex arrays.  ``x``: (N, 2 or 3) points;
    ``cells``: (T, 3) triangles or (T, 4) tetrahedra (0-based);
    ``point_data``: name -> (N,) or (N, c) arrays; ``field_data``: name ->
    scalars."""
    x = np.asarray(x, np.float64)
    if x.shape[1] == 2:
        x = np.hstack([x, np.zeros((len(x), 1))])
    cells = np.asarray(cells, np.int64)
    nv = cells.shape[1]
    if nv not in (3, 4):
        raise ValueError("cells must be triangles (3) or tetrahedra (4)")
    root = ET.Element("VTKFile", type="UnstructuredGrid", version="1.0", byte_order="LittleEndian",
                      header_type="UInt64")
    grid = ET.SubElement(root, "UnstructuredGrid")
    if field_data:
        fd = ET.SubElement(grid, "FieldData")
        for name, v in field_data.items():
            a = np.atleast_1d(np.asarray(v, np.float64))
            el = _array(fd, name, a, 1)
            el.set("NumberOfTuples", str(a.size))
    piece = ET.SubElement(grid, "Piece", NumberOfPoints=str(len(x)), NumberOfCells=str(len(cells)))
    if point_data:
        pd = ET.SubElement(piece, "PointData")
        for name, v in point_data.items():
            a = np.asarray(v)
            if a.dtype not in _TYPES:
                a = a.astype(np.float64)
            if a.shape[0] != len(x):
                raise ValueError(f"point data {name!r} has {a.shape[0]} rows, the mesh {len(x)} points")
            _array(pd, name, a, 1 if a.ndim == 1 else a.shape[1])
    _array(ET.SubElement(piece, "Points"), "Points", x, 3)
    ce = ET.SubElement(piece, "Cells")
    _array(ce, "connectivity", cells, 1)
    _array(ce, "offsets", np.arange(1, len(cells) + 1, dtype=np.int64) * nv, 1)
    _array(ce, "types", np.full(len(cells), VTK_TRIANGLE if nv == 3 else VTK_TETRA, np.uint8), 1)
    ET.ElementTree(root).write(path, xml_declaration=True, encoding="utf-8")


def _read_array(el):
    dtype = _DTYPES[el.get("type")]
    fmt = el.get("format", "ascii")
    if fmt == "binary":
        a = _decode(el.text or "", dtype)
    elif fmt == "ascii":
        a = np.array((el.text or "").split(), dtype=dtype)
    else:
        raise ValueError(f"unsupported DataArray format {fmt!r}")
    nc = int(el.get("NumberOfComponents", "1"))
    return a.reshape(-1, nc) if nc > 1 else a


def read_vtu(path):
    """Read a .vtu written by ``write_vtu`` (or any single-piece unstructured
    grid of one cell type with inline binary or ASCII arrays).  Returns
    (x (N, 3), cells (T, 3|4) int32, point_data dict, field_data dict)."""
    root = ET.parse(path).getroot()
    if root.get("type") != "UnstructuredGrid":
        raise ValueError("not a VTK unstructured grid")
    if root.get("header_type", "UInt32") != "UInt64" and any(
            el.get("format") == "binary" for el in root.iter("DataArray")):
        raise ValueError("binary arrays need UInt64 headers")
    grid = root.find("UnstructuredGrid")
    pieces = grid.findall("Piece")
    if len(pieces) != 1:
        raise ValueError("exactly one Piece is supported")
    piece = pieces[0]
    x = _read_array(piece.find("Points/DataArray")).astype(np.float64).reshape(-1, 3)
    arrays = {el.get("Name"): _read_array(el) for el in piece.findall("Cells/DataArray")}
    types = np.unique(arrays["types"])
    if len(types) != 1 or int(types[0]) not in (VTK_TRIANGLE, VTK_TETRA):
        raise ValueError("cells must all be triangles or all tetrahedra")
    nv = 3 if int(types[0]) == VTK_TRIANGLE else 4
    off = arrays["offsets"].astype(np.int64)
    if not np.array_equal(off, np.arange(1, len(off) + 1) * nv):
        raise ValueError("cell offsets do not match the cell type")
    cells = arrays["connectivity"].astype(np.int64).reshape(-1, nv)
    if cells.size and (cells.min() < 0 or cells.max() >= len(x)):
        raise ValueError("cell connectivity out of range")
    pdata = {el.get("Name"): _read_array(el) for el in piece.findall("PointData/DataArray")}
    fdata = {el.get("Name"): _read_array(el) for el in grid.findall("FieldData/DataArray")}
    return x, cells.astype(np.int32), pdata, fdata


def state_point_data(psi, A=None, V=None):
    """Point data of a state: psi (2N interleaved) as (N, 2) (Re, Im), and
    the fields when given."""
    psi = np.asarray(psi, np.float64)
    out = {"psi": psi.reshape(-1, 2)}
    if A is not None:
        out["A"] = np.asarray(A, np.float64).reshape(-1, 3)
    if V is not None:
        out["V"] = np.asarray(V, np.float64).reshape(-1)
    return out


def read_state(path):
    """(x, cells, psi (2N interleaved), fields dict, field data) of a state
    file; ``fields`` holds A and V when present."""
    x, cells, pd, fd = read_vtu(path)
    if "psi" not in pd:
        raise ValueError("no psi array")
    psi = np.ascontiguousarray(pd["psi"], np.float64).reshape(-1)
    fields = {k: pd[k] for k in ("A", "V") if k in pd}
    return x, cells, psi, fields, fd


class DataSaver:
    """Per-step state files, as the reference's continuation data saver:
    ``<prefix>0000.vtu``, ``<prefix>0001.vtu``, ... in ``directory``, each
    with psi, the fields and the step's mu.  Call it with (index, x, mu) like
    the stepper's observer (it chains to ``observer`` when given)."""

    def __init__(self, x, cells, directory=".", prefix="out", A=None, V=None, observer=None):
        self.x, self.cells = np.asarray(x), np.asarray(cells)
        self.directory, self.prefix = directory, prefix
        self.A, self.V = A, V
        self.observer = observer
        self.index = 0
        self.paths = []

    def __call__(self, index, psi, mu):
        path = os.path.join(self.directory, f"{self.prefix}{self.index:04d}.vtu")
        write_vtu(path, self.x, self.cells, state_point_data(psi, self.A, self.V),
                  {"mu": float(mu), "step": float(index)})
        self.paths.append(path)
        self.index += 1
        if self.observer:
            self.observer(index, psi, mu)

    def close(self):
        if self.observer:
            self.observer.close()
