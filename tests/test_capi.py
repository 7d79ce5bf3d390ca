"""C-ABI checks that need no GPU: the library loads, exports every entry
point ``include/nosh_gb300.h`` declares, and reports the missing GPU as an
error instead of falling back to the CPU."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "nosh_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nosh_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_boundary():
    names = declared_symbols()
    for required in ("nosh_mesh_create", "nosh_keo_set_parameters", "nosh_jacobian_apply",
                     "nosh_nls_compute_f", "nosh_keo_regularized_apply", "nosh_newton_solve"):
        assert required in names


def test_library_exports_every_declared_symbol():
    import nosh_gb300 as ng

    lib = ng.lib()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_library_is_in_tree():
    import nosh_gb300 as ng

    assert os.path.dirname(ng.LIB_PATH) == os.path.join(ROOT, "nosh_gb300")


def test_no_gpu_is_an_error_not_a_fallback():
    import numpy as np
    import nosh_gb300 as ng

    if ng.device_count() > 0:
        pytest.skip("a GPU is present")
    x = np.zeros((3, 3))
    c = np.array([[0, 1, 2]], np.int32)
    with pytest.raises(ng.NoshError) as e:
        ng.mesh(x, c)
    assert e.value.code == ng.ERR_CUDA


@pytest.mark.parametrize("cells,nv,code", [
    ([[0, 1, 3]], 3, "ERR_INVALID"),        # vertex index out of range
    ([[0, -1, 2]], 3, "ERR_INVALID"),       # negative vertex index
    ([[0, 1, 1]], 3, "ERR_MESH"),           # a triangle repeating a vertex
    ([[0, 1, 2, 0]], 4, "ERR_MESH"),        # a tetrahedron repeating a vertex
    (np.zeros((0, 3), np.int32), 3, "ERR_INVALID"),  # no cells
])
def test_malformed_mesh_is_rejected_on_the_host(cells, nv, code):
    # nosh_mesh_create validates the description before it needs a device,
    # so these codes are the same with or without a GPU
    import nosh_gb300 as ng

    x = np.zeros((nv, 3))
    with pytest.raises(ng.NoshError) as e:
        ng.mesh(x, np.asarray(cells, np.int32))
    assert e.value.code == getattr(ng, code)


def test_cell_type_is_checked_by_the_abi():
    import ctypes as C

    import nosh_gb300 as ng

    x = np.zeros((3, 3))
    c = np.array([0, 1], np.int32)
    h = C.c_void_p()
    rc = ng.lib().nosh_mesh_create(x.ctypes.data_as(C.c_void_p), C.c_int64(3), c.ctypes.data_as(C.c_void_p),
                                   C.c_int64(1), 2, C.byref(h))
    assert rc == ng.ERR_INVALID and not h.value


def test_version():
    import nosh_gb300 as ng

    assert ng.lib().nosh_version() >= 100
