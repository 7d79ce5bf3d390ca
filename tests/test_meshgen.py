"""The product's numpy mesh generator reproduces the oracle's C generator
bit for bit (coordinates, cells, initial state)."""
import numpy as np
import pytest

from nosh_gb300 import meshgen
from oracle import oracle as O


@pytest.mark.parametrize("s,seed", [(5, 1), (17, 7), (65, 1)])
def test_square_matches_oracle(s, seed):
    a = meshgen.square(s, seed)
    b = O.gen_square(s, seed)
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)


@pytest.mark.parametrize("m,seed", [(2, 3), (6, 11), (24, 2)])
def test_cube_matches_oracle(m, seed):
    a = meshgen.cube(m, seed)
    b = O.gen_cube(m, seed)
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)


def test_sizes_match_the_configs():
    x, c, _ = meshgen.square(65, 1)
    assert x.shape[0] == 4225 and c.shape[0] == 8192
    x, c, _ = meshgen.cube(48, 4)
    assert x.shape[0] == 117649 and c.shape[0] == 663552


def test_edges_count_formula():
    # 3-D Kuhn: 3m(m+1)^2 + 3m^2(m+1) + m^3 edges
    m = 6
    x, c, _ = meshgen.cube(m, 1)
    mesh = O.finish_mesh(x, c)
    assert mesh.E == 3 * m * (m + 1) ** 2 + 3 * m * m * (m + 1) + m**3


def test_numpy_modules_do_not_map_the_cuda_library():
    """The CPU arm of the benchmark builds its meshes with meshgen; importing
    it (and batch) must not map libnosh_gb300.so into the process."""
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys; sys.path.insert(0, sys.argv[1]); "
            "from nosh_gb300 import meshgen, batch; meshgen.cube(2, 1); "
            "print(open('/proc/self/maps').read())")
    out = subprocess.run([sys.executable, "-c", code, root], capture_output=True, text=True, check=True).stdout
    assert "libnosh_gb300" not in out
    code_lib = ("import sys; sys.path.insert(0, sys.argv[1]); import nosh_gb300 as ng; ng.lib(); "
                "print(open('/proc/self/maps').read())")
    out = subprocess.run([sys.executable, "-c", code_lib, root], capture_output=True, text=True, check=True).stdout
    assert "libnosh_gb300" in out
