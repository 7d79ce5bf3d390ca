"""The committed golden vectors (tests/golden/small_cases.npz, written by
tests/golden/make_golden.py) against the oracle and the reference's own
known-answer constants.

The fixture is what the GPU tests compare with; here it is pinned: the
oracle run now reproduces every array (integer arrays bit-exact, FP64 to
1e-13 relative), and on the reference's two test meshes its KEO sums are the
constants of test/keo.cpp:137-138 and :163-164.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, HERE)

import make_golden  # noqa: E402

GOLD = np.load(os.path.join(HERE, "small_cases.npz"))


@pytest.fixture(scope="module")
def fresh():
    return make_golden.generate()


def test_fixture_is_reproduced_by_the_oracle(fresh):
    assert sorted(fresh) == sorted(GOLD.files)
    for k in GOLD.files:
        a, b = fresh[k], GOLD[k]
        assert a.shape == b.shape and a.dtype == b.dtype, k
        if np.issubdtype(b.dtype, np.integer):
            np.testing.assert_array_equal(a, b, err_msg=k)
        else:
            scale = max(np.abs(b).max(), 1e-300)
            assert np.abs(a - b).max() <= 1e-13 * scale, k


@pytest.mark.parametrize("name,ones,even", [
    ("rect", 0.01262434246161348, 0.0063121712308067401),
    ("cube", 1.67083246311428e-4, 8.3541623155714007e-05),
])
def test_fixture_keo_matches_reference_constants(name, ones, even):
    # the real 2N form of a complex entry a is [[Re a, -Im a], [Im a, Re a]]:
    # 1'K1 sums 2 Re a over all entries and e'Ke (e = ones on the real
    # slots) sums Re a
    re = GOLD[f"{name}/keo"].real
    assert abs(2.0 * re.sum() - ones) < 1e-12
    assert abs(re.sum() - even) < 1e-12


def test_fixture_newton_state_solves_f():
    from oracle import oracle as O

    m = O.finish_mesh(GOLD["newton/x"], GOLD["newton/cells"])
    P = O.Problem(m, O.mvp_constant_curl(m.x))
    f = P.compute_f(GOLD["newton/psi"], 1.0, float(GOLD["newton/mu"]))
    assert np.linalg.norm(f) <= 1e-12
