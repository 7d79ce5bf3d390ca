"""Writes ``small_cases.npz``: inputs and oracle outputs of the hot path on
four small meshes, the committed golden vectors of the parity tests.

Cases: the reference's two known-answer meshes ("rectanglesmall", 4 vertices;
"cubesmall", 8 vertices, as rebuilt by the oracle from test/keo.cpp and
test/mesh.cpp), a jittered 17 x 17 triangle square (seed 7) and a jittered
6^3-cube tetrahedral mesh (seed 11).  Per case, with A = 1/2 (-y, x, 0),
V = -1, thickness 1, g = 1:

* inputs: points, cells, A, a seeded state ``psi`` (1 + 0.2 N(0,1) noise on
  the real part, 0.2 N(0,1) on the imaginary part) and a seeded direction
  ``v``;
* the KEO values (complex CSR order: row_ptr / cols) at mu = 0.01 and
  mu = 7 (the series and the sincos branch of the edge phases), dK/dmu at
  mu = 0.01;
* at mu = 0.01: F(psi), J(psi) v, dF/dmu and dF/dg, the Gibbs energy and
  the row-sum scale of |J|;
* the square only: a converged state of F = 0 at mu = 0.5 (exact-LU Newton
  to 1e-12 from the oracle's seeded start) and that start.

Run from the repository root: ``python tests/golden/make_golden.py``.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

MU, MU_LARGE, G = 0.01, 7.0, 1.0
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "small_cases.npz")


def meshes():
    yield "rect", O.rectanglesmall()
    yield "cube", O.cubesmall()
    x, c, _ = O.gen_square(17, 7)
    yield "square17", O.finish_mesh(x, c)
    x, c, _ = O.gen_cube(6, 11)
    yield "cube6", O.finish_mesh(x, c)


def case_arrays(name, m, seed):
    A = O.mvp_constant_curl(m.x)
    P = O.Problem(m, A)
    rng = np.random.default_rng(seed)
    psi = np.zeros(2 * m.N)
    psi[0::2] = 1.0
    psi += 0.2 * rng.standard_normal(psi.size)
    v = rng.standard_normal(2 * m.N)
    out = {
        "x": m.x,
        "cells": m.cells.astype(np.int32),
        "A": A,
        "psi": psi,
        "v": v,
        "row_ptr": P.row_ptr,
        "cols": P.cols,
        "keo": P.keo_values(MU),
        "keo_large": P.keo_values(MU_LARGE),
        "dkeo": P.dkeo_values(MU),
        "f": P.compute_f(psi, G, MU),
        "jv": P.jac_apply(psi, G, MU, v),
        "dfdmu": P.dfdp(psi, G, MU, "mu"),
        "dfdg": P.dfdp(psi, G, MU, "g", deriv_param="mu"),
        "energy": np.array(P.energy(psi)),
        "jscale": np.array(np.abs(P.jac_csr_real(psi, G, MU)).sum(axis=1).max()),
    }
    return {f"{name}/{k}": np.asarray(a) for k, a in out.items()}


def converged_square():
    x, c, psi0 = O.gen_square(9, 1)
    m = O.finish_mesh(x, c)
    P = O.Problem(m, O.mvp_constant_curl(m.x))
    ref, _ = O.newton_exact(P, psi0, G, 0.5, tol=1e-12)
    return {"newton/x": m.x, "newton/cells": m.cells.astype(np.int32), "newton/psi0": psi0,
            "newton/psi": ref, "newton/mu": np.array(0.5)}


def generate():
    arrays = {"mu": np.array(MU), "mu_large": np.array(MU_LARGE), "g": np.array(G)}
    for k, (name, m) in enumerate(meshes()):
        arrays.update(case_arrays(name, m, 100 + k))
    arrays.update(converged_square())
    return arrays


if __name__ == "__main__":
    np.savez_compressed(OUT, **generate())
    print(OUT, os.path.getsize(OUT), "bytes")
