"""The rounding bound of the mixed path's residual update, on the CPU.

Close to convergence a Newton step's residual takes K dx from an FP32
product of the FP32 update with the FP32 KEO (K rounded per component).  Its
deviation from the exact product is bounded by
e = 3 (n_max + 1) 2^-24 R ||dx||_2, n_max the largest off-diagonal row
length and R the largest row sum of |K|.  Here the FP32 product is simulated
with every multiply and add rounded to FP32 (one rounding more per term than
the kernel's fused multiply-adds), over the oracle's KEO at a few meshes,
fields and update shapes, and its error against the FP64 product of the same
FP32 update stays within e.
"""
import numpy as np
import pytest

from oracle import oracle as O


def _offdiag(P, mu):
    vals = P.keo_values(mu)
    rp, ci = P.row_ptr, P.cols
    rows = np.repeat(np.arange(P.m.N), np.diff(rp))
    keep = ci != rows
    return rows[keep], ci[keep], vals[keep]


def _fp32_product(rows, cols, k32, dx32, N):
    """Row by row, in column order, every operation rounded to FP32."""
    order = np.lexsort((cols, rows))
    rows, cols, k32 = rows[order], cols[order], k32[order]
    counts = np.bincount(rows, minlength=N)
    nmax = int(counts.max())
    start = np.concatenate([[0], np.cumsum(counts)[:-1]])
    slot = np.arange(rows.size) - start[rows]
    a = np.zeros((N, nmax), np.float32)
    b = np.zeros((N, nmax), np.float32)
    x = np.zeros((N, nmax), np.float32)
    y = np.zeros((N, nmax), np.float32)
    a[rows, slot] = k32.real
    b[rows, slot] = k32.imag
    x[rows, slot] = dx32.real[cols]
    y[rows, slot] = dx32.imag[cols]
    sr = np.zeros(N, np.float32)
    si = np.zeros(N, np.float32)
    for k in range(nmax):
        sr = sr + a[:, k] * x[:, k]
        sr = sr - b[:, k] * y[:, k]
        si = si + a[:, k] * y[:, k]
        si = si + b[:, k] * x[:, k]
    return sr.astype(np.float64) + 1j * si.astype(np.float64), nmax


@pytest.mark.parametrize("name,mu", [("cube10", 0.5), ("cube10", 7.0), ("square33", 0.1)])
@pytest.mark.parametrize("shape", ["noise", "smooth", "aligned"])
def test_fp32_update_product_within_bound(name, mu, shape):
    if name == "cube10":
        x, c, _ = O.gen_cube(10, 3)
    else:
        x, c, _ = O.gen_square(33, 1)
    m = O.finish_mesh(x, c)
    P = O.Problem(m, O.mvp_constant_curl(m.x))
    rows, cols, k = _offdiag(P, mu)
    k32 = (k.real.astype(np.float32) + 1j * k.imag.astype(np.float32)).astype(np.complex64)
    rng = np.random.default_rng(7)
    N = m.N
    if shape == "noise":
        d = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    elif shape == "smooth":
        d = np.exp(1j * 3.0 * m.x[:, 0]) * (1.0 + m.x[:, 1])
    else:
        # every term of a row with the same sign: the product's terms do not
        # cancel, the sum of |K_ij||dx_j| is as large as the row allows
        d = np.ones(N) * (1.0 + 0.5j)
    dx32 = (1e-6 * d).astype(np.complex64)
    got, nmax = _fp32_product(rows, cols, k32, dx32, N)
    exact = np.zeros(N, np.complex128)
    np.add.at(exact, rows, k * dx32[cols].astype(np.complex128))
    R = np.bincount(rows, weights=np.abs(k), minlength=N).max()
    norm_dx = np.linalg.norm(dx32.astype(np.complex128))
    e = 3.0 * (nmax + 1) * 2.0**-24 * R * norm_dx
    err = np.linalg.norm(got - exact)
    assert err <= e, (err, e)
    # the worst case the constant rests on, sqrt(2) (2 n_max + 1) u R ||dx||,
    # lies below e
    assert np.sqrt(2.0) * (2 * nmax + 1) <= 3.0 * (nmax + 1)
