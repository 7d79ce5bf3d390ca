"""Synthetic structured meshes for the benchmark workloads (numpy).

* :func:`square` -- unit square, ``s x s`` vertices, each square cut into two
  right triangles;
* :func:`cube` -- unit cube, ``m^3`` cubes, each cut into the 6 Kuhn
  tetrahedra sharing the (0,0,0)-(1,1,1) diagonal.

Interior vertices are jittered by ``U(-j h, j h)`` per coordinate, boundary
vertices only tangentially.  Random numbers come from splitmix64 in vertex-id
order (one draw per coordinate, used or not), followed by the initial state
``psi = 1 + U(-0.01, 0.01) + i U(-0.01, 0.01)`` per vertex.  The stream is
fully determined by the seed, so meshes are reproducible across languages.
"""
from __future__ import annotations

import numpy as np

_GOLD = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64_stream(seed: int, count: int) -> np.ndarray:
    """The first ``count`` outputs of splitmix64 seeded with ``seed``."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + _GOLD * np.arange(1, count + 1, dtype=np.uint64)
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def _uniform(bits: np.ndarray, lo, hi) -> np.ndarray:
    u = (bits >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    return lo + (hi - lo) * u


def square(s: int, seed: int, jitter: float = 0.1):
    """(x (N,3), cells (T,3) int32, psi (2N,)) for the jittered unit square."""
    N = s * s
    h = 1.0 / (s - 1)
    r = splitmix64_stream(seed, 2 * N + 2 * N)
    d = _uniform(r[: 2 * N], -jitter * h, jitter * h).reshape(N, 2)
    j, i = np.divmod(np.arange(N), s)
    x = np.zeros((N, 3))
    x[:, 0] = i * h + np.where((i > 0) & (i < s - 1), d[:, 0], 0.0)
    x[:, 1] = j * h + np.where((j > 0) & (j < s - 1), d[:, 1], 0.0)
    p = _uniform(r[2 * N :], -0.01, 0.01).reshape(N, 2)
    psi = np.empty(2 * N)
    psi[0::2] = 1.0 + p[:, 0]
    psi[1::2] = p[:, 1]
    jj, ii = np.meshgrid(np.arange(s - 1), np.arange(s - 1), indexing="ij")
    v00 = (ii + s * jj).ravel()
    v10, v01 = v00 + 1, v00 + s
    v11 = v01 + 1
    cells = np.empty((2 * v00.size, 3), np.int32)
    cells[0::2] = np.stack([v00, v10, v11], axis=1)
    cells[1::2] = np.stack([v00, v11, v01], axis=1)
    return x, cells, psi


_PERMS = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))


def cube(m: int, seed: int, jitter: float = 0.1):
    """(x (N,3), cells (T,4) int32, psi (2N,)) for the jittered unit cube."""
    n = m + 1
    N = n**3
    h = 1.0 / m
    r = splitmix64_stream(seed, 3 * N + 2 * N)
    d = _uniform(r[: 3 * N], -jitter * h, jitter * h).reshape(N, 3)
    v = np.arange(N)
    k, rem = np.divmod(v, n * n)
    j, i = np.divmod(rem, n)
    x = np.empty((N, 3))
    for ax, idx in enumerate((i, j, k)):
        x[:, ax] = idx * h + np.where((idx > 0) & (idx < m), d[:, ax], 0.0)
    p = _uniform(r[3 * N :], -0.01, 0.01).reshape(N, 2)
    psi = np.empty(2 * N)
    psi[0::2] = 1.0 + p[:, 0]
    psi[1::2] = p[:, 1]
    kk, jj, ii = np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij")
    ii, jj, kk = ii.ravel(), jj.ravel(), kk.ravel()
    base = ii + n * (jj + n * kk)
    top = (ii + 1) + n * ((jj + 1) + n * (kk + 1))
    cells = np.empty((6 * base.size, 4), np.int32)
    for q, perm in enumerate(_PERMS):
        o = np.zeros((3, base.size), np.int64)
        t = cells[q::6]
        t[:, 0] = base
        for s2 in range(2):
            o[perm[s2]] = 1
            t[:, 1 + s2] = (ii + o[0]) + n * ((jj + o[1]) + n * (kk + o[2]))
        t[:, 3] = top
    return x, cells, psi


def mvp_constant_curl(x: np.ndarray) -> np.ndarray:
    """A = 1/2 (-y, x, 0) per vertex (the field scaled by mu, B = (0,0,mu))."""
    A = np.zeros_like(x)
    A[:, 0] = -0.5 * x[:, 1]
    A[:, 1] = 0.5 * x[:, 0]
    return A


def mvp_stress(x: np.ndarray) -> np.ndarray:
    """A = 1/2 (-y, x, 0) + 0.05 sin(2 pi z) (1, 0, 0) per vertex."""
    A = mvp_constant_curl(x)
    A[:, 0] += 0.05 * np.sin(2.0 * np.pi * x[:, 2])
    return A
