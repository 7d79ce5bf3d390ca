"""Batched independent solves: many meshes (each with its own mu) in one
handle, and their distribution over ranks.

The GPU path solves the batch as the disjoint union of the systems (one
block-diagonal operator; every kernel covers all systems in one launch, see
``nls.set_systems``).  Across GPUs the systems are the shardable unit: each
rank takes a subset with no collective in the data path, and only the
per-system results are gathered at the end.
"""
from __future__ import annotations

import numpy as np

from . import meshgen


def union(meshes):
    """Disjoint union of meshes ``[(x (N_k,3), cells (T_k,c)), ...]``:
    returns (x, cells, vertex_offsets) with system k owning vertices
    [offsets[k], offsets[k+1])."""
    xs, cs, off = [], [], [0]
    for x, c in meshes:
        cs.append(np.asarray(c, np.int64) + off[-1])
        xs.append(np.asarray(x, np.float64))
        off.append(off[-1] + len(x))
    return np.concatenate(xs), np.concatenate(cs).astype(np.int32), np.asarray(off, np.int64)


def squares(sides, mus, seed0=1000):
    """The batch of jittered unit squares with ``sides[k]`` vertices per side
    (seed ``seed0 + k``): (x, cells, offsets, psi0, A, mu)."""
    meshes, psis = [], []
    for k, s in enumerate(sides):
        x, c, p = meshgen.square(int(s), seed0 + k)
        meshes.append((x, c))
        psis.append(p)
    x, c, off = union(meshes)
    return x, c, off, np.concatenate(psis), meshgen.mvp_constant_curl(x), np.asarray(mus, np.float64)


def config_squares(count=256, lo=33, hi=257, seed=1000):
    """Sides drawn uniformly from {lo..hi} and mu uniformly from [0, 1]
    (splitmix64 stream ``seed``), the batched-solve workload's sampling."""
    r = meshgen.splitmix64_stream(seed, 2 * count)
    u = (r >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    sides = lo + np.minimum((u[:count] * (hi - lo + 1)).astype(np.int64), hi - lo)
    return sides, u[count:]


def partition(weights, world):
    """Systems -> ranks by longest-processing-time: heaviest first onto the
    least-loaded rank (ties to the lower rank).  Returns one sorted index
    list per rank."""
    w = np.asarray(weights, np.float64)
    load = np.zeros(world)
    parts = [[] for _ in range(world)]
    for k in sorted(range(len(w)), key=lambda i: (-w[i], i)):
        r = int(np.argmin(load))
        parts[r].append(k)
        load[r] += w[k]
    return [sorted(p) for p in parts]


def split_state(x, offsets):
    """Per-system slices of a union state (2N interleaved)."""
    return [x[2 * offsets[k] : 2 * offsets[k + 1]] for k in range(len(offsets) - 1)]
