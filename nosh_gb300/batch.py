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


def squares(sides, mus, seed0=1000, seeds=None):
    """The batch of jittered unit squares with ``sides[k]`` vertices per side
    (seed ``seeds[k]``, default ``seed0 + k``): (x, cells, offsets, psi0, A,
    mu)."""
    meshes, psis = [], []
    if seeds is None:
        seeds = [seed0 + k for k in range(len(sides))]
    for k, s in enumerate(sides):
        x, c, p = meshgen.square(int(s), int(seeds[k]))
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


def solve_union(sides, mus, seeds, tol=1e-10, precision=None, repeats=1, timer=None):
    """Solve the squares ``sides`` (seeds ``seeds``, parameters ``mus``) as one
    batched handle on the GPU, from their initial states, to ``||F_s|| <=
    tol`` in every system.  The solve runs ``repeats`` times from the same
    initial states (the set-up is not repeated); ``timer``, when given, is
    called as ``timer(phase)`` with phase "start" / "stop" around each.
    Returns (per-system norms, the last solve's stats, the states)."""
    import nosh_gb300 as ng

    x, c, off, psi0, A, mu = squares(sides, mus, seeds=seeds)
    model = ng.nls(ng.mesh(x, c), A, -1.0, 1.0, 1.0, mu=0.0,
                   precision=ng.PREC_MIXED if precision is None else precision)
    model.set_systems(off, mu)
    st, psi = None, None
    for _ in range(repeats):
        psi = psi0.copy()
        if timer:
            timer("start")
        st = model.newton(psi, {"mu": 0.0}, tol=tol)
        if timer:
            timer("stop")
        if st["status"] != 0:
            raise RuntimeError(f"batched solve failed: {st}")
    return model.system_norms(), st, split_state(psi, off)


def sharded_solve(sides, mus, rank, world, seed0=1000, solve=None, gather=None):
    """The batched-solve workload sharded over ranks: rank ``rank`` of
    ``world`` takes ``partition(sides^2, world)[rank]`` (longest processing
    time by vertex count), solves those systems with ``solve(sides, mus,
    seeds)`` -- by default :func:`solve_union` on this rank's GPU -- and the
    per-system norms of every rank are gathered (``gather(obj) -> list`` of
    every rank's obj, by default ``torch.distributed.all_gather_object``).
    No collective touches the data path: the only exchange is that gather.
    Returns {system index: norm} over all systems on every rank."""
    sides = np.asarray(sides)
    parts = partition(sides.astype(np.float64) ** 2, world)
    mine = parts[rank]
    if solve is None:
        def solve(s, m, sd):
            return solve_union(s, m, sd)[0]
    norms = solve([int(sides[k]) for k in mine], [float(mus[k]) for k in mine], [seed0 + k for k in mine]) \
        if mine else []
    local = {int(k): float(v) for k, v in zip(mine, norms)}
    if world == 1:
        return local
    if gather is None:
        import torch.distributed as dist

        def gather(obj):
            out = [None] * world
            dist.all_gather_object(out, obj)
            return out
    merged = {}
    for g in gather(local):
        if set(g) & set(merged):
            raise RuntimeError("a system was solved by two ranks")
        merged.update(g)
    return merged
