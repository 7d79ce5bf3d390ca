"""Host logic of batched solves (no GPU): the union mesh, the workload
sampling, the rank partition, and a 2-rank gloo run that shards the systems
with no data-path collective and gathers the per-system results."""
import os

import numpy as np
import pytest


def test_union_offsets_and_cells():
    from nosh_gb300 import batch, meshgen

    a = meshgen.square(5, 1)
    b = meshgen.square(7, 2)
    x, c, off = batch.union([a[:2], b[:2]])
    assert list(off) == [0, 25, 74]
    assert x.shape == (74, 3) and c.shape == (len(a[1]) + len(b[1]), 3)
    assert c[: len(a[1])].max() < 25 and c[len(a[1]) :].min() >= 25
    np.testing.assert_array_equal(c[len(a[1]) :] - 25, b[1])


def test_config_sampling_is_deterministic_and_in_range():
    from nosh_gb300 import batch

    s1, m1 = batch.config_squares(256)
    s2, m2 = batch.config_squares(256)
    np.testing.assert_array_equal(s1, s2)
    np.testing.assert_array_equal(m1, m2)
    assert s1.min() >= 33 and s1.max() <= 257 and len(set(s1.tolist())) > 100
    assert m1.min() >= 0.0 and m1.max() < 1.0


def test_partition_balances_and_covers():
    from nosh_gb300 import batch

    sides, _ = batch.config_squares(256)
    w = sides.astype(float) ** 2
    for world in (1, 2, 4, 8):
        parts = batch.partition(w, world)
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(256))
        loads = [w[p].sum() for p in parts]
        assert max(loads) <= min(loads) + w.max()


def _cpu_solve(sides, mus, seeds):
    """Rank-local solve injected in place of the GPU one: the oracle's FP64
    CPU Newton-MINRES on each square, returning each system's ||F||."""
    from nosh_gb300 import meshgen
    from oracle import oracle as O

    norms = []
    for s, mu, seed in zip(sides, mus, seeds):
        x, c, psi = meshgen.square(int(s), int(seed))
        m = O.finish_mesh(x, c)
        P = O.Problem(m, O.mvp_constant_curl(m.x))
        st = O.CpuSolver(P).newton(psi, mu, tol=1e-10)
        assert st["status"] == 0, st
        norms.append(float(np.linalg.norm(P.compute_f(psi, 1.0, mu))))
    return norms


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    from nosh_gb300 import batch

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sides, mus = batch.config_squares(12, lo=5, hi=17)
    merged = batch.sharded_solve(sides, mus, rank, world, solve=_cpu_solve)
    if rank == 0:
        out.put(sorted(merged.items()))
    dist.destroy_process_group()


def test_two_rank_sharding_gathers_every_system():
    import multiprocessing as mp
    import socket

    pytest.importorskip("torch")
    from nosh_gb300 import batch

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [k for k, _ in merged] == list(range(12))
    assert all(v <= 1e-10 for _, v in merged)
    # the same function on one rank solves the same systems to the same norms
    sides, mus = batch.config_squares(12, lo=5, hi=17)
    single = batch.sharded_solve(sides, mus, 0, 1, solve=_cpu_solve)
    assert sorted(single) == list(range(12))
    for k, v in merged:
        assert abs(v - single[k]) <= 1e-14


def test_sharded_solve_rejects_overlapping_shards():
    from nosh_gb300 import batch

    sides, mus = batch.config_squares(4, lo=5, hi=9)

    def fake_solve(s, m, sd):
        return [0.0] * len(s)

    # a gather that returns this rank's shard twice: every system twice
    with pytest.raises(RuntimeError):
        batch.sharded_solve(sides, mus, 0, 2, solve=fake_solve, gather=lambda obj: [obj, obj])
