"""bench.py's multi-rank path on the CPU: two gloo ranks (the GPU pool runs
one GPU, so N > 1 is exercised here). Every rank steps its own replica; the
job time is the slowest rank's and the value counts every rank's points."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist            # noqa: E402
import torch.multiprocessing as mp          # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 10.0 + 5.0 * rank                    # rank 1 is the slower one
        slow = bench.allmax(dist, ms)
        q.put((rank, bench.dist_env(), slow, bench.job_value(world, 1000, 20, slow)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, env, slow, value in out:
        assert env == (rank, world, rank)
        assert slow == 15.0
        assert value == pytest.approx(2 * 1000 * 20 / 0.015 / 1e6)
    assert bench_single() == 10.0


def bench_single():
    import bench
    return bench.allmax(None, 10.0)


def _replica(rank, world, port, q):
    """One rank's replica: its own seeded scene, stepped on its own (the
    oracle stands in for the GPU step on this CPU-only host), no exchange;
    the ranks meet only in the timing reduction."""
    import hashlib
    import time

    import bench
    from fluids3_gb300 import scenes
    from oracle import oracle as O
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sc = scenes.dam_break(n=2000, seed=100 + rank)
        st = O.State.new(sc.params, sc.pos, sc.vel, sc.veval, sc.clr)
        t0 = time.perf_counter()
        O.run(sc.params, st, 3, 0.0)
        ms = (time.perf_counter() - t0) * 1e3
        slow = bench.allmax(dist, ms)
        digest = hashlib.sha256(st.pos.tobytes() + st.vel.tobytes() + st.veval.tobytes()).hexdigest()
        q.put((rank, digest, ms, slow, bench.job_value(world, sc.n, 3, slow)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_step_independently():
    """Replicas only: each of two gloo ranks steps its own scene; each final
    state equals the same scene stepped alone in this process (nothing
    crosses ranks but the timing), the job time is the slower rank's and
    the value counts both ranks' points."""
    import hashlib

    from fluids3_gb300 import scenes
    from oracle import oracle as O
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=180) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    slowest = max(ms for _, _, ms, _, _ in out)
    for rank, digest, ms, slow, value in out:
        sc = scenes.dam_break(n=2000, seed=100 + rank)
        st = O.State.new(sc.params, sc.pos, sc.vel, sc.veval, sc.clr)
        O.run(sc.params, st, 3, 0.0)
        assert digest == hashlib.sha256(st.pos.tobytes() + st.vel.tobytes() + st.veval.tobytes()).hexdigest()
        assert slow == pytest.approx(slowest)
        assert value == pytest.approx(world * sc.n * 3 / (slowest / 1e3) / 1e6)
    assert out[0][1] != out[1][1]   # different replicas, different states
