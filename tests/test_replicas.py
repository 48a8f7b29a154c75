"""The multi-rank side of bench.py on CPU: world_size-2 gloo ranks meet only
for the barrier and the timing reductions, and a batch's scenes are split
over the ranks with every scene on exactly one rank."""

import multiprocessing as mp
import os
import socket


SIZES = [2048, 65536, 30000, 4096, 4096, 12000, 9000, 50000, 2100, 33000]


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench

    w, r, _ = bench.dist_setup("gloo")
    got_max = bench.max_over_ranks(1.5 * (r + 1), w)
    got_sum = bench.sum_over_ranks(10.0 * (r + 1), w)
    bench.barrier(w)
    parts = bench.partition_scenes(SIZES, w)
    q.put((r, w, got_max, got_sum, parts))
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_and_partition():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    for _, w, mx, sm, parts in out:
        assert w == 2 and mx == 3.0 and sm == 30.0
        assert parts == out[0][4]  # every rank computes the same split
    parts = out[0][4]
    assert sorted(k for p in parts for k in p) == list(range(len(SIZES)))
    loads = [sum(SIZES[k] for k in p) for p in parts]
    assert max(loads) - min(loads) <= max(SIZES)


def test_partition_single_rank_keeps_everything():
    import bench

    assert bench.partition_scenes(SIZES, 1) == [list(range(len(SIZES)))]
    parts = bench.partition_scenes(SIZES, 4)
    assert sorted(k for p in parts for k in p) == list(range(len(SIZES)))
    assert all(p for p in parts)
