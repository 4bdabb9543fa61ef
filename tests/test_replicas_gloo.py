"""The multi-rank path of bench.py on CPU: two gloo ranks (127.0.0.1), each a
replica with its own terrain id.  Checks the job time (slowest rank), the
whole-job throughput and that replicas draw independent rain streams."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch.distributed as dist
    import bench
    import oracle as O
    r, ws, local = bench.dist_env()
    dist.init_process_group("gloo", rank=r, world_size=ws)
    slowest = bench.max_over_ranks(dist, 1.5 + r, "cpu")  # rank r "took" 1.5 + r seconds
    word = O.rain_word(17, 5, 3, r, 0)  # the replica's terrain id keys its rain
    words = [None] * ws
    dist.all_gather_object(words, word)
    dist.destroy_process_group()
    out.put((r, slowest, words))


def test_two_gloo_replicas():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, slowest, words in res:
        assert slowest == 2.5
        assert words[0] != words[1]
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_throughput(2, 4096 * 4096, 500, 0.25) == 2 * 4096 * 4096 * 500 / 0.25
