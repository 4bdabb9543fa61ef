"""The ragged batch split over ranks by area (hydrogen.shard_by_area), on CPU.

The assignment's properties on the 64-terrain manifest, and two gloo ranks
(127.0.0.1) that each step their share on the float oracle (terrains scaled
down 32x): together they step every terrain exactly once, with results equal
to one process stepping them all."""
import hashlib
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SCALE = 32  # oracle worlds of side / 32: 8 .. 64 cells
STEPS = 6


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def step_terrain(O, t, i):
    """A config-3 terrain's physics and rain on the float oracle; digest of its fields."""
    import math
    n = t["n"] // SCALE
    s = O.settings_config2()
    s.Kc = t["Kc"]
    s.Ks[0] = s.Ks[1] = t["Ks"]
    s.Kd[0] = s.Kd[1] = t["Kd"]
    s.Ke = t["Ke"]
    s.Kalpha[0] = s.Kalpha[1] = math.atan(t["talus_tan"])
    o = O.options(2, 1, 0.5, p=0.01, seed=t["seed"], terrain_id=i)
    w = O.OracleWorld(n, 32)
    w.set("rock", O.fbm(n, seed=t["seed"], frequency=1.0 / 8))
    w.step(s, o, STEPS)
    h = hashlib.sha1()
    for f in ("rock", "water", "sediment"):
        h.update(w.get(f).astype(np.float32).tobytes())
    return h.hexdigest()


def rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, os.path.join(ROOT, "hydro-gen_gb300"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch.distributed as dist
    import hydrogen as H
    import oracle as O
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ts = H.config3_terrains(count=64, seed=0)
    owner = H.shard_by_area([t["n"] for t in ts], world)
    mine = {i: step_terrain(O, ts[i], i) for i in range(len(ts)) if owner[i] == rank}
    owners = [None] * world
    dist.all_gather_object(owners, owner)
    shares = [None] * world
    dist.all_gather_object(shares, mine)
    dist.destroy_process_group()
    out.put((rank, owners, shares))


def test_shard_by_area_properties():
    sys.path.insert(0, os.path.join(ROOT, "hydro-gen_gb300"))
    import hydrogen as H
    ts = H.config3_terrains(count=64, seed=0)
    sides = [t["n"] for t in ts]
    area = [s * s for s in sides]
    for nranks in (1, 2, 3, 4, 8):
        owner = H.shard_by_area(sides, nranks)
        assert owner == H.shard_by_area(sides, nranks)  # every rank computes the same split
        assert len(owner) == len(sides) and all(0 <= r < nranks for r in owner)
        loads = [sum(a for a, r in zip(area, owner) if r == k) for k in range(nranks)]
        assert sum(loads) == sum(area)
        assert max(loads) <= sum(area) / nranks + max(area)  # greedy LPT bound
    assert H.shard_by_area(sides, 1) == [0] * len(sides)
    assert H.shard_by_area([], 4) == []
    with pytest.raises(ValueError):
        H.shard_by_area(sides, 0)


def test_two_gloo_ranks_step_the_batch_once():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    _, owners, shares = res[0]
    assert owners[0] == owners[1]
    done = {}
    for share in shares:
        assert not set(share) & set(done)  # no terrain stepped twice
        done.update(share)
    assert sorted(done) == list(range(64))
    sys.path.insert(0, os.path.join(ROOT, "hydro-gen_gb300"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import hydrogen as H
    import oracle as O
    ts = H.config3_terrains(count=64, seed=0)
    for i in (0, 17, 63):  # one process stepping the same terrains gets the same fields
        assert done[i] == step_terrain(O, ts[i], i)
