"""One world split into row slabs over two gloo ranks on CPU (slabs.py).

Each rank runs the float oracle's passes on its own rows only and gets the
rows around them from its neighbour before each pass that reads them; the
eroded sediment's halo follows the back-trace reach, with an all-gather when
the reach leaves the halo.  After the steps every rank's rows equal one
process stepping the whole world, bit for bit, and both sediment paths ran.
"""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
N, STEPS = 48, 12
FIELDS = ("rock", "water", "sediment", "flux_l", "flux_r", "flux_t", "flux_b", "vel_u", "vel_v")


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def workload(O, films):
    """Talus slippage and smoothing on a small world, with dense Bernoulli rain
    (thin films, back-traces across the grid) or uniform rain (every cell
    keeps water, back-traces of a cell or two)."""
    s = O.settings_config2()
    s.Kspeed[1] = 2.0
    o = O.options(2, 1, 0.5, p=0.05, seed=3) if films else O.options(1, 1, 0.01)
    return s, o


class OracleSlab:
    """A slab stepper on the float oracle: passes restricted to own rows."""

    def __init__(self, O, rows, rank, s, o, dt):
        self.O, self.s, self.o, self.dt = O, s, o, dt
        self.lo, self.hi = rows[rank]
        self.w = O.OracleWorld(N, 32)
        self.w.set("rock", O.fbm(N, seed=1, frequency=1.0 / 16))
        self.w.set_rows(self.lo, self.hi)

    def run_pass(self, name, layer):
        self.w.run_pass(name, self.s, self.o, layer)

    def get_rows(self, field, y0, y1):
        return self.w.tex_rows(field, y0, y1)

    def set_rows(self, field, y0, rows):
        self.w.set_tex_rows(field, y0, rows)

    def max_reach_rows(self):
        v = self.w.tex_rows("vel", self.lo, self.hi)[..., 1]
        return int(np.ceil(np.max(np.abs(v)) * self.dt)) + 1 if v.size else 0


def rank_main(rank, nranks, port, halo_max, films, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(nranks))
    sys.path.insert(0, os.path.join(ROOT, "hydro-gen_gb300"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch.distributed as dist
    import oracle as O
    import slabs
    dist.init_process_group("gloo", rank=rank, world_size=nranks)
    rows = slabs.slab_rows(N, nranks)
    s, o = workload(O, films)
    st = OracleSlab(O, rows, rank, s, o, s.d_t)
    comm = slabs.SlabComm(dist, rank, nranks, rows, N)
    for k in range(STEPS):
        st.w.step_count = k
        slabs.slab_step(st, comm, k + 1, s, o.rain_period, halo_max=halo_max)
        st.w.step_count = k + 1
    lo, hi = rows[rank]
    mine = {f: st.w.get(f)[lo:hi] for f in FIELDS}
    dist.destroy_process_group()
    out.put((rank, lo, hi, mine, comm.exchanges, comm.gathers))


def run_ranks(nranks, halo_max, films):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, nranks, port, halo_max, films, q)) for r in range(nranks)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return res


def test_slab_rows():
    sys.path.insert(0, os.path.join(ROOT, "hydro-gen_gb300"))
    import slabs
    assert slabs.slab_rows(10, 3) == [(0, 4), (4, 7), (7, 10)]
    assert slabs.slab_rows(8, 1) == [(0, 8)]
    with pytest.raises(ValueError):
        slabs.slab_rows(4, 5)


@pytest.mark.parametrize("films", [True, False])
def test_two_ranks_equal_one_world(films):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    res = run_ranks(2, 8, films)
    s, o = workload(O, films)
    w = O.OracleWorld(N, 32)
    w.set("rock", O.fbm(N, seed=1, frequency=1.0 / 16))
    w.step(s, o, STEPS)
    exchanges = gathers = 0
    covered = np.zeros(N, bool)
    for rank, lo, hi, mine, ex, ga in res:
        exchanges, gathers = exchanges + ex, gathers + ga
        covered[lo:hi] = True
        for f in FIELDS:
            ref = w.get(f)[lo:hi]
            bad = np.argwhere(mine[f] != ref)
            assert bad.size == 0, f"rank {rank} {f}: {len(bad)} cells differ"
    assert covered.all()
    assert exchanges > 0
    # thin films send back-traces past the halo (the all-gather ran); with
    # uniform rain every step's sediment halo was a neighbour exchange
    assert (gathers > 0) == films
