"""One world split into row slabs over gloo ranks on CPU (slabs.py).

Per-pass schedule: each rank runs the float oracle's passes on its own rows
only and gets the rows around them from its neighbours before each pass
that reads them; the eroded sediment's halo follows the back-trace reach,
with an all-gather when the reach leaves the halo.  Deep-halo schedule: one
exchange of the state's halo per block of steps, the passes computing a
shrinking range of rows, and a roll-back to the per-pass schedule when a
back-trace leaves the block's budget.  After the steps every rank's rows
equal one process stepping the whole world, bit for bit, and each schedule's
paths ran.
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

    def set_compute_rows(self, a, b):
        self.w.set_rows(a, b)

    def set_step(self, done):
        self.w.step_count = done

    def get_rows(self, field, y0, y1):
        return self.w.tex_rows(field, y0, y1)

    def set_rows(self, field, y0, rows):
        self.w.set_tex_rows(field, y0, rows)

    def max_reach_rows(self, y0=None, y1=None):
        y0 = self.lo if y0 is None else y0
        y1 = self.hi if y1 is None else y1
        v = self.w.tex_rows("vel", y0, y1)[..., 1]
        return int(np.ceil(np.max(np.abs(v)) * self.dt)) + 1 if v.size else 0


def rank_main(rank, nranks, port, halo_max, films, out, deep=0):
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
    k = 0
    while k < STEPS:
        if deep:
            k += slabs.deep_block(st, comm, k + 1, min(deep, STEPS - k), s, o.rain_period, sed_budget=3,
                                  halo_max=halo_max)
        else:
            slabs.slab_step(st, comm, k + 1, s, o.rain_period, halo_max=halo_max)
            k += 1
        st.w.step_count = k
    lo, hi = rows[rank]
    mine = {f: st.w.get(f)[lo:hi] for f in FIELDS}
    dist.destroy_process_group()
    out.put((rank, lo, hi, mine, comm.exchanges, comm.gathers, comm.deep_blocks, comm.rollbacks))


def run_ranks(nranks, halo_max, films, deep=0):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, nranks, port, halo_max, films, q, deep)) for r in range(nranks)]
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


def one_world(films):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    s, o = workload(O, films)
    w = O.OracleWorld(N, 32)
    w.set("rock", O.fbm(N, seed=1, frequency=1.0 / 16))
    w.step(s, o, STEPS)
    return w


def check_equal(res, w):
    """Every rank's rows equal the one world's; the ranks' counters summed."""
    covered = np.zeros(N, bool)
    tot = np.zeros(4, int)
    for rank, lo, hi, mine, *counters in res:
        tot += np.array(counters)
        covered[lo:hi] = True
        for f in FIELDS:
            bad = np.argwhere(mine[f] != w.get(f)[lo:hi])
            assert bad.size == 0, f"rank {rank} {f}: {len(bad)} cells differ"
    assert covered.all()
    return tot  # exchanges, gathers, deep blocks, roll-backs


@pytest.mark.parametrize("films", [True, False])
def test_two_ranks_equal_one_world(films):
    exchanges, gathers, _, _ = check_equal(run_ranks(2, 8, films), one_world(films))
    assert exchanges > 0
    # thin films send back-traces past the halo (the all-gather ran); with
    # uniform rain every step's sediment halo was a neighbour exchange
    assert (gathers > 0) == films


@pytest.mark.parametrize("nranks,films", [(2, False), (2, True), (3, False)])
def test_deep_halo_blocks_equal_one_world(nranks, films):
    """Blocks of up to 4 steps per exchange (10 halo rows a step at a
    back-trace budget of 3 rows, the uniform-rain workload's largest reach:
    two steps on 24-row slabs, one on 16-row ones)."""
    exchanges, gathers, deep_blocks, rollbacks = check_equal(run_ranks(nranks, 8, films, deep=4), one_world(films))
    assert exchanges > 0
    if films:  # thin-film back-traces overrun the budget: blocks redone pass by pass
        assert rollbacks > 0 and gathers > 0
    else:  # uniform rain: every block completed after its one exchange
        assert deep_blocks > 0 and rollbacks == 0 and gathers == 0


@pytest.mark.parametrize("nranks,deep", [(2, 0), (3, 4)])
def test_thread_ranks_equal_one_world(nranks, deep):
    """The same schedules with the ranks as threads of one process
    (slabs.ThreadComm: rows through host memory), thin films included: bit
    for bit one world."""
    import threading
    sys.path.insert(0, os.path.join(ROOT, "hydro-gen_gb300"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    import slabs
    films = True
    rows = slabs.slab_rows(N, nranks)
    s, o = workload(O, films)
    group = slabs.ThreadGroup(nranks, timeout=120.0)
    out, errors = [None] * nranks, []

    def rank_main(r):
        try:
            st = OracleSlab(O, rows, r, s, o, s.d_t)
            comm = slabs.ThreadComm(group, r, rows, N)
            k = 0
            while k < STEPS:
                if deep:
                    k += slabs.deep_block(st, comm, k + 1, min(deep, STEPS - k), s, o.rain_period, sed_budget=3)
                else:
                    slabs.slab_step(st, comm, k + 1, s, o.rain_period, halo_max=8)
                    k += 1
            lo, hi = rows[r]
            out[r] = {f: st.w.get(f)[lo:hi] for f in FIELDS}
        except BaseException as e:  # let the other ranks' waits end
            errors.append(e)
            group.abort()

    threads = [threading.Thread(target=rank_main, args=(r,)) for r in range(nranks)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    w = one_world(films)
    for r, (lo, hi) in enumerate(rows):
        for f in FIELDS:
            assert np.array_equal(out[r][f], w.get(f)[lo:hi]), (r, f)


def test_thread_rank_failure_ends_the_others_waits():
    """A rank that raises in the middle of a step (here: its stepper fails on
    the third flux pass) aborts the group; the other rank's next wait raises
    BrokenBarrierError at once instead of waiting out the timeout."""
    import threading
    import time
    sys.path.insert(0, os.path.join(ROOT, "hydro-gen_gb300"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    import slabs
    rows = slabs.slab_rows(N, 2)
    s, o = workload(O, False)
    group = slabs.ThreadGroup(2, timeout=60.0)
    seen = [None, None]

    class Failing(OracleSlab):
        flux_passes = 0

        def run_pass(self, name, layer):
            if name == "flux":
                self.flux_passes += 1
                if self.flux_passes == 3:
                    raise RuntimeError("planted failure")
            super().run_pass(name, layer)

    def rank_main(r):
        st = (Failing if r == 1 else OracleSlab)(O, rows, r, s, o, s.d_t)
        comm = slabs.ThreadComm(group, r, rows, N)
        try:
            for k in range(STEPS):
                slabs.slab_step(st, comm, k + 1, s, o.rain_period, halo_max=8)
        except BaseException as e:
            seen[r] = e
            group.abort()

    t0 = time.perf_counter()
    threads = [threading.Thread(target=rank_main, args=(r,)) for r in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=120)
    assert not any(t.is_alive() for t in threads)
    assert isinstance(seen[1], RuntimeError)
    assert isinstance(seen[0], threading.BrokenBarrierError)
    assert time.perf_counter() - t0 < 30.0  # well inside the 60 s timeout


@pytest.mark.parametrize("reach,expect", [(2, "exchange"), (50, "gather")])
def test_fused_slab_step_schedule(reach, expect):
    """slabs.fused_slab_step on two thread ranks with a stepper that records
    what it is asked: the rank's rows, a one-row exchange of height and flux,
    k_hydro, the eroded rock two rows deep, the agreed back-trace reach, the
    eroded sediment that deep (or the all-gather past the halo limit), then
    k_transport."""
    import threading
    sys.path.insert(0, os.path.join(ROOT, "hydro-gen_gb300"))
    import slabs
    n = 64
    rows = slabs.slab_rows(n, 2)
    group = slabs.ThreadGroup(2, timeout=60.0)
    logs, errors = [[], []], []

    class Recorder:
        def __init__(self, r):
            self.r = r

        def set_compute_rows(self, a, b):
            logs[self.r].append(("rows", a, b))

        def get_rows(self, tex, y0, y1):
            logs[self.r].append(("get", tex, y1 - y0))
            return np.zeros((y1 - y0, n, 4))

        def set_rows(self, tex, y0, data):
            logs[self.r].append(("set", tex, data.shape[0]))

        def fused_half(self, which):
            logs[self.r].append(("half", which))

        def max_reach_rows(self):
            return reach if self.r == 1 else 1

    def rank_main(r):
        try:
            slabs.fused_slab_step(Recorder(r), slabs.ThreadComm(group, r, rows, n), thermal=True, halo_max=8)
        except BaseException as e:
            errors.append(e)
            group.abort()

    threads = [threading.Thread(target=rank_main, args=(r,)) for r in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=60)
    assert not errors, errors
    for r in range(2):
        ev = logs[r]
        assert ev[0] == ("rows",) + rows[r]
        halves = [i for i, e in enumerate(ev) if e[0] == "half"]
        assert [ev[i][1] for i in halves] == [0, 1]
        before, between = ev[:halves[0]], ev[halves[0] + 1:halves[1]]
        assert ("set", "height", 1) in before and ("set", "flux", 1) in before
        assert ("set", "ero_rock", 2) in between
        if expect == "exchange":  # the agreed reach (the larger rank's) deep
            assert ("set", "ero_sed", reach) in between
        else:  # past the halo limit: every other rank's rows
            assert ("set", "ero_sed", rows[1 - r][1] - rows[1 - r][0]) in between
