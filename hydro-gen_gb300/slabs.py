"""Row-slab decomposition of one world over ranks: the schedule of one step.

The reference dispatches every pass over the whole grid at once
(src/erosion.cpp:92-101, 158-200).  Split over R ranks, rank r owns rows
[lo_r, hi_r) of an n x n world and computes only those; before each pass it
needs its neighbours' rows of the fields that pass reads around a cell:

  pass                     reads outside the cell            halo rows
  rain                     nothing                           0
  hydro_flux               total height, flux (4-nbhd)       1 of height and flux
  hydro_erosion            total height (4-nbhd, normal)     1 of height
  sediment_transport       eroded sediment at the back-trace the back-trace's reach
  thermal_erosion (layer)  total height (8-nbhd)             1 of height
  thermal_transport        outflows (8-nbhd)                 1 of both outflow maps
  smoothing                total height (4-nbhd)             1 of height

The sediment back-trace reach |v| dt is unbounded (velocity divides by the
water depth), so after the flux pass every rank takes the largest reach over
its rows, the ranks agree on the maximum (an all-reduce), and the eroded
sediment's halo is exchanged that deep when it fits inside the neighbours'
slabs and `halo_max`, else every rank gathers the whole field (all-gather):
the fallback the unbounded reach needs.  Halos come from the two neighbours
only; no other data moves.

`deep_block` trades the per-pass exchanges for one exchange every T steps:
each rank receives D rows of the state from each neighbour, D the sum of
the read radii of the block's passes (the sediment pass counted at a fixed
back-trace budget), and every pass computes the rows that its inputs still
determine, a range that shrinks by the pass's radius; the own rows come out
as one world's.  Before each sediment pass the ranks agree on the largest
back-trace reach over the rows it computes (all-reduce); above the budget,
every rank restores its rows from the block's start and steps the block
with the per-pass schedule instead.

The schedule drives any `stepper` that runs one pass over a row range and
reads and writes rows of a field (`run_pass`, `set_compute_rows`,
`get_rows`, `set_rows`, `max_reach_rows`, `set_step`) through a `comm` that
moves row blocks between ranks: `SlabComm` (torch.distributed, ranks as
processes; gloo on CPU, NCCL between GPUs) or `ThreadComm` (ranks as threads
of one process, rows through host memory).  `GpuSlabStepper` steps a rank's
rows with the library's per-pass kernels (hg_set_rows, hg_pass,
hg_world_rows); `fused_slab_step` steps them with its two fused kernels
instead (hg_fused_pass), exchanging the hand-off between them.  The tests
drive the schedules with the float oracle's passes on gloo ranks and on
threads (tests/test_slabs_gloo.py) and with GPU steppers on threads
(tests/test_gpu_slabs.py), bit for bit against one world stepped whole.
"""
import threading

import numpy as np

# (pass, layer, [(field, halo rows or "reach"), ...]) in the step's order
STEP_PLAN = [
    ("rain", 0, []),
    ("flux", 0, [("height", 1), ("flux", 1)]),
    ("erosion", 0, [("height", 1)]),
    ("sediment", 0, [("sed", "reach")]),
    ("thermal_flux", 0, [("height", 1)]),
    ("thermal_transport", 0, [("thc", 1), ("thd", 1)]),
    ("thermal_flux", 1, [("height", 1)]),
    ("thermal_transport", 1, [("thc", 1), ("thd", 1)]),
    ("smoothing", 0, [("height", 1)]),
]


# rows a pass reads around the rows it writes (the sediment pass: its
# back-trace reach, bounded per block by the caller's budget)
PASS_RADIUS = {"rain": 0, "flux": 1, "erosion": 1, "thermal_flux": 1, "thermal_transport": 1, "smoothing": 1}
# the carried state (the thermal outflows are rewritten before every read)
STATE_TEXTURES = ("height", "flux", "vel", "sed")


def slab_rows(n, nranks):
    """Row ranges [lo, hi) of an even split of n rows over nranks ranks."""
    if nranks < 1 or nranks > n:
        raise ValueError("need 1 <= ranks <= rows")
    base, extra = divmod(n, nranks)
    out, lo = [], 0
    for r in range(nranks):
        hi = lo + base + (1 if r < extra else 0)
        out.append((lo, hi))
        lo = hi
    return out


def passes_of_step(step1, settings, rain_period, rain_on=True):
    """The passes one step runs (the reference's cadence and the identity
    passes it skips: a talus layer with no slippage, smoothing with
    Kspeed[1] == 0): the plan's entries for step number step1 (1-based)."""
    out = []
    for name, layer, halos in STEP_PLAN:
        if name == "rain" and not (rain_on and rain_period > 0 and step1 % rain_period == 0):
            continue
        if name.startswith("thermal") and settings.Kspeed[layer] == 0.0:
            continue
        if name == "smoothing" and settings.Kspeed[1] == 0.0:
            continue
        out.append((name, layer, halos))
    return out


class SlabComm:
    """Halo exchange and gather of row blocks between the ranks of a slab
    decomposition (torch.distributed: buffers on the current GPU under NCCL,
    in host memory under gloo)."""

    def __init__(self, dist, rank, nranks, rows, n, channels=4):
        import torch
        self.torch = torch
        self.dist = dist
        self.rank, self.nranks, self.rows, self.n, self.ch = rank, nranks, rows, n, channels
        self.min_rows = min(hi - lo for lo, hi in rows)
        # NCCL moves device buffers, gloo host ones
        nccl = dist.is_initialized() and dist.get_backend() == "nccl"
        self.dev = torch.device("cuda", torch.cuda.current_device()) if nccl else torch.device("cpu")
        self.gathers = 0
        self.exchanges = 0
        self.deep_blocks = 0  # blocks of steps after one exchange
        self.rollbacks = 0    # blocks redone pass by pass (a back-trace beyond the budget)

    def agree_max(self, value):
        t = self.torch.tensor([float(value)], dtype=self.torch.float64, device=self.dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def exchange(self, stepper, field, depth):
        """Refresh `depth` rows on each side of the own slab from the two
        neighbours (depth <= the smallest slab): point-to-point, one block
        each way per neighbour, nothing to the other ranks."""
        torch, dist = self.torch, self.dist
        lo, hi = self.rows[self.rank]
        reqs, recv = [], []
        for nb, send_rows, recv_at in ((self.rank - 1, (lo, lo + depth), lo - depth),
                                       (self.rank + 1, (hi - depth, hi), hi)):
            if 0 <= nb < self.nranks:
                out = torch.from_numpy(np.ascontiguousarray(stepper.get_rows(field, *send_rows))).to(self.dev)
                inc = torch.empty_like(out)
                reqs += [dist.isend(out, nb), dist.irecv(inc, nb)]
                recv.append((recv_at, inc))
        for r in reqs:
            r.wait()
        for at, inc in recv:
            stepper.set_rows(field, at, inc.cpu().numpy())
        self.exchanges += 1

    def gather(self, stepper, field):
        """Every rank receives every row of the field."""
        torch = self.torch
        lo, hi = self.rows[self.rank]
        h = max(b - a for a, b in self.rows)
        blk = np.zeros((h, self.n, self.ch))
        blk[: hi - lo] = stepper.get_rows(field, lo, hi)
        mine = torch.from_numpy(blk).to(self.dev)
        allb = [torch.empty_like(mine) for _ in range(self.nranks)]
        self.dist.all_gather(allb, mine)
        for r, (a, b) in enumerate(self.rows):
            if r != self.rank:
                stepper.set_rows(field, a, allb[r][: b - a].cpu().numpy())
        self.gathers += 1


def slab_step(stepper, comm, step1, settings, rain_period, halo_max=8, rain_on=True):
    """One step of the owned rows: each pass after the halos it reads."""
    lo, hi = comm.rows[comm.rank]
    stepper.set_step(step1 - 1)
    stepper.set_compute_rows(lo, hi)
    for name, layer, halos in passes_of_step(step1, settings, rain_period, rain_on):
        for field, depth in halos:
            if depth == "reach":
                reach = int(comm.agree_max(stepper.max_reach_rows()))
                if reach <= min(halo_max, comm.min_rows):
                    if reach > 0:
                        comm.exchange(stepper, field, reach)
                else:
                    comm.gather(stepper, field)
            else:
                comm.exchange(stepper, field, depth)
        stepper.run_pass(name, layer)


def fused_slab_step(stepper, comm, thermal=True, halo_max=8):
    """One step of the owned rows with the two fused kernels (whole tile rows:
    slabs of multiples of 16 rows; no smoothing).  k_hydro reads its tile's
    total height and flux one row around; k_transport reads the eroded rock
    two rows around (the talus passes, when on) and the eroded sediment at
    the back-traces (an exchange as deep as they reach, else the all-gather)."""
    lo, hi = comm.rows[comm.rank]
    stepper.set_compute_rows(lo, hi)
    comm.exchange(stepper, "height", 1)
    comm.exchange(stepper, "flux", 1)
    stepper.fused_half(0)
    if thermal:
        comm.exchange(stepper, "ero_rock", 2)
    reach = int(comm.agree_max(stepper.max_reach_rows()))
    if reach <= min(halo_max, comm.min_rows):
        if reach > 0:
            comm.exchange(stepper, "ero_sed", reach)
    else:
        comm.gather(stepper, "ero_sed")
    stepper.fused_half(1)


def block_depth(plans, sed_budget):
    """Halo rows a block of steps needs: the read radii of its passes."""
    return sum(sed_budget if name == "sediment" else PASS_RADIUS[name] for plan in plans for name, _, _ in plan)


def deep_block(stepper, comm, step1, nsteps, settings, rain_period, sed_budget=2, halo_max=8, rain_on=True):
    """Steps step1 .. step1 + nsteps - 1 of the owned rows after one halo
    exchange (as many steps per exchange as the smallest slab allows, at
    least one); returns the number of steps done.  A back-trace beyond
    `sed_budget` rows sends every rank back to the block's start and through
    slab_step (per-pass exchanges, `halo_max` as there)."""
    lo, hi = comm.rows[comm.rank]
    n = comm.n
    plans = []
    for k in range(nsteps):
        p = passes_of_step(step1 + k, settings, rain_period, rain_on)
        if block_depth(plans + [p], sed_budget) > comm.min_rows:
            break
        plans.append(p)
    if not plans:  # not even one step's halo fits a slab
        slab_step(stepper, comm, step1, settings, rain_period, halo_max, rain_on)
        return 1
    depth = block_depth(plans, sed_budget)
    saved = {f: stepper.get_rows(f, lo, hi) for f in STATE_TEXTURES}
    for f in STATE_TEXTURES:
        comm.exchange(stepper, f, depth)
    a, b = max(0, lo - depth), min(n, hi + depth)  # rows whose inputs are known

    def shrink(r):  # the grid's own edges need no rows beyond them
        return (a if a == 0 else a + r), (b if b == n else b - r)

    for k, plan in enumerate(plans):
        stepper.set_step(step1 + k - 1)
        for name, layer, _ in plan:
            if name == "sediment":
                na, nb = shrink(sed_budget)
                reach = int(comm.agree_max(stepper.max_reach_rows(na, nb)))
                if reach > sed_budget:  # every rank sees the same maximum
                    for f, rows in saved.items():
                        stepper.set_rows(f, lo, rows)
                    comm.rollbacks += 1
                    for j in range(len(plans)):
                        slab_step(stepper, comm, step1 + j, settings, rain_period, halo_max, rain_on)
                    return len(plans)
            else:
                na, nb = shrink(PASS_RADIUS[name])
            a, b = na, nb
            stepper.set_compute_rows(a, b)
            stepper.run_pass(name, layer)
    assert a <= lo and b >= hi
    stepper.set_compute_rows(lo, hi)
    comm.deep_blocks += 1
    return len(plans)


class GpuSlabStepper:
    """A rank's rows stepped by the library's one-layer per-pass kernels: a
    world the size of the whole grid whose passes compute only the rows the
    schedule names.  Fields travel as row blocks of four channels per cell,
    packed as height (rock, water), flux (L, R, T, B), vel (u, v, depth),
    sed (sediment) and the two talus outflow planes."""
    PACK = {"height": ("rock", "water"), "flux": ("flux_l", "flux_r", "flux_t", "flux_b"),
            "vel": ("vel_u", "vel_v", "vel_z"), "sed": ("sediment",),
            "ero_rock": ("eroded_rock",), "ero_sed": ("eroded_sediment",)}
    PLANES = {"thc": "thermal_c", "thd": "thermal_d"}

    def __init__(self, world, rows, rank, dt):
        self.w = world
        self.lo, self.hi = rows[rank]
        self.dt = dt

    def run_pass(self, name, layer):
        self.w.run_pass(name, layer)

    def fused_half(self, which):
        self.w.fused_pass(which)

    def set_compute_rows(self, a, b):
        self.w.restrict_rows(a, b)

    def set_step(self, done):
        self.w.step_count = done

    def get_rows(self, tex, y0, y1):
        out = np.zeros((y1 - y0, self.w.n, 4))
        if tex in self.PLANES:
            out[:] = self.w.get_rows(self.PLANES[tex], y0, y1)
        else:
            for k, f in enumerate(self.PACK[tex]):
                out[..., k] = self.w.get_rows(f, y0, y1)
        return out

    def set_rows(self, tex, y0, rows):
        if tex in self.PLANES:
            self.w.put_rows(self.PLANES[tex], y0, rows)
        else:
            for k, f in enumerate(self.PACK[tex]):
                self.w.put_rows(f, y0, rows[..., k])

    def max_reach_rows(self, y0=None, y1=None):
        y0 = self.lo if y0 is None else y0
        y1 = self.hi if y1 is None else y1
        v = self.w.get_rows("vel_v", y0, y1)
        return int(np.ceil(np.max(np.abs(v)) * self.dt)) + 1 if v.size else 0


class ThreadGroup:
    """The ranks of one slab decomposition as threads of one process (one
    GPU each, or several on one GPU): a barrier and a mailbox.  A rank that
    fails calls abort(), and the others' next wait raises instead of
    hanging; every wait also gives up after `timeout` seconds."""

    def __init__(self, nranks, timeout=300.0):
        self.nranks = nranks
        self.timeout = timeout
        self.barrier = threading.Barrier(nranks)
        self.box = {}

    def abort(self):
        self.barrier.abort()


class ThreadComm:
    """SlabComm's operations between the threads of a ThreadGroup: halo rows
    from the two neighbours, the all-gather and the maximum, through host
    memory."""

    def __init__(self, group, rank, rows, n):
        self.g = group
        self.rank, self.nranks, self.rows, self.n = rank, group.nranks, rows, n
        self.min_rows = min(hi - lo for lo, hi in rows)
        self.gathers = 0
        self.exchanges = 0
        self.deep_blocks = 0
        self.rollbacks = 0

    def _sync(self):
        self.g.barrier.wait(self.g.timeout)

    def agree_max(self, value):
        self.g.box[("max", self.rank)] = float(value)
        self._sync()
        m = max(self.g.box[("max", r)] for r in range(self.nranks))
        self._sync()  # every rank has read before the box is reused
        return m

    def exchange(self, stepper, field, depth):
        lo, hi = self.rows[self.rank]
        self.g.box[("lo", self.rank)] = stepper.get_rows(field, lo, lo + depth)
        self.g.box[("hi", self.rank)] = stepper.get_rows(field, hi - depth, hi)
        self._sync()
        if self.rank > 0:
            stepper.set_rows(field, lo - depth, self.g.box[("hi", self.rank - 1)])
        if self.rank < self.nranks - 1:
            stepper.set_rows(field, hi, self.g.box[("lo", self.rank + 1)])
        self._sync()
        self.exchanges += 1

    def gather(self, stepper, field):
        lo, hi = self.rows[self.rank]
        self.g.box[("all", self.rank)] = stepper.get_rows(field, lo, hi)
        self._sync()
        for r, (a, b) in enumerate(self.rows):
            if r != self.rank:
                stepper.set_rows(field, a, self.g.box[("all", r)])
        self._sync()
        self.gathers += 1
