"""One grid split into row slabs and stepped by the library's per-pass kernels
(slabs.GpuSlabStepper: hg_set_rows, hg_pass, hg_world_rows): the ranks are
threads of one process on one GPU, each with its own world computing only
the rows the schedule names, halo rows moved through host memory between
passes (slabs.ThreadComm).  No kernel waits on another: every row moves on
the host between launches.  With the per-pass schedule and the deep-halo
blocks, under uniform rain and under thin films (back-traces past the halo:
all-gathers and roll-backs), every rank's own rows equal one world stepped
whole with the per-pass kernels, bit for bit."""
import threading

import numpy as np
import pytest

import hydrogen as H
import slabs

pytestmark = pytest.mark.gpu

N, STEPS = 96, 10
FIELDS = ["rock", "water", "sediment", "flux_l", "flux_r", "flux_t", "flux_b", "vel_u", "vel_v"]


def make(films):
    """Config-2 physics with smoothing (Kspeed[1] = 2) on a small world; dense
    Bernoulli rain (thin films) or uniform rain."""
    w = H.World(N)
    w.init_heightmap(H.noise(seed=1, frequency=1.0 / 16))
    H.configure(w, "config2")
    s = H.settings_config2()
    s.Kspeed[1] = 2.0
    w.set_erosion(s)
    if films:
        w.set_rain(H.rain_uniform(0.5, 1))
        w.set_options(H.options(H.RAIN_BERNOULLI, p=0.05, seed=3))
    else:
        w.set_rain(H.rain_uniform(0.01, 1))
        w.set_options(H.options(H.RAIN_UNIFORM))
    return w, s


def run_ranks(nranks, films, deep):
    rows = slabs.slab_rows(N, nranks)
    group = slabs.ThreadGroup(nranks, timeout=120.0)
    worlds, s = [], None
    for _ in range(nranks):
        w, s = make(films)
        worlds.append(w)
    out, errors = [None] * nranks, []

    def rank_main(r):
        try:
            st = slabs.GpuSlabStepper(worlds[r], rows, r, s.d_t)
            comm = slabs.ThreadComm(group, r, rows, N)
            k = 0
            while k < STEPS:
                if deep:
                    k += slabs.deep_block(st, comm, k + 1, min(deep, STEPS - k), s, 1, sed_budget=3, halo_max=8)
                else:
                    slabs.slab_step(st, comm, k + 1, s, 1, halo_max=8)
                    k += 1
            worlds[r].sync()
            lo, hi = rows[r]
            out[r] = ({f: worlds[r].get_rows(f, lo, hi) for f in FIELDS},
                      (comm.exchanges, comm.gathers, comm.deep_blocks, comm.rollbacks))
        except BaseException as e:  # let the other ranks' waits end
            errors.append(e)
            group.abort()

    threads = [threading.Thread(target=rank_main, args=(r,)) for r in range(nranks)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for w in worlds:
        w.close()
    return rows, out


@pytest.mark.parametrize("nranks,films,deep", [(2, False, 0), (2, True, 0), (3, False, 4), (2, True, 4)])
def test_gpu_slabs_equal_one_world(nranks, films, deep):
    rows, out = run_ranks(nranks, films, deep)
    ref, _ = make(films)
    ref.step(STEPS, H.MODE_PLAIN)
    counters = np.zeros(4, int)
    for r, (lo, hi) in enumerate(rows):
        fields, c = out[r]
        counters += np.array(c)
        for f in FIELDS:
            g = ref.download(f)[lo:hi]
            bad = np.argwhere(fields[f].view(np.uint32) != g.view(np.uint32))
            assert bad.size == 0, f"rank {r} {f}: {len(bad)} cells differ, first {bad[:3].tolist()}"
    exchanges, gathers, deep_blocks, rollbacks = counters
    assert exchanges > 0
    if films:  # back-traces past the halo: the all-gather (and, in blocks, the roll-back) ran
        assert gathers > 0 and (rollbacks > 0 or not deep)
    elif deep:
        assert deep_blocks > 0


def test_row_restricted_world_refuses_whole_world_paths():
    w = H.World(128)
    w.init_heightmap(H.noise(seed=1))
    H.configure(w, "config2")
    w.restrict_rows(0, 64)
    with pytest.raises(H.HydrogenError) as e:
        w.step(1, H.MODE_FUSED)
    assert e.value.code == -5 and "row-restricted" in str(e.value)
    w.step(1, H.MODE_PLAIN)  # the per-pass step honours the range
    with pytest.raises(H.HydrogenError):
        w.restrict_rows(4, 2)
    w.restrict_rows()
    w.step(1, H.MODE_FUSED)
    w.close()


def make_fused(films, n=128):
    """Config-2 physics (talus slippage, no smoothing) for the fused halves."""
    w = H.World(n)
    w.init_heightmap(H.noise(seed=1, frequency=1.0 / 16))
    H.configure(w, "config2")
    if films:
        w.set_options(H.options(H.RAIN_BERNOULLI, p=0.05, seed=3))
    else:
        w.set_rain(H.rain_uniform(0.01, 1))
        w.set_options(H.options(H.RAIN_UNIFORM))
    return w


@pytest.mark.parametrize("nranks,films", [(2, False), (2, True), (4, True)])
def test_gpu_fused_slabs_equal_one_world(nranks, films):
    """The fused step on row slabs (hg_fused_pass; slabs.fused_slab_step):
    k_hydro on each rank's tile rows after a one-row exchange of height and
    flux, the eroded rock two rows deep and the eroded sediment as deep as
    the back-traces reach (or the all-gather) between the kernels, then
    k_transport; every rank's rows equal one world stepped with the fused
    kernels, bit for bit."""
    n = 128
    rows = slabs.slab_rows(n, nranks)
    group = slabs.ThreadGroup(nranks, timeout=120.0)
    worlds = [make_fused(films, n) for _ in range(nranks)]
    dt = H.settings_config2().d_t
    out, errors = [None] * nranks, []

    def rank_main(r):
        try:
            st = slabs.GpuSlabStepper(worlds[r], rows, r, dt)
            comm = slabs.ThreadComm(group, r, rows, n)
            for _ in range(STEPS):
                slabs.fused_slab_step(st, comm, thermal=True, halo_max=8)
            worlds[r].sync()
            lo, hi = rows[r]
            out[r] = ({f: worlds[r].get_rows(f, lo, hi) for f in FIELDS}, (comm.exchanges, comm.gathers))
        except BaseException as e:  # let the other ranks' waits end
            errors.append(e)
            group.abort()

    threads = [threading.Thread(target=rank_main, args=(r,)) for r in range(nranks)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    ref = make_fused(films, n)
    ref.step(STEPS, H.MODE_FUSED)
    gathers = 0
    for r, (lo, hi) in enumerate(rows):
        fields, (ex, ga) = out[r]
        gathers += ga
        assert worlds[r].step_count == STEPS
        for f in FIELDS:
            g = ref.download(f)[lo:hi]
            bad = np.argwhere(fields[f].view(np.uint32) != g.view(np.uint32))
            assert bad.size == 0, f"rank {r} {f}: {len(bad)} cells differ, first {bad[:3].tolist()}"
    assert (gathers > 0) == films
    for w in worlds:
        w.close()
