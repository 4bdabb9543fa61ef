"""Failure detection without a GPU fault.

A fused-step block waits for its TMA tile with a bounded number of barrier
polls; if the tile never arrives it records an error flag, skips the tile and
returns, and hg_sync reports HG_ERR_TIMEOUT.  Here the same wait runs on a
barrier phase that nothing completes (no copy in flight, no trap, no fault):
it must give up, say so, and leave the device usable."""
import ctypes

import numpy as np
import pytest

import hydrogen as H

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_the_device_stays_usable():
    flag, ns = ctypes.c_int(-1), ctypes.c_double()
    H.check(H.lib.hg_selftest_bounded_wait(1 << 12, ctypes.byref(flag), ctypes.byref(ns)))
    assert flag.value == 1
    assert ns.value > 0
    bound_s = (1 << 18) * ns.value / 1e9  # the kernels' limit
    print(f"bounded wait: {ns.value:.1f} ns per poll; a lost tile is given up after {bound_s:.2f} s")
    assert bound_s < 5
    # the context still runs the library's kernels: the fused step equals the per-pass one
    a, b = H.World(128), H.World(128)
    for w in (a, b):
        w.init_heightmap(H.noise(seed=3))
        H.configure(w, "config2")
    a.step(10, H.MODE_PLAIN)
    b.step(10, H.MODE_FUSED)
    for f in ("rock", "water", "sediment"):
        assert np.array_equal(a.download(f), b.download(f)), f
    b.sync()  # no tile of the fused steps timed out


def test_timeout_leaves_the_world_undefined_until_reinitialised():
    """hg_sync's HG_ERR_TIMEOUT contract, exercised without a lost copy: the
    host sets the device flag a giving-up wait would set.  The world then
    refuses to step until it is re-initialised, and steps again after."""
    w = H.World(128)
    w.init_heightmap(H.noise(seed=1))
    H.configure(w, "config2")
    w.step(4, H.MODE_FUSED)
    w.sync()
    H.check(H.lib.hg_selftest_report_timeout(w.h))
    assert H.lib.hg_sync(w.h) == -4
    for mode in (H.MODE_PLAIN, H.MODE_FUSED):
        with pytest.raises(H.HydrogenError) as e:
            w.step(1, mode)
        assert e.value.code == -4
    tape = H.Tape(w, 4, 4)
    with pytest.raises(H.HydrogenError) as e:
        tape.forward()
    assert e.value.code == -4
    tape.close()
    w.init_heightmap(H.noise(seed=1))
    w.step(4, H.MODE_FUSED)
    w.sync()
    ref = H.World(128)
    ref.init_heightmap(H.noise(seed=1))
    H.configure(ref, "config2")
    ref.step(4, H.MODE_FUSED)
    assert np.array_equal(w.download("rock"), ref.download("rock"))


def test_tape_outliving_its_world():
    """A world destroyed before its tape frees the tape's device memory; the
    tape then reports HG_ERR_STATE and its own destruction only drops the
    handle (through the C ABI directly, past the wrapper's ordering)."""
    import ctypes
    w = H.World(64)
    w.init_heightmap(H.noise(seed=1))
    H.configure(w, "config1")
    t = ctypes.c_void_p()
    H.check(H.lib.hg_tape_create(w.h, 4, 2, ctypes.byref(t)))
    H.check(H.lib.hg_world_destroy(w.h))
    w.h = None
    assert H.lib.hg_forward(t) == -7
    a, b = ctypes.c_int(), ctypes.c_int()
    assert H.lib.hg_tape_info(t, ctypes.byref(a), ctypes.byref(b)) == -7
    H.check(H.lib.hg_tape_destroy(t))


def two_layer_world(n):
    s = H.ErosionSettings()
    H.check(H.lib.hg_default_erosion_settings(ctypes.byref(s)))
    w = H.World(n, layers=2)
    w.init_reference_heightmap(H.map_settings(hmap_dims=(n, n)))
    w.set_erosion(s)
    w.set_rain(H.rain_uniform(0.01, 1))
    w.set_options(H.options(H.RAIN_UNIFORM))
    return w


def one_layer_world(n, smooth=False):
    w = H.World(n)
    w.init_heightmap(H.noise(seed=5))
    H.configure(w, "config2")
    if smooth:
        s = H.settings_config2()
        s.Kspeed[1] = 1.0
        w.set_erosion(s)
    return w


@pytest.mark.parametrize("layers,smooth,mode", [(1, False, H.MODE_PLAIN), (1, False, H.MODE_FUSED),
                                                (1, True, H.MODE_FUSED), (2, False, H.MODE_PLAIN),
                                                (2, False, H.MODE_FUSED)])
def test_every_output_cell_is_written(layers, smooth, mode):
    """Before each step every buffer the step writes is filled with NaN; after
    it no carried field holds a NaN and the fields equal a world stepped
    without poison, bit for bit: no cell is left unwritten or read before
    it is written (192 = 3 x 64: edge and interior tiles)."""
    n = 192
    make = (lambda: two_layer_world(n)) if layers == 2 else (lambda: one_layer_world(n, smooth))
    a, b = make(), make()
    bad = ctypes.c_uint64()
    for _ in range(3):
        H.check(H.lib.hg_world_poison_scratch(b.h))
        b.step(1, mode)
        H.check(H.lib.hg_world_count_nonfinite(b.h, ctypes.byref(bad)))
        assert bad.value == 0
    a.step(3, mode)
    fields = ["rock", "water", "sediment", "flux_l", "flux_r", "flux_t", "flux_b"]
    if layers == 2:
        fields += ["dirt", "sediment_dirt"]
    for f in fields:
        assert np.array_equal(a.download(f), b.download(f)), f


def particle_world(n, count):
    w = H.World(n, layers=2)
    w.init_heightmap(H.noise(seed=2))
    w.upload("dirt", np.full((n, n), 0.5, np.float32))
    w.particles_init(count)
    w.set_erosion(H.settings_particles())
    w.set_options(H.options(H.RAIN_UNIFORM, seed=7))
    return w


def same_bits(x, y):
    return np.array_equal(np.ascontiguousarray(x).view(np.uint32), np.ascontiguousarray(y).view(np.uint32))


def test_every_output_cell_is_written_particles():
    """Particle mode: the droplet records' sediment and layer masks and the
    step's alternate buffers start each step as NaN; afterwards the fields,
    the momentum map and every droplet equal an unpoisoned world's, bit for
    bit, and hold no NaN (4096 droplets on 128² so texels share records)."""
    n, count = 128, 4096
    a, b = particle_world(n, count), particle_world(n, count)
    bad = ctypes.c_uint64()
    for _ in range(4):
        H.check(H.lib.hg_world_poison_scratch(b.h))
        b.step(1, H.MODE_PARTICLES)
        H.check(H.lib.hg_world_count_nonfinite(b.h, ctypes.byref(bad)))
        assert bad.value == 0
    a.step(4, H.MODE_PARTICLES)
    for f in ("rock", "dirt", "water", "momentum_x", "momentum_y"):
        assert same_bits(a.download(f), b.download(f)), f
    for x, y, name in zip(a.particles(), b.particles(), ("state", "iters", "kill")):
        assert same_bits(x, y), name


def test_every_output_cell_is_written_batch_table_launch():
    """One table launch per fused kernel for two worlds of different sizes
    (128² and 192², tile height 16, no graph: no autotuning, so every step is
    the table form): each world's scratch is NaN before each batch step,
    afterwards no carried field holds a NaN and both worlds equal an
    unpoisoned batch's, bit for bit."""
    def worlds():
        out = []
        for i, n in enumerate((128, 192)):
            w = H.World(n)
            w.init_heightmap(H.noise(seed=10 + i))
            H.configure(w, "config2")
            w.set_options(H.options(H.RAIN_BERNOULLI, p=0.02, seed=i, terrain_id=i, tile=(64, 16), graph=0))
            out.append(w)
        return out
    wa, wb = worlds(), worlds()
    ba, bb = H.Batch(wa), H.Batch(wb)
    bad = ctypes.c_uint64()
    for _ in range(3):
        for w in wb:
            H.check(H.lib.hg_world_poison_scratch(w.h))
        bb.step(1, H.MODE_FUSED)
        bb.sync()
        for w in wb:
            H.check(H.lib.hg_world_count_nonfinite(w.h, ctypes.byref(bad)))
            assert bad.value == 0
    ba.step(3, H.MODE_FUSED)
    ba.sync()
    assert bb.tuning()[0] == 0  # never tuned: the table launch ran
    for x, y in zip(wa, wb):
        for f in ("rock", "water", "sediment", "flux_l", "flux_r", "flux_t", "flux_b"):
            assert np.array_equal(x.download(f), y.download(f)), (x.n, f)
    ba.close()
    bb.close()
