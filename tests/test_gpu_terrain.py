"""hydro-gen's own terrain generator and rain on the GPU against the CPU
restatement (oracle/hg_terrain_ref.cpp): bit for bit where no exp() enters,
within float tolerance through the exponential mask; the reference rain in
the per-pass and fused steps against the oracle's world."""
import numpy as np
import pytest

import hydrogen as H
import oracle as O

pytestmark = pytest.mark.gpu


def gpu_heightmap(n, layers, ms):
    w = H.World(n, layers=layers)
    w.init_reference_heightmap(ms)
    rock = w.download("rock")
    dirt = w.download("dirt") if layers == 2 else None
    assert not np.any(w.download("water")) and w.step_count == 0
    return rock, dirt


@pytest.mark.parametrize("kw", [dict(mask_exp=0), dict(mask_exp=0, mask_round=1, mask_slope=1, terrace=5),
                                dict(mask_exp=0, uplift=1, domain_warp=2, seed=3.5, octaves=6)])
def test_reference_heightmap_bitwise(kw):
    ms = H.map_settings(scale=0.00075 * 8, **kw)
    rock, dirt = gpu_heightmap(128, 2, ms)
    ref_rock, ref_dirt = O.ref_heightmap(ms, 128)
    assert np.array_equal(rock, ref_rock), np.max(np.abs(rock - ref_rock))
    assert np.array_equal(dirt, ref_dirt)


def test_reference_heightmap_defaults_within_float_tolerance():
    ms = H.map_settings(scale=0.00075 * 8)  # the reference defaults: exponential and power masks
    rock, _ = gpu_heightmap(128, 1, ms)
    ref_rock, _ = O.ref_heightmap(ms, 128)
    # exp() of the GPU and of the host's libm may differ in the last bits
    assert np.max(np.abs(rock - ref_rock)) <= 1e-5 * ms.max_height
    assert rock.std() > 0.0


def make_rain_pair(layers, mode_fused=False):
    n = 128
    ms = H.map_settings(scale=0.00075 * 8, mask_exp=0, max_height=64.0)
    w = H.World(n, layers=layers)
    w.init_reference_heightmap(ms)
    H.configure(w, "config1")
    r = H.rain_uniform(0.01, 3)
    r.mountain_thresh, r.mountain_multip, r.drops = 0.3, 0.05, 0.05
    w.set_rain(r)
    w.set_options(H.options(H.RAIN_REFERENCE, time0=0.37, time_step=1.0 / 60.0))
    ow = O.OracleWorld(n, 32)
    ow.set("rock", w.download("rock"))
    if layers == 2:
        ow.set("dirt", w.download("dirt"))
    s, _ = O.workload("config1")
    oo = O.options(3, 3, 0.01, time0=0.37, time_step=1.0 / 60.0, mountain_thresh=0.3, mountain_multip=0.05,
                   drops=0.05, max_height=64.0)
    return w, ow, s, oo


@pytest.mark.parametrize("layers", [1, 2])
def test_reference_rain_plain_bitwise(layers):
    w, ow, s, oo = make_rain_pair(layers)
    for k in range(7):
        w.step(1, H.MODE_PLAIN)
        ow.step(s, oo, 1)
    fields = ["rock", "water", "sediment", "flux_l", "flux_r", "vel_u", "vel_v"] + (["dirt"] if layers == 2 else [])
    for f in fields:
        assert np.array_equal(w.download(f).astype(np.float64), ow.get(f)), f
    assert w.totals()[1] > 0.0


def test_reference_rain_fused_equals_plain():
    a, _, _, _ = make_rain_pair(1)
    b, _, _, _ = make_rain_pair(1)
    a.step(13, H.MODE_PLAIN)
    b.step(13, H.MODE_FUSED)  # rain on steps 3, 6, 9, 12 inserted before the fused launches
    for f in H.STATE_FIELDS:
        assert np.array_equal(a.download(f), b.download(f)), f


def test_standalone_rain_pass_matches_the_restatement():
    # hg_rain is Erosion::dispatch_grid_rain: one pass at the given frame
    # time, whatever the period; water starts at 0, so it holds the increment
    n = 128
    w = H.World(n, layers=2)
    ms = H.map_settings(hmap_dims=(n, n), max_height=64.0)
    w.init_reference_heightmap(ms)
    r = H.rain_uniform(0.02, 0)
    r.mountain_thresh, r.mountain_multip, r.drops = 0.3, 0.05, 0.05
    w.set_rain(r)
    w.set_options(H.options(H.RAIN_REFERENCE))
    w.rain(2.5)
    total = (w.download("rock") + w.download("dirt")).astype(np.float32)
    expect = O.ref_rain(total, 2.5, r, 64.0)
    assert np.array_equal(w.download("water"), expect)
    assert w.step_count == 0 and np.any(expect > 0)
    w.step(2, H.MODE_PLAIN)  # period 0: the step adds no rain of its own
