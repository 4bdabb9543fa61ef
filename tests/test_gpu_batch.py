"""Batches: one fused launch pair per step over worlds of different sizes and
settings, CUDA-graph replay, both tile heights and the autotuner all give the
same fields as stepping each world alone with the per-pass kernels."""
import numpy as np
import pytest

import hydrogen as H

pytestmark = pytest.mark.gpu

STATE = ["rock", "water", "sediment", "flux_l", "flux_r", "flux_t", "flux_b", "vel_u", "vel_v"]


def terrains():
    ts = H.config3_terrains(count=6, seed=5)
    sizes = [64, 128, 256, 192, 64, 128]  # small sides keep the test fast; 192 = 3 x 64
    for t, n in zip(ts, sizes):
        t["n"] = n
    return ts


def make(ts, p=0.02, **opt):
    ws = []
    for i, t in enumerate(ts):
        w = H.make_config3_world(t, terrain_id=i)
        w.set_options(H.options(H.RAIN_BERNOULLI, p=p, seed=t["seed"], terrain_id=i, **opt))
        if i == 1:  # one world without thermal erosion
            s = w.get_erosion()
            s.Kspeed[0] = 0.0
            w.set_erosion(s)
        if i in (2, 4):  # two worlds with smoothing (Kspeed[1] != 0), one of them without thermal
            s = w.get_erosion()
            s.Kspeed[1] = 3.0
            if i == 4:
                s.Kspeed[0] = 0.0
            w.set_erosion(s)
        ws.append(w)
    return ws


def same(a, b):
    for f in STATE:
        x, y = a.download(f), b.download(f)
        assert np.array_equal(x, y), f"{f}: {np.count_nonzero(x != y)} cells differ"


@pytest.mark.parametrize("tile_y,graph", [(16, 0), (16, 1), (8, 0), (8, 1)])
def test_batch_fused_equals_individual_plain(tile_y, graph):
    ts = terrains()
    ref = make(ts)
    for w in ref:
        w.step(13, H.MODE_PLAIN)
    ws = make(ts, tile=(64, tile_y), graph=graph)
    b = H.Batch(ws)
    b.step(13, H.MODE_FUSED)  # odd count: graph pairs plus one direct step
    b.sync()
    for a, c in zip(ref, ws):
        same(a, c)
        assert c.step_count == 13


def test_batch_modes_agree_and_interleave_with_world_steps():
    ts = terrains()
    a = make(ts)
    b = make(ts)
    ba = H.Batch(a)
    ba.step(5, H.MODE_FUSED)
    a[0].step(2, H.MODE_PLAIN)  # a world stepped alone between batch steps
    a[2].step(3, H.MODE_FUSED)
    ba.step(4, H.MODE_FUSED)
    bb = H.Batch(b)
    bb.step(5, H.MODE_FUSED_PER_WORLD)
    b[0].step(2, H.MODE_PLAIN)
    b[2].step(3, H.MODE_PLAIN)
    bb.step(4, H.MODE_PLAIN)
    ba.sync()
    bb.sync()
    for x, y in zip(a, b):
        same(x, y)
        assert x.step_count == y.step_count


def test_autotuner_picks_a_variant_and_keeps_results():
    ts = terrains()
    ref = make(ts)
    for w in ref:
        w.step(27, H.MODE_PLAIN)
    ws = make(ts)
    b = H.Batch(ws)
    b.step(20, H.MODE_FUSED)  # first 12 steps time per-world launches and the four table variants
    b.sync()
    th, graph, ms = b.tuning()
    assert th in (16, 8) and graph in (0, 1)
    assert all(m > 0 for m in ms)
    per_world, ms_pw = b.launch_form()
    assert per_world in (0, 1) and ms_pw > 0
    assert per_world == (ms_pw < min(ms))
    b.step(7, H.MODE_FUSED)  # the chosen form
    b.sync()
    for a, c in zip(ref, ws):
        same(a, c)
        assert c.step_count == 27


def test_world_autotune_and_settings_change_rebuilds_tables():
    ref = H.World(256)
    w = H.World(256)
    for x in (ref, w):
        x.init_heightmap(H.noise(seed=2))
        H.configure(x, "config2")
    ref.step(10, H.MODE_PLAIN)
    w.step(10, H.MODE_FUSED)
    assert w.tuning()[0] in (16, 8)
    s = H.settings_config2()
    s.Kc = 0.3  # new settings must reach the fused descriptors
    for x in (ref, w):
        x.set_erosion(s)
    ref.step(6, H.MODE_PLAIN)
    w.step(6, H.MODE_FUSED)
    same(ref, w)


def test_batch_rejects_unfusable_world():
    w = H.World(40)
    H.configure(w, "config1")
    b = H.Batch([w])
    b.step(1, H.MODE_PLAIN)
    with pytest.raises(H.HydrogenError) as e:
        b.step(1, H.MODE_FUSED)
    assert e.value.code == -5


def test_largest_batch_in_one_launch():
    """128 worlds (the most a batch holds; a 129th is refused) of 64² with
    their own settings and seeds: one table launch per kernel for all of them,
    the terrain lookup spanning its whole table, over 17 steps (two eight-step
    graph replays and a direct step), equals each world's per-pass steps."""
    ts = H.config3_terrains(count=129, seed=11)
    for t in ts:
        t["n"] = 64

    def worlds(k):
        out = []
        for i, t in enumerate(ts[:k]):
            w = H.make_config3_world(t, terrain_id=i)
            w.set_options(H.options(H.RAIN_BERNOULLI, p=0.05, seed=t["seed"], terrain_id=i, tile=(64, 16), graph=1))
            out.append(w)
        return out
    ref = worlds(128)
    for w in ref:
        w.step(17, H.MODE_PLAIN)
    ws = worlds(128)
    b = H.Batch(ws)
    b.step(17, H.MODE_FUSED)
    b.sync()
    assert b.tuning()[0] == 0 and b.launch_form()[0] == 0  # the table launch ran
    for a, c in zip(ref, ws):
        same(a, c)
    b.close()
    extra = worlds(129)
    with pytest.raises(H.HydrogenError) as e:
        H.Batch(extra)
    assert e.value.code == -5  # HG_ERR_UNSUPPORTED
    for w in ref + ws + extra:
        w.close()
