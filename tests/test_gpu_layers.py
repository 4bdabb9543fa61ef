"""Two-layer worlds (rock + dirt, both sediment channels): the per-pass
kernels and the fused three-kernel step against the float oracle's two-layer
model, bit for bit, with the reference's default settings (Kconv, both
slippage rates, smoothing) and with the config-2 rain; plus what the
two-layer world does not support."""
import numpy as np
import pytest

import hydrogen as H
import oracle as O

pytestmark = pytest.mark.gpu

FIELDS = ["rock", "dirt", "water", "sediment", "sediment_dirt", "flux_l", "flux_r", "flux_t", "flux_b", "vel_u",
          "vel_v", "vel_z"]


def make(n, settings, rain, opts, oopts, seed=0):
    w = H.World(n, layers=2)
    w.init_heightmap(H.noise(seed=seed))
    dirt = (O.fbm(n, seed=seed + 3, lo=0.0, hi=4.0)).astype(np.float32)
    w.upload("dirt", dirt)
    w.set_erosion(settings)
    w.set_rain(rain)
    w.set_options(opts)
    ow = O.OracleWorld(n, 32)
    ow.set("rock", w.download("rock"))
    ow.set("dirt", dirt)
    return w, ow, O.erosion_from(settings), oopts


def check(w, ow, ctx):
    for f in FIELDS:
        g, r = w.download(f).astype(np.float64), ow.get(f)
        bad = np.argwhere(g != r)
        assert bad.size == 0, f"{ctx} {f}: {len(bad)} cells differ, first {bad[:3].tolist()}"


def reference_defaults():
    s = H.ErosionSettings()
    H.check(H.lib.hg_default_erosion_settings(H.ctypes.byref(s)))
    return s


@pytest.mark.parametrize("case", ["defaults", "config2_rain"])
def test_two_layer_plain_bitwise_vs_float_oracle(case):
    if case == "defaults":  # src/state.cpp:81-92: Kconv 0.001, Kspeed (0.5, 2.0), dt 0.001
        s = reference_defaults()
        w, ow, os_, oo = make(128, s, H.rain_uniform(0.01, 1), H.options(H.RAIN_UNIFORM), O.options(1, 1, 0.01))
        steps = 40
    else:
        s = H.settings_config2()
        s.Kconv = 0.01
        s.Kspeed[1] = 1.0
        s.Kalpha[1] = 0.4
        w, ow, os_, oo = make(128, s, H.rain_uniform(0.5, 1), H.options(H.RAIN_BERNOULLI, p=0.02),
                              O.options(2, 1, 0.5, p=0.02))
        steps = 30
    for k in range(steps):
        w.step(1, H.MODE_PLAIN)
        ow.step(os_, oo, 1)
        if k in (0, steps - 1):
            check(w, ow, f"{case} step {k + 1}")
    assert np.any(w.download("sediment_dirt"))


def test_two_layer_limits_and_checkpoint(tmp_path):
    w = H.World(64, layers=2)
    w.init_heightmap(H.noise(seed=1))
    w.upload("dirt", np.full((64, 64), 0.5, np.float32))
    w.step(5, H.MODE_PLAIN)
    with pytest.raises(H.HydrogenError) as e:
        H.Tape(w, 4)
    assert e.value.code == -5
    path = str(tmp_path / "w2.bin")
    w.save(path)
    v = H.World(64, layers=2)
    v.load(path)
    w.step(7, H.MODE_PLAIN)
    v.step(7, H.MODE_PLAIN)
    for f in FIELDS:
        assert np.array_equal(w.download(f), v.download(f)), f
    one = H.World(64)
    with pytest.raises(H.HydrogenError):
        one.load(path)  # layer count differs
    with pytest.raises(H.HydrogenError):
        one.download("dirt")  # no dirt layer


FUSED_FIELDS = ["rock", "dirt", "water", "sediment", "sediment_dirt", "flux_l", "flux_r", "flux_t", "flux_b", "vel_u",
                "vel_v"]


def check_fused(w, ow, ctx):
    for f in FUSED_FIELDS:
        g, r = w.download(f).astype(np.float64), ow.get(f)
        bad = np.argwhere(g != r)
        assert bad.size == 0, f"{ctx} {f}: {len(bad)} cells differ, first {bad[:3].tolist()}"


@pytest.mark.parametrize("case", ["defaults", "config2_rain", "no_dirt_talus", "rock_talus_off"])
def test_two_layer_fused_bitwise_vs_float_oracle(case):
    # 192 = 3 x 64: edge tiles on every side and interior tiles
    n = 192
    if case == "config2_rain":
        s = H.settings_config2()
        s.Kconv = 0.01
        s.Kspeed[1] = 1.0
        s.Kalpha[1] = 0.4
        w, ow, os_, oo = make(n, s, H.rain_uniform(0.5, 1), H.options(H.RAIN_BERNOULLI, p=0.02, seed=9),
                              O.options(2, 1, 0.5, p=0.02, seed=9), seed=1)
        steps = 25
    else:
        s = reference_defaults()
        if case == "no_dirt_talus":
            s.Kspeed[1] = 0.0  # no dirt pass, no smoothing: two kernels per step
        if case == "rock_talus_off":
            s.Kspeed[0] = 0.0
        w, ow, os_, oo = make(n, s, H.rain_uniform(0.01, 1), H.options(H.RAIN_UNIFORM), O.options(1, 1, 0.01))
        steps = 30
    for k in range(steps):
        w.step(1, H.MODE_FUSED)
        ow.step(os_, oo, 1)
        if k in (0, 1, steps - 1):
            check_fused(w, ow, f"{case} step {k + 1}")
    assert np.any(w.download("sediment_dirt"))


def test_two_layer_fused_matches_plain_with_reference_rain():
    n = 128
    ms = H.map_settings(hmap_dims=(n, n), max_height=64.0)
    worlds = []
    for mode in (H.MODE_PLAIN, H.MODE_FUSED):
        w = H.World(n, layers=2)
        w.init_reference_heightmap(ms)
        w.set_erosion(reference_defaults())
        w.set_rain(H.rain_uniform(0.2, 3))
        w.set_options(H.options(H.RAIN_REFERENCE, time0=1.0, time_step=0.25))
        w.step(20, mode)
        worlds.append(w)
    for f in FUSED_FIELDS:
        assert np.array_equal(worlds[0].download(f), worlds[1].download(f)), f
    assert worlds[0].step_count == worlds[1].step_count == 20


def test_two_layer_batch_fused_runs_each_world():
    ws, solo = [], []
    for i, n in enumerate((64, 128)):
        for group in (ws, solo):
            w = H.World(n, layers=2)
            w.init_heightmap(H.noise(seed=i))
            w.upload("dirt", np.full((n, n), 0.5, np.float32))
            w.set_erosion(reference_defaults())
            w.set_rain(H.rain_uniform(0.01, 1))
            w.set_options(H.options(H.RAIN_UNIFORM))
            group.append(w)
    b = H.Batch(ws)
    b.step(6, H.MODE_FUSED)
    b.sync()
    for w in solo:
        w.step(6, H.MODE_PLAIN)
    for w, v in zip(ws, solo):
        for f in FUSED_FIELDS:
            assert np.array_equal(w.download(f), v.download(f)), f
