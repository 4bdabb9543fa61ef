"""Two-layer worlds (rock + dirt, both sediment channels): the per-pass
kernels against the float oracle's two-layer model, bit for bit, with the
reference's default settings (Kconv, both slippage rates, smoothing) and with
the config-2 rain; plus what the two-layer world does not support."""
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
    for bad in (lambda: w.step(1, H.MODE_FUSED), lambda: H.Tape(w, 4)):
        with pytest.raises(H.HydrogenError) as e:
            bad()
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
