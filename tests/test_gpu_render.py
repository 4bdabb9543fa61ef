"""The headless ray-marcher (glsl/rendering.glsl) on the GPU against its CPU
restatement, bit for bit: RGBA8 pixels and the float colours (NaN colours of
the shader's undefined pow included), over cameras that exercise the
terrain, water refraction / reflection, shadows, sky, the low-resolution form
and the sediment tint, on one- and two-layer worlds."""
import numpy as np
import pytest

import hydrogen as H
import oracle as O

pytestmark = pytest.mark.gpu


def fields_of(w, two_layer):
    names = ["rock", "water", "sediment"] + (["dirt", "sediment_dirt"] if two_layer else [])
    return {k: w.download(k) for k in names}


def check(w, two_layer, cam, width, height, max_height, hmap_dim_x, ctx):
    rgba, rgb = w.render(cam, width, height, rgb=True)
    orgba, orgb = O.render(fields_of(w, two_layer), w.n, cam, width, height, max_height, hmap_dim_x)
    bad = np.argwhere(np.any(rgba != orgba, axis=2))
    assert bad.size == 0, f"{ctx}: {len(bad)} pixels differ, first {bad[:3].tolist()}"
    bad = np.argwhere(np.any(rgb.view(np.uint32) != orgb.view(np.uint32), axis=2))
    assert bad.size == 0, f"{ctx}: {len(bad)} float colours differ, first {bad[:3].tolist()}"
    return rgba


@pytest.fixture(scope="module")
def two_layer_world():
    n = 128
    w = H.World(n, layers=2)
    ms = H.map_settings(hmap_dims=(n, n), max_height=64.0)
    w.init_reference_heightmap(ms)
    rock = w.download("rock")
    w.upload("water", np.where(rock < 30.0, 30.0 - rock, 0.0).astype(np.float32))
    w.set_erosion(H.settings_config1())
    w.set_rain(H.rain_uniform(0.01, 1))
    w.set_options(H.options(H.RAIN_UNIFORM))
    w.step(20, H.MODE_PLAIN)
    return w


CAMERAS = {
    "diagonal": ((-12.0, 90.0, -12.0), (1.0, -0.55, 1.0)),
    "grazing": ((-30.0, 36.0, 64.0), (1.0, -0.12, 0.05)),
    "overhead": ((64.0, 120.0, 64.0), (0.05, -1.0, 0.02)),
    "away": ((-10.0, 80.0, -10.0), (-1.0, 0.2, -1.0)),
}


@pytest.mark.parametrize("name", list(CAMERAS))
def test_render_bitwise_two_layer(two_layer_world, name):
    pos, d = CAMERAS[name]
    cam = H.camera(pos, d, aspect=16 / 9)
    img = check(two_layer_world, True, cam, 160, 90, 64.0, 128, name)
    if name != "away":
        assert len(np.unique(img[..., :3].reshape(-1, 3), axis=0)) > 100


def test_render_forms_and_sediment(two_layer_world):
    cam = H.camera(*CAMERAS["diagonal"], aspect=4 / 3)
    cam.low_res_div3 = 1
    low = check(two_layer_world, True, cam, 121, 91, 64.0, 128, "low-res")
    assert np.all(low[:90, :120, 3] == 255) and np.all(low[90:, :, 3] == 0)
    cam.low_res_div3 = 0
    cam.display_sediment = 1
    cam.sediment_max_cap = 0.002
    check(two_layer_world, True, cam, 120, 90, 64.0, 128, "sediment")
    cam.display_sediment = 0
    cam.draw_water = 0
    cam.prec = 0.8
    check(two_layer_world, True, cam, 120, 90, 64.0, 128, "no water, coarse steps")


def test_render_one_layer_fused_world():
    n = 128
    w = H.World(n)
    w.init_heightmap(H.noise(seed=4))
    s = H.settings_config2()
    w.set_erosion(s)
    w.set_rain(H.rain_uniform(0.5, 1))
    w.set_options(H.options(H.RAIN_BERNOULLI, p=0.02, seed=3))
    w.step(30, H.MODE_FUSED)
    cam = H.camera((-5.0, 100.0, 48.0), (1.0, -0.7, 0.1), aspect=1.0)
    check(w, False, cam, 96, 96, 256.0, 1024, "one layer")
    with pytest.raises(H.HydrogenError):
        w.render(cam, 0, 10)
