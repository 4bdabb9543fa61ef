"""The ray-marcher's CPU restatement (oracle/hg_render_ref.cpp) and the
camera builder of the C-ABI: accuracy of the series exp2 / log2 / pow that
both sides share, the glm conventions of hg_camera_look_at, and properties
of rendered images (sky above the horizon, low-resolution 3x3 blocks,
sediment tint) that hold whatever the terrain."""
import ctypes

import numpy as np
import pytest

import hydrogen as H
import oracle as O


def test_series_exp2_log2_pow_accuracy():
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(-126, 127.9, 4000), rng.uniform(-2, 2, 4000)]).astype(np.float32)
    got = np.array([O.render_exp2(float(x)) for x in xs])
    ref = np.exp2(xs.astype(np.float64))
    ulp = np.abs(got - ref) / np.spacing(ref.astype(np.float32)).astype(np.float64)
    assert ulp.max() <= 2.0
    xs = np.exp(rng.uniform(np.log(1e-40), np.log(1e38), 8000)).astype(np.float32)
    got = np.array([O.render_log2(float(x)) for x in xs])
    ref = np.log2(xs.astype(np.float64))
    assert np.all(np.abs(got - ref) <= 4 * np.spacing(np.maximum(np.abs(ref), 1.0).astype(np.float32)))
    assert O.render_log2(1.0) == 0.0 and O.render_log2(0.25) == -2.0 and O.render_exp2(3.0) == 8.0
    bx = rng.uniform(0, 2, 6000).astype(np.float32)
    by = rng.choice(np.array([2.5, 4.0, 5.0, 64.0, 512.0, 16.0, 2.0, 1 / 2.2], np.float32), 6000)
    got = np.array([O.render_pow(float(a), float(b)) for a, b in zip(bx, by)])
    ref = np.power(bx.astype(np.float64), by.astype(np.float64))
    m = (ref > 1e-30) & (ref < 3e38)
    mag = np.abs(by[m] * np.log2(bx[m].astype(np.float64)))
    assert np.all(np.abs(got[m] - ref[m]) <= ref[m] * 3e-7 * (1.0 + mag))
    # the shader's undefined cases: negative base NaN, 0^y
    assert np.isnan(O.render_pow(-0.5, 2.0)) and O.render_pow(0.0, 2.5) == 0.0 and O.render_pow(0.0, 0.0) == 1.0


def test_camera_builder_follows_glm():
    pos, d, up = np.array([3.0, 50.0, -7.0]), np.array([1.0, -0.4, 0.7]), np.array([0.0, 1.0, 0.0])
    cam = H.camera(tuple(pos), tuple(d), tuple(up), fov=90.0, aspect=1.5, z_near=0.1, z_far=2048.0)
    f = d / np.linalg.norm(d)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    V = np.eye(4)
    V[0, :3], V[1, :3], V[2, :3] = s, u, -f
    V[:3, 3] = [-s @ pos, -u @ pos, f @ pos]
    t = np.tan(np.radians(90.0) / 2)
    P = np.zeros((4, 4))
    P[0, 0], P[1, 1] = 1 / (1.5 * t), 1 / t
    P[2, 2], P[2, 3] = -(2048.1) / (2047.9), -(2 * 2048.0 * 0.1) / 2047.9
    P[3, 2] = -1.0
    # column-major storage: m[c*4 + r] = M[r, c]
    assert np.allclose(np.array(cam.view).reshape(4, 4).T, V, atol=1e-5)
    assert np.allclose(np.array(cam.perspective).reshape(4, 4).T, P, rtol=1e-6)
    assert abs(cam.prec - 0.35) < 1e-7 and cam.draw_water == 1 and cam.low_res_div3 == 0


def scene(n=64, seed=0):
    rock = O.fbm(n, seed=seed, lo=0.0, hi=40.0)
    dirt = O.fbm(n, seed=seed + 1, lo=0.0, hi=2.0)
    water = np.where(rock < 12.0, 12.0 - rock, 0.0).astype(np.float32)
    sed = np.zeros((n, n), np.float32)
    return dict(rock=rock, dirt=dirt, water=water, sediment=sed, sediment_dirt=sed.copy())


def test_render_properties():
    n = 64
    f = scene(n)
    cam = H.camera((-8.0, 70.0, -8.0), (1.0, -0.5, 1.0), aspect=4 / 3)
    rgba, rgb = O.render(f, n, cam, 96, 72, max_height=64.0)
    again, _ = O.render(f, n, cam, 96, 72, max_height=64.0)
    assert np.array_equal(rgba, again)
    assert np.all(rgba[..., 3] == 0)
    # a ray through the top row rises above the map: sky colours, blue-dominant
    top = rgba[-1, :, :3].astype(int)
    assert np.all(top[:, 2] > top[:, 0])
    # terrain in view: the image is not one colour
    assert len(np.unique(rgba[..., :3].reshape(-1, 3), axis=0)) > 50
    # NaN colours (GLSL pow of a negative mix) store as 0; finite ones round
    fin = np.isfinite(rgb)
    q = np.floor(np.clip(rgb[fin], 0, 1) * 255 + 0.5).astype(np.uint8)
    assert np.array_equal(rgba[..., :3][fin], q)
    # low-resolution form: 3x3 blocks of one colour, alpha 255
    cam.low_res_div3 = 1
    low, _ = O.render(f, n, cam, 96, 72, max_height=64.0)
    blocks = low.reshape(24, 3, 32, 3, 4)
    assert np.all(blocks == blocks[:, :1, :, :1, :]) and np.all(low[..., 3] == 255)
    # sediment tint: full rock sediment turns terrain pixels red
    cam.low_res_div3 = 0
    cam.display_sediment = 1
    g = dict(f, sediment=np.full((n, n), 1.0, np.float32))
    red, _ = O.render(g, n, cam, 96, 72, max_height=64.0)
    hit = np.any(rgba[..., :3] != red[..., :3], axis=2)
    assert hit.sum() > 100
    # full red except where the bilinear tap blends in the zeros beyond the map's edge
    assert np.mean(red[hit][:, 0] == 255) > 0.95
