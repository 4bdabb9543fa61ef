"""The CPU restatement of hydro-gen's terrain generator and rain
(oracle/hg_terrain_ref.cpp) pinned without a GPU: the simplex noise against an
independent float64 implementation of the published algorithm (McEwan et al.,
JGT 2012), the gradient noise's analytic derivatives against central
differences of its value, and properties of the generator and the rain."""
import math

import numpy as np

import oracle as O


def simplex64(x, y):
    """2-D simplex noise in float64 from the published description."""
    F, G, G2, R = 0.366025403784439, 0.211324865405187, -0.577350269189626, 0.024390243902439
    s = (x + y) * F
    i, j = math.floor(x + s), math.floor(y + s)
    t = (i + j) * G
    x0, y0 = x - i + t, y - j + t
    ox, oy = (1.0, 0.0) if x0 > y0 else (0.0, 1.0)
    corners = [(x0, y0), (x0 + G - ox, y0 + G - oy), (x0 + G2, y0 + G2)]
    perm = lambda v: ((v * 34.0 + 1.0) * v) % 289.0
    im, jm = i % 289.0, j % 289.0
    hashes = [perm(perm(jm + dj) + im + di) for di, dj in ((0.0, 0.0), (ox, oy), (1.0, 1.0))]
    total = 0.0
    for (cx, cy), h in zip(corners, hashes):
        w = max(0.5 - (cx * cx + cy * cy), 0.0) ** 4
        gx = 2.0 * ((h * R) % 1.0) - 1.0
        gy = abs(gx) - 0.5
        a = gx - math.floor(gx + 0.5)
        w *= 1.79284291400159 - 0.85373472095314 * (a * a + gy * gy)
        total += w * (a * cx + gy * cy)
    return 130.0 * total


def test_simplex_is_the_published_algorithm():
    rng = np.random.default_rng(3)
    # the float restatement loses precision with the coordinates' magnitude
    # (|v| = 300 has a 3e-5 ulp); the tolerance follows it
    for span, tol in ((40.0, 2e-5), (300.0, 2e-4)):
        pts = rng.uniform(-span, span, size=(2000, 2)).astype(np.float32)
        err = max(abs(O.ref_simplex(float(x), float(y)) - simplex64(float(x), float(y))) for x, y in pts)
        assert err < tol, (span, err)
    vals = [O.ref_simplex(float(x), float(y)) for x, y in pts]
    assert -1.0 <= min(vals) < -0.5 and 0.5 < max(vals) <= 1.0


def test_gradient_noise_derivatives():
    rng = np.random.default_rng(4)
    h = 1e-2
    for x, y in rng.uniform(-50, 50, size=(300, 2)):
        v, dx, dy = O.ref_noised(x, y)
        fx = (O.ref_noised(x + h, y)[0] - O.ref_noised(x - h, y)[0]) / (2 * h)
        fy = (O.ref_noised(x, y + h)[0] - O.ref_noised(x, y - h)[0]) / (2 * h)
        assert abs(fx - dx) < 2e-3 and abs(fy - dy) < 2e-3, (x, y, dx, fx, dy, fy)


def test_heightmap_properties():
    import ctypes

    class Map(ctypes.Structure):
        _fields_ = [("max_height", ctypes.c_float), ("max_dirt", ctypes.c_float), ("hmap_dims", ctypes.c_int32 * 2),
                    ("height_mult", ctypes.c_float), ("water_lvl", ctypes.c_float), ("seed", ctypes.c_float),
                    ("persistance", ctypes.c_float), ("lacunarity", ctypes.c_float), ("scale", ctypes.c_float),
                    ("redistribution", ctypes.c_float), ("octaves", ctypes.c_int32), ("fake_erosion", ctypes.c_uint32),
                    ("mask_round", ctypes.c_uint32), ("mask_exp", ctypes.c_uint32), ("mask_power", ctypes.c_uint32),
                    ("mask_slope", ctypes.c_uint32), ("uplift", ctypes.c_uint32), ("uplift_scale", ctypes.c_float),
                    ("domain_warp", ctypes.c_int32), ("domain_warp_scale", ctypes.c_float),
                    ("terrace", ctypes.c_int32), ("terrace_scale", ctypes.c_float), ("pad", ctypes.c_float)]
    assert ctypes.sizeof(Map) == 96
    m = Map(256.0, 2.0, (64, 64), 1.0, 96.0, 0.0, 0.44, 2.0, 0.00075 * 16, 1.0, 8, 0, 0, 1, 1, 0, 0, 1.16, 1,
            100.0, 0, 0.5, 0.0)
    rock, dirt = O.ref_heightmap(m, 64)
    rock2, dirt2 = O.ref_heightmap(m, 64)
    assert np.array_equal(rock, rock2) and np.array_equal(dirt, dirt2)
    assert rock.max() <= 256.0 and rock.min() >= 0.0 and rock.std() > 0.0
    assert 0.0 < dirt.min() and dirt.max() < 2.0 * 2.5
    m.seed = 7.0
    assert not np.array_equal(O.ref_heightmap(m, 64)[0], rock)
    m.seed, m.terrace = 0.0, 4
    terraced = O.ref_heightmap(m, 64)[0]
    assert len(np.unique(terraced)) > 1 and not np.array_equal(terraced, rock)


def test_rain_increment_properties():
    class Rain:
        amount, mountain_thresh, mountain_multip, drops = 0.01, 0.55, 0.05, 0.02
    n = 64
    low = np.zeros((n, n), np.float32)
    high = np.full((n, n), 200.0, np.float32)  # above 0.55 * 256
    a = O.ref_rain(low, 0.37, Rain, 256.0)
    b = O.ref_rain(high, 0.37, Rain, 256.0)
    assert a.min() >= 0.0 and a.max() > 0.0
    assert np.all(b >= a) and np.any(b > a)  # the mountain bonus
    assert np.array_equal(np.nonzero(a)[0], np.nonzero(b)[0])  # both scale the same noise r
    assert not np.array_equal(O.ref_rain(low, 0.52, Rain, 256.0), a)  # the frame time seeds it
