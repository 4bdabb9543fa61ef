"""Known-answer tests that pin the oracle to the reference's GLSL passes.

hydro-gen ships no tests or golden vectors, so each case here is derived by
hand from the cited shader lines on a micro-grid whose outcome has a closed
form, and checked against the FP64 oracle (and the float oracle where the
case is exact in float).
"""
import math

import numpy as np
import pytest

import oracle as O



def f32(x):
    """The settings travel as float32 (std140 UBO); the FP64 oracle widens them."""
    return float(np.float32(x))


DT, G = f32(0.02), f32(9.81)
KC, KS, KD, KE = f32(0.1), f32(0.05), f32(0.05), f32(0.015)
KALPHA, KSPEED = f32(math.atan(0.65)), f32(0.3)


def settings(**kw):
    s = O.settings_config1()
    for k, v in kw.items():
        if isinstance(v, (tuple, list)):
            arr = getattr(s, k)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(s, k, v)
    return s


def world(n, prec=64, **fields):
    w = O.OracleWorld(n, prec)
    for k, v in fields.items():
        a = np.broadcast_to(np.asarray(v, dtype=np.float64), (n, n)).copy()
        w.set(k, a)
    return w


# ---- hydro_flux, glsl/hydro_flux.glsl:77-166 -------------------------------------

def test_flux_flat_lake_is_still():
    w = world(8, rock=5.0, water=1.0)
    w.run_pass("flux", settings())
    for f in ("flux_l", "flux_r", "flux_t", "flux_b", "vel_u", "vel_v"):
        assert np.all(w.get(f) == 0.0), f
    assert np.all(w.get("water") == 1.0)
    assert np.all(w.get("vel_z") == 2.0)  # d1 + d2


def test_flux_single_bump_outflow():
    rock = np.zeros((8, 8)); rock[3, 3] = 1.0
    w = world(8, rock=rock, water=1.0)
    w.run_pass("flux", settings())
    f = DT * G * 1.0  # :100-107, A = L = 1, old flux 0, dh = 1
    for name in ("flux_l", "flux_r", "flux_t", "flux_b"):
        got = w.get(name)
        assert got[3, 3] == pytest.approx(f, rel=1e-15)
        assert np.count_nonzero(got) == 1
    # K = min(1, d / (sum_out dt)) = 1 here; :133-134
    assert w.get("water")[3, 3] == pytest.approx(1.0 - DT * 4 * f, rel=1e-15)
    # inflow to the neighbours uses the OLD flux (0): their water is unchanged
    assert w.get("water")[3, 4] == 1.0
    # velocity uses the old flux too (:146-158): zero everywhere
    assert np.all(w.get("vel_u") == 0.0) and np.all(w.get("vel_v") == 0.0)


def test_flux_scaled_to_available_water():
    rock = np.zeros((8, 8)); rock[3, 3] = 1.0
    water = np.zeros((8, 8)); water[3, 3] = 0.001
    w = world(8, rock=rock, water=water)
    w.run_pass("flux", settings())
    f = DT * G * (1.0 + 0.001)  # dh includes the water column
    K = 0.001 / (4 * f * DT)
    assert K < 1
    assert w.get("flux_r")[3, 3] == pytest.approx(f * K, rel=1e-13)
    assert w.get("water")[3, 3] == pytest.approx(0.0, abs=1e-18)  # max(0, d + dt(0 - d/dt))


def test_flux_zero_over_zero_keeps_k_one():
    # d = 0 and no outflow: K = min(1, 0/0); GLSL min(x, y) = y < x ? y : x -> 1
    w = world(8, rock=2.0, water=0.0)
    w.run_pass("flux", settings())
    assert np.all(np.isfinite(w.get("flux_l")))
    assert np.all(w.get("water") == 0.0)
    assert np.all(w.get("vel_u") == 0.0)


def test_flux_closed_boundaries():
    # a tilted lake: every border outflow through the grid edge is zeroed (:110-119)
    x = np.arange(8)
    rock = np.broadcast_to(x[None, :] * 0.1, (8, 8))
    w = world(8, rock=rock, water=1.0)
    w.run_pass("flux", settings())
    assert np.all(w.get("flux_l")[:, 0] == 0.0)
    assert np.all(w.get("flux_r")[:, -1] == 0.0)
    assert np.all(w.get("flux_b")[0, :] == 0.0)
    assert np.all(w.get("flux_t")[-1, :] == 0.0)
    assert np.all(w.get("flux_l")[:, 1:] > 0.0)  # downhill to the left


def test_flux_velocity_from_old_flux():
    fr = np.zeros((8, 8)); fr[2, 2] = 0.5  # old right-flux of cell (x=2, y=2)
    w = world(8, rock=0.0, water=1.0, flux_r=fr)
    w.run_pass("flux", settings())
    # cell (3, 2): inl = 0.5; d2 = 1 + dt*(0.5 - 0) ; u = 0.5 / (d1 + d2)
    d2 = 1.0 + DT * 0.5
    assert w.get("water")[2, 3] == pytest.approx(d2, rel=1e-15)
    assert w.get("vel_u")[2, 3] == pytest.approx(0.5 / (1.0 + d2), rel=1e-15)
    # cell (2, 2) itself: u = (0 - 0 + 0.5 - 0) / vz
    assert w.get("vel_u")[2, 2] > 0


# ---- hydro_erosion, glsl/hydro_erosion.glsl:37-92 --------------------------------

def erosion_world(u, v, vz, sed=0.0, rock=10.0):
    w = world(8, rock=rock, water=vz / 2, vel_u=u, vel_v=v, vel_z=vz, sediment=sed)
    return w


def test_erosion_dissolve_flat():
    w = erosion_world(3.0, 4.0, 1.0)
    w.run_pass("erosion", settings())
    c = KC * 0.02 * 5.0  # Kc * max(0.02, sin_a = 0) * |v|
    delta = DT * KS * c
    assert w.get("rock")[4, 4] == pytest.approx(10.0 - delta, rel=1e-15)
    assert w.get("sediment")[4, 4] == pytest.approx(delta, rel=1e-15)
    assert np.all(w.get("dirt") == 0.0) and np.all(w.get("sediment_dirt") == 0.0)


def test_erosion_deposit():
    w = erosion_world(3.0, 4.0, 1.0, sed=0.05)
    w.run_pass("erosion", settings())
    c = KC * 0.02 * 5.0
    delta = DT * KD * (0.05 - c)
    assert w.get("rock")[4, 4] == pytest.approx(10.0 + delta, rel=1e-15)
    assert w.get("sediment")[4, 4] == pytest.approx(0.05 - delta, rel=1e-15)


def test_erosion_shallow_water_fade():
    # dd = 7.5e-4 < 1e-3: ero_vel = mix(|v|, 0, smoothstep(1e-3, 5e-4, dd)) = 5 * (1 - 0.5)
    w = erosion_world(3.0, 4.0, 7.5e-4)
    w.run_pass("erosion", settings())
    c = KC * 0.02 * 2.5
    assert w.get("sediment")[4, 4] == pytest.approx(DT * KS * c, rel=1e-12)


def test_erosion_tilted_normal():
    # rock slope 1 per cell along x: dx = 2, dz = 0 -> n = (4, -4, 0)/|.|, sin_a = sqrt(1/2)
    x = np.arange(8, dtype=np.float64)
    rock = np.broadcast_to(10.0 + x[None, :], (8, 8))
    w = world(8, rock=rock, water=0.5, vel_u=3.0, vel_v=4.0, vel_z=1.0)
    w.run_pass("erosion", settings())
    c = KC * math.sqrt(0.5) * 5.0
    assert w.get("sediment")[4, 4] == pytest.approx(DT * KS * c, rel=1e-12)


def test_erosion_border_normal_reads_zero():
    # out-of-range imageLoad returns 0: at x = 7 the right neighbour height is 0
    w = world(8, rock=10.0, water=0.5, vel_u=3.0, vel_v=4.0, vel_z=1.0)
    w.run_pass("erosion", settings())
    # dx = 0 - 10 = -10 -> sin_a = sqrt(1 - 16/(400+16))
    sin_a = math.sqrt(1 - 16 / 416)
    assert w.get("sediment")[4, 7] == pytest.approx(DT * KS * KC * sin_a * 5.0, rel=1e-12)


def test_erosion_layer_exhausted():
    # rock 1e-6 cannot supply the dissolve amount: sediment takes what is left
    w = erosion_world(3000.0, 4000.0, 1.0, rock=1e-6)
    w.run_pass("erosion", settings())
    c = KC * 0.02 * 5000.0
    delta = DT * KS * c
    assert w.get("rock")[4, 4] == 0.0
    assert w.get("sediment")[4, 4] == pytest.approx(delta + (1e-6 - delta), rel=1e-9)


# ---- sediment_transport + img_bilinear -----------------------------------------------

def test_sediment_semi_lagrangian_shift():
    x = np.arange(8, dtype=np.float64)
    sed = np.broadcast_to(x[None, :] * 0.01, (8, 8))
    w = world(8, rock=1.0, water=2.0, sediment=sed, vel_u=10.0, vel_v=0.0)
    w.run_pass("sediment", settings())
    # back-trace x - 0.2: bilinear between x-1 (weight 0.2) and x (0.8)
    got = w.get("sediment")
    fx = 1.0 - 10.0 * DT  # fract(x - u dt), ~0.8
    for xx in range(1, 8):
        expect = 0.01 * (xx - 1) * (1 - fx) + 0.01 * xx * fx
        assert got[3, xx] == pytest.approx(expect, rel=1e-12)
    assert got[3, 0] == 0.0  # clamped to 0
    assert np.all(w.get("water") == pytest.approx(2.0 * (1 - KE * DT), rel=1e-15))


def test_sediment_clamped_edge_tap():
    # back-trace beyond N-1 clamps to N-1: fract = 0, the +1 tap is outside (0)
    sed = np.full((8, 8), 0.3)
    w = world(8, rock=1.0, water=1.0, sediment=sed, vel_u=-1e4, vel_v=0.0)
    w.run_pass("sediment", settings())
    assert np.all(w.get("sediment") == 0.3)


def test_sediment_half_cell_both_axes():
    sed = np.zeros((8, 8)); sed[2, 2] = 1.0
    w = world(8, rock=1.0, water=1.0, sediment=sed, vel_u=-25.0, vel_v=-25.0)
    w.run_pass("sediment", settings())
    # cell (2, 2) traces back to (2 + 25 dt, 2 + 25 dt) ~ (2.5, 2.5): weight (1-f)^2 on its own value
    f = 25.0 * DT
    assert w.get("sediment")[2, 2] == pytest.approx((1 - f) * (1 - f), rel=1e-12)


# ---- thermal_erosion / thermal_transport (layer 0) --------------------------------------

def test_thermal_spike_all_marked():
    rock = np.zeros((5, 5)); rock[2, 2] = 2.0
    s = settings(Kspeed=(0.3, 0.0))
    w = world(5, rock=rock)
    w.run_pass("thermal_flux", s, layer=0)
    cross, diag = w.thermal()
    K = KALPHA
    sharp = 1 + math.atan(2.0) - K
    S = DT * KSPEED * sharp ** 3 * 1.0 * 2.0 / 2
    out = S * 2.0 / 16.0
    assert np.allclose(cross[2, 2], out, rtol=1e-12)
    assert np.allclose(diag[2, 2], out, rtol=1e-12)
    w.run_pass("thermal_transport", s, layer=0)
    r = w.get("rock")
    assert r[2, 2] == pytest.approx(2.0 - 8 * out, rel=1e-12)
    for dy, dx in [(0, 1), (1, 0), (1, 1), (-1, 1)]:
        assert r[2 + dy, 2 + dx] == pytest.approx(out, rel=1e-12)


def test_thermal_below_talus_no_flow():
    rock = np.zeros((5, 5)); rock[2, 2] = 0.5  # atan(0.5) < atan(0.65)
    s = settings(Kspeed=(0.3, 0.0))
    w = world(5, rock=rock)
    w.run_pass("thermal_flux", s, layer=0)
    cross, diag = w.thermal()
    assert np.all(cross == 0) and np.all(diag == 0)


def test_thermal_cross_only():
    # drop 0.8: cross slope 0.8 > 0.65 marked, diagonal 0.8/sqrt(2) = 0.566 not
    rock = np.zeros((5, 5)); rock[2, 2] = 0.8
    s = settings(Kspeed=(0.3, 0.0))
    w = world(5, rock=rock)
    w.run_pass("thermal_flux", s, layer=0)
    cross, diag = w.thermal()
    sharp = 1 + math.atan(0.8) - KALPHA
    S = DT * KSPEED * sharp ** 3 * 0.8 / 2
    assert np.allclose(cross[2, 2], S * 0.8 / 3.2, rtol=1e-12)
    assert np.all(diag[2, 2] == 0)


def test_thermal_border_neighbour_is_far():
    # out-of-range neighbours read 999999999999: no outflow through the edge
    rock = np.zeros((5, 5)); rock[0, 0] = 3.0
    s = settings(Kspeed=(0.3, 0.0))
    w = world(5, rock=rock)
    w.run_pass("thermal_flux", s, layer=0)
    cross, diag = w.thermal()
    assert cross[0, 0][0] == 0 and cross[0, 0][3] == 0  # L and B leave the grid
    assert cross[0, 0][1] > 0 and cross[0, 0][2] > 0


# ---- smoothing, glsl/smoothing.glsl:22-103 ---------------------------------------------

def test_smoothing_asymmetric_pit():
    rock = np.zeros((5, 5))
    rock[2, 1], rock[2, 3], rock[3, 2], rock[1, 2] = 2.0, 1.0, 1.0, 1.0
    s = settings(Kspeed=(0.0, 25.0))  # multip = clamp(25 * 0.02, 0, 1) = 0.5
    w = world(5, rock=rock)
    w.run_pass("smoothing", s)
    m = 25.0 * DT  # clamp(Kspeed[1] * d_t, 0, 1), ~0.5
    assert w.get("rock")[2, 2] == pytest.approx(m * (0 + 2 + 1 + 1 + 1) / 5.0, rel=1e-12)


def test_smoothing_identity_when_blend_zero():
    rng = np.random.default_rng(1)
    rock = rng.random((8, 8))
    w = world(8, rock=rock)
    w.run_pass("smoothing", settings())
    assert np.array_equal(w.get("rock"), rock)


# ---- rain and step sequencing --------------------------------------------------------------

def test_rain_uniform_and_period():
    w = world(8, rock=1.0)
    s = settings()
    o = O.options(rain_mode=1, period=3, amount=0.01)
    w.step(s, o, 2)
    assert np.all(w.get("water") == 0.0)  # steps 1, 2: no rain
    w.step(s, o, 1)
    assert np.all(w.get("water") > 0.0)  # step 3 rains (src/main.cpp:315-319)


def test_bernoulli_rain_rate():
    n = 256
    thr = O.bernoulli_threshold(0.01)
    words = np.array([[O.rain_word(x, y, 7, 0, 123) for x in range(n)] for y in range(0, n, 8)])
    rate = np.mean(words < thr)
    assert abs(rate - 0.01) < 4 * math.sqrt(0.01 * 0.99 / words.size)


def test_philox_words_distinct_per_cell():
    a = [O.rain_word(x, 5, 1, 0, 0) for x in range(64)]
    assert len(set(a)) == 64
    assert O.rain_word(0, 0, 1, 0, 0) != O.rain_word(0, 0, 2, 0, 0)


# ---- single-material form of the two-layer model -------------------------------------------

def test_empty_dirt_layer_stays_empty():
    n = 64
    rock = O.fbm(n)
    w = world(n, prec=32, rock=rock)
    s, o = O.workload("config2")
    o.skip_identity = 0  # run all reference passes, thermal layer 1 and smoothing included
    w.step(s, o, 50)
    assert np.all(w.get("dirt") == 0.0)
    assert np.all(w.get("sediment_dirt") == 0.0)


def test_skipping_identity_passes_is_exact():
    n = 64
    rock = O.fbm(n)
    s, o = O.workload("config2")
    a = world(n, prec=32, rock=rock)
    b = world(n, prec=32, rock=rock)
    o_full = O.options(2, 1, 0.5, p=0.001, skip_identity=0)
    a.step(s, o, 40)
    b.step(s, o_full, 40)
    for f in ("rock", "water", "sediment", "flux_l", "vel_u"):
        assert np.array_equal(a.get(f), b.get(f)), f


# ---- helpers of the restatement ---------------------------------------------------------------

def test_poly_atan_accuracy():
    xs = np.r_[np.linspace(0, 4, 4001), np.geomspace(4, 1e8, 2000)].astype(np.float32)
    for x in xs:
        got = O.atanf(float(x))
        ref = math.atan(float(x))
        assert abs(got - ref) <= 3 * float(np.spacing(np.float32(ref)))


def test_poly_atan_monotone_every_positive_float():
    # the fused kernel's one-arctangent-per-cell talus test relies on this
    assert O.atan_monotone_violations() == 0


def test_fbm_range_and_determinism():
    a = O.fbm(128, seed=3)
    b = O.fbm(128, seed=3)
    c = O.fbm(128, seed=4)
    assert a.min() == 0.0 and a.max() == 64.0
    assert np.array_equal(a, b) and not np.array_equal(a, c)
