"""Particle (droplet) erosion on two-layer worlds against the oracle's
sequential restatement (droplets in id order, corners 0..3), bit for bit:
droplet state, rock, dirt, water and the momentum map, with the reference's
particle defaults and with denser droplets sharing texels."""
import numpy as np
import pytest

import hydrogen as H
import oracle as O

pytestmark = pytest.mark.gpu

FIELDS = [("rock", "rock"), ("dirt", "dirt"), ("water", "water"), ("momentum_x", "vel_u"), ("momentum_y", "vel_v")]


def make(n, count, settings, seed=0, rain=True, rain_seed=7):
    w = H.World(n, layers=2)
    w.init_heightmap(H.noise(seed=seed))
    dirt = O.fbm(n, seed=seed + 3, lo=0.0, hi=2.0).astype(np.float32)
    w.upload("dirt", dirt)
    w.particles_init(count)
    w.set_erosion(settings)
    w.set_options(H.options(H.RAIN_UNIFORM if rain else H.RAIN_OFF, seed=rain_seed))
    ow = O.OracleWorld(n, 32)
    ow.set("rock", w.download("rock"))
    ow.set("dirt", dirt)
    ow.particles_init(count)
    oo = O.options(1 if rain else 0, 1, 0.0, seed=rain_seed)
    return w, ow, O.erosion_from(settings), oo


def check(w, ow, ctx):
    gs, gi, gk = w.particles()
    rs, ri, rk = ow.particles()
    for name, a, b in (("state", gs, rs), ("iters", gi, ri), ("kill", gk, rk)):
        bad = np.argwhere(a.view(np.uint32) != b.view(np.uint32)) if a.dtype == np.float32 else np.argwhere(a != b)
        assert bad.size == 0, f"{ctx} droplet {name}: {len(bad)} differ, first {bad[:3].tolist()}"
    for gf, of in FIELDS:
        g, r = w.download(gf), ow.get(of).astype(np.float32)
        bad = np.argwhere(g.view(np.uint32) != r.view(np.uint32))
        assert bad.size == 0, f"{ctx} {gf}: {len(bad)} cells differ, first {bad[:3].tolist()}"


@pytest.mark.parametrize("n,count,steps", [(64, 256, 40), (128, 4096, 25)])
def test_particles_bitwise_vs_oracle(n, count, steps):
    s = H.settings_particles()
    w, ow, os_, oo = make(n, count, s)
    for k in range(steps):
        w.step(1, H.MODE_PARTICLES)
        ow.particle_step(os_, oo, 1)
        if k in (0, 1, steps // 2, steps - 1):
            check(w, ow, f"n={n} count={count} step {k + 1}")
    st, it, kl = w.particles()
    assert np.all(it > 0) and np.any(st[:, 6] != 0.0)
    assert np.any(w.download("momentum_x") != 0.0)


def test_particles_crowded_texels_and_kills():
    # few texels, many droplets: long per-texel record lists; short ttl and
    # fast evaporation exercise the kill path and respawns
    s = H.settings_particles()
    s.ttl = 6
    s.Ke = 0.2
    s.Kspeed[0] = 0.0
    w, ow, os_, oo = make(16, 2048, s, seed=2)
    for k in range(20):
        w.step(1, H.MODE_PARTICLES)
        ow.particle_step(os_, oo, 1)
    check(w, ow, "crowded")
    _, it, _ = w.particles()
    assert it.max() <= 6


@pytest.mark.parametrize("count", [16384, 65536])
def test_particles_pile_up_beyond_shared_sort(count):
    # thousands of droplets on an 8x8 map: every live droplet sits on the
    # same few texels, buckets of thousands to tens of thousands of records
    # (several of the 2048-record chunks a warp sorts in shared memory,
    # merged by rank)
    s = H.settings_particles()
    s.Kspeed[0] = 0.0
    w, ow, os_, oo = make(8, count, s, seed=5)
    for k in range(3):
        w.step(1, H.MODE_PARTICLES)
        ow.particle_step(os_, oo, 1)
        check(w, ow, f"pile-up step {k + 1}")


def test_particles_rain_off_keeps_idle_and_limits():
    s = H.settings_particles()
    w, ow, os_, oo = make(64, 256, s, rain=False)
    rock0 = w.download("rock")
    w.step(3, H.MODE_PARTICLES)
    ow.particle_step(os_, oo, 3)
    check(w, ow, "rain off")
    _, it, _ = w.particles()
    assert np.all(it == 0)
    # thermal passes still move rock on a rough map
    assert w.download("rock").shape == rock0.shape
    one = H.World(64, layers=1)
    with pytest.raises(H.HydrogenError) as e:
        one.particles_init(16)
    assert e.value.code == -5
    v = H.World(64, layers=2)
    with pytest.raises(H.HydrogenError):
        v.step(1, H.MODE_PARTICLES)
    s.particle_count = 256
    w.set_erosion(s)  # the droplet count is accepted
    s.particle_count = 255
    with pytest.raises(H.HydrogenError):
        w.set_erosion(s)


def test_particles_checkpoint_resume_is_bitwise(tmp_path):
    s = H.settings_particles()
    a, _, _, _ = make(64, 512, s, seed=3)
    a.step(10, H.MODE_PARTICLES)
    path = str(tmp_path / "p.bin")
    a.save(path)
    a.step(12, H.MODE_PARTICLES)
    b = H.World(64, layers=2)
    b.load(path)  # sets up the droplets from the file
    b.step(12, H.MODE_PARTICLES)
    sa, ia, ka = a.particles()
    sb, ib, kb = b.particles()
    assert np.array_equal(sa.view(np.uint32), sb.view(np.uint32)) and np.array_equal(ia, ib)
    assert np.array_equal(ka, kb)
    for f in ("rock", "dirt", "water", "momentum_x", "momentum_y"):
        assert np.array_equal(a.download(f), b.download(f)), f
