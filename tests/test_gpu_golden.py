"""The GPU's grid step against the committed golden vectors (tests/golden/)
with no oracle at run time: per-pass and fused kernels, every state field
bit for bit (SHA-256 of the float32 field; on a mismatch the crops say
where).  Worlds start from the library's own fBm init (bit-identical to the
oracle's) and the named workloads' settings."""
import hashlib
import json
import os

import numpy as np
import pytest

import hydrogen as H

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
G = json.load(open(os.path.join(GOLDEN, "grid_golden.json")))
GRID = sorted(k for k, v in G.items() if v["kind"] == "grid")


def sha(a, dtype):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=dtype).tobytes()).hexdigest()


def make_world(name, g):
    n = g["n"]
    if g["layers"] == 1:
        w = H.World(n)
        w.init_heightmap(H.noise(seed=g["init_seeds"]["rock"]))
        H.configure(w, name.split("_")[0])
        return w
    w = H.World(n, layers=2)
    w.init_heightmap(H.noise(seed=g["init_seeds"]["rock"]))
    tmp = H.World(n)
    tmp.init_heightmap(H.noise(seed=g["init_seeds"]["dirt"], lo=0.0, hi=4.0))
    w.upload("dirt", tmp.download("rock"))
    tmp.close()
    s = H.ErosionSettings()
    H.check(H.lib.hg_default_erosion_settings(H.ctypes.byref(s)))
    w.set_erosion(s)
    w.set_rain(H.rain_uniform(0.01, 1))
    w.set_options(H.options(H.RAIN_UNIFORM))
    return w


@pytest.mark.parametrize("mode", [H.MODE_PLAIN, H.MODE_FUSED])
@pytest.mark.parametrize("name", GRID)
def test_gpu_matches_golden(name, mode):
    g = G[name]
    crops = np.load(os.path.join(GOLDEN, "grid_crops.npz"))
    w = make_world(name, g)
    w.step(g["steps"], mode)
    w.sync()
    bad = []
    for f, h in g["sha256"].items():
        a = np.ascontiguousarray(w.download(f), dtype=np.float32)
        if hashlib.sha256(a.tobytes()).hexdigest() != h:
            c = g["n"] // 2 - 4
            where = {"lo_lo": (0, 0), "lo_hi": (0, g["n"] - 8), "hi_lo": (g["n"] - 8, 0),
                     "hi_hi": (g["n"] - 8, g["n"] - 8), "mid": (c, c)}
            crop_bad = [k for k, (y, x) in where.items()
                        if not np.array_equal(a[y:y + 8, x:x + 8].view(np.uint32),
                                              crops[f"{name}/{f}/{k}"].view(np.uint32))]
            bad.append((f, crop_bad))
    w.close()
    assert not bad, f"fields differing from the golden vectors (field, crops that differ): {bad}"


def test_gpu_particles_match_golden():
    """Particle mode on the vectors' 128² two-layer world (4096 droplets, the
    reference's particle defaults, 25 steps): fields, momentum map and
    droplet state bit for bit."""
    g = G["particles_128x25"]
    n = g["n"]
    w = H.World(n, layers=2)
    w.init_heightmap(H.noise(seed=g["rock_seed"]))
    tmp = H.World(n)
    tmp.init_heightmap(H.noise(seed=g["dirt_seed"], lo=0.0, hi=g["dirt_hi"]))
    w.upload("dirt", tmp.download("rock"))
    tmp.close()
    w.particles_init(g["count"])
    w.set_erosion(H.settings_particles())
    w.set_options(H.options(H.RAIN_UNIFORM, seed=g["rain_seed"]))
    for _ in range(g["steps"]):
        w.step(1, H.MODE_PARTICLES)
    names = {"rock": "rock", "dirt": "dirt", "water": "water", "vel_u": "momentum_x", "vel_v": "momentum_y"}
    got = {f: sha(w.download(gf), np.float32) for f, gf in names.items()}
    st, it, kl = w.particles()
    got["droplet_state"] = sha(st, np.float32)
    got["droplet_iters"] = sha(it, np.uint32)
    got["droplet_kill"] = sha(kl, np.int32)
    w.close()
    bad = [k for k in g["sha256"] if got[k] != g["sha256"][k]]
    assert not bad, f"differ from the golden vectors: {bad}"


@pytest.mark.parametrize("mode", [H.MODE_PLAIN, H.MODE_FUSED])
def test_gpu_render_matches_golden(mode):
    """The ray-marcher over the GPU's own config2_256x100 world: RGBA8 pixels
    and float colours bit for bit."""
    g = G["render_config2_256x100"]
    src = G[g["of"]]
    w = make_world(g["of"], src)
    w.step(src["steps"], mode)
    cam = H.camera(tuple(g["pos"]), tuple(g["dir"]), aspect=g["aspect"])
    rgba, rgb = w.render(cam, g["width"], g["height"], rgb=True)
    w.close()
    assert sha(rgba, np.uint8) == g["sha256"]["rgba8"]
    assert hashlib.sha256(np.ascontiguousarray(rgb, dtype=np.float32).view(np.uint32).tobytes()).hexdigest() == \
        g["sha256"]["rgb_bits"]
