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
@pytest.mark.parametrize("name", sorted(G))
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
