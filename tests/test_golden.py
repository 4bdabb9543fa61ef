"""The float oracle against the committed golden vectors (tests/golden/,
made by tests/golden/make_golden.py): after each workload's steps every
state field equals the vectors bit for bit (SHA-256, the crops and the FP64
sum of the field), and the FP64 oracle's totals agree within 1e-9 relative.
This pins the restatement against drift; the GPU side of the same vectors is
tests/test_gpu_golden.py."""
import importlib.util
import json
import os

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
G = json.load(open(os.path.join(GOLDEN, "grid_golden.json")))
GRID = sorted(k for k, v in G.items() if v["kind"] == "grid")


def maker():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.mark.parametrize("name", GRID)
def test_float_oracle_reproduces_golden(name):
    m, g = maker(), G[name]
    crops = np.load(os.path.join(GOLDEN, "grid_crops.npz"))
    s, o = m.settings_from(O, g["settings"]), m.options_from(O, g["options"])
    w = m.run_oracle(O, g["n"], g["steps"], g["layers"], s, o, 32)
    for f, h in g["sha256"].items():
        a = w.get(f).astype(np.float32)
        for cname, (y, x) in m.crop_corners(g["n"]).items():
            ref = crops[f"{name}/{f}/{cname}"]
            assert np.array_equal(a[y:y + 8, x:x + 8].view(np.uint32), ref.view(np.uint32)), (f, cname)
        assert m.digest(a) == h, f
        assert float(np.sum(a, dtype=np.float64)) == pytest.approx(g["sum_f64"][f], rel=1e-12, abs=1e-12)


@pytest.mark.parametrize("name", GRID)
def test_fp64_oracle_totals_match_golden(name):
    m, g = maker(), G[name]
    s, o = m.settings_from(O, g["settings"]), m.options_from(O, g["options"])
    t = m.run_oracle(O, g["n"], g["steps"], g["layers"], s, o, 64).totals()
    got = dict(zip(("rock", "dirt", "water", "sediment"), t))
    for k, v in g["fp64_oracle_totals"].items():
        assert got[k] == pytest.approx(v, rel=1e-9, abs=1e-9), k


def test_golden_settings_are_the_workloads():
    """The vectors' settings are the named workloads' (config1, config2) and
    the reference defaults the library states, so the GPU test's worlds,
    configured by name, step the same inputs."""
    import hydrogen as H
    m = maker()
    for cfg in ("config1", "config2"):
        s, o = O.workload(cfg)
        assert G[f"{cfg}_256x100"]["settings"] == m.settings_dict(s)
        assert G[f"{cfg}_256x100"]["options"] == m.options_dict(o)
    d = H.ErosionSettings()
    H.check(H.lib.hg_default_erosion_settings(H.ctypes.byref(d)))
    assert G["two_layer_128x40"]["settings"] == m.settings_dict(O.erosion_from(d))


def test_oracle_particles_reproduce_golden():
    """The oracle's particle mode (droplets in id order) on the vectors' 128²
    two-layer world: fields, momentum map and droplet state bit for bit."""
    import hydrogen as H
    m = maker()
    w = m.particle_run(O, H)
    st, it, kl = w.particles()
    got = m.particle_digests({f: w.get(f).astype(np.float32) for f in m.DROPLETS}, st, it, kl)
    assert got == G["particles_128x25"]["sha256"]


def test_oracle_render_reproduces_golden():
    """The ray-marcher's restatement over config2_256x100's final fields:
    RGBA8 pixels and float colours bit for bit."""
    import hydrogen as H
    m, g = maker(), G["render_config2_256x100"]
    src = G[g["of"]]
    s, o = m.settings_from(O, src["settings"]), m.options_from(O, src["options"])
    w = m.run_oracle(O, src["n"], src["steps"], src["layers"], s, o, 32)
    rgba, rgb = O.render({f: w.get(f).astype(np.float32) for f in ("rock", "water", "sediment")}, src["n"],
                         m.render_camera(H), g["width"], g["height"], g["max_height"], g["hmap_dim_x"])
    assert m.render_digests(rgba, rgb) == g["sha256"]
