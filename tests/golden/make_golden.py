"""Golden vectors of the grid step, made by the float oracle (the C++
restatement of the reference's passes) and checked in for the parity tests.

    python tests/golden/make_golden.py        (from the repository root)

The reference (hydro-gen) ships no tests, fixtures or golden vectors and its
GLSL passes need an OpenGL context, so these vectors come from the oracle.
They freeze its output: `tests/test_golden.py` re-runs the oracle against
them on the host, and `tests/test_gpu_golden.py` checks the GPU's fields
against them with no oracle at run time.  Per workload:

- SHA-256 of every float32 state field after the steps (bit-exact pin),
- 8 x 8 crops of every field at the four corners and the centre
  (`grid_crops.npz`, float32; they locate a difference the hashes report),
- the FP64 sums of the float fields, and the FP64 oracle's totals of rock,
  water and sediment on the same inputs (a cross-check with a tolerance:
  libm's double-precision functions may differ between hosts),
- the settings and options themselves, so the check needs only the oracle.

Workloads (seeded simplex fBm heightmaps, seed 0, scaled to [0, 64]):
config1_256x100 (uniform rain 0.01, no thermal, 100 steps), config2_256x100
(thermal, Bernoulli rain 0.5 at p = 0.001, 100 steps) and two_layer_128x40
(rock + dirt, the reference's default settings of src/state.cpp:81-92,
uniform rain 0.01, 40 steps); then particles_128x25 (4096 droplets on a
two-layer 128² world with the reference's particle defaults, 25 steps:
fields, momentum map and droplet state) and render_config2_256x100 (a
96 x 96 frame of the ray-marcher over config2_256x100's final fields: the
RGBA8 pixels and the float colours' bits).
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

ONE = ["rock", "water", "sediment", "flux_l", "flux_r", "flux_t", "flux_b", "vel_u", "vel_v"]
TWO = ONE + ["dirt", "sediment_dirt"]


def settings_dict(s):
    out = {}
    for name, _ in s._fields_:
        v = getattr(s, name)
        out[name] = list(v) if hasattr(v, "__len__") else v
    return out


def settings_from(O, d):
    s = O.OracleErosion()
    for k, v in d.items():
        if isinstance(v, list):
            for i, x in enumerate(v):
                getattr(s, k)[i] = x
        else:
            setattr(s, k, v)
    return s


def options_dict(o):
    return {name: getattr(o, name) for name, _ in o._fields_}


def options_from(O, d):
    o = O.OracleOptions()
    for k, v in d.items():
        setattr(o, k, v)
    return o


def cases(O):
    """name -> (n, steps, layers, settings, options)."""
    out = {}
    for cfg in ("config1", "config2"):
        s, o = O.workload(cfg)
        out[f"{cfg}_256x100"] = (256, 100, 1, s, o)
    # the reference's grid defaults (src/state.cpp:81-92) as the library
    # states them (a host-only call)
    sys.path.insert(0, os.path.join(ROOT, "hydro-gen_gb300"))
    import hydrogen as H
    d = H.ErosionSettings()
    H.check(H.lib.hg_default_erosion_settings(H.ctypes.byref(d)))
    out["two_layer_128x40"] = (128, 40, 2, O.erosion_from(d), O.options(1, 1, 0.01))
    return out


def initial(O, n, layers):
    init = {"rock": O.fbm(n, seed=0)}
    if layers == 2:
        init["dirt"] = O.fbm(n, seed=3, lo=0.0, hi=4.0)
    return init


def run_oracle(O, n, steps, layers, s, o, precision):
    w = O.OracleWorld(n, precision)
    for f, a in initial(O, n, layers).items():
        w.set(f, a)
    w.step(s, o, steps)
    return w


def crop_corners(n):
    c = n // 2 - 4
    return {"lo_lo": (0, 0), "lo_hi": (0, n - 8), "hi_lo": (n - 8, 0), "hi_hi": (n - 8, n - 8), "mid": (c, c)}


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float32).tobytes()).hexdigest()


PARTICLES = {"n": 128, "count": 4096, "steps": 25, "rain_seed": 7, "rock_seed": 0, "dirt_seed": 3, "dirt_hi": 2.0}
RENDER = {"of": "config2_256x100", "pos": [-10.0, 120.0, 96.0], "dir": [1.0, -0.7, 0.1], "aspect": 1.0,
          "width": 96, "height": 96, "max_height": 256.0, "hmap_dim_x": 1024}
DROPLETS = ["rock", "dirt", "water", "vel_u", "vel_v"]  # vel_u / vel_v: the momentum map's x / y


def particle_run(O, H):
    """The oracle's particle mode (droplets in id order) on PARTICLES."""
    P = PARTICLES
    s = H.settings_particles()
    w = O.OracleWorld(P["n"], 32)
    w.set("rock", O.fbm(P["n"], seed=P["rock_seed"]))
    w.set("dirt", O.fbm(P["n"], seed=P["dirt_seed"], lo=0.0, hi=P["dirt_hi"]))
    w.particles_init(P["count"])
    o = O.options(1, 1, 0.0, seed=P["rain_seed"])
    for _ in range(P["steps"]):
        w.particle_step(O.erosion_from(s), o, 1)
    return w


def particle_digests(fields, state, iters, kill):
    out = {f: digest(a) for f, a in fields.items()}
    out["droplet_state"] = hashlib.sha256(np.ascontiguousarray(state, dtype=np.float32).tobytes()).hexdigest()
    out["droplet_iters"] = hashlib.sha256(np.ascontiguousarray(iters, dtype=np.uint32).tobytes()).hexdigest()
    out["droplet_kill"] = hashlib.sha256(np.ascontiguousarray(kill, dtype=np.int32).tobytes()).hexdigest()
    return out


def render_digests(rgba, rgb):
    return {"rgba8": hashlib.sha256(np.ascontiguousarray(rgba, dtype=np.uint8).tobytes()).hexdigest(),
            "rgb_bits": hashlib.sha256(np.ascontiguousarray(rgb, dtype=np.float32).view(np.uint32).tobytes()).hexdigest()}


def render_camera(H):
    return H.camera(tuple(RENDER["pos"]), tuple(RENDER["dir"]), aspect=RENDER["aspect"])


def main():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "hydro-gen_gb300"))
    import oracle as O
    import hydrogen as H
    golden, crops = {}, {}
    for name, (n, steps, layers, s, o) in cases(O).items():
        fields = TWO if layers == 2 else ONE
        w = run_oracle(O, n, steps, layers, s, o, 32)
        w64 = run_oracle(O, n, steps, layers, s, o, 64)
        t64 = w64.totals()  # rock, dirt, water, sediment (both channels)
        entry = {"kind": "grid", "n": n, "steps": steps, "layers": layers, "init_seeds": {"rock": 0, "dirt": 3},
                 "settings": settings_dict(s), "options": options_dict(o), "sha256": {}, "sum_f64": {},
                 "fp64_oracle_totals": {"rock": t64[0], "dirt": t64[1], "water": t64[2], "sediment": t64[3]}}
        for f in fields:
            a = w.get(f).astype(np.float32)
            entry["sha256"][f] = digest(a)
            entry["sum_f64"][f] = float(np.sum(a, dtype=np.float64))
            for cname, (y, x) in crop_corners(n).items():
                crops[f"{name}/{f}/{cname}"] = a[y:y + 8, x:x + 8].copy()
        golden[name] = entry
        print(name, {f: entry["sha256"][f][:12] for f in fields})
        if name == RENDER["of"]:
            rgba, rgb = O.render({f: w.get(f).astype(np.float32) for f in ("rock", "water", "sediment")}, n,
                                 render_camera(H), RENDER["width"], RENDER["height"], RENDER["max_height"],
                                 RENDER["hmap_dim_x"])
            golden["render_" + name] = dict(RENDER, kind="render", sha256=render_digests(rgba, rgb))
            print("render_" + name, golden["render_" + name]["sha256"])
    pw = particle_run(O, H)
    st, it, kl = pw.particles()
    golden["particles_128x25"] = dict(PARTICLES, kind="particles", sha256=particle_digests(
        {f: pw.get(f).astype(np.float32) for f in DROPLETS}, st, it, kl))
    print("particles_128x25", {k: v[:12] for k, v in golden["particles_128x25"]["sha256"].items()})
    with open(os.path.join(HERE, "grid_golden.json"), "w") as fh:
        json.dump(golden, fh, indent=1, sort_keys=True)
        fh.write("\n")
    np.savez_compressed(os.path.join(HERE, "grid_crops.npz"), **crops)


if __name__ == "__main__":
    main()
