"""ctypes wrapper of the oracle library — TEST INFRASTRUCTURE ONLY.

The oracle (hg_oracle.cpp) restates hydro-gen's GLSL grid-erosion passes on
the CPU, in float (the reference's precision) or double.  Only tests, the
smoke check and the benchmark's CPU-baseline legs use it, always as the
checker or the timed CPU baseline, never as part of the product path.

Parity unpinned: the reference ships no tests or golden vectors and its GLSL
passes cannot run without an OpenGL driver, so the restatement is pinned by
the hand-derived known-answer cases in tests/test_oracle_kat.py instead.
"""
import ctypes
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhg_oracle.so")

FIELDS = {"rock": 0, "water": 1, "sediment": 2, "flux_l": 3, "flux_r": 4, "flux_t": 5, "flux_b": 6,
          "vel_u": 7, "vel_v": 8, "dirt": 9, "sediment_dirt": 10, "vel_z": 11, "total": 12, "vel_w": 13}
PASSES = {"rain": 0, "flux": 1, "erosion": 2, "sediment": 3, "thermal_flux": 4, "thermal_transport": 5,
          "smoothing": 6}


class OracleErosion(ctypes.Structure):
    """Erosion_data, glsl/bindings.glsl:39-60 (std140, 96 bytes)."""
    _fields_ = [("particle_count", ctypes.c_uint32), ("Kc", ctypes.c_float),
                ("Kalpha", ctypes.c_float * 2), ("Kconv", ctypes.c_float), ("pad0", ctypes.c_float),
                ("Ks", ctypes.c_float * 2), ("Kd", ctypes.c_float * 2), ("Ke", ctypes.c_float),
                ("ENERGY_KEPT", ctypes.c_float), ("Kspeed", ctypes.c_float * 2), ("G", ctypes.c_float),
                ("d_t", ctypes.c_float), ("density", ctypes.c_float), ("init_volume", ctypes.c_float),
                ("friction", ctypes.c_float), ("inertia", ctypes.c_float), ("min_volume", ctypes.c_float),
                ("min_velocity", ctypes.c_float), ("ttl", ctypes.c_uint32), ("pad1", ctypes.c_uint32)]


class OracleOptions(ctypes.Structure):
    _fields_ = [("rain_mode", ctypes.c_int32), ("rain_period", ctypes.c_int32), ("rain_amount", ctypes.c_float),
                ("rain_threshold", ctypes.c_uint32), ("rain_seed", ctypes.c_uint64),
                ("terrain_id", ctypes.c_uint32), ("skip_identity", ctypes.c_int32),
                ("rain_time0", ctypes.c_float), ("rain_time_step", ctypes.c_float),
                ("mountain_thresh", ctypes.c_float), ("mountain_multip", ctypes.c_float), ("drops", ctypes.c_float),
                ("max_height", ctypes.c_float)]


def build():
    import importlib.util
    spec = importlib.util.spec_from_file_location("_oracle_build", os.path.join(HERE, "build.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m.build()


def _load():
    if not os.path.exists(LIB_PATH):
        build()
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    sig = {
        "hgo_create": (P, [ctypes.c_int, ctypes.c_int]),
        "hgo_destroy": (None, [P]),
        "hgo_set_field": (ctypes.c_int, [P, ctypes.c_int, P]),
        "hgo_get_field": (ctypes.c_int, [P, ctypes.c_int, P]),
        "hgo_set_ks_field": (ctypes.c_int, [P, P]),
        "hgo_set_step": (None, [P, ctypes.c_uint64]),
        "hgo_get_step": (ctypes.c_uint64, [P]),
        "hgo_step": (ctypes.c_int, [P, ctypes.POINTER(OracleErosion), ctypes.POINTER(OracleOptions), ctypes.c_int]),
        "hgo_pass": (ctypes.c_int, [P, ctypes.POINTER(OracleErosion), ctypes.POINTER(OracleOptions), ctypes.c_int,
                                    ctypes.c_int]),
        "hgo_set_rows": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int]),
        "hgo_tex_rows": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, ctypes.c_int]),
        "hgo_get_thermal": (ctypes.c_int, [P, P, P]),
        "hgo_totals": (None, [P, ctypes.POINTER(ctypes.c_double)]),
        "hgo_atanf": (ctypes.c_float, [ctypes.c_float]),
        "hgo_set_float_atan_libm": (ctypes.c_int, [ctypes.c_int]),
        "hgo_set_film_guard": (ctypes.c_double, [ctypes.c_double]),
        "hgo_philox4x32_10": (None, [ctypes.POINTER(ctypes.c_uint32)] * 3),
        "hgo_atan_monotone_violations": (ctypes.c_uint64, [ctypes.c_uint32, ctypes.c_uint32]),
        "hgo_rain_word": (ctypes.c_uint32, [ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint32,
                                            ctypes.c_uint64]),
        "hgo_simplex2f": (ctypes.c_float, [ctypes.c_float, ctypes.c_float, ctypes.c_uint32]),
        "hgo_fbm_raw": (None, [P, ctypes.c_int, ctypes.c_int, ctypes.c_uint32, ctypes.c_int, ctypes.c_float,
                               ctypes.c_float, ctypes.c_float]),
        "hgo_fbm_scaled": (None, [P, ctypes.c_int, ctypes.c_uint32, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                  ctypes.c_float, ctypes.c_float, ctypes.c_float]),
        "hgo_particles_init": (ctypes.c_int, [P, ctypes.c_int]),
        "hgo_particle_step": (ctypes.c_int, [P, ctypes.POINTER(OracleErosion), ctypes.POINTER(OracleOptions),
                                             ctypes.c_int]),
        "hgo_particles_get": (ctypes.c_int, [P, P, P, P]),
        "hgo_num_threads": (ctypes.c_int, []),
        "hgo_set_num_threads": (None, [ctypes.c_int]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def erosion_from(s):
    """Copy any ctypes struct with Erosion_data's fields into an OracleErosion."""
    o = OracleErosion()
    ctypes.memmove(ctypes.byref(o), ctypes.byref(s), ctypes.sizeof(OracleErosion))
    return o


def bernoulli_threshold(p):
    t = math.floor(p * 4294967296.0)
    return int(min(max(t, 0), 4294967295))


def options(rain_mode=1, period=1, amount=0.01, p=0.0, seed=0, terrain_id=0, skip_identity=1, time0=0.0,
            time_step=0.0, mountain_thresh=0.55, mountain_multip=0.05, drops=0.02, max_height=256.0):
    """Rain and pass options; rain_mode 3 is the reference's rain (frame time
    time0 + n * time_step at step n, mountain bonus above mountain_thresh of
    max_height)."""
    return OracleOptions(rain_mode, period, amount, bernoulli_threshold(p), seed, terrain_id, skip_identity,
                         time0, time_step, mountain_thresh, mountain_multip, drops, max_height)


def settings_config1():
    s = OracleErosion()
    s.Kc = 0.1
    s.Ks[0] = s.Ks[1] = 0.05
    s.Kd[0] = s.Kd[1] = 0.05
    s.Ke = 0.015
    s.ENERGY_KEPT = 1.0
    s.G = 9.81
    s.d_t = 0.02
    s.Kalpha[0] = s.Kalpha[1] = math.atan(0.65)
    return s


def settings_config2():
    s = settings_config1()
    s.Kspeed[0] = 0.3
    return s


def workload(cfg, seed=0):
    """(settings, options) of a named workload, matching hydrogen.configure."""
    if cfg == "config1":
        return settings_config1(), options(1, 1, 0.01)
    if cfg == "config2":
        return settings_config2(), options(2, 1, 0.5, p=0.001, seed=seed)
    raise ValueError(cfg)


def fbm(n, seed=0, octaves=6, frequency=1.0 / 128, lacunarity=2.0, gain=0.5, lo=0.0, hi=64.0):
    out = np.empty((n, n), dtype=np.float32)
    lib.hgo_fbm_scaled(out.ctypes.data, n, seed, octaves, frequency, lacunarity, gain, lo, hi)
    return out


def fbm_raw(w, h, seed, octaves, frequency, lacunarity, gain):
    out = np.empty((h, w), dtype=np.float32)
    lib.hgo_fbm_raw(out.ctypes.data, w, h, seed, octaves, frequency, lacunarity, gain)
    return out


class OracleWorld:
    def __init__(self, n, precision=64):
        self.n = n
        self.precision = precision
        self.h = lib.hgo_create(n, precision)
        if not self.h:
            raise ValueError("oracle create failed")

    def __del__(self):
        if getattr(self, "h", None):
            lib.hgo_destroy(self.h)
            self.h = None

    def set(self, field, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        assert a.size == self.n * self.n
        assert lib.hgo_set_field(self.h, FIELDS[field], a.ctypes.data) == 0

    def get(self, field):
        a = np.empty((self.n, self.n), dtype=np.float64)
        assert lib.hgo_get_field(self.h, FIELDS[field], a.ctypes.data) == 0
        return a

    def set_ks(self, ks):
        if ks is None:
            lib.hgo_set_ks_field(self.h, None)
            return
        self._ks = np.ascontiguousarray(ks, dtype=np.float32)
        lib.hgo_set_ks_field(self.h, self._ks.ctypes.data)

    @property
    def step_count(self):
        return lib.hgo_get_step(self.h)

    @step_count.setter
    def step_count(self, v):
        lib.hgo_set_step(self.h, v)

    def step(self, settings, opts, nsteps=1):
        rc = lib.hgo_step(self.h, ctypes.byref(settings), ctypes.byref(opts), nsteps)
        if rc != 0:
            raise RuntimeError(f"oracle step failed ({rc})")

    def run_pass(self, name, settings, opts=None, layer=0):
        opts = opts or options()
        assert lib.hgo_pass(self.h, ctypes.byref(settings), ctypes.byref(opts), PASSES[name], layer) == 0

    def set_rows(self, lo=0, hi=-1):
        """Restrict the grid passes to rows [lo, hi) (hi = -1: all rows)."""
        assert lib.hgo_set_rows(self.h, lo, hi) == 0

    TEXTURES = {"height": 0, "flux": 1, "vel": 2, "sed": 3, "thc": 4, "thd": 5}

    def tex_rows(self, tex, y0, y1):
        """Rows [y0, y1) of a current texture as (rows, n, 4) doubles."""
        a = np.empty((y1 - y0, self.n, 4), dtype=np.float64)
        assert lib.hgo_tex_rows(self.h, self.TEXTURES[tex], y0, y1, a.ctypes.data, 0) == 0
        return a

    def set_tex_rows(self, tex, y0, rows):
        a = np.ascontiguousarray(rows, dtype=np.float64)
        assert lib.hgo_tex_rows(self.h, self.TEXTURES[tex], y0, y0 + a.shape[0], a.ctypes.data, 1) == 0

    def particles_init(self, count):
        assert lib.hgo_particles_init(self.h, count) == 0
        self.count_particles = count

    def particle_step(self, settings, opts, nsteps=1):
        assert lib.hgo_particle_step(self.h, ctypes.byref(settings), ctypes.byref(opts), nsteps) == 0

    def particles(self):
        """(state[count, 8] = x, y, vx, vy, volume, rock sed, dirt sed, capacity; iters; kill)"""
        c = self.count_particles
        st = np.empty((c, 8), np.float32)
        it = np.empty(c, np.uint32)
        kl = np.empty(c, np.int32)
        assert lib.hgo_particles_get(self.h, st.ctypes.data, it.ctypes.data, kl.ctypes.data) == 0
        return st, it, kl

    def thermal(self):
        c = np.empty((self.n, self.n, 4))
        d = np.empty((self.n, self.n, 4))
        lib.hgo_get_thermal(self.h, c.ctypes.data, d.ctypes.data)
        return c, d

    def totals(self):
        out = (ctypes.c_double * 4)()
        lib.hgo_totals(self.h, out)
        return list(out)

    def state(self, fields=("rock", "water", "sediment", "flux_l", "flux_r", "flux_t", "flux_b", "vel_u",
                            "vel_v")):
        return {f: self.get(f) for f in fields}


def atanf(x):
    return lib.hgo_atanf(x)


class libm_atan:
    """Context in which the float oracle takes its arctangent from the C
    library (atanf) instead of the kernels' polynomial; for measuring how
    much the arctangent moves the float result, never for parity."""

    def __enter__(self):
        self.prev = lib.hgo_set_float_atan_libm(1)
        return self

    def __exit__(self, *a):
        lib.hgo_set_float_atan_libm(self.prev)


class film_guard:
    """Context in which the oracle's flux pass sets the velocity to 0 where
    the depth d1 + d2 is below `depth` (both precisions): a change to the
    scheme, for measuring how much of the float-vs-FP64 distance comes from
    the velocity of thin films, never for parity."""

    def __init__(self, depth):
        self.depth = depth

    def __enter__(self):
        self.prev = lib.hgo_set_film_guard(self.depth)
        return self

    def __exit__(self, *a):
        lib.hgo_set_film_guard(self.prev)


def rain_word(x, y, step, terrain, seed):
    return lib.hgo_rain_word(x, y, step, terrain, seed)


def philox(ctr, key):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib.hgo_philox4x32_10(c, k, o)
    return list(o)


def atan_monotone_violations(lo_bits=0, hi_bits=0x7F800000):
    """Number of consecutive positive float pairs (by bit pattern) in
    [lo_bits, hi_bits] where the polynomial arctangent decreases."""
    return lib.hgo_atan_monotone_violations(lo_bits, hi_bits)


def num_threads():
    return lib.hgo_num_threads()


def set_num_threads(t):
    lib.hgo_set_num_threads(t)


# ---- FP64 reference adjoint (hg_adjoint_ref.cpp) ------------------------------------
lib.hgo_adjoint_ref.restype = ctypes.c_int
lib.hgo_adjoint_ref.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_int,
                                ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                ctypes.c_void_p, ctypes.c_void_p]
lib.hgo_fd_ref.restype = ctypes.c_int
lib.hgo_fd_ref.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_int,
                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                           ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p]
lib.hgo_fd_ref_final.restype = ctypes.c_int
lib.hgo_fd_ref_final.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_int,
                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                 ctypes.c_void_p, ctypes.c_void_p]
lib.hgo_forward_ref.restype = ctypes.c_int
lib.hgo_forward_ref.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_int,
                                ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]


lib.hgo_ref_heightmap.restype = None
lib.hgo_ref_heightmap.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
lib.hgo_ref_rain.restype = None
lib.hgo_ref_rain.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                             ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_void_p]
lib.hgo_ref_simplex.restype = ctypes.c_float
lib.hgo_ref_simplex.argtypes = [ctypes.c_float, ctypes.c_float]
lib.hgo_ref_noised.restype = None
lib.hgo_ref_noised.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_void_p]


def ref_heightmap(map_settings, n):
    """The reference's terrain generator (glsl/heightmap.glsl): (rock, dirt),
    map_settings any ctypes struct with Map_settings_data's 96-byte layout."""
    rock = np.empty((n, n), np.float32)
    dirt = np.empty((n, n), np.float32)
    lib.hgo_ref_heightmap(ctypes.byref(map_settings), n, rock.ctypes.data, dirt.ctypes.data)
    return rock, dirt


def ref_rain(total, time, rain, max_height):
    """The reference's rain increment (glsl/rain.glsl) of every cell."""
    n = total.shape[0]
    t = np.ascontiguousarray(total, np.float32)
    out = np.empty((n, n), np.float32)
    lib.hgo_ref_rain(n, t.ctypes.data, time, rain.amount, rain.mountain_thresh, rain.mountain_multip, rain.drops,
                     max_height, out.ctypes.data)
    return out


def ref_simplex(x, y):
    return lib.hgo_ref_simplex(x, y)


def ref_noised(x, y):
    out = (ctypes.c_float * 3)()
    lib.hgo_ref_noised(x, y, out)
    return tuple(out)


lib.hgo_render.restype = ctypes.c_int
lib.hgo_render.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int, ctypes.c_float, ctypes.c_int, ctypes.c_void_p,
                                                   ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
for _f in ("hgo_render_pow",):
    getattr(lib, _f).restype = ctypes.c_float
    getattr(lib, _f).argtypes = [ctypes.c_float, ctypes.c_float]
for _f in ("hgo_render_exp2", "hgo_render_log2"):
    getattr(lib, _f).restype = ctypes.c_float
    getattr(lib, _f).argtypes = [ctypes.c_float]


def render(fields, n, camera, width, height, max_height=256.0, hmap_dim_x=1024):
    """The ray-marcher (glsl/rendering.glsl) on host fields: dict with rock,
    water, sediment and, for two-layer worlds, dirt and sediment_dirt;
    camera any ctypes struct with hg_camera's layout.  Returns (rgba[h, w, 4]
    uint8, rgb[h, w, 3] float32), row 0 first."""
    keep = []

    def ptr(name):
        if name not in fields:
            return None
        a = np.ascontiguousarray(fields[name], dtype=np.float32)
        assert a.size == n * n
        keep.append(a)
        return a.ctypes.data

    rgba = np.zeros((height, width, 4), np.uint8)
    rgb = np.zeros((height, width, 3), np.float32)
    rc = lib.hgo_render(ptr("rock"), ptr("dirt"), ptr("water"), ptr("sediment"), ptr("sediment_dirt"), n,
                        max_height, hmap_dim_x, ctypes.byref(camera), width, height, rgba.ctypes.data,
                        rgb.ctypes.data)
    assert rc == 0, "singular camera matrices"
    return rgba, rgb


def render_pow(x, y):
    return lib.hgo_render_pow(x, y)


def render_exp2(x):
    return lib.hgo_render_exp2(x)


def render_log2(x):
    return lib.hgo_render_log2(x)


def _adj_settings(s, amount):
    return np.array([s.d_t, s.G, s.ENERGY_KEPT, s.Kc, s.Kd[0], s.Ke, amount, s.Kalpha[0], s.Kspeed[0]],
                    dtype=np.float32)


def adjoint_ref(settings, amount, period, b0, ks, target, nsteps, step0=0):
    """FP64 reference: loss = mean((rock_final - target)^2) after nsteps of the
    single-material step (thermal layer 0 when Kspeed[0] != 0); returns
    (loss, dL/dKs, dL/drock0)."""
    n = b0.shape[0]
    st = _adj_settings(settings, amount)
    b0 = np.ascontiguousarray(b0, dtype=np.float64)
    ks = np.ascontiguousarray(ks, dtype=np.float32)
    tg = np.ascontiguousarray(target, dtype=np.float64)
    loss = ctypes.c_double()
    dks = np.empty((n, n)); db0 = np.empty((n, n))
    rc = lib.hgo_adjoint_ref(n, st.ctypes.data, period, step0, nsteps, b0.ctypes.data, ks.ctypes.data, tg.ctypes.data,
                             ctypes.byref(loss), dks.ctypes.data, db0.ctypes.data)
    assert rc == 0
    return loss.value, dks, db0


def fd_ref(settings, amount, period, b0, ks, target, nsteps, cells, params, eps, step0=0):
    """Central finite differences of the FP64 reference's loss (mean squared
    rock error after nsteps) for each (flat cell index, parameter) pair:
    parameter 0 = the cell's Ks, 1 = its initial rock; pairs run in parallel
    over the host's threads.  Returns dL/dparam per pair."""
    n = b0.shape[0]
    st = _adj_settings(settings, amount)
    b0 = np.ascontiguousarray(b0, dtype=np.float64)
    ks = np.ascontiguousarray(ks, dtype=np.float32)
    tg = np.ascontiguousarray(target, dtype=np.float64)
    cells = np.ascontiguousarray(cells, dtype=np.int32)
    params = np.ascontiguousarray(params, dtype=np.int32)
    out = np.empty(len(cells))
    rc = lib.hgo_fd_ref(n, st.ctypes.data, period, step0, nsteps, b0.ctypes.data, ks.ctypes.data, tg.ctypes.data,
                        len(cells), cells.ctypes.data, params.ctypes.data, eps, out.ctypes.data)
    assert rc == 0
    return out


def fd_ref_final(settings, amount, period, b0, ks, nsteps, cell, param, delta, step0=0):
    """Final rock of fd_ref's windowed forward for one perturbation (flat
    cell, parameter 0 = Ks / 1 = initial rock, signed delta) and the number
    of cells its window grew to."""
    n = b0.shape[0]
    st = _adj_settings(settings, amount)
    b0 = np.ascontiguousarray(b0, dtype=np.float64)
    ks = np.ascontiguousarray(ks, dtype=np.float32)
    out = np.empty((n, n))
    rc_cells = ctypes.c_int()
    rc = lib.hgo_fd_ref_final(n, st.ctypes.data, period, step0, nsteps, b0.ctypes.data, ks.ctypes.data, cell,
                              param, delta, out.ctypes.data, ctypes.byref(rc_cells))
    assert rc == 0
    return out, rc_cells.value


def forward_ref(settings, amount, period, b0, ks, nsteps, step0=0):
    n = b0.shape[0]
    st = _adj_settings(settings, amount)
    b0 = np.ascontiguousarray(b0, dtype=np.float64)
    ks = np.ascontiguousarray(ks, dtype=np.float32)
    out = np.empty((n, n))
    lib.hgo_forward_ref(n, st.ctypes.data, period, step0, nsteps, b0.ctypes.data, ks.ctypes.data, out.ctypes.data)
    return out
