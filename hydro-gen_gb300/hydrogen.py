"""Python binding of libhydrogen_gb300.so (ctypes over the C ABI in include/hydrogen.h).

This mirrors the reference's erosion interface: an ErosionSettings struct
with Erosion_data's fields and std140 layout (glsl/bindings.glsl:39-60), a
RainSettings struct mirroring Rain_data (glsl/bindings.glsl:62-68), a World
that owns the device fields (State::World::Textures, src/state.hpp:59-76),
World.init_heightmap for World::gen_heightmap (src/state.cpp:116-147) and
World.step for Erosion::dispatch_grid (src/erosion.cpp:158-200).

Errors raise HydrogenError carrying the library's status code and message.
The library must be built (build.build()); importing this module without it
raises ImportError: there is no CPU fallback.
"""
import atexit
import ctypes
import weakref
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhydrogen_gb300.so")
HEADER = os.path.join(HERE, "..", "include", "hydrogen.h")

HG_OK = 0
STATUS = {-1: "HG_ERR_INVALID", -2: "HG_ERR_OOM", -3: "HG_ERR_CUDA", -4: "HG_ERR_TIMEOUT",
          -5: "HG_ERR_UNSUPPORTED", -6: "HG_ERR_IO", -7: "HG_ERR_STATE"}
HG_AUTO = -1
RAIN_OFF, RAIN_UNIFORM, RAIN_BERNOULLI, RAIN_REFERENCE = 0, 1, 2, 3
MODE_PLAIN, MODE_FUSED, MODE_FUSED_PER_WORLD, MODE_PARTICLES = 0, 1, 2, 3
FIELDS = {"rock": 0, "water": 1, "sediment": 2, "flux_l": 3, "flux_r": 4, "flux_t": 5, "flux_b": 6,
          "vel_u": 7, "vel_v": 8, "vel_z": 9, "ks": 10, "dirt": 11, "sediment_dirt": 12,
          "momentum_x": 13, "momentum_y": 14}
STATE_FIELDS = ["rock", "water", "sediment", "flux_l", "flux_r", "flux_t", "flux_b", "vel_u", "vel_v"]
# single passes of the per-pass step (hg_pass) and the talus outflow planes' row ids (hg_world_rows)
PASSES = {"rain": 0, "flux": 1, "erosion": 2, "sediment": 3, "thermal_flux": 4, "thermal_transport": 5,
          "smoothing": 6}
# row-transfer ids beyond FIELDS: (id, floats per cell)
ROWS_EXTRA = {"thermal_c": (100, 4), "thermal_d": (101, 4), "eroded_rock": (102, 1), "eroded_sediment": (103, 1)}


class Camera(ctypes.Structure):
    """hg_camera: the ray-marcher's uniforms (glsl/rendering.glsl:15-23)."""
    _fields_ = [("view", ctypes.c_float * 16), ("perspective", ctypes.c_float * 16), ("pos", ctypes.c_float * 3),
                ("prec", ctypes.c_float), ("draw_water", ctypes.c_int32), ("display_sediment", ctypes.c_int32),
                ("sediment_max_cap", ctypes.c_float), ("low_res_div3", ctypes.c_int32)]


class HydrogenError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class ErosionSettings(ctypes.Structure):
    """Erosion_data, glsl/bindings.glsl:39-60 (std140, 96 bytes)."""
    _fields_ = [("particle_count", ctypes.c_uint32), ("Kc", ctypes.c_float),
                ("Kalpha", ctypes.c_float * 2), ("Kconv", ctypes.c_float), ("_pad0", ctypes.c_float),
                ("Ks", ctypes.c_float * 2), ("Kd", ctypes.c_float * 2), ("Ke", ctypes.c_float),
                ("ENERGY_KEPT", ctypes.c_float), ("Kspeed", ctypes.c_float * 2), ("G", ctypes.c_float),
                ("d_t", ctypes.c_float), ("density", ctypes.c_float), ("init_volume", ctypes.c_float),
                ("friction", ctypes.c_float), ("inertia", ctypes.c_float), ("min_volume", ctypes.c_float),
                ("min_velocity", ctypes.c_float), ("ttl", ctypes.c_uint32), ("_pad1", ctypes.c_uint32)]


class RainSettings(ctypes.Structure):
    """Rain_data, glsl/bindings.glsl:62-68 (20 bytes)."""
    _fields_ = [("amount", ctypes.c_float), ("mountain_thresh", ctypes.c_float),
                ("mountain_multip", ctypes.c_float), ("period", ctypes.c_int32), ("drops", ctypes.c_float)]


class StepOptions(ctypes.Structure):
    _fields_ = [("rain_mode", ctypes.c_int32), ("rain_probability", ctypes.c_float),
                ("rain_seed", ctypes.c_uint64), ("terrain_id", ctypes.c_uint32), ("thermal", ctypes.c_int32),
                ("tile_x", ctypes.c_int32), ("tile_y", ctypes.c_int32), ("graph", ctypes.c_int32),
                ("rain_time0", ctypes.c_float), ("rain_time_step", ctypes.c_float), ("reserved", ctypes.c_int32 * 4)]


class MapSettings(ctypes.Structure):
    """Map_settings_data, glsl/bindings.glsl:70-99 (std140, 96 bytes)."""
    _fields_ = [("max_height", ctypes.c_float), ("max_dirt", ctypes.c_float), ("hmap_dims", ctypes.c_int32 * 2),
                ("height_mult", ctypes.c_float), ("water_lvl", ctypes.c_float), ("seed", ctypes.c_float),
                ("persistance", ctypes.c_float), ("lacunarity", ctypes.c_float), ("scale", ctypes.c_float),
                ("redistribution", ctypes.c_float), ("octaves", ctypes.c_int32), ("fake_erosion", ctypes.c_uint32),
                ("mask_round", ctypes.c_uint32), ("mask_exp", ctypes.c_uint32), ("mask_power", ctypes.c_uint32),
                ("mask_slope", ctypes.c_uint32), ("uplift", ctypes.c_uint32), ("uplift_scale", ctypes.c_float),
                ("domain_warp", ctypes.c_int32), ("domain_warp_scale", ctypes.c_float), ("terrace", ctypes.c_int32),
                ("terrace_scale", ctypes.c_float), ("pad0", ctypes.c_float)]


class NoiseSettings(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint32), ("octaves", ctypes.c_int32), ("frequency", ctypes.c_float),
                ("lacunarity", ctypes.c_float), ("gain", ctypes.c_float), ("out_min", ctypes.c_float),
                ("out_max", ctypes.c_float)]


class FitSettings(ctypes.Structure):
    _fields_ = [("nsteps", ctypes.c_int32), ("ckpt_every", ctypes.c_int32), ("iters", ctypes.c_int32),
                ("ks_step", ctypes.c_float), ("ks_min", ctypes.c_float), ("ks_max", ctypes.c_float),
                ("rock_step", ctypes.c_float)]


# hg_log_fn: level (0 error, 1 info), message, user pointer
LOG_FN = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.c_char_p, ctypes.c_void_p)


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with hydro-gen_gb300/build.py (no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    sig = {
        "hg_version": (ctypes.c_char_p, []),
        "hg_last_error": (ctypes.c_char_p, []),
        "hg_launch_count": (ctypes.c_uint64, []),
        "hg_default_erosion_settings": (ctypes.c_int, [ctypes.POINTER(ErosionSettings)]),
        "hg_default_rain_settings": (ctypes.c_int, [ctypes.POINTER(RainSettings)]),
        "hg_default_step_options": (ctypes.c_int, [ctypes.POINTER(StepOptions)]),
        "hg_world_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(P)]),
        "hg_world_destroy": (ctypes.c_int, [P]),
        "hg_world_size": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_int)]),
        "hg_world_stream": (ctypes.c_int, [P, ctypes.POINTER(P)]),
        "hg_set_erosion_settings": (ctypes.c_int, [P, ctypes.POINTER(ErosionSettings)]),
        "hg_get_erosion_settings": (ctypes.c_int, [P, ctypes.POINTER(ErosionSettings)]),
        "hg_set_rain_settings": (ctypes.c_int, [P, ctypes.POINTER(RainSettings)]),
        "hg_set_step_options": (ctypes.c_int, [P, ctypes.POINTER(StepOptions)]),
        "hg_init_heightmap": (ctypes.c_int, [P, ctypes.POINTER(NoiseSettings)]),
        "hg_init_heightmap_host": (ctypes.c_int, [P, P]),
        "hg_init_ks_field": (ctypes.c_int, [P, ctypes.POINTER(NoiseSettings), ctypes.c_float, ctypes.c_float]),
        "hg_clear_ks_field": (ctypes.c_int, [P]),
        "hg_world_upload": (ctypes.c_int, [P, ctypes.c_int, P]),
        "hg_world_download": (ctypes.c_int, [P, ctypes.c_int, P]),
        "hg_world_upload_device": (ctypes.c_int, [P, ctypes.c_int, P]),
        "hg_world_download_device": (ctypes.c_int, [P, ctypes.c_int, P]),
        "hg_world_get_step": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_uint64)]),
        "hg_world_set_step": (ctypes.c_int, [P, ctypes.c_uint64]),
        "hg_step": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int]),
        "hg_set_rows": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int]),
        "hg_pass": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int]),
        "hg_world_rows": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, ctypes.c_int]),
        "hg_fused_pass": (ctypes.c_int, [P, ctypes.c_int]),
        "hg_sync": (ctypes.c_int, [P]),
        "hg_world_totals": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_double)]),
        "hg_field_totals_noalloc": (ctypes.c_int, [ctypes.POINTER(P), ctypes.c_int, ctypes.c_size_t, P, P]),
        "hg_world_tuning": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                           ctypes.POINTER(ctypes.c_double)]),
        "hg_batch_create": (ctypes.c_int, [ctypes.POINTER(P), ctypes.c_int, ctypes.POINTER(P)]),
        "hg_batch_destroy": (ctypes.c_int, [P]),
        "hg_batch_step": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int]),
        "hg_batch_sync": (ctypes.c_int, [P]),
        "hg_batch_stream": (ctypes.c_int, [P, ctypes.POINTER(P)]),
        "hg_default_map_settings": (ctypes.c_int, [ctypes.POINTER(MapSettings)]),
        "hg_set_map_settings": (ctypes.c_int, [P, ctypes.POINTER(MapSettings)]),
        "hg_init_reference_heightmap": (ctypes.c_int, [P, ctypes.POINTER(MapSettings)]),
        "hg_particles_init": (ctypes.c_int, [P, ctypes.c_int]),
        "hg_rain": (ctypes.c_int, [P, ctypes.c_float]),
        "hg_camera_look_at": (ctypes.c_int, [ctypes.POINTER(Camera), P, P, P, ctypes.c_float, ctypes.c_float,
                                             ctypes.c_float, ctypes.c_float]),
        "hg_render": (ctypes.c_int, [P, ctypes.POINTER(Camera), ctypes.c_int, ctypes.c_int, P, P]),
        "hg_render_device": (ctypes.c_int, [P, ctypes.POINTER(Camera), ctypes.c_int, ctypes.c_int, P, P]),
        "hg_default_particle_settings": (ctypes.c_int, [ctypes.POINTER(ErosionSettings)]),
        "hg_particles_count": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_int)]),
        "hg_particles_get": (ctypes.c_int, [P, P, P, P]),
        "hg_selftest_division": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]),
        "hg_selftest_bounded_wait": (ctypes.c_int, [ctypes.c_uint32, ctypes.POINTER(ctypes.c_int),
                                                    ctypes.POINTER(ctypes.c_double)]),
        "hg_selftest_report_timeout": (ctypes.c_int, [P]),
        "hg_selftest_paired": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]),
        "hg_batch_launch_form": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]),
        "hg_batch_tuning": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                           ctypes.POINTER(ctypes.c_double)]),
        "hg_tape_create": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(P)]),
        "hg_tape_destroy": (ctypes.c_int, [P]),
        "hg_tape_info": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
        "hg_forward": (ctypes.c_int, [P]),
        "hg_backward": (ctypes.c_int, [P, P, P, P]),
        "hg_mse": (ctypes.c_int, [P, P, ctypes.POINTER(ctypes.c_double), P]),
        "hg_default_fit_settings": (ctypes.c_int, [ctypes.POINTER(FitSettings)]),
        "hg_set_log_callback": (ctypes.c_int, [LOG_FN, P]),
        "hg_world_poison_scratch": (ctypes.c_int, [P]),
        "hg_world_count_nonfinite": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_uint64)]),
        "hg_inverse_fit": (ctypes.c_int, [P, P, P, P, ctypes.POINTER(FitSettings), ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_double)]),
        "hg_world_save": (ctypes.c_int, [P, ctypes.c_char_p]),
        "hg_world_load": (ctypes.c_int, [P, ctypes.c_char_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def check(code):
    if code != HG_OK:
        raise HydrogenError(code, lib.hg_last_error().decode())
    return code


def header_functions(path=HEADER):
    """Names of the functions declared in include/hydrogen.h."""
    import re
    text = open(path).read()
    return sorted(set(re.findall(r"^\w[\w\s\*]*?\b(hg_\w+)\s*\(", text, re.M)))


# ---- workload presets --------------------------------------------------------------
TALUS_TAN = 0.65


def settings_config1():
    """Plain virtual-pipe erosion workload: dt 0.02, G 9.81, A = L = 1, Kc 0.1,
    Ks = Kd = 0.05, Ke 0.015, thermal off (Kspeed 0), single material."""
    s = ErosionSettings()
    check(lib.hg_default_erosion_settings(ctypes.byref(s)))
    s.Kc = 0.1
    s.Ks[0] = s.Ks[1] = 0.05
    s.Kd[0] = s.Kd[1] = 0.05
    s.Ke = 0.015
    s.ENERGY_KEPT = 1.0
    s.G = 9.81
    s.d_t = 0.02
    s.Kconv = 0.0
    s.Kalpha[0] = s.Kalpha[1] = math.atan(TALUS_TAN)
    s.Kspeed[0] = s.Kspeed[1] = 0.0
    return s


def settings_config2():
    """Config-1 physics with thermal erosion: talus tan 0.65, slippage 0.3."""
    s = settings_config1()
    s.Kspeed[0] = 0.3
    return s


def settings_particles():
    """The reference's particle-model defaults (src/state.cpp:61-79)."""
    s = ErosionSettings()
    check(lib.hg_default_particle_settings(ctypes.byref(s)))
    return s


def camera(pos, dir, up=(0.0, 1.0, 0.0), fov=90.0, aspect=16.0 / 9.0, z_near=0.1, z_far=2048.0):
    """hg_camera of glm::lookAt(pos, pos + dir, up) and glm::perspective
    (src/rendering.cpp:89-99; FOV 90, Z_NEAR 0.1, Z_FAR 2048)."""
    c = Camera()
    f3 = ctypes.c_float * 3
    check(lib.hg_camera_look_at(ctypes.byref(c), f3(*pos), f3(*dir), f3(*up), fov, aspect, z_near, z_far))
    return c


def save_ppm(path, rgba):
    """Writes an RGBA8 image (row 0 = bottom, as rendered) as a binary PPM."""
    img = np.ascontiguousarray(rgba[::-1, :, :3])
    with open(path, "wb") as f:
        f.write(f"P6 {img.shape[1]} {img.shape[0]} 255\n".encode())
        f.write(img.tobytes())


def rain_uniform(amount=0.01, period=1):
    r = RainSettings()
    check(lib.hg_default_rain_settings(ctypes.byref(r)))
    r.amount = amount
    r.period = period
    return r


def options(rain_mode=RAIN_UNIFORM, p=0.0, seed=0, terrain_id=0, thermal=HG_AUTO, tile=(HG_AUTO, HG_AUTO),
            graph=HG_AUTO, time0=0.0, time_step=0.0):
    o = StepOptions()
    check(lib.hg_default_step_options(ctypes.byref(o)))
    o.rain_mode = rain_mode
    o.rain_probability = p
    o.rain_seed = seed
    o.terrain_id = terrain_id
    o.thermal = thermal
    o.tile_x, o.tile_y = tile
    o.graph = graph
    o.rain_time0 = time0
    o.rain_time_step = time_step
    return o


def map_settings(**kw):
    """The reference's map defaults (seed 0) with fields overridden by keyword."""
    m = MapSettings()
    check(lib.hg_default_map_settings(ctypes.byref(m)))
    for k, v in kw.items():
        setattr(m, k, v)
    return m


def noise(seed=0, octaves=6, frequency=1.0 / 128, lacunarity=2.0, gain=0.5, lo=0.0, hi=64.0):
    return NoiseSettings(seed, octaves, frequency, lacunarity, gain, lo, hi)


def bernoulli_threshold(p):
    t = math.floor(p * 4294967296.0)
    return int(min(max(t, 0), 4294967295))


# Live handles, closed at interpreter exit dependents first (tapes and
# batches before the worlds they use) while the CUDA runtime is still up;
# garbage collection of reference cycles would otherwise finalise them in
# any order.
_live = {"tapes": weakref.WeakSet(), "batches": weakref.WeakSet(), "worlds": weakref.WeakSet()}


@atexit.register
def _close_all():
    for kind in ("tapes", "batches", "worlds"):
        for obj in list(_live[kind]):
            try:
                obj.close()
            except Exception:
                pass


class World:
    """An n x n erosion world on the current CUDA device."""

    def __init__(self, n, layers=1):
        h = ctypes.c_void_p()
        check(lib.hg_world_create(n, layers, ctypes.byref(h)))
        self.h = h
        self.n = n
        self._tapes = weakref.WeakSet()
        _live["worlds"].add(self)

    def close(self):
        if self.h:
            for t in list(self._tapes):  # a tape's handle before its world's
                t.close()
            lib.hg_world_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_erosion(self, s):
        check(lib.hg_set_erosion_settings(self.h, ctypes.byref(s)))

    def get_erosion(self):
        s = ErosionSettings()
        check(lib.hg_get_erosion_settings(self.h, ctypes.byref(s)))
        return s

    def set_rain(self, r):
        check(lib.hg_set_rain_settings(self.h, ctypes.byref(r)))

    def set_options(self, o):
        check(lib.hg_set_step_options(self.h, ctypes.byref(o)))

    def init_heightmap(self, ns):
        check(lib.hg_init_heightmap(self.h, ctypes.byref(ns)))

    def init_from_heightmap(self, rock):
        """Every field zero, ROCK from a host heightmap (n x n float32 array or
        a pointer to n*n floats, pinned for the fastest copy), step 0."""
        if isinstance(rock, int):
            check(lib.hg_init_heightmap_host(self.h, ctypes.c_void_p(rock)))
            return
        a = np.ascontiguousarray(rock, dtype=np.float32)
        assert a.size == self.n * self.n
        check(lib.hg_init_heightmap_host(self.h, ctypes.c_void_p(a.ctypes.data)))

    def init_reference_heightmap(self, ms):
        """The reference's terrain generator (glsl/heightmap.glsl)."""
        check(lib.hg_init_reference_heightmap(self.h, ctypes.byref(ms)))

    def set_map(self, ms):
        check(lib.hg_set_map_settings(self.h, ctypes.byref(ms)))

    def render(self, cam, width, height, rgb=False):
        """Ray-marched image: rgba[h, w, 4] uint8 (row 0 = bottom), and the
        float colour rgb[h, w, 3] when asked."""
        img = np.empty((height, width, 4), np.uint8)
        col = np.empty((height, width, 3), np.float32) if rgb else None
        check(lib.hg_render(self.h, ctypes.byref(cam), width, height, img.ctypes.data,
                            col.ctypes.data if rgb else None))
        return (img, col) if rgb else img

    def particles_init(self, count):
        """`count` idle droplets and a zero momentum map (two-layer worlds)."""
        check(lib.hg_particles_init(self.h, count))

    def particles(self):
        """(state[count, 8] = x, y, vx, vy, volume, rock sed, dirt sed, capacity; iters; kill)"""
        c = ctypes.c_int()
        check(lib.hg_particles_count(self.h, ctypes.byref(c)))
        st = np.empty((c.value, 8), np.float32)
        it = np.empty(c.value, np.uint32)
        kl = np.empty(c.value, np.int32)
        check(lib.hg_particles_get(self.h, st.ctypes.data, it.ctypes.data, kl.ctypes.data))
        return st, it, kl

    def init_ks_field(self, ns, base, k):
        check(lib.hg_init_ks_field(self.h, ctypes.byref(ns), base, k))

    def clear_ks_field(self):
        check(lib.hg_clear_ks_field(self.h))

    def upload(self, field, arr):
        a = np.ascontiguousarray(arr, dtype=np.float32)
        assert a.size == self.n * self.n
        check(lib.hg_world_upload(self.h, FIELDS[field], a.ctypes.data))

    def download(self, field):
        a = np.empty((self.n, self.n), dtype=np.float32)
        check(lib.hg_world_download(self.h, FIELDS[field], a.ctypes.data))
        return a

    def upload_device(self, field, ptr):
        check(lib.hg_world_upload_device(self.h, FIELDS[field], ctypes.c_void_p(ptr)))

    def download_device(self, field, ptr):
        check(lib.hg_world_download_device(self.h, FIELDS[field], ctypes.c_void_p(ptr)))

    def restrict_rows(self, lo=0, hi=-1):
        """Per-pass kernels compute rows [lo, hi) only (hi = -1: all rows)."""
        check(lib.hg_set_rows(self.h, lo, hi))

    def run_pass(self, name, layer=0):
        """One pass of the one-layer per-pass step (PASSES)."""
        check(lib.hg_pass(self.h, PASSES[name], layer))

    def fused_pass(self, which):
        """One kernel of the fused step over the restricted rows (0: k_hydro,
        1: k_transport, after which the step is done)."""
        check(lib.hg_fused_pass(self.h, which))

    def get_rows(self, field, y0, y1):
        """Rows [y0, y1) of a field as float32 (rows, n), or (rows, n, 4) for
        the talus outflow planes."""
        fid, per = ROWS_EXTRA.get(field, (FIELDS.get(field), 1))
        a = np.empty((y1 - y0, self.n) if per == 1 else (y1 - y0, self.n, per), np.float32)
        check(lib.hg_world_rows(self.h, fid, y0, y1, a.ctypes.data, 0))
        return a

    def put_rows(self, field, y0, rows):
        fid, per = ROWS_EXTRA.get(field, (FIELDS.get(field), 1))
        a = np.ascontiguousarray(rows, dtype=np.float32)
        y1 = y0 + a.shape[0]
        assert a.size == (y1 - y0) * self.n * per
        check(lib.hg_world_rows(self.h, fid, y0, y1, a.ctypes.data, 1))

    def state(self, fields=STATE_FIELDS):
        return {f: self.download(f) for f in fields}

    def step(self, nsteps=1, mode=MODE_PLAIN):
        check(lib.hg_step(self.h, nsteps, mode))

    def rain(self, time=0.0):
        """One rain pass now (Erosion::dispatch_grid_rain), whatever the period."""
        check(lib.hg_rain(self.h, time))

    def sync(self):
        check(lib.hg_sync(self.h))

    @property
    def step_count(self):
        v = ctypes.c_uint64()
        check(lib.hg_world_get_step(self.h, ctypes.byref(v)))
        return v.value

    @step_count.setter
    def step_count(self, v):
        check(lib.hg_world_set_step(self.h, v))

    def totals(self):
        out = (ctypes.c_double * 3)()
        check(lib.hg_world_totals(self.h, out))
        return list(out)

    def tuning(self):
        th, g, ms = ctypes.c_int(), ctypes.c_int(), (ctypes.c_double * 4)()
        check(lib.hg_world_tuning(self.h, ctypes.byref(th), ctypes.byref(g), ms))
        return th.value, g.value, list(ms)

    def save(self, path):
        check(lib.hg_world_save(self.h, str(path).encode()))

    def load(self, path):
        check(lib.hg_world_load(self.h, str(path).encode()))

    @property
    def stream(self):
        p = ctypes.c_void_p()
        check(lib.hg_world_stream(self.h, ctypes.byref(p)))
        return p.value or 0


class Tape:
    """Checkpointed record of nsteps steps of a world for hg_backward."""

    def __init__(self, world, nsteps, ckpt_every=HG_AUTO):
        h = ctypes.c_void_p()
        check(lib.hg_tape_create(world.h, nsteps, ckpt_every, ctypes.byref(h)))
        self.h = h
        self.world = world
        world._tapes.add(self)
        _live["tapes"].add(self)

    def close(self):
        if self.h:
            lib.hg_tape_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def ckpt_every(self):
        a, b = ctypes.c_int(), ctypes.c_int()
        check(lib.hg_tape_info(self.h, ctypes.byref(a), ctypes.byref(b)))
        return b.value

    def forward(self):
        check(lib.hg_forward(self.h))

    def backward(self, dl_drock_ptr, dl_dks_ptr=None, dl_drock0_ptr=None):
        """Device pointers (e.g. torch tensors' data_ptr())."""
        check(lib.hg_backward(self.h, ctypes.c_void_p(dl_drock_ptr), ctypes.c_void_p(dl_dks_ptr or 0),
                              ctypes.c_void_p(dl_drock0_ptr or 0)))


def mse(world, target_ptr, grad_ptr=None):
    loss = ctypes.c_double()
    check(lib.hg_mse(world.h, ctypes.c_void_p(target_ptr), ctypes.byref(loss), ctypes.c_void_p(grad_ptr or 0)))
    return loss.value


_log_keep = None


def set_log(fn):
    """Route the library's reports (hg_set_log_callback) to fn(level, text);
    None turns them off.  Level 0 is a failure, 1 an autotuner choice."""
    global _log_keep
    _log_keep = LOG_FN(lambda level, msg, user: fn(level, msg.decode())) if fn else LOG_FN()
    check(lib.hg_set_log_callback(_log_keep, None))


def fit_settings(**kw):
    """hg_fit_settings with the library defaults, fields overridden by keyword."""
    s = FitSettings()
    check(lib.hg_default_fit_settings(ctypes.byref(s)))
    for k, v in kw.items():
        if not hasattr(s, k):
            raise AttributeError(f"hg_fit_settings has no field {k}")
        setattr(s, k, v)
    return s


def inverse_fit(world, target_ptr, ks_ptr, rock0_ptr, settings=None, grad_norms=False):
    """Native inverse-erosion descent (hg_inverse_fit) on device buffers;
    returns the per-iteration losses (and, with grad_norms, the FP64 norms
    of each iteration's gradient)."""
    s = settings or fit_settings()
    out = (ctypes.c_double * s.iters)()
    gn = (ctypes.c_double * s.iters)() if grad_norms else None
    check(lib.hg_inverse_fit(world.h, ctypes.c_void_p(target_ptr), ctypes.c_void_p(ks_ptr or 0),
                             ctypes.c_void_p(rock0_ptr), ctypes.byref(s), out, gn))
    return (list(out), list(gn)) if grad_norms else list(out)


class Batch:
    """Several worlds stepped together (one fused launch pair per step for all)."""

    def __init__(self, worlds):
        self.worlds = list(worlds)
        arr = (ctypes.c_void_p * len(self.worlds))(*[w.h for w in self.worlds])
        h = ctypes.c_void_p()
        check(lib.hg_batch_create(arr, len(self.worlds), ctypes.byref(h)))
        self.h = h
        _live["batches"].add(self)

    def close(self):
        if self.h:
            lib.hg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, nsteps=1, mode=MODE_FUSED):
        check(lib.hg_batch_step(self.h, nsteps, mode))

    def sync(self):
        check(lib.hg_batch_sync(self.h))

    @property
    def stream(self):
        p = ctypes.c_void_p()
        check(lib.hg_batch_stream(self.h, ctypes.byref(p)))
        return p.value or 0

    def tuning(self):
        th, g, ms = ctypes.c_int(), ctypes.c_int(), (ctypes.c_double * 4)()
        check(lib.hg_batch_tuning(self.h, ctypes.byref(th), ctypes.byref(g), ms))
        return th.value, g.value, list(ms)

    def launch_form(self):
        """(per_world, ms_per_world): 1 when the autotuner kept every world's
        own launches over one table launch."""
        pw, ms = ctypes.c_int(), ctypes.c_double()
        check(lib.hg_batch_launch_form(self.h, ctypes.byref(pw), ctypes.byref(ms)))
        return pw.value, ms.value


def config3_terrains(count=64, seed=0):
    """Ragged multi-terrain workload: side drawn from {256, 512, 1024, 2048},
    own fBm seed, Kc log-uniform [0.05, 0.5], Ks and Kd log-uniform
    [0.01, 0.1], Ke uniform [0.005, 0.03], talus tan uniform [0.4, 0.9],
    config-2 rain and slippage.  Returns a list of dicts (the manifest)."""
    import random
    rng = random.Random(seed)
    lu = lambda a, b: math.exp(rng.uniform(math.log(a), math.log(b)))
    out = []
    for i in range(count):
        out.append(dict(n=rng.choice([256, 512, 1024, 2048]), seed=1000 + i, Kc=lu(0.05, 0.5), Ks=lu(0.01, 0.1),
                        Kd=lu(0.01, 0.1), Ke=rng.uniform(0.005, 0.03), talus_tan=rng.uniform(0.4, 0.9)))
    return out


def shard_by_area(sides, nranks):
    """Owner rank of each terrain for a job of nranks ranks: greedy longest
    processing time on cell counts (largest terrain first, ties by index,
    each to the least-loaded rank, ties by rank).  Every rank computes the
    same assignment from the manifest; terrains are independent, so the
    ranks step their shares with no data exchange.  The largest load is
    within one terrain of the mean."""
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    area = [int(s) * int(s) for s in sides]
    load = [0] * nranks
    owner = [0] * len(area)
    for i in sorted(range(len(area)), key=lambda k: (-area[k], k)):
        r = min(range(nranks), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += area[i]
    return owner


def make_config3_world(t, terrain_id=0):
    w = World(t["n"])
    w.init_heightmap(noise(seed=t["seed"]))
    s = settings_config2()
    s.Kc = t["Kc"]
    s.Ks[0] = s.Ks[1] = t["Ks"]
    s.Kd[0] = s.Kd[1] = t["Kd"]
    s.Ke = t["Ke"]
    s.Kalpha[0] = s.Kalpha[1] = math.atan(t["talus_tan"])
    w.set_erosion(s)
    w.set_rain(rain_uniform(0.5, 1))
    w.set_options(options(RAIN_BERNOULLI, p=0.001, seed=t["seed"], terrain_id=terrain_id))
    return w


def configure(world, cfg, seed=0):
    """Apply a named workload ('config1', 'config2') to a world."""
    if cfg == "config1":
        world.set_erosion(settings_config1())
        world.set_rain(rain_uniform(0.01, 1))
        world.set_options(options(RAIN_UNIFORM))
    elif cfg == "config2":
        world.set_erosion(settings_config2())
        world.set_rain(rain_uniform(0.5, 1))
        world.set_options(options(RAIN_BERNOULLI, p=0.001, seed=seed))
    else:
        raise ValueError(cfg)
