"""The C-ABI library loads and exports every entry point declared in
include/hydrogen.h, and the settings structs keep the reference's layout.
No compute calls: these run without a GPU."""
import ctypes
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "hydro-gen_gb300", "libhydrogen_gb300.so")


@pytest.fixture(scope="module")
def hg():
    if not os.path.exists(LIB):
        import importlib.util
        spec = importlib.util.spec_from_file_location("hg_build", os.path.join(ROOT, "hydro-gen_gb300", "build.py"))
        m = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(m)
        m.build()
    import hydrogen
    return hydrogen


def test_every_declared_function_is_exported(hg):
    names = hg.header_functions()
    assert len(names) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", LIB], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    lib = ctypes.CDLL(LIB)
    for n in names:
        assert getattr(lib, n) is not None


def test_erosion_settings_std140_layout(hg):
    # Erosion_data offsets (glsl/bindings.glsl:39-60 under std140)
    S = hg.ErosionSettings
    assert ctypes.sizeof(S) == 96
    expect = {"particle_count": 0, "Kc": 4, "Kalpha": 8, "Kconv": 16, "Ks": 24, "Kd": 32, "Ke": 40,
              "ENERGY_KEPT": 44, "Kspeed": 48, "G": 56, "d_t": 60, "density": 64, "ttl": 88}
    for f, off in expect.items():
        assert getattr(S, f).offset == off, f
    assert ctypes.sizeof(hg.RainSettings) == 20


def test_reference_defaults(hg):
    s = hg.ErosionSettings()
    assert hg.lib.hg_default_erosion_settings(ctypes.byref(s)) == 0
    # src/state.cpp:81-92
    assert s.Kc == pytest.approx(0.2) and s.G == 1.0 and s.d_t == pytest.approx(0.001)
    assert list(s.Ks) == pytest.approx([0.03, 0.09]) and list(s.Kspeed) == pytest.approx([0.5, 2.0])
    r = hg.RainSettings()
    assert hg.lib.hg_default_rain_settings(ctypes.byref(r)) == 0
    assert r.period == 512 and r.amount == pytest.approx(0.01)


def test_error_paths_without_a_device(hg):
    # argument checks run before any CUDA call
    h = ctypes.c_void_p()
    assert hg.lib.hg_world_create(12, 1, ctypes.byref(h)) == -1  # not a multiple of 8
    assert b"multiple of 8" in hg.lib.hg_last_error()
    assert hg.lib.hg_world_create(64, 3, ctypes.byref(h)) == -5  # layers 1 (rock) or 2 (rock + dirt)
    assert hg.lib.hg_step(None, 1, 0) == -1
    assert hg.lib.hg_world_destroy(None) == 0
    flag, ns = ctypes.c_int(), ctypes.c_double()
    assert hg.lib.hg_selftest_bounded_wait(0, ctypes.byref(flag), ctypes.byref(ns)) == -1
    assert hg.lib.hg_selftest_bounded_wait((1 << 18) + 1, ctypes.byref(flag), ctypes.byref(ns)) == -1
    fs = hg.FitSettings()
    assert hg.lib.hg_default_fit_settings(ctypes.byref(fs)) == 0
    assert (fs.nsteps, fs.ckpt_every, fs.iters) == (256, 32, 8)
    assert hg.lib.hg_inverse_fit(None, None, None, None, ctypes.byref(fs), None, None) == -1
    assert hg.lib.hg_init_heightmap_host(None, None) == -1
    # the row-slab entry points refuse a null world before any CUDA call
    assert hg.lib.hg_set_rows(None, 0, 8) == -1
    assert hg.lib.hg_pass(None, 1, 0) == -1
    assert hg.lib.hg_fused_pass(None, 0) == -1
    assert hg.lib.hg_world_rows(None, 0, 0, 1, None, 0) == -1
    # the allocation-free totals check their arguments before any CUDA call
    out = ctypes.c_void_p(1)
    ptrs = (ctypes.c_void_p * 9)(*([1] * 9))
    assert hg.lib.hg_field_totals_noalloc(None, 1, 16, out, None) == -1
    assert hg.lib.hg_field_totals_noalloc(ptrs, 0, 16, out, None) == -1
    assert hg.lib.hg_field_totals_noalloc(ptrs, 9, 16, out, None) == -1  # more than HG_NOALLOC_MAX_FIELDS
    assert b"nfields" in hg.lib.hg_last_error()
    nulls = (ctypes.c_void_p * 2)(1, None)
    assert hg.lib.hg_field_totals_noalloc(nulls, 2, 16, out, None) == -1


def test_log_callback_receives_failures(hg):
    got = []
    hg.set_log(lambda level, text: got.append((level, text)))
    try:
        h = ctypes.c_void_p()
        assert hg.lib.hg_world_create(12, 1, ctypes.byref(h)) == -1
        assert got and got[-1][0] == 0 and "multiple of 8" in got[-1][1]
        assert got[-1][1] == hg.lib.hg_last_error().decode()
    finally:
        hg.set_log(None)
    n = len(got)
    assert hg.lib.hg_world_create(12, 1, ctypes.byref(ctypes.c_void_p())) == -1
    assert len(got) == n  # off again


def test_header_cites_reference():
    text = open(os.path.join(ROOT, "include", "hydrogen.h")).read()
    for cite in ("glsl/bindings.glsl:39-60", "src/erosion.cpp", "src/state.cpp:116-147"):
        assert cite in text
