"""Full-size workloads (4096², 8192²) through a size-independent property:
the fused step equals the per-pass kernels bit for bit on every state field.
Fields are compared on the device (torch.equal), not downloaded; the oracle
itself is checked at sizes it finishes in seconds (test_gpu_parity,
test_gpu_layers)."""
import numpy as np
import pytest

import hydrogen as H

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

ONE = ["rock", "water", "sediment", "flux_l", "flux_r", "flux_t", "flux_b", "vel_u", "vel_v"]
TWO = ONE + ["dirt", "sediment_dirt"]


def device_field(w, f):
    t = torch.empty((w.n, w.n), dtype=torch.float32, device="cuda")
    w.download_device(f, t.data_ptr())
    w.sync()
    return t


def run_pair(make, steps, fields):
    out = []
    for mode in (H.MODE_PLAIN, H.MODE_FUSED):
        w = make()
        w.step(steps, mode)
        w.sync()
        out.append({f: device_field(w, f) for f in fields})
        w.close()
    for f in fields:
        a, b = out[0][f], out[1][f]
        assert torch.equal(a.view(torch.int32), b.view(torch.int32)), f"{f}: fused and per-pass differ"
        assert torch.isfinite(a).all(), f
    return out[1]


def test_config2_4096_fused_equals_plain():
    def make():
        w = H.World(4096)
        w.init_heightmap(H.noise(seed=0))
        H.configure(w, "config2")
        return w
    f = run_pair(make, 6, ONE)
    assert float(f["water"].max()) > 0.0 and float(f["sediment"].abs().max()) > 0.0


def test_large_8192_thermal_fused_equals_plain():
    def make():
        w = H.World(8192)
        w.init_heightmap(H.noise(seed=5))
        s = H.settings_config1()
        s.Kspeed[0] = 0.3
        s.Kalpha[0] = float(np.arctan(0.65))
        w.set_erosion(s)
        w.set_rain(H.rain_uniform(0.01, 1))
        w.set_options(H.options(H.RAIN_UNIFORM))
        return w
    run_pair(make, 4, ONE)


def test_two_layer_4096_reference_defaults_fused_equals_plain():
    def make():
        w = H.World(4096, layers=2)
        w.init_reference_heightmap(H.map_settings(hmap_dims=(4096, 4096)))
        s = H.ErosionSettings()
        H.check(H.lib.hg_default_erosion_settings(H.ctypes.byref(s)))
        w.set_erosion(s)
        w.set_rain(H.rain_uniform(0.01, 1))
        w.set_options(H.options(H.RAIN_UNIFORM))
        return w
    f = run_pair(make, 4, TWO)
    assert float(f["sediment_dirt"].abs().max()) > 0.0
