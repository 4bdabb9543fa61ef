"""Full-size workloads (4096², 8192², 16384²).

The headline workload (4096², Bernoulli rain p = 0.001, talus slippage) is
compared bit for bit with the float oracle on every state field after 20
steps, per-pass and fused (the oracle takes a few seconds per 20 steps on
the host's cores).  The other full sizes go through a size-independent
property: the fused step equals the per-pass kernels bit for bit on every
state field, compared on the device (torch.equal)."""
import numpy as np
import pytest

import hydrogen as H
import oracle as O

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


@pytest.mark.parametrize("mode", [H.MODE_PLAIN, H.MODE_FUSED])
def test_config2_4096_bitwise_vs_float_oracle(mode):
    """The metric's workload at its own size: every state field (and, for the
    per-pass kernels, the velocity map's depth channel) equals the float
    restatement of the GLSL passes bit for bit after 20 steps."""
    n, steps = 4096, 20
    w = H.World(n)
    w.init_heightmap(H.noise(seed=0))
    H.configure(w, "config2")
    s, o = O.workload("config2")
    ow = O.OracleWorld(n, 32)
    ow.set("rock", w.download("rock"))
    w.step(steps, mode)
    ow.step(s, o, steps)
    fields = ONE + (["vel_z"] if mode == H.MODE_PLAIN else [])
    for f in fields:
        g = w.download(f).astype(np.float64)
        r = ow.get(f)
        bad = np.argwhere(g != r)
        assert bad.size == 0, f"{f}: {len(bad)} cells differ, first {bad[:3].tolist()}"
    assert w.step_count == steps
    # the workload is not trivial at this point: rain fell, sediment moved,
    # talus slippage changed rock
    assert float(np.max(ow.get("water"))) > 0.0 and float(np.max(np.abs(ow.get("sediment")))) > 0.0
    w.close()


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


def test_largest_16384_fused_equals_plain():
    """The largest size the tests step: 16384² (268 M cells, 2^28, about
    35 GB of fields and scratch per world; the cell index is 64-bit and a
    launch has 262,144 tiles), the metric's physics and rain."""
    def make():
        w = H.World(16384)
        w.init_heightmap(H.noise(seed=0))
        H.configure(w, "config2")
        return w
    f = run_pair(make, 3, ONE)
    assert float(f["water"].max()) > 0.0 and float(f["sediment"].abs().max()) > 0.0


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
