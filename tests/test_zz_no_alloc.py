"""hg_field_totals_noalloc: the allocation-free variant of the FP64 totals.

Some callers cannot allocate device memory: an engine or content tool that
owns the GPU's memory budget and gives plugins only buffers it allocated,
or a frame loop that cannot afford the device-wide synchronisation that
cudaMalloc/cudaFree bring.  They call hg_field_totals_noalloc with their own
input and output buffers; its scratch is a fixed array inside the library.
This test checks it through the C ABI against hg_world_totals (the existing
entry point, whose scratch the world allocated) on two calls in a row, the
second with different inputs and fewer fields so the shared scratch still
holds the first call's partial sums.  Kept in its own file, collected last.
"""
import ctypes

import numpy as np
import pytest

import hydrogen as H

pytestmark = pytest.mark.gpu

TOL = 1e-12  # same reduction tree on both sides: expect equality, allow FP64 rounding noise


def device_fields(w, names):
    import torch
    out = []
    for f in names:
        t = torch.empty((w.n, w.n), dtype=torch.float32, device="cuda")
        w.download_device(f, t.data_ptr())
        out.append(t)
    return out


def noalloc_totals(w, tensors):
    import torch
    ptrs = (ctypes.c_void_p * len(tensors))(*[t.data_ptr() for t in tensors])
    out = torch.full((len(tensors),), float("nan"), dtype=torch.float64, device="cuda")
    H.check(H.lib.hg_field_totals_noalloc(ptrs, len(tensors), w.n * w.n, ctypes.c_void_p(out.data_ptr()),
                                          ctypes.c_void_p(w.stream)))
    w.sync()
    return out.cpu().numpy()


def test_noalloc_totals_match_world_totals_twice():
    import torch
    torch.cuda.set_device(0)
    w = H.World(256)
    w.init_heightmap(H.noise(seed=5))
    H.configure(w, "config2")
    w.set_options(H.options(H.RAIN_BERNOULLI, p=0.02))
    w.step(30, H.MODE_FUSED)

    ref1 = np.array(w.totals())  # rock, water, sediment
    got1 = noalloc_totals(w, device_fields(w, ["rock", "water", "sediment"]))
    assert np.allclose(got1, ref1, rtol=TOL, atol=0), (got1, ref1)

    w.step(10, H.MODE_FUSED)
    ref2 = np.array(w.totals())
    got2 = noalloc_totals(w, device_fields(w, ["water", "sediment"]))
    assert np.allclose(got2, ref2[1:], rtol=TOL, atol=0), (got2, ref2)
    assert not np.allclose(ref1[1:], ref2[1:])  # the second call really saw new data


def test_noalloc_rejects_too_many_fields():
    import torch
    t = torch.zeros(64, dtype=torch.float32, device="cuda")
    out = torch.zeros(16, dtype=torch.float64, device="cuda")
    ptrs = (ctypes.c_void_p * 9)(*([t.data_ptr()] * 9))
    rc = H.lib.hg_field_totals_noalloc(ptrs, 9, 64, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == -1
    assert b"HG_NOALLOC_MAX_FIELDS" in H.lib.hg_last_error()
