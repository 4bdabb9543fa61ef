"""Failure detection without a GPU fault.

A fused-step block waits for its TMA tile with a bounded number of barrier
polls; if the tile never arrives it records an error flag, skips the tile and
returns, and hg_sync reports HG_ERR_TIMEOUT.  Here the same wait runs on a
barrier phase that nothing completes (no copy in flight, no trap, no fault):
it must give up, say so, and leave the device usable."""
import ctypes

import numpy as np
import pytest

import hydrogen as H

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_the_device_stays_usable():
    flag, ns = ctypes.c_int(-1), ctypes.c_double()
    H.check(H.lib.hg_selftest_bounded_wait(1 << 12, ctypes.byref(flag), ctypes.byref(ns)))
    assert flag.value == 1
    assert ns.value > 0
    bound_s = (1 << 18) * ns.value / 1e9  # the kernels' limit
    print(f"bounded wait: {ns.value:.1f} ns per poll; a lost tile is given up after {bound_s:.2f} s")
    assert bound_s < 5
    # the context still runs the library's kernels: the fused step equals the per-pass one
    a, b = H.World(128), H.World(128)
    for w in (a, b):
        w.init_heightmap(H.noise(seed=3))
        H.configure(w, "config2")
    a.step(10, H.MODE_PLAIN)
    b.step(10, H.MODE_FUSED)
    for f in ("rock", "water", "sediment"):
        assert np.array_equal(a.download(f), b.download(f)), f
    b.sync()  # no tile of the fused steps timed out
