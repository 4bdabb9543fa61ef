"""Checkpoint / resume: a run interrupted by save + load into a fresh world
continues bit for bit like the uninterrupted run (rain is keyed by step)."""
import numpy as np
import pytest

import hydrogen as H

pytestmark = pytest.mark.gpu

STATE = ["rock", "water", "sediment", "flux_l", "flux_r", "flux_t", "flux_b", "vel_u", "vel_v"]


def world(n=256):
    w = H.World(n)
    w.init_heightmap(H.noise(seed=3))
    H.configure(w, "config2")
    w.set_options(H.options(H.RAIN_BERNOULLI, p=0.02, seed=11))
    return w


@pytest.mark.parametrize("mode", [H.MODE_PLAIN, H.MODE_FUSED])
def test_resume_is_bit_identical(tmp_path, mode):
    a = world()
    a.step(40, mode)
    path = tmp_path / "w.hgw"
    a.save(path)
    a.step(40, mode)
    b = H.World(256)  # fresh world, default settings: everything comes from the file
    b.load(path)
    assert b.step_count == 40
    assert b.get_erosion().Kspeed[0] == pytest.approx(0.3)
    b.step(40, mode)
    for f in STATE:
        assert np.array_equal(a.download(f), b.download(f)), f


def test_checkpoint_keeps_ks_field(tmp_path):
    a = world(128)
    a.init_ks_field(H.noise(seed=7, octaves=3, frequency=1.0 / 256), 0.05, 0.5)
    a.save(tmp_path / "k.hgw")
    b = H.World(128)
    b.load(tmp_path / "k.hgw")
    assert np.array_equal(a.download("ks"), b.download("ks"))
    a.step(10, H.MODE_FUSED)
    b.step(10, H.MODE_FUSED)
    assert np.array_equal(a.download("rock"), b.download("rock"))


def test_checkpoint_errors(tmp_path):
    a = world(128)
    a.save(tmp_path / "a.hgw")
    with pytest.raises(H.HydrogenError) as e:
        H.World(256).load(tmp_path / "a.hgw")
    assert e.value.code == -1
    (tmp_path / "bad.hgw").write_bytes(b"not a checkpoint")
    with pytest.raises(H.HydrogenError) as e:
        a.load(tmp_path / "bad.hgw")
    assert e.value.code == -6
    with pytest.raises(H.HydrogenError) as e:
        a.load(tmp_path / "missing.hgw")
    assert e.value.code == -6
