"""GPU adjoint (FP32, through the C ABI) against the FP64 reference adjoint,
which is itself checked against finite differences of the oracle forward
(tests/test_adjoint_reference.py), without and with thermal erosion.  Bar:
relative L2 error of each gradient field within 1e-3 of the FP64
reference."""
import numpy as np
import pytest

import hydrogen as H
import oracle as O

pytestmark = pytest.mark.gpu


def torch_dev():
    import torch
    torch.cuda.set_device(0)
    return torch


def make_world(n, ks_seed=7, rock_seed=1, freq=1.0 / 32, thermal=False):
    w = H.World(n)
    w.init_heightmap(H.noise(seed=rock_seed, frequency=freq))
    H.configure(w, "config1")
    if thermal:  # the uniform-rain physics with talus slippage
        s = H.settings_config1()
        s.Kspeed[0] = 0.3
        w.set_erosion(s)
    w.init_ks_field(H.noise(seed=ks_seed, octaves=3, frequency=1.0 / 64), 0.05, 0.5)
    return w


def ref_settings(thermal):
    s = O.settings_config1()
    if thermal:
        s.Kspeed[0] = 0.3
    return s


def gpu_gradients(w, target, nsteps, ckpt):
    torch = torch_dev()
    n = w.n
    tgt = torch.from_numpy(target.astype(np.float32)).cuda()
    g = torch.empty((n, n), dtype=torch.float32, device="cuda")
    dks = torch.empty_like(g)
    db0 = torch.empty_like(g)
    tape = H.Tape(w, nsteps, ckpt)
    tape.forward()
    loss = H.mse(w, tgt.data_ptr(), g.data_ptr())
    tape.backward(g.data_ptr(), dks.data_ptr(), db0.data_ptr())
    w.sync()
    return loss, dks.cpu().numpy().astype(np.float64), db0.cpu().numpy().astype(np.float64), tape


def rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("n,nsteps,ckpt,thermal", [(64, 24, 8, False), (128, 40, 7, False),
                                                   (64, 24, 8, True), (128, 40, 7, True)])
def test_gpu_adjoint_matches_fp64_reference(n, nsteps, ckpt, thermal):
    w = make_world(n, thermal=thermal)
    b0 = w.download("rock").astype(np.float64)
    ks = w.download("ks")
    rng = np.random.default_rng(n)
    target = b0 - 0.02 * rng.random((n, n))
    loss, dks, db0, tape = gpu_gradients(w, target, nsteps, ckpt)
    assert tape.ckpt_every == ckpt
    rloss, rdks, rdb0 = O.adjoint_ref(ref_settings(thermal), 0.01, 1, b0, ks, target, nsteps)
    assert abs(loss - rloss) <= 1e-4 * rloss
    e_ks, e_b0 = rel_l2(dks, rdks), rel_l2(db0, rdb0)
    print(f"{n}^2 x {nsteps} thermal={thermal}: rel L2 error dKs {e_ks:.2e}, drock0 {e_b0:.2e}")
    assert e_ks <= 1e-3 and e_b0 <= 1e-3


def test_checkpoint_interval_does_not_change_gradients():
    n, nsteps = 64, 20
    outs = []
    for ckpt in (1, 6, 20, H.HG_AUTO):
        w = make_world(n)
        target = w.download("rock") * 0.99
        outs.append(gpu_gradients(w, target, nsteps, ckpt))
    for loss, dks, db0, _ in outs[1:]:
        assert loss == outs[0][0]
        assert rel_l2(dks, outs[0][1]) <= 1e-5  # only atomic-add order differs
        assert rel_l2(db0, outs[0][2]) <= 1e-5


@pytest.mark.parametrize("thermal", [False, True])
def test_tape_forward_is_the_fused_step(thermal):
    a = make_world(128, thermal=thermal)
    b = make_world(128, thermal=thermal)
    tape = H.Tape(a, 30, 8)
    tape.forward()
    b.step(30, H.MODE_FUSED)
    for f in H.STATE_FIELDS:
        assert np.array_equal(a.download(f), b.download(f)), f


def test_inverse_fit_reduces_loss():
    """Fit per-cell Ks to a target made with a noise Ks field (config-4 form, small)."""
    torch = torch_dev()
    n, nsteps = 64, 32
    truth = make_world(n, ks_seed=7)
    truth.step(nsteps, H.MODE_FUSED)
    target = torch.from_numpy(truth.download("rock")).cuda()
    w = make_world(n)
    b0 = w.download("rock")
    ks = torch.full((n, n), 0.05, dtype=torch.float32, device="cuda")
    g = torch.empty_like(ks)
    dks = torch.empty_like(ks)
    losses = []
    for it in range(6):
        w.upload("rock", b0)
        for f in ("water", "sediment", "flux_l", "flux_r", "flux_t", "flux_b"):
            w.upload(f, np.zeros((n, n), np.float32))
        w.step_count = 0
        w.upload_device("ks", ks.data_ptr())
        tape = H.Tape(w, nsteps, 8)
        tape.forward()
        losses.append(H.mse(w, target.data_ptr(), g.data_ptr()))
        tape.backward(g.data_ptr(), dks.data_ptr(), None)
        w.sync()
        step = 1e-3 / max(float(dks.abs().max()), 1e-30)
        ks = torch.clamp(ks - step * dks, 0.005, 0.5)
    print("inverse fit losses", losses)
    assert losses[-1] < losses[0]


def test_adjoint_rejects_smoothing():
    w = H.World(64)
    H.configure(w, "config1")
    s = H.settings_config1()
    s.Kspeed[1] = 1.0
    w.set_erosion(s)
    with pytest.raises(H.HydrogenError) as e:
        H.Tape(w, 4)
    assert e.value.code == -5


@pytest.mark.parametrize("nsteps,ckpt", [(20, 5), (8, 4), (6, 6)])
def test_second_backward_recomputes_the_same_gradients(nsteps, ckpt):
    """The forward leaves its last segment in the tape; a second backward over
    the same tape recomputes every segment (two segment buffers alternate
    between the recompute stream and the reverse sweep)."""
    torch = torch_dev()
    w = make_world(64, thermal=True)
    target = torch.from_numpy(w.download("rock") * 0.99).cuda()
    g = torch.empty_like(target)
    tape = H.Tape(w, nsteps, ckpt)
    tape.forward()
    H.mse(w, target.data_ptr(), g.data_ptr())
    outs = []
    for _ in range(2):
        dks = torch.empty_like(g)
        db0 = torch.empty_like(g)
        tape.backward(g.data_ptr(), dks.data_ptr(), db0.data_ptr())
        w.sync()
        outs.append((dks.cpu().numpy().astype(np.float64), db0.cpu().numpy().astype(np.float64)))
    assert rel_l2(outs[1][0], outs[0][0]) <= 1e-5  # only atomic-add order differs
    assert rel_l2(outs[1][1], outs[0][1]) <= 1e-5
