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


@pytest.mark.parametrize("n, nsteps", [(256, 60), (1024, 40)])
def test_gradients_finite_under_intermittent_rain(n, nsteps):
    """Bernoulli rain (the 4096^2 workload's physics: p = 0.001, talus
    slippage) leaves water films down to ~1e-35 deep, where the derivatives
    of the velocity (flux difference / depth) and of the flux scale grow
    like 1/depth and overflow float; below 5e-4 of water (where the erosion
    ignores the velocity) the reverse holds both constant, so the gradients
    stay finite and non-zero."""
    w = H.World(n)
    w.init_heightmap(H.noise(seed=0))
    H.configure(w, "config2")
    w.init_ks_field(H.noise(seed=7, octaves=3, frequency=1.0 / 256), 0.05, 0.5)
    target = w.download("rock") * 0.999
    loss, dks, db0, tape = gpu_gradients(w, target, nsteps, H.HG_AUTO)
    assert np.isfinite(loss)
    assert np.all(np.isfinite(dks)) and np.all(np.isfinite(db0))
    assert np.abs(dks).max() > 0 and np.abs(db0).max() > 0


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


def test_ragged_segments_under_step_keyed_rain():
    """Bernoulli rain is keyed on the step number, so every segment's steps
    must take their own numbers in the forward, the recompute and the
    reverse.  With checkpoint intervals that leave a short first segment
    (29 = 3 + 2 x 13 = 1 + 4 x 7) the gradients equal those of the whole
    tape in memory (interval 29, nothing recomputed) up to the order of the
    sediment adjoint's atomic adds, and the forward's final state equals 29
    plain fused steps bit for bit."""
    n, nsteps = 128, 29
    torch_dev()

    def world():
        w = H.World(n)
        w.init_heightmap(H.noise(seed=1, frequency=1.0 / 32))
        H.configure(w, "config2")
        w.set_options(H.options(H.RAIN_BERNOULLI, p=0.05, seed=5))
        w.init_ks_field(H.noise(seed=7, octaves=3, frequency=1.0 / 64), 0.05, 0.5)
        return w

    ref = world()
    ref.step(nsteps, H.MODE_FUSED)
    final = {f: ref.download(f) for f in H.STATE_FIELDS}
    target = world().download("rock") * 0.999
    outs = {}
    for ckpt in (29, 13, 7):
        w = world()
        outs[ckpt] = gpu_gradients(w, target, nsteps, ckpt)
        assert outs[ckpt][3].ckpt_every == ckpt
        for f in H.STATE_FIELDS:
            assert np.array_equal(w.download(f), final[f]), (ckpt, f)
    loss, dks, db0, _ = outs[29]
    assert np.abs(dks).max() > 0
    for ckpt in (13, 7):
        assert outs[ckpt][0] == loss
        assert rel_l2(outs[ckpt][1], dks) <= 1e-5 and rel_l2(outs[ckpt][2], db0) <= 1e-5, ckpt


@pytest.mark.parametrize("thermal", [False, True])
def test_tape_forward_is_the_fused_step(thermal):
    a = make_world(128, thermal=thermal)
    b = make_world(128, thermal=thermal)
    tape = H.Tape(a, 30, 8)
    tape.forward()
    b.step(30, H.MODE_FUSED)
    for f in H.STATE_FIELDS:
        assert np.array_equal(a.download(f), b.download(f)), f


def fit_problem(n, nsteps):
    """Target: nsteps of the uniform-rain physics with a noise Ks field; the
    fit starts from uniform Ks = 0.05 and the same initial rock."""
    torch = torch_dev()
    truth = make_world(n, ks_seed=7)
    truth.step(nsteps, H.MODE_FUSED)
    target = torch.from_numpy(truth.download("rock")).cuda()
    w = make_world(n)
    b0 = torch.from_numpy(w.download("rock")).cuda()
    ks = torch.full((n, n), 0.05, dtype=torch.float32, device="cuda")
    return torch, w, target, b0, ks


def descend(x, g, step, lo, hi):
    """The normalised step of hg_inverse_fit in float32: x - (step / max|g|) g, clamped."""
    a = np.float32(step) / np.maximum(np.abs(g).max(), np.float32(1e-30))
    return np.minimum(np.maximum(x - np.float32(a) * g, np.float32(lo)), np.float32(hi))


@pytest.mark.parametrize("rock_step", [0.0, 0.05])
def test_inverse_fit_is_the_tape_loop(rock_step):
    """hg_inverse_fit equals the same descent driven by hand through
    hg_forward / hg_mse / hg_backward and a float32 update.  The sediment
    adjoint scatters with float atomics, so the gradients' last bits follow
    the atomics' order: the bar is a few ulps (rtol 1e-5), against a Ks
    change of up to 1e-2 per iteration."""
    n, nsteps, iters = 64, 24, 3
    torch, w, target, b0, ks = fit_problem(n, nsteps)
    s = H.fit_settings(nsteps=nsteps, ckpt_every=8, iters=iters, ks_step=0.01, rock_step=rock_step)
    ks_fit, b_fit = ks.clone(), b0.clone()
    torch.cuda.synchronize()  # the fit reads the buffers on the world's stream
    losses, norms = H.inverse_fit(w, target.data_ptr(), ks_fit.data_ptr(), b_fit.data_ptr(), s, grad_norms=True)
    w_end = w.download("rock")

    m = make_world(n)
    ks_np, b_np = ks.cpu().numpy(), b0.cpu().numpy()
    g = torch.empty_like(ks)
    dks = torch.empty_like(ks)
    db0 = torch.empty_like(ks)
    tape = H.Tape(m, nsteps, 8)
    ref, ref_norms = [], []
    for _ in range(iters):
        m.upload("rock", b_np)
        for f in ("water", "sediment", "flux_l", "flux_r", "flux_t", "flux_b", "vel_u", "vel_v"):
            m.upload(f, np.zeros((n, n), np.float32))
        m.step_count = 0
        m.upload("ks", ks_np)
        tape.forward()
        ref.append(H.mse(m, target.data_ptr(), g.data_ptr()))
        tape.backward(g.data_ptr(), dks.data_ptr(), db0.data_ptr())
        m.sync()
        sq = np.sum(dks.cpu().numpy().astype(np.float64) ** 2)
        if rock_step:
            sq += np.sum(db0.cpu().numpy().astype(np.float64) ** 2)
        ref_norms.append(np.sqrt(sq))
        ks_np = descend(ks_np, dks.cpu().numpy(), 0.01, 0.005, 0.5)
        if rock_step:
            b_np = descend(b_np, db0.cpu().numpy(), rock_step, -np.finfo(np.float32).max, np.finfo(np.float32).max)
    np.testing.assert_allclose(losses, ref, rtol=1e-5)
    np.testing.assert_allclose(norms, ref_norms, rtol=1e-4)  # FP64 on the device, FP64 here
    np.testing.assert_allclose(ks_fit.cpu().numpy(), ks_np, rtol=1e-5, atol=0)
    np.testing.assert_allclose(b_fit.cpu().numpy(), b_np, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(w_end, m.download("rock"), rtol=1e-5, atol=1e-5)
    assert np.array_equal(w.download("ks"), ks_fit.cpu().numpy())


def test_inverse_fit_reduces_loss():
    """Fit per-cell Ks and the initial rock to a target made with a noise Ks
    field (the inverse-erosion workload's form, small)."""
    n, nsteps = 64, 32
    torch, w, target, b0, ks = fit_problem(n, nsteps)
    s = H.fit_settings(nsteps=nsteps, ckpt_every=8, iters=8, ks_step=0.01, rock_step=0.02)
    torch.cuda.synchronize()
    losses = H.inverse_fit(w, target.data_ptr(), ks.data_ptr(), b0.data_ptr(), s)
    print("inverse fit losses", losses)
    assert losses[-1] < 0.5 * losses[0]
    assert float(ks.min()) >= 0.005 and float(ks.max()) <= 0.5


def test_inverse_fit_rejects_bad_arguments():
    n = 64
    torch, w, target, b0, ks = fit_problem(n, 4)
    for kw in (dict(iters=0), dict(ks_step=-1.0), dict(ks_min=0.5, ks_max=0.1)):
        s = H.fit_settings(nsteps=4, ckpt_every=2, **kw)
        with pytest.raises(H.HydrogenError) as e:
            H.inverse_fit(w, target.data_ptr(), ks.data_ptr(), b0.data_ptr(), s)
        assert e.value.code == -1
    with pytest.raises(H.HydrogenError):  # fitting Ks needs a Ks buffer
        H.inverse_fit(w, target.data_ptr(), None, b0.data_ptr(), H.fit_settings(nsteps=4, iters=1))


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


def inverse_workload(nsteps):
    """The 1024^2 inverse-erosion workload: target = nsteps of config-1
    physics with Ks = 0.05 exp(0.5 n(x)); gradients at uniform Ks 0.05."""
    torch = torch_dev()
    n = 1024
    w = H.World(n)
    w.init_heightmap(H.noise(seed=0))
    H.configure(w, "config1")
    w.init_ks_field(H.noise(seed=7, octaves=3, frequency=1.0 / 256), 0.05, 0.5)
    w.step(nsteps, H.MODE_FUSED)
    target = w.download("rock").astype(np.float64)
    w.init_heightmap(H.noise(seed=0))
    b0 = w.download("rock").astype(np.float64)
    ks = np.full((n, n), 0.05, np.float32)
    w.upload("ks", ks)
    return w, b0, ks, target


def test_gpu_adjoint_matches_fp64_reference_at_workload_size():
    """The inverse workload's grid and physics over 32 steps (checkpoints
    every 8).  The float and FP64 forwards have barely parted: the relative
    L2 error stays within 2e-3 (measured: 3.6e-4 for Ks, 1.1e-3 for the
    initial rock, against 1.5e-4 at the small sizes above)."""
    w, b0, ks, target = inverse_workload(32)
    loss, dks, db0, _ = gpu_gradients(w, target, 32, 8)
    rloss, rdks, rdb0 = O.adjoint_ref(O.settings_config1(), 0.01, 1, b0, ks, target, 32)
    assert abs(loss - rloss) <= 1e-4 * rloss
    for name, g, r in (("dKs", dks, rdks), ("drock0", db0, rdb0)):
        rel = np.abs(g - r) / np.maximum(np.abs(r), 1e-2 * np.abs(r).max())
        print(f"1024^2 x 32 {name}: rel L2 error {rel_l2(g, r):.2e}, within 1e-3 {np.mean(rel <= 1e-3):.4f}")
        assert rel_l2(g, r) <= 2e-3


def test_gpu_adjoint_full_inverse_workload():
    """All 256 steps.  The float model the GPU differentiates and the FP64
    model part at a few hundred cells (final rock apart by more than 1e-4,
    where a dissolve/deposit switch, a clamp or a maximum went the other
    way), and there the two exact gradients differ.  Bar: at least 90 % of
    the cells within 1e-3 relative (floor 1e-2 of the largest gradient) and
    most of the squared difference within 8 cells of where the forwards
    parted."""
    w, b0, ks, target = inverse_workload(256)
    loss, dks, db0, _ = gpu_gradients(w, target, 256, 32)
    final = w.download("rock").astype(np.float64)
    _, rdks, rdb0 = O.adjoint_ref(O.settings_config1(), 0.01, 1, b0, ks, target, 256)
    f64 = O.forward_ref(O.settings_config1(), 0.01, 1, b0, ks, 256)
    parted = np.abs(final - f64) > 1e-4
    near = parted.copy()
    for _ in range(8):
        t = near.copy()
        t[1:] |= near[:-1]
        t[:-1] |= near[1:]
        t[:, 1:] |= near[:, :-1]
        t[:, :-1] |= near[:, 1:]
        near = t
    for name, g, r in (("dKs", dks, rdks), ("drock0", db0, rdb0)):
        rel = np.abs(g - r) / np.maximum(np.abs(r), 1e-2 * np.abs(r).max())
        d2 = (g - r) ** 2
        share = d2[near].sum() / d2.sum()
        print(f"1024^2 x 256 {name}: within 1e-3 {np.mean(rel <= 1e-3):.4f}, median rel {np.median(rel):.1e}, "
              f"squared difference within 8 cells of the {int(parted.sum())} parted cells {share:.3f} "
              f"({near.mean():.3f} of the area)")
        assert np.mean(rel <= 1e-3) >= 0.9
        assert share >= 0.75
