"""The FP64 reference adjoint (oracle/hg_adjoint_ref.cpp) against central
finite differences of the oracle's own FP64 forward restatement of the GLSL
passes (an independent implementation), eps = 1e-3, on 64 random cells, for
the gradients with respect to the initial rock heights and the per-cell
rock solubility.  CPU only."""
import numpy as np

import oracle as O

N, STEPS, EPS = 32, 16, 1e-3


def setup():
    rng = np.random.default_rng(4)
    b0 = O.fbm(N, frequency=1.0 / 16).astype(np.float64)
    ks = (0.05 * np.exp(0.5 * O.fbm_raw(N, N, 7, 3, 1.0 / 16, 2.0, 0.5) / 1.75)).astype(np.float32)
    target = b0 - 0.02 * rng.random((N, N))
    return rng, b0, ks, target


def oracle_loss(b0, ks, target):
    w = O.OracleWorld(N, 64)
    w.set("rock", b0)
    w.set_ks(ks)
    s, o = O.workload("config1")
    w.step(s, o, STEPS)
    return np.mean((w.get("rock") - target) ** 2)


def test_reference_forward_is_the_oracle_forward():
    _, b0, ks, _ = setup()
    w = O.OracleWorld(N, 64)
    w.set("rock", b0)
    w.set_ks(ks)
    s, o = O.workload("config1")
    w.step(s, o, STEPS)
    ref = O.forward_ref(O.settings_config1(), 0.01, 1, b0, ks, STEPS)
    assert np.array_equal(ref, w.get("rock"))


def test_reference_adjoint_vs_finite_differences():
    rng, b0, ks, target = setup()
    loss, dks, db0 = O.adjoint_ref(O.settings_config1(), 0.01, 1, b0, ks, target, STEPS)
    assert abs(loss - oracle_loss(b0, ks, target)) <= 1e-12 * loss
    cells = rng.choice(N * N, size=64, replace=False)
    scale_b = np.abs(db0).max()
    scale_k = np.abs(dks).max()
    bad = []
    for c in cells:
        y, x = divmod(int(c), N)
        bp, bm = b0.copy(), b0.copy()
        bp[y, x] += EPS
        bm[y, x] -= EPS
        fd = (oracle_loss(bp, ks, target) - oracle_loss(bm, ks, target)) / (2 * EPS)
        if abs(fd - db0[y, x]) > 1e-3 * max(abs(fd), 1e-2 * scale_b):
            bad.append(("rock", y, x, db0[y, x], fd))
        kp, km = ks.copy(), ks.copy()
        kp[y, x] += np.float32(EPS)
        km[y, x] -= np.float32(EPS)
        h = float(kp[y, x]) - float(km[y, x])
        fd = (oracle_loss(b0, kp, target) - oracle_loss(b0, km, target)) / h
        if abs(fd - dks[y, x]) > 1e-3 * max(abs(fd), 1e-2 * scale_k):
            bad.append(("ks", y, x, dks[y, x], fd))
    # a central difference can straddle a dissolve/deposit or clamp switch;
    # allow at most 2 of the 128 comparisons to do so
    assert len(bad) <= 2, bad[:5]
