"""Fit the coefficients of the single-precision arctangent used by the talus test.

The thermal pass compares atan(slope) with the talus angle and uses the angle in
its sharpness factor.  GLSL leaves atan's precision to the driver, so the
library defines its own float atan and the float oracle evaluates the same
operations, which keeps the GPU and the float CPU restatement bit-identical.

Method (own design).  Three branches keep the polynomial's argument within
|u| <= tan(pi/8), where the correction term u*s*P(s) is below 6% of u:
    x <= tan(pi/8)              atan(x) = poly(x)
    tan(pi/8) < x <= tan(3pi/8) atan(x) = pi/4 + poly((x - 1) / (x + 1))
    x > tan(3pi/8)              atan(x) = pi/2 - poly(1 / x)
with poly(u) = u + u*(s*P(s)), s = u*u and P a degree-5 polynomial fitted by
Lawson's iteratively reweighted least squares (a standard route to a
near-minimax fit) on Chebyshev nodes, weighted for relative error in atan.
Evaluation is Horner with separate multiply and add (no fused multiply-add).
The small correction keeps the float evaluation monotone non-decreasing on
x >= 0; the oracle's exhaustive check over every positive float confirms it.

Run:  python fit_atan.py   (prints the float32 coefficients and the error)
"""
import numpy as np

DEG = 5
T8 = np.tan(np.pi / 8)


def fit(deg=DEG, npts=4000, iters=60):
    smax = T8 * T8
    k = np.arange(npts)
    s = smax * 0.5 * (1 - np.cos(np.pi * (k + 0.5) / npts))
    s = s[s > 1e-9]
    t = np.sqrt(s)
    target = (np.arctan(t) - t) / (t * s)
    w0 = s / (np.arctan(t) / t)
    A = np.vander(s, deg + 1, increasing=True)
    lw = np.ones_like(s)
    for _ in range(iters):
        W = np.sqrt(lw) * w0
        c, *_ = np.linalg.lstsq(A * W[:, None], target * W, rcond=None)
        err = np.abs((A @ c - target) * w0)
        lw = lw * err
        lw /= lw.sum()
    return c


def f32(x):
    return np.asarray(x, dtype=np.float32)


def poly(u, c32):
    s = f32(u * u)
    p = np.full_like(s, c32[-1])
    for ci in c32[-2::-1]:
        p = f32(p * s)
        p = f32(p + ci)
    return f32(u + f32(u * f32(s * p)))


def atan_f32(x, c32):
    x = f32(x)
    ax = np.abs(x)
    lo, hi = np.float32(0.414213562), np.float32(2.41421356)
    with np.errstate(divide="ignore", invalid="ignore"):
        r1 = poly(ax, c32)
        u2 = f32(f32(ax - np.float32(1)) / f32(ax + np.float32(1)))
        r2 = f32(np.float32(0.785398163) + poly(u2, c32))
        r3 = f32(np.float32(1.57079637) - poly(f32(np.float32(1) / ax), c32))
    r = np.where(ax <= lo, r1, np.where(ax <= hi, r2, r3))
    return np.copysign(r, x).astype(np.float32)


def ulp_err(x, c32):
    got = atan_f32(x, c32).astype(np.float64)
    ref = np.arctan(x.astype(np.float64))
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    return np.abs(got - ref) / ulp


if __name__ == "__main__":
    c = fit()
    c32 = c.astype(np.float32)
    print("coefficients (float32, s^0 .. s^%d):" % DEG)
    for i, ci in enumerate(c32):
        print("  c%d = %.9ef" % (i, ci))
    xs = np.concatenate([
        np.linspace(0, 3, 6_000_001, dtype=np.float32),
        np.float32(1) / np.linspace(1e-6, 1, 2_000_001, dtype=np.float32),
        np.logspace(-30, 30, 200_001).astype(np.float32),
    ])
    e = ulp_err(xs, c32)
    print("max error %.3f ulp, mean %.3f ulp" % (e.max(), e.mean()))
    ys = atan_f32(np.sort(xs[xs >= 0]), c32)
    print("non-monotone steps in sample:", int(np.sum(np.diff(ys) < 0)))
