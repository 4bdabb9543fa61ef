"""Where the float scheme's deviation from FP64 comes from (config-2 physics,
256², 100 steps; oracle only, no GPU).

The kernels equal the float restatement bit for bit, so the float
restatement's distance from the FP64 one is the product's.  On this workload
it exceeds the workload's bar (1e-4 of the height range after 100 steps) at
a few dozen cells.  Candidate causes, each switched on its own in both
precisions:

* the arctangent of the talus test: the float restatement uses the kernels'
  polynomial (2.5 ulp).  Replacing it by the C library's atanf leaves the
  largest deviation where it is, so the arctangent is not the cause;
* the velocity of thin water films: glsl/hydro_flux.glsl:144-158 divides the
  old-flux difference by the depth d1 + d2, Bernoulli rain leaves cells
  whose FP64 depth decays to 1e-30 and below (float: exactly 0 or
  ulp-sized), and the sediment back-trace (glsl/sediment_transport.glsl:70)
  follows that velocity across the grid.  Zeroing the velocity below a depth
  of 1e-4 (a change to the scheme, test only) removes about two thirds of
  the maximum;
* the talus test (glsl/thermal_erosion.glsl:78-88) is a step function of the
  slope, and slippage drives slopes onto the talus angle, where a last-bit
  difference flips a direction's mark.  With thermal erosion off as well
  only a couple of cells remain above the bar.

So the miss is the scheme's conditioning (a division by a vanishing depth
and a discontinuous threshold), not the library's arithmetic: every float
implementation of these passes meets the same cells.
"""
import numpy as np

import oracle as O

N, STEPS = 256, 100


def deviation(thermal=True, guard=0.0, libm=False):
    rock = O.fbm(N)
    s, o = O.workload("config2")
    if not thermal:
        s.Kspeed[0] = 0.0
    with O.film_guard(guard):
        w64 = O.OracleWorld(N, 64)
        w64.set("rock", rock)
        w64.step(s, o, STEPS)
        w32 = O.OracleWorld(N, 32)
        w32.set("rock", rock)
        if libm:
            with O.libm_atan():
                w32.step(s, o, STEPS)
        else:
            w32.step(s, o, STEPS)
    r = w64.get("rock")
    return np.abs(w32.get("rock") - r) / (r.max() - r.min())


def summary(e):
    return float(e.max()), int(np.sum(e > 1e-4))


def test_fp64_deviation_is_the_schemes_conditioning_not_the_arctangent():
    base_max, base_n = summary(deviation())
    libm_max, libm_n = summary(deviation(libm=True))
    film_max, film_n = summary(deviation(guard=1e-4))
    calm_max, calm_n = summary(deviation(thermal=False, guard=1e-4))
    # the workload's 1e-4 bar is missed by the faithful float scheme ...
    assert base_max > 1e-4 and base_n >= 20
    # ... whatever the arctangent
    assert abs(libm_max - base_max) <= 0.05 * base_max
    assert abs(libm_n - base_n) <= 0.25 * base_n
    # thin-film velocities carry most of the maximum
    assert film_max <= 0.5 * base_max and film_n <= 0.5 * base_n
    # without them and the talus threshold, only a few cells are left
    assert calm_n <= 5 and calm_max <= 0.15 * base_max
    print(f"config2 256^2 @100 vs FP64 (max, cells > 1e-4): poly_atanf {base_max:.3e} {base_n}, "
          f"libm atanf {libm_max:.3e} {libm_n}, film guard 1e-4 {film_max:.3e} {film_n}, "
          f"film guard + thermal off {calm_max:.3e} {calm_n}")
