"""Mass budget of the reference scheme, on the oracle (CPU).

The reference's flux pass is not conservative: a cell adds its neighbours'
stored outflow of the previous step (glsl/hydro_flux.glsl:94-98) but removes
its own outflow of this step (:100-127), so the water in flight is lost
while the flux grows.  The semi-Lagrangian sediment gather
(glsl/sediment_transport.glsl:70-72) is not conservative either.  A
conservation bar therefore cannot hold for any faithful implementation; these
tests pin what does hold: how much water the reference scheme itself loses,
and how far the float scheme's mass totals sit from the FP64 scheme's.
"""
import numpy as np

import oracle as O


def test_flux_pass_loses_water_in_fp64_and_float():
    """No rain, no evaporation: 50 flux passes over a tilted lake lose about
    13 % of the water, in FP64 and in float alike (it is the scheme)."""
    s = O.settings_config1()
    s.Ke = 0.0
    o = O.options(0)
    lost = {}
    for prec in (64, 32):
        w = O.OracleWorld(256, prec)
        w.set("rock", O.fbm(256))
        w.set("water", np.full((256, 256), 0.5))
        w0 = w.totals()[2]
        for _ in range(50):
            w.run_pass("flux", s, o)
        lost[prec] = (w0 - w.totals()[2]) / w0
    assert 0.12 < lost[64] < 0.14, lost
    assert abs(lost[32] - lost[64]) < 1e-6, lost


def test_float_mass_totals_against_fp64():
    """The uniform-rain workload (256², rain 0.01 per cell and step, no
    thermal): after 100 steps the float scheme's water total is within 1e-6
    of the FP64 scheme's and its sediment total within 5e-6 (measured 2.9e-7
    and 1.2e-6); the rock total within 1e-8."""
    s, o = O.workload("config1")
    a, b = O.OracleWorld(256, 32), O.OracleWorld(256, 64)
    r = O.fbm(256)
    a.set("rock", r)
    b.set("rock", r)
    a.step(s, o, 100)
    b.step(s, o, 100)
    ta, tb = a.totals(), b.totals()
    rel = [abs(x - y) / abs(y) for x, y in zip(ta, tb) if y]
    rock, water, sediment = rel
    assert rock <= 1e-8, rel
    assert water <= 1e-6, rel
    assert sediment <= 5e-6, rel
