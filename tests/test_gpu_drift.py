"""NVE energy drift of the FP64 GPU path against the oracle from the same start.

The reference's scheme (5-value Gear predictor-corrector with the coefficients 0.1583 / 0.757 of
src/move.f90:224-225, an unshifted molecular cutoff) drifts in total energy on its own; this test
shows that the drift of the library's resident steps is the oracle's drift, not an artefact of the
GPU arithmetic.  Both run 6,000 steps of 1 fs from the same equilibrated 256-water start (the
oracle in its parity build, the same arithmetic as the GPU's FP64 form to ~1e-15); htot is sampled
every 250 steps.  The trajectories stay close for the first picoseconds and then decorrelate as
any chaotic trajectory does, so the early samples are compared point by point and the whole run
through its least-squares drift rate.
"""
import numpy as np
import pytest

from md_sim_gb300 import abi, configs

pytestmark = pytest.mark.gpu

STEPS, EVERY = 6000, 250


def _series(ctx):
    return np.array([ctx.run(EVERY)["htot"] for _ in range(STEPS // EVERY)])


def test_nve_drift_matches_oracle(gpulib, oracle):
    s, prm = configs.bulk_water()
    g = abi.Context(gpulib, s, prm)
    configs.equilibrate(g, s, steps=300, every=10)
    s0 = s.copy()
    g.set_state(s0.copy())
    r = abi.Context(oracle, s0.copy(), prm)
    r.set_state(s0.copy())
    hg, hr = _series(g), _series(r)
    t_ns = np.arange(1, len(hg) + 1) * EVERY * s.dt * 1e-6
    slope_g = np.polyfit(t_ns, hg, 1)[0] / s.nrig
    slope_r = np.polyfit(t_ns, hr, 1)[0] / s.nrig
    rel = (hg[-1] - hg[0]) / abs(hg[0])
    print(f"drift per molecule: GPU {slope_g:.2f}, oracle {slope_r:.2f} kJ/mol/ns; htot change over "
          f"{STEPS} steps {rel:+.3e} (GPU)")
    print("htot GPU   ", " ".join(f"{x:.6f}" for x in hg))
    print("htot oracle", " ".join(f"{x:.6f}" for x in hr))
    # the first picosecond: the same trajectory, so the same drift
    np.testing.assert_allclose(hg[:4], hr[:4], rtol=1e-8)
    # the whole run: after the trajectories decorrelate, a drift rate of the same sign and size
    # (a 6 ps slope of a 256-water system varies by tens of percent between trajectories)
    assert slope_g > 0 and slope_r > 0, (slope_g, slope_r)
    assert 0.5 < slope_g / slope_r < 2.0, (slope_g, slope_r)
