"""The drop-in MD step as a Fortran host makes it (src/main.f90:58-68): the integrator on the
host (mdg_host_predict / mdg_host_correct), the force evaluation and SHAKE on the GPU through
mdg_force_get / mdg_shake with host arrays, against the oracle's production loop and against the
library's resident steps (mdg_run) from the same start."""
import numpy as np
import pytest

from md_sim_gb300 import abi, configs

pytestmark = pytest.mark.gpu

CASES = {
    "bulk256_nve": (lambda: configs.bulk_water(), 15),
    "slab512_nvt": (lambda: configs.slab_water(nwat=512, cells=6, nvt=True), 10),
    "electrolyte": (lambda: configs.slab_electrolyte(), 10),
    "shake256": (lambda: configs.shake_water(nwat=256, cells=6), 8),
}


def _close(a, b, tol):
    L = a.lx
    for x, y in ((a.x0, b.x0), (a.y0, b.y0), (a.z0, b.z0)):
        assert np.abs(x - y).max() < tol * L
    if a.nrig:
        for k in range(5):
            assert np.abs(a.c[k] - b.c[k]).max() <= tol * max(np.abs(b.c[k]).max(), 1e-300) + tol * (L if k == 0 else 0)
            assert np.abs(a.q[k] - b.q[k]).max() <= 10 * tol * max(np.abs(b.q[k]).max(), 1e-300)
            assert np.abs(a.w[k] - b.w[k]).max() <= 10 * tol * max(np.abs(b.w[k]).max(), 1e-300)


@pytest.mark.parametrize("name", list(CASES))
def test_dropin_loop_matches_oracle_and_resident(name, oracle, gpulib):
    make, steps = CASES[name]
    s, prm = make()
    sd, so, sr = s.copy(), s.copy(), s.copy()
    # drop-in: host integrator + GPU force calls
    g = abi.Context(gpulib, sd, prm)
    hg = abi.HostGear(gpulib, sd)
    hg.step(g, steps)
    hg.write_back(sd)
    rd = hg.report()
    # the oracle's loop
    o = abi.Context(oracle, so, prm)
    o.set_state(so)
    ro = o.run(steps)
    o.get_state(so)
    # the library's resident steps
    r = abi.Context(gpulib, sr, prm)
    r.set_state(sr)
    rr = r.run(steps)
    r.get_state(sr)
    _close(sd, so, 1e-9)
    _close(sd, sr, 1e-9)
    for key in ("kp", "kw", "uconf"):
        assert abs(rd[key] - ro[key]) <= 1e-9 * (abs(ro[key]) + 1.0), (key, rd[key], ro[key])
        assert abs(rd[key] - rr[key]) <= 1e-9 * (abs(rr[key]) + 1.0), (key, rd[key], rr[key])
