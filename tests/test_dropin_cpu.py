"""The drop-in MD step with the host integrator of the library (mdg_host_predict /
mdg_host_correct) around the oracle's force_get and move_shake, against the oracle's own
restatement of the production loop (src/main.f90:58-68 with move_predict and move_correct,
src/move.f90:48-383).  The host integrator touches no GPU, so this runs on the CPU; both follow
the reference's arithmetic order without contraction, so the states agree bit for bit.
"""
import numpy as np
import pytest

from md_sim_gb300 import abi, configs

CASES = {
    "bulk256_nve": (lambda: configs.bulk_water(), 12),
    "slab512_nvt": (lambda: configs.slab_water(nwat=512, cells=6, nvt=True), 8),
    # flexible point ions between the waters (atoms nriga+1..nliqa)
    "electrolyte": (lambda: configs.slab_electrolyte(), 8),
    # surface atoms: Verlet + SHAKE through the context after the corrector
    "shake256": (lambda: configs.shake_water(nwat=256, cells=6), 6),
}


def _state_arrays(s):
    out = [s.x0, s.y0, s.z0, s.xd, s.xold, s.yold, s.zold, s.rsx, s.rsy, s.rsz, np.asarray(s.s), np.asarray(s.rs)]
    if s.nrig:
        out += [s.c, s.q, s.w]
    return out


@pytest.mark.parametrize("threads", ["1", "2", "3", "8"])
@pytest.mark.parametrize("name", list(CASES))
def test_host_integrator_matches_oracle_loop(name, threads, oracle, gpulib, monkeypatch):
    """The host threads split the molecules into ranges, and the seven kinetic sums run as
    separate chains (several per thread below seven threads, one per thread from seven on); the
    result does not depend on their number (MDG_HOST_THREADS is read when the integrator is
    created)."""
    monkeypatch.setenv("MDG_HOST_THREADS", threads)
    make, steps = CASES[name]
    s, prm = make()
    sa, sb = s.copy(), s.copy()
    ra = abi.Context(oracle, sa, prm)
    ra.set_state(sa)
    rep_a = ra.run(steps)
    ra.get_state(sa)
    rb = abi.Context(oracle, sb, prm)
    hg = abi.HostGear(gpulib, sb)
    hg.step(rb, steps)
    hg.write_back(sb)
    rep_b = hg.report()
    for a, b in zip(_state_arrays(sa), _state_arrays(sb)):
        np.testing.assert_array_equal(a, b)
    # tempnow is 0/0 in both for a system of surface atoms only, as in the reference
    for key in ("kp", "kw", "ke", "htot", "tempnow", "uconf"):
        np.testing.assert_equal(rep_a[key], rep_b[key], err_msg=key)


def test_host_gear_rejects_bad_description(gpulib):
    import ctypes as C

    h = C.c_void_p()
    assert gpulib.host_gear_create(None, None, C.byref(h)) == -1  # MDG_E_ARG
