"""Resident mode (move_predict -> force_get -> move_correct -> move_shake on the device, replayed
through CUDA graphs) against the oracle's restatement of the same loop (src/main.f90:58-68)."""
import numpy as np
import pytest

from md_sim_gb300 import abi, configs

pytestmark = pytest.mark.gpu


def _pair(fn, oracle, gpulib):
    s, prm = fn()
    sg, sr = s.copy(), s.copy()
    g, r = abi.Context(gpulib, sg, prm), abi.Context(oracle, sr, prm)
    g.set_state(sg)
    r.set_state(sr)
    return sg, sr, g, r


def _compare(sg, sr, tol=1e-9):
    L = sg.lx
    for a, b in ((sg.x0, sr.x0), (sg.y0, sr.y0), (sg.z0, sr.z0)):
        assert np.abs(a - b).max() < tol * L
    if sg.nrig:
        for k in range(5):
            sc = np.abs(sr.c[k]).max() + 1e-300
            assert np.abs(sg.c[k] - sr.c[k]).max() <= tol * max(sc, L if k == 0 else sc)
            sw = np.abs(sr.w[k]).max() + 1e-300
            assert np.abs(sg.w[k] - sr.w[k]).max() <= tol * sw * 10
            sq = np.abs(sr.q[k]).max() + 1e-300
            assert np.abs(sg.q[k] - sr.q[k]).max() <= tol * sq * 10
    assert np.abs(sg.xold - sr.xold).max() < tol * L


@pytest.mark.parametrize("name,fn,steps", [
    ("bulk256_nve", lambda: configs.bulk_water(), 20),
    ("slab512_nvt", lambda: configs.slab_water(nwat=512, cells=6, nvt=True), 12),
    ("slab512_nve", lambda: configs.slab_water(nwat=512, cells=6), 12),
    ("shake256", lambda: configs.shake_water(nwat=256, cells=6), 10),
])
def test_run_matches_oracle(name, fn, steps, oracle, gpulib):
    sg, sr, g, r = _pair(fn, oracle, gpulib)
    rg = g.run(steps)
    rr = r.run(steps)
    g.get_state(sg)
    r.get_state(sr)
    _compare(sg, sr)
    for key in ("kp", "kw", "ke", "uconf"):
        assert abs(rg[key] - rr[key]) <= 1e-9 * (abs(rr[key]) + 1.0), (key, rg[key], rr[key])
    if sg.temper != -1.0:
        assert abs(rg["htot"] - rr["htot"]) <= 1e-8 * (abs(rr["htot"]) + 1.0)
    assert rg["steps"] == steps


def test_run_in_chunks_equals_one_call(gpulib):
    """Graph replay and chunking do not change the trajectory."""
    s, prm = configs.bulk_water()
    a, b = s.copy(), s.copy()
    ga, gb = abi.Context(gpulib, a, prm), abi.Context(gpulib, b, prm)
    ga.set_state(a)
    gb.set_state(b)
    ga.run(30)
    for _ in range(3):
        gb.run(10)
    ga.get_state(a)
    gb.get_state(b)
    assert np.abs(a.x0 - b.x0).max() < 1e-10


def test_nve_energy_drift(gpulib):
    """Bulk water NVE after a short rescaled equilibration: htot drift stays small."""
    s, prm = configs.bulk_water()
    g = abi.Context(gpulib, s, prm)
    configs.equilibrate(g, s, steps=300, every=10)
    h0 = g.run(50)["htot"]
    h1 = g.run(400)["htot"]
    assert abs(h1 - h0) < 0.01 * abs(h0)


def _compare_mixed(sg, sr, rg, rr, pos_tol=1e-6, e_tol=2e-5):
    """Mixed precision against the FP64 oracle: the same trajectory to within what the FP32 force
    arithmetic moves it in a few steps (positions relative to the box, energies relative)."""
    L = sg.lx
    for a, b in ((sg.x0, sr.x0), (sg.y0, sr.y0), (sg.z0, sr.z0)):
        assert np.abs(a - b).max() < pos_tol * L
    for key in ("kp", "kw", "ke", "uconf"):
        assert abs(rg[key] - rr[key]) <= e_tol * (abs(rr[key]) + 1.0), (key, rg[key], rr[key])


@pytest.mark.parametrize("name,fn,steps", [
    # the predictor packs the force records (walls: wall-packing blocks), molecules on lane pairs,
    # the corrector fused with the final merge
    ("slab512_nve", lambda: configs.slab_water(nwat=512, cells=6), 10),
    ("slab512_nvt", lambda: configs.slab_water(nwat=512, cells=6, nvt=True), 10),
    # point ions among the waters: flexible units beside the molecule pairs
    ("electrolyte", lambda: configs.slab_electrolyte(), 10),
    # no walls: packing blocks only for molecules
    ("bulk256", lambda: configs.bulk_water(), 10),
    # SHAKE surface molecules: the separate packing kernel, merge fused with the corrector
    ("shake256", lambda: configs.shake_water(nwat=256, cells=6), 8),
])
def test_mixed_run_matches_oracle(name, fn, steps, oracle, gpulib):
    s, prm = fn()
    sg, sr = s.copy(), s.copy()
    pg = abi.RunParams(**{f: getattr(prm, f) for f in prm.__dataclass_fields__})
    pg.precision = abi.MDG_MIXED
    g, r = abi.Context(gpulib, sg, pg), abi.Context(oracle, sr, prm)
    g.set_state(sg)
    r.set_state(sr)
    rg, rr = g.run(steps), r.run(steps)
    g.get_state(sg)
    r.get_state(sr)
    _compare_mixed(sg, sr, rg, rr)
    assert rg["steps"] == steps


@pytest.mark.parametrize("nwat,cells", [
    (3000, 12),   # 20 molecules per warp: one lane each, one warp per block
    (5200, 16),   # 32 molecules per warp, blocks of four warps
])
def test_integrator_layouts_match_oracle(nwat, cells, oracle, gpulib):
    """The integrator's other lane layouts (larger systems) against the oracle, FP64."""
    sg, sr, g, r = _pair(lambda: configs.slab_water(nwat=nwat, cells=cells), oracle, gpulib)
    rg = g.run(3)
    rr = r.run(3)
    g.get_state(sg)
    r.get_state(sr)
    _compare(sg, sr)
    for key in ("kp", "kw", "ke", "uconf"):
        assert abs(rg[key] - rr[key]) <= 1e-9 * (abs(rr[key]) + 1.0), (key, rg[key], rr[key])
