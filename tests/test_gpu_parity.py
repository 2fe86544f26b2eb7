"""GPU parity: the CUDA library against the oracle on the same seeded inputs, through the C ABI.

Bars: neighbour lists bit-exact (same (i, j) sets); FP64 forces within 1e-12 relative
(||dF|| / ||F||) and energies within 1e-12 of the energy scale; SHAKE positions within 1e-12
relative to the box and the same sweep count.
"""
import numpy as np
import pytest

from md_sim_gb300 import abi, configs
from tests.golden.fixture import y_n_case

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-12
ENERGY_RTOL = 1e-12


def _cases():
    return {
        "bulk256": lambda: configs.bulk_water(),
        "bulk_sc512": lambda: configs.bulk_water(8, "sc", box=8 * 3.103, seeds=(5, 6, 7), rcut=10.0,
                                                 alpha=0.32, kmax=8),
        "slab512": lambda: configs.slab_water(nwat=512, cells=6),
        "slab2048": lambda: configs.slab_water(),
        "shake256": lambda: configs.shake_water(nwat=256, cells=6),
        "y_n": lambda: y_n_case()[:2],
        # ions between the walls (site types 3 and 4 among waters)
        "electrolyte": lambda: configs.slab_electrolyte(),
        # point ions only, with a cutoff below the closest approach: empty real-space sum
        "ions_empty_real": lambda: configs.ion_lattice(),
    }


CASES = _cases()


def _pairs(ctx):
    (li, lj), (wi, wj) = ctx.get_lists()
    hh = set(zip(li.tolist(), lj.tolist()))
    hw = set(zip(wi.tolist(), wj.tolist()))
    return hh, hw


def _both(name, oracle, gpulib, mutate=None):
    s, prm = CASES[name]()
    if mutate:
        mutate(s, prm)
    sg, sr = s.copy(), s.copy()
    g = abi.Context(gpulib, sg, prm)
    r = abi.Context(oracle, sr, prm)
    return sg, sr, g, r


def _check_forces(og, orf):
    f_err = np.linalg.norm(og["f"] - orf["f"]) / np.linalg.norm(orf["f"])
    assert f_err < FORCE_RTOL, f"site force rel err {f_err:.3e}"
    for key in ("ft", "fc", "torque"):
        a, b = og[key], orf[key]
        if b.size:
            e = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)
            assert e < FORCE_RTOL * 10, f"{key} rel err {e:.3e}"
    scale = np.abs(orf["elj"]).sum() + np.abs(orf["eqq"]).sum() + abs(orf["uewa"]) + 1.0
    for key in ("elj", "eqq"):
        d = np.abs(og[key] - orf[key]).max()
        assert d <= ENERGY_RTOL * scale, f"{key} diff {d:.3e} (scale {scale:.3e})"
    # uself includes the rigid-molecule and constraint exclusions with the transposed constraint
    # read of src/forcem.f90:812-813 (Q7)
    for key in ("uewa", "urf", "ulr", "uself", "uconf", "uavex", "ewqLL", "ewqWW", "ewqWL"):
        d = abs(og[key] - orf[key])
        assert d <= ENERGY_RTOL * scale, f"{key}: {og[key]!r} vs {orf[key]!r}"
    fs = np.abs(orf["fws"]).max() + 1.0
    assert np.abs(og["fws"] - orf["fws"]).max() <= 1e-11 * fs * 10, (og["fws"], orf["fws"])
    assert abs(og["press"] - orf["press"]) <= 1e-10 * (abs(orf["press"]) + 1.0)


@pytest.mark.parametrize("name", list(CASES))
def test_neighbour_list_bit_exact(name, oracle, gpulib):
    sg, sr, g, r = _both(name, oracle, gpulib)
    hg, wg = _pairs(g)
    hr, wr = _pairs(r)
    assert len(hg) == len(hr) and hg == hr
    assert len(wg) == len(wr) and wg == wr


@pytest.mark.parametrize("name", list(CASES))
def test_force_get_fp64(name, oracle, gpulib):
    sg, sr, g, r = _both(name, oracle, gpulib)
    og, orf = g.force_get(sg), r.force_get(sr)
    _check_forces(og, orf)
    # force_sum leaves rsx(1:3) holding the last rigid molecule's site offsets
    np.testing.assert_allclose(sg.rsx[:3], sr.rsx[:3], rtol=0, atol=1e-13)


def test_stale_rsx_quirk(oracle, gpulib):
    """Second evaluation: rsx(1) of molecule 1 is stale (src/forcem.f90:1006 + src/move.f90:157)."""
    sg, sr, g, r = _both("bulk256", oracle, gpulib)
    g.force_get(sg)
    r.force_get(sr)
    assert abs(sg.rsx[0]) > 1e-3  # the quirk is live
    _check_forces(g.force_get(sg), r.force_get(sr))


def test_rebuild_trigger_sequence(oracle, gpulib):
    """Moving the molecules step by step: the list is rebuilt when 4*max|dr|^2 > skin^2 and the
    lists and forces stay identical to the oracle's."""
    sg, sr, g, r = _both("slab512", oracle, gpulib)
    rng = np.random.default_rng(3)
    for step in range(6):
        dx = rng.normal(0.0, 0.12, size=(3, sg.nrig))
        for s in (sg, sr):
            s.c[0] += dx
            s.quatsite()
            s.rsx_after_predict()
        og, orf = g.force_get(sg), r.force_get(sr)
        _check_forces(og, orf)
        assert _pairs(g) == _pairs(r), f"lists differ at step {step}"


@pytest.mark.parametrize("pbcz", [0, 1])
def test_list_z_image_switch(pbcz, oracle, gpulib):
    def mut(s, prm):
        prm.pbc_z_list = pbcz

    sg, sr, g, r = _both("bulk_sc512", oracle, gpulib, mut)
    assert _pairs(g) == _pairs(r)


def test_nnlist_make_explicit(oracle, gpulib):
    sg, sr, g, r = _both("shake256", oracle, gpulib)
    for s in (sg, sr):
        s.x0[: s.nmove] += 0.3
    assert g.nnlist_make(sg) == r.nnlist_make(sr)
    assert _pairs(g) == _pairs(r)


@pytest.mark.parametrize("clean", [False, True])
def test_shake_parity(clean, oracle, gpulib):
    def mut(s, prm):
        prm.quirks = 1 if clean else 0
        prm.shake_maxit = 100

    sg, sr, g, r = _both("shake256", oracle, gpulib, mut)
    og, orf = g.force_get(sg), r.force_get(sr)
    assert np.abs(og["ft"] - orf["ft"]).max() <= 1e-11 * np.abs(orf["ft"]).max()
    # the same forces into both SHAKEs: the sweep count of the reference stop rule depends on the
    # last bits of one molecule's iteration, so force rounding is kept out of this comparison
    a = g.shake(sg, orf["ft"])
    b = r.shake(sr, orf["ft"])
    assert a["sweeps"] == b["sweeps"]
    for u, w in ((sg.x0, sr.x0), (sg.y0, sr.y0), (sg.z0, sr.z0), (sg.xold, sr.xold)):
        assert np.abs(u - w).max() < 1e-12 * sg.lx
    np.testing.assert_allclose(a["kps"], b["kps"], rtol=1e-12, atol=1e-9)
    assert abs(a["tkps"] - b["tkps"]) <= 1e-11 * abs(b["tkps"])


def test_shake_reference_stop_rule(oracle, gpulib):
    """Reference mode: sweeps are decided by the last molecule (src/move.f90:458)."""
    def mut(s, prm):
        prm.quirks = 0
        prm.shake_maxit = 100

    sg, sr, g, r = _both("shake256", oracle, gpulib, mut)
    og, orf = g.force_get(sg), r.force_get(sr)
    a, b = g.shake(sg, orf["ft"]), r.shake(sr, orf["ft"])
    assert a["sweeps"] == b["sweeps"]
    assert np.abs(sg.x0 - sr.x0).max() < 1e-12 * sg.lx


def test_shake_errors(gpulib):
    """A stretched bond trips the rptol test; a sweep limit of 1 trips the iteration limit."""
    s, prm = configs.shake_water(nwat=64, cells=4, seed=5)
    prm.shake_maxit = 1
    g = abi.Context(gpulib, s, prm)
    og = g.force_get(s)
    with pytest.raises(abi.MdgError) as ei:
        g.shake(s.copy(), og["ft"])
    assert ei.value.code == -4
    s2, prm2 = configs.shake_water(nwat=64, cells=4, seed=5)
    prm2.shake_maxit = 100
    g2 = abi.Context(gpulib, s2, prm2)
    og2 = g2.force_get(s2)
    # previous position of one H chosen so that the Verlet step reflects it through its O:
    # the new O-H bond then points against the old one (rpab < 0)
    s2.xold[1] = s2.x0[1] + 2.0 * (s2.x0[1] - s2.x0[0])
    s2.yold[1] = s2.y0[1] + 2.0 * (s2.y0[1] - s2.y0[0])
    s2.zold[1] = s2.z0[1] + 2.0 * (s2.z0[1] - s2.z0[0])
    with pytest.raises(abi.MdgError) as ei:
        g2.shake(s2, og2["ft"])
    assert ei.value.code == -5


def test_list_capacity_growth(oracle, gpulib):
    """An undersized list capacity is grown on the fly; results stay exact."""
    def mut(s, prm):
        prm.list_capacity = 8
        prm.wlist_capacity = 8

    sg, sr, g, r = _both("slab512", oracle, gpulib, mut)
    _check_forces(g.force_get(sg), r.force_get(sr))
    assert _pairs(g) == _pairs(r)


def test_golden_y_n(gpulib):
    """The reference's own interfacial sample against the committed oracle record."""
    s, prm, z = y_n_case()
    g = abi.Context(gpulib, s, prm)
    o = g.force_get(s)
    e = np.linalg.norm(o["f"] - z["ref_f"]) / np.linalg.norm(z["ref_f"])
    assert e < FORCE_RTOL
    np.testing.assert_allclose(o["elj"], z["ref_elj"], rtol=1e-11, atol=1e-8)
    np.testing.assert_allclose(o["eqq"], z["ref_eqq"], rtol=1e-11, atol=1e-8)
    assert abs(o["uconf"] - float(z["ref_uconf"])) < 1e-10 * abs(float(z["ref_uconf"]))
