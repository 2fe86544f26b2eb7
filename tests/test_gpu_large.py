"""Parity at the full sizes of the benchmark systems.

At these sizes the tensor-core reciprocal sum takes the branches that the small parity systems
never reach: 32,768 waters (98,304 atoms) with kmax 24 give 29,038 k vectors and 768 atom tiles of
128, so the force pass runs five whole waves of 152 tiles and cuts only the 8 tiles of its last,
partial wave into pieces; the structure-factor pass splits 98,304 atoms over its CTAs.  The
mixed form is compared with the FP64 form of the library and with the oracle directly (its
OpenMP build, -O2 -ffast-math, which agrees with the parity build far below these tolerances).
The bars are those of the metric: force rel-RMS ||dF|| / ||F|| <= 1e-5 over all moving sites;
the configurational energy within 1e-5 of the energy scale |sum elj| + |sum eqq| + |uewa|; the
reciprocal energy's own relative error is printed and held under 1e-5.  The FP64 form itself is
pinned against the parity oracle at 1e-12 on a bulk system large enough (20,577 atoms) for more
than one wave of force tiles.
"""
import numpy as np
import pytest

from md_sim_gb300 import abi, configs

pytestmark = pytest.mark.gpu

MIXED_FORCE_RTOL = 1e-5
MIXED_ENERGY_RTOL = 1e-5
FP64_FORCE_RTOL = 1e-12


def _with(prm, precision):
    return abi.RunParams(**{**prm.__dict__, "precision": precision})


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _scale(e):
    return np.abs(e["elj"]).sum() + np.abs(e["eqq"]).sum() + abs(e["uewa"])


@pytest.fixture(scope="module")
def oracle_omp():
    import build as oracle_build

    oracle_build.build()
    return abi.Lib(oracle_build.path("libmdref_omp.so"), "ref_")


@pytest.fixture(scope="module")
def bulk32k():
    return configs.large_bulk_water()


def test_bulk32k_kset(gpulib, bulk32k):
    s, prm = bulk32k
    kl, km, kn, ak = abi.Context(gpulib, s.copy(), _with(prm, abi.MDG_MIXED)).kvectors()
    assert len(kl) == 29038
    assert kl.max() == 24 and km.min() == -24 and kn.max() == 24


def test_bulk32k_mixed_vs_fp64_and_oracle(gpulib, oracle_omp, bulk32k):
    s, prm = bulk32k
    s64, s32, so = s.copy(), s.copy(), s.copy()
    a = abi.Context(gpulib, s64, _with(prm, abi.MDG_FP64)).force_get(s64)
    b = abi.Context(gpulib, s32, _with(prm, abi.MDG_MIXED)).force_get(s32)
    r = abi.Context(oracle_omp, so, _with(prm, abi.MDG_FP64)).force_get(so)
    e_mx64, e_mxo, e_64o = _rel(b["f"], a["f"]), _rel(b["f"], r["f"]), _rel(a["f"], r["f"])
    print(f"bulk32k dF_rms: mixed vs FP64 GPU {e_mx64:.3e}, mixed vs oracle {e_mxo:.3e}, "
          f"FP64 GPU vs oracle {e_64o:.3e}")
    assert e_mx64 <= MIXED_FORCE_RTOL
    assert e_mxo <= MIXED_FORCE_RTOL
    assert e_64o <= 1e-10
    for key in ("fc", "torque"):
        assert _rel(b[key], r[key]) <= MIXED_FORCE_RTOL, key
    ue = abs(b["uewa"] - r["uewa"]) / abs(r["uewa"])
    uc = abs(b["uconf"] - r["uconf"]) / _scale(r)
    print(f"bulk32k energies: uewa rel {ue:.3e}, uconf / scale {uc:.3e}")
    assert uc <= MIXED_ENERGY_RTOL
    assert ue <= MIXED_ENERGY_RTOL
    assert abs(a["uself"] - r["uself"]) <= 1e-12 * abs(r["uself"])


def test_bulk32k_box_reciprocal_only(gpulib):
    """97,336 point ions (charges dealt to a jittered lattice at random) in the 99.3 A box at kmax
    24 with no pair inside the cutoff: the forces are the tensor-core reciprocal forces alone (761
    atom tiles: five whole waves + one tile cut into pieces), against the FP64 reciprocal sum."""
    s, prm = configs.ion_lattice(n_side=46, spacing=99.3 / 46, rcut=1.5, alpha=0.32, kmax=24, jitter=0.05,
                                 shuffle=True)
    s64, s32 = s.copy(), s.copy()
    a = abi.Context(gpulib, s64, _with(prm, abi.MDG_FP64)).force_get(s64)
    b = abi.Context(gpulib, s32, _with(prm, abi.MDG_MIXED)).force_get(s32)
    assert a["eqq"].max() == 0.0 and a["eqq"].min() == 0.0  # empty real-space sum
    e = _rel(b["f"], a["f"])
    ue = abs(b["uewa"] - a["uewa"]) / abs(a["uewa"])
    print(f"reciprocal-only 97,336 ions, kmax 24: dF_rms {e:.3e}, uewa rel {ue:.3e}")
    assert e <= MIXED_FORCE_RTOL
    assert ue <= MIXED_ENERGY_RTOL


def test_bulk32k_resident_steps_mixed_vs_fp64(gpulib, bulk32k):
    """Three resident MD steps (predictor that packs the records, graph branches, corrector) of
    the mixed form against the FP64 form from the same start."""
    s, prm = bulk32k
    sg, s64 = s.copy(), s.copy()
    g = abi.Context(gpulib, sg, _with(prm, abi.MDG_MIXED))
    f = abi.Context(gpulib, s64, _with(prm, abi.MDG_FP64))
    scale = _scale(f.force_get(s64.copy()))
    g.set_state(sg)
    f.set_state(s64)
    rg, rf = g.run(3), f.run(3)
    g.get_state(sg)
    f.get_state(s64)
    assert np.abs(sg.x0 - s64.x0).max() < 1e-6 * sg.lx
    for key in ("kp", "kw"):
        assert abs(rg[key] - rf[key]) <= 1e-5 * abs(rf[key]), (key, rg[key], rf[key])
    assert abs(rg["uconf"] - rf["uconf"]) <= MIXED_ENERGY_RTOL * scale, (rg["uconf"], rf["uconf"], scale)


def test_bulk7k_fp64_vs_oracle(gpulib, oracle):
    """FP64 parity on a bulk system shaped like the 32,768-water one (simple-cubic water lattice,
    alpha 0.32, rcut 10) with 6,859 waters = 20,577 atoms > 152 x 128, kmax 16; the mixed form on
    the same system against the oracle directly (161 force tiles: one whole wave + 9 cut)."""
    n = 19
    s, prm = configs.bulk_water(n, "sc", box=n * 3.103, seeds=(5, 6, 7), rcut=10.0, alpha=0.32, kmax=16)
    sg, sr, sm = s.copy(), s.copy(), s.copy()
    og = abi.Context(gpulib, sg, _with(prm, abi.MDG_FP64)).force_get(sg)
    orf = abi.Context(oracle, sr, _with(prm, abi.MDG_FP64)).force_get(sr)
    om = abi.Context(gpulib, sm, _with(prm, abi.MDG_MIXED)).force_get(sm)
    e64 = _rel(og["f"], orf["f"])
    emx = _rel(om["f"], orf["f"])
    print(f"bulk 6859 waters: FP64 GPU vs oracle {e64:.3e}, mixed vs oracle {emx:.3e}")
    assert e64 < FP64_FORCE_RTOL
    for key in ("fc", "torque"):
        assert _rel(og[key], orf[key]) < FP64_FORCE_RTOL * 10, key
    scale = _scale(orf) + 1.0
    for key in ("uewa", "uself", "uconf"):
        assert abs(og[key] - orf[key]) <= 1e-12 * scale, (key, og[key], orf[key])
    assert emx <= MIXED_FORCE_RTOL
    assert abs(om["uconf"] - orf["uconf"]) <= MIXED_ENERGY_RTOL * scale


def test_shake8k_mixed_vs_fp64(gpulib):
    """The full SHAKE-water system (8,192 constrained waters on 11,552 wall sites, 8 x 8 nm walls)
    in the mixed form against FP64: forces of the force evaluation, then one SHAKE step each from
    those forces at the 1e-10 tolerance."""
    s, prm = configs.shake_water()
    s64, s32 = s.copy(), s.copy()
    c64 = abi.Context(gpulib, s64, _with(prm, abi.MDG_FP64))
    c32 = abi.Context(gpulib, s32, _with(prm, abi.MDG_MIXED))
    a, b = c64.force_get(s64), c32.force_get(s32)
    e = _rel(b["f"], a["f"])
    print(f"shake8k dF_rms mixed vs FP64 {e:.3e}")
    assert e <= MIXED_FORCE_RTOL
    assert abs(b["uconf"] - a["uconf"]) <= MIXED_ENERGY_RTOL * _scale(a)
    sa, sb = c64.shake(s64, a["ft"]), c32.shake(s32, b["ft"])
    assert abs(sa["sweeps"] - sb["sweeps"]) <= 2, (sa["sweeps"], sb["sweeps"])
    assert np.abs(s64.x0 - s32.x0).max() < 1e-6 * s64.lx
