"""Independent physics checks of the oracle (oracle/mdref.cpp), which has no reference outputs to
be pinned against: the NaCl Madelung constant from its Ewald sum, forces as the negative energy
gradient, independence of the total from the Ewald splitting parameter, Newton's third law and
translation invariance.  CPU only."""
import numpy as np
import pytest

from md_sim_gb300 import abi, configs
from md_sim_gb300 import system as S

MADELUNG_NACL = 1.747564594633  # rocksalt, per ion pair, nearest-neighbour distance units


def _facq():
    return S.PH_4epi * S.PH_e * S.PH_e * S.PH_NA / (1000.0 * S.PH_A2m)


def _coulomb(e):
    # uconf leaves the self term out (src/forcem.f90 energy bookkeeping); add it back
    return float(np.sum(e["eqq"]) + e["uewa"] + e["uself"])


def _energy(oracle, s, prm):
    ctx = abi.Context(oracle, s, prm)
    try:
        return ctx.force_get(s)
    finally:
        ctx.close()


def test_madelung_constant(oracle):
    s, prm = configs.ion_lattice(n_side=6, spacing=2.8, rcut=8.0, alpha=0.45, kmax=10, jitter=0.0)
    e = _energy(oracle, s, prm)
    n = s.nmove
    m = -2.0 * _coulomb(e) * 2.8 / (n * _facq())
    assert abs(m - MADELUNG_NACL) < 2e-6 * MADELUNG_NACL, m
    # a perfect lattice is a force-free configuration
    assert np.abs(e["f"]).max() < 1e-7 * _facq() / 2.8 ** 2


def test_total_independent_of_ewald_split(oracle):
    base = dict(n_side=6, spacing=2.8, rcut=8.0, jitter=0.25, seed=4)
    s1, p1 = configs.ion_lattice(alpha=0.45, kmax=10, **base)
    s2, p2 = configs.ion_lattice(alpha=0.55, kmax=13, **base)
    e1, e2 = _energy(oracle, s1, p1), _energy(oracle, s2, p2)
    u1, u2 = _coulomb(e1), _coulomb(e2)
    assert abs(u1 - u2) < 2e-6 * abs(u1), (u1, u2)
    f1, f2 = e1["f"], e2["f"]
    assert np.linalg.norm(f1 - f2) < 2e-5 * np.linalg.norm(f1)


def test_forces_are_negative_energy_gradient(oracle):
    s, prm = configs.ion_lattice(n_side=4, spacing=2.8, rcut=5.2, alpha=0.55, kmax=9, jitter=0.25, seed=7)
    e0 = _energy(oracle, s.copy(), prm)
    f = e0["f"]
    h = 2e-5
    rng = np.random.default_rng(0)
    for atom in rng.choice(s.nmove, 4, replace=False):
        for d, arr in enumerate(("x0", "y0", "z0")):
            sp, sm = s.copy(), s.copy()
            getattr(sp, arr)[atom] += h
            getattr(sm, arr)[atom] -= h
            up, um = _coulomb(_energy(oracle, sp, prm)), _coulomb(_energy(oracle, sm, prm))
            fd = -(up - um) / (2 * h)
            assert abs(fd - f[d, atom]) < 1e-4 * (abs(f[d, atom]) + 1.0), (atom, d, fd, f[d, atom])


def test_newton_third_law_and_translation(oracle):
    s, prm = configs.bulk_water()
    e = _energy(oracle, s.copy(), prm)
    f = e["f"]
    scale = np.sqrt((f ** 2).mean())
    assert np.abs(f.sum(1)).max() < 1e-9 * scale * f.shape[1]
    st = s.copy()
    shift = np.array([0.37, -1.21, 2.03])
    for d, arr in enumerate(("x0", "y0", "z0")):
        getattr(st, arr)[: st.nmove] += shift[d]
    if st.nrig:
        for d in range(3):
            st.c[0, d] += shift[d]
    et = _energy(oracle, st, prm)
    assert abs(et["uconf"] - e["uconf"]) < 1e-9 * abs(e["uconf"])
    assert np.linalg.norm(et["f"] - f) < 1e-8 * np.linalg.norm(f)
