"""The k-vector set of force_fouri_init (src/forcem.f90:743-776) in the oracle, against the counts
the benchmark systems must have and against an independent numpy restatement of the selection.

The selection runs in real(4) arithmetic in the reference (src/forcem.f90:756,759): a vector
(kl, km, kn) of the half space (kl >= 0; kl = 0 -> km >= 0; kl = km = 0 -> kn >= 1) is kept when
real(kl^2 + km^2) + real(kn^2 kmax^2) / real(knmax^2) < real(kmax^2) + 2.01, all in float32,
with klmax, kmmax, knmax = nint(kmax L / min L) (src/forcem.f90:673-678).  The k set depends only
on the box and kmax, so the 32,768-water box is checked on a small ion lattice of the same box.
"""
import numpy as np
import pytest

from md_sim_gb300 import abi, configs


def _oracle_kset(oracle, s, prm):
    return abi.Context(oracle, s, prm).kvectors()


def _numpy_kset(lx, ly, lz, kmax):
    lmin = min(lx, ly, lz)
    rk = float(np.float32(kmax))
    KL, KM, KN = (int(np.floor(rk * L / lmin + 0.5)) for L in (lx, ly, lz))
    lim = np.float32(np.float32(kmax * kmax) + np.float32(2.01))
    out = []
    kmmin, knmin = 0, 1
    for kl in range(KL + 1):
        for km in range(kmmin, KM + 1):
            for kn in range(knmin, KN + 1):
                a = np.float32(kl * kl + km * km)
                b = np.float32(np.float32(kn * kn * kmax * kmax) / np.float32(KN * KN))
                if np.float32(a + b) < lim:
                    out.append((kl, km, kn))
            knmin = -KN
        kmmin = -KM
    return np.array(out, dtype=np.int32).reshape(-1, 3)


SYSTEMS = {
    # name: (builder, expected N_k)
    "bulk256 (256 waters, kmax 7)": (lambda: configs.bulk_water(), 775),
    "slab2048 (kmax 10/10/20)": (lambda: configs.slab_water(), 4338),
    # the 99.3 A box of the 32,768-water system at kmax 24
    "bulk32k box (kmax 24)": (lambda: configs.ion_lattice(n_side=2, spacing=99.3 / 2, rcut=10.0, alpha=0.32,
                                                          kmax=24), 29038),
}


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_kset_counts_and_order(name, oracle):
    make, nk = SYSTEMS[name]
    s, prm = make()
    kl, km, kn, ak = _oracle_kset(oracle, s, prm)
    assert len(kl) == nk
    ref = _numpy_kset(s.lx, s.ly, s.lz, prm.kmax)
    assert len(ref) == nk
    np.testing.assert_array_equal(np.stack([kl, km, kn], 1), ref)
    assert np.all(ak > 0) and np.all(np.isfinite(ak))


def test_kset_boundary_vector_included(oracle):
    """Q2: (7, 1, 1) at kmax 7 has kl^2 + km^2 + kn^2 = 51 < 49 + 2.01 in float32: it is kept."""
    s, prm = configs.bulk_water()
    kl, km, kn, _ = _oracle_kset(oracle, s, prm)
    keys = set(zip(kl.tolist(), km.tolist(), kn.tolist()))
    assert (7, 1, 1) in keys
    assert (7, 2, 1) not in keys  # 54 > 51.01
