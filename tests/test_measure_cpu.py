"""Measurement histograms of the oracle against independent numpy restatements of the reference's
formulas (CPU only): ngc of the site-wall pairs (src/forcem.f90:493-495) and of the bulk pair loop
(src/forcem_back.f90:348-349,380-382), the ion field profiles efipos / tefipos / nefipos
(src/forcem.f90:347-354,388-395,486-489,930-934,1094-1098), ngang (:617-625) and measure_do's
z-profiles (src/measure.f90:283-312)."""
import numpy as np
import pytest

from md_sim_gb300 import abi, configs
from tests.golden.fixture import y_n_case

RDEL = 0.1


def anint(x):
    """Fortran ANINT (half away from zero), exact."""
    t = np.trunc(x)
    return t + np.where(np.abs(x - t) >= 0.5, np.sign(x), 0.0)


def minimg(d, L):
    return d - L * anint(d * (1.0 / L))


def ij(s, a, b):
    """0-based pair id of 1-based site types a, b."""
    return s.ijtype[(a - 1) + s.nit * (b - 1)] - 1


def heads(s):
    return np.nonzero(s.nsi[s.itype[: s.nmove] - 1] > 0)[0]


def zbin(s, z):
    return ((z + s.lwh) * (1.0 / RDEL) + 0.5).astype(np.int64)


def rbin(r):
    return (r * (1.0 / RDEL) + 0.5).astype(np.int64)


def lmax(s):
    return int(s.lw * (1.0 / RDEL) + 0.5) + 1


def _ctx(lib, s, prm, **kw):
    c = abi.Context(lib, s.copy(), prm)
    dims = c.measure_init(RDEL, **kw)
    return c, dims


def _wall_ngc(s, rsx, rsy, rsz, rcut, bulk=False):
    out = np.zeros((s.nijt, lmax(s) + 1), np.int64)
    w = np.arange(s.nmove, s.ntota)
    for i in heads(s):
        it = s.itype[i]
        xi = minimg(s.x0[i] - s.x0[w], s.lx)
        yi = minimg(s.y0[i] - s.y0[w], s.ly)
        zi = s.z0[i] - s.z0[w]
        if bulk:
            zi = minimg(zi, s.lz)
        ok = xi * xi + yi * yi + zi * zi <= rcut * rcut
        for a in range(s.nsi[it - 1]):
            xd, yd, zd = xi[ok] + rsx[i + a], yi[ok] + rsy[i + a], zi[ok] + rsz[i + a]
            rr = np.sqrt(xd * xd + yd * yd + zd * zd)
            np.add.at(out, (ij(s, s.itype[i + a], s.itype[w[ok]]), rbin(rr)), 1)
    return out


def test_wall_ngc_matches_numpy(oracle):
    s, prm = configs.slab_water(nwat=192, cells=5, kmax=5, placement="lattice")
    rs = (s.rsx.copy(), s.rsy.copy(), s.rsz.copy())
    c, d = _ctx(oracle, s, prm)
    c.force_get(s.copy())
    h = c.measure_get()
    want = _wall_ngc(s, *rs, prm.rcut)
    assert h["ngc"].sum() > 0
    np.testing.assert_array_equal(h["ngc"], want)
    assert h["calls_force"] == 1 and h["out_of_range"] == 0
    assert h["efipos"].any() == False  # no ions
    c.close()


def test_bulk_pair_ngc_matches_numpy(oracle):
    s, prm = configs.bulk_water(n_side=2, box=9.9, rcut=4.5, kmax=4)
    rs = (s.rsx.copy(), s.rsy.copy(), s.rsz.copy())
    c, d = _ctx(oracle, s, prm)
    c.force_get(s.copy())
    h = c.measure_get()
    want = np.zeros_like(h["ngc"])
    hd = heads(s)
    rc2 = prm.rcut ** 2
    oor = 0
    for i in hd:
        for j in hd[hd > i]:
            xio = minimg(np.array([s.x0[i] - s.x0[j]]), s.lx)[0]
            yio = minimg(np.array([s.y0[i] - s.y0[j]]), s.ly)[0]
            zio = minimg(np.array([s.z0[i] - s.z0[j]]), s.lz)[0]
            rsq = xio * xio + yio * yio + zio * zio
            if rsq > rc2:
                continue
            pairs = [(0, 0, np.sqrt(rsq))]
            for a in range(3):
                for b in range(1 if a == 0 else 0, 3):
                    xd = (xio + rs[0][i + a]) - rs[0][j + b]
                    yd = (yio + rs[1][i + a]) - rs[1][j + b]
                    zd = (zio + rs[2][i + a]) - rs[2][j + b]
                    pairs.append((a, b, np.sqrt(xd * xd + yd * yd + zd * zd)))
            for a, b, r in pairs:
                l = int(r * (1.0 / RDEL) + 0.5)
                if l > d["lmax"]:
                    oor += 1
                    continue
                want[ij(s, s.itype[i + a], s.itype[j + b]), l] += 1
    assert want.sum() > 0
    np.testing.assert_array_equal(h["ngc"], want)
    assert h["out_of_range"] == oor
    c.close()


def _ion_realspace_fz(s, rsx, rsy, rsz, prm):
    """z component of the real-space force on each liquid ion, summed the way efipos books it."""
    alfa = prm.alpha
    facq = s_facq(s)
    spii = 2.0 / np.sqrt(float(np.float32(3.1415926535898)))
    out = {}
    hd = heads(s)
    allj = np.concatenate([hd, np.arange(s.nmove, s.ntota)])
    A = [np.float32(x) for x in (0.254829592, -0.284496736, 1.421413741, -1.453152027, 1.061405429)]
    P = float(np.float32(0.3275911))

    def erfc_f(rr, au, r2i):
        ar = alfa * rr
        t = 1.0 / (1.0 + P * ar)
        e2 = np.exp(-ar * ar)
        ef = ((((float(A[4]) * t + float(A[3])) * t + float(A[2])) * t + float(A[1])) * t + float(A[0])) * t * e2
        return (spii * ar * e2 + ef) * au * r2i

    for i in range(s.nriga, s.nliqa):
        fz = 0.0
        for j in allj:
            if j == i:
                continue
            dz = s.z0[i] - s.z0[j]
            dx = minimg(np.array([s.x0[i] - s.x0[j]]), s.lx)[0]
            dy = minimg(np.array([s.y0[i] - s.y0[j]]), s.ly)[0]
            rsq = dx * dx + dy * dy + dz * dz
            if rsq > prm.rcut ** 2:
                continue
            ijt = ij(s, s.itype[i], s.itype[j])
            rij = np.sqrt(rsq)
            f = 0.0
            vk = s.vdwnum[ijt]
            if vk == 1:
                r6 = s.sig[ijt] * (1.0 / rsq) ** 3
                f = 6.0 / rsq * s.eps[ijt] * r6 * (2.0 * r6 - 1.0)
            elif vk == 2:
                r6 = s.cc[ijt] * (1.0 / rsq) ** 3
                aux = s.aa[ijt] * np.exp(-rij * s.rhoi[ijt])
                f = aux * s.rhoi[ijt] / rij - 6.0 / rsq * r6
            f += erfc_f(rij, facq * s.qs[i] * s.qs[j] / rij, 1.0 / rsq)
            fz += dz * f
            nsj = s.nsi[s.itype[j] - 1] if j < s.nmove else 1
            for b in range(1, nsj):  # the other sites of a molecule
                xd = (dx + rsx[i]) - rsx[j + b]
                yd = (dy + rsy[i]) - rsy[j + b]
                zd = (dz + rsz[i]) - rsz[j + b]
                r2 = xd * xd + yd * yd + zd * zd
                rr = np.sqrt(r2)
                fz += zd * erfc_f(rr, facq * s.qs[i] * s.qs[j + b] / rr, 1.0 / r2)
        out[i] = fz
    return out


def s_facq(s):
    """facq of force_init (src/forcem.f90:60) from the single-precision constants of src/global.f90."""
    f = np.float32
    k4, e, na, a2m = (float(f(x)) for x in (8.987551784952e+9, 1.6021892e-19, 6.022045e23, 1.0e-10))
    return k4 * e * e * na / (1000.0 * a2m)


def test_ion_profiles(oracle):
    s, prm = configs.slab_electrolyte(nwat=96, npair=6, cells=4, kmax=4, rcut=7.0)
    rs = (s.rsx.copy(), s.rsy.copy(), s.rsz.copy())
    c, d = _ctx(oracle, s, prm)
    out = c.force_get(s.copy())
    h = c.measure_get()
    ions = np.arange(s.nriga, s.nliqa)
    t = s.itype[ions] - 3
    l = zbin(s, s.z0[ions])
    nef = np.zeros((2, d["lmax"] + 1), np.int64)
    np.add.at(nef, (t, l), 1)
    np.testing.assert_array_equal(h["nefipos"], nef)
    ftz = out["ft"][2, ions - s.nriga]
    tef = np.zeros((2, d["lmax"] + 1))
    np.add.at(tef, (t, l), ftz)
    scale = np.abs(ftz).max()
    assert np.abs(h["tefipos"] - tef).max() <= 1e-12 * scale
    # efipos = real-space z force on the ions (pair and wall terms) + whole fz after force_fouri
    real = _ion_realspace_fz(s, *rs, prm)
    ef = tef.copy()
    np.add.at(ef, (t, l), np.array([real[i] for i in ions]))
    assert np.abs(h["efipos"] - ef).max() <= 1e-9 * scale, np.abs(h["efipos"] - ef).max() / scale
    assert h["out_of_range"] == 0
    c.close()


def test_ngang_and_profiles(oracle):
    s, prm = y_n_case()[:2]
    c, d = _ctx(oracle, s, prm, profiles=True, l2d=True, rfrst=3.0, rscnd=6.0)
    s2 = s.copy()
    c.force_get(s2)
    c.measure_do(s)
    h = c.measure_get()
    # ngang from the angle terms
    ng = np.zeros((d["ntz"], d["langmax"] + 1), np.int64)
    for ia in range(s.nang):
        it = s.iatype[ia] - 1
        for k in range(s.nangt[it]):
            i, j, kk = (s.ang[:, k, ia] - 1)
            ax = minimg(np.array([s.x0[kk] - s.x0[j]]), s.lx)[0]
            ay = minimg(np.array([s.y0[kk] - s.y0[j]]), s.ly)[0]
            az = s.z0[kk] - s.z0[j]
            bx = minimg(np.array([s.x0[j] - s.x0[i]]), s.lx)[0]
            by = minimg(np.array([s.y0[j] - s.y0[i]]), s.ly)[0]
            bz = s.z0[j] - s.z0[i]
            ai = 1.0 / np.sqrt(ax * ax + ay * ay + az * az)
            bi = 1.0 / np.sqrt(bx * bx + by * by + bz * bz)
            cang = -(ax * bx + ay * by + az * bz) * ai * bi
            ng[it, int((cang + 1.0) * 100.0) + 1] += 1
    assert ng.sum() == 54
    np.testing.assert_array_equal(h["ngang"], ng)
    # measure_do z-profile and dipole profile
    n = s.nmove
    it = s.itype[:n]
    l = zbin(s, s.z0[:n])
    ngz = np.zeros((d["ntz"], d["lmax"] + 1), np.int64)
    inr = (l >= 0) & (l <= d["lmax"])  # surface groups beyond the wall planes fall outside the bins
    np.add.at(ngz, (it[inr] - 1, l[inr]), 1)
    np.testing.assert_array_equal(h["ngz"], ngz)
    assert h["out_of_range"] == int((~inr).sum())
    o = np.nonzero((it == 1) & inr)[0]
    mu = [np.zeros(d["lmax"] + 1) for _ in range(3)]
    for k, a in enumerate((s.x0, s.y0, s.z0)):
        np.add.at(mu[k], l[o], a[o] - 0.5 * (a[o + 1] + a[o + 2]))
    for k, key in enumerate(("ndipx", "ndipy", "ndipz")):
        assert np.allclose(h[key], mu[k], rtol=0, atol=1e-12)
    assert np.allclose(h["ndipsq"], mu[0] ** 2 + mu[1] ** 2 + mu[2] ** 2, rtol=1e-12, atol=1e-12)
    # 2-D maps: atoms within rscnd of a wall
    rij = s.lwh - np.abs(s.z0[:n])
    near = rij < 6.0
    assert h["ng2d1"].sum() + h["ng2d2"].sum() == int(near.sum())
    assert h["ng2d1"].sum() == int((rij < 3.0).sum())
    assert h["calls_do"] == 1 and h["calls_force"] == 1
    c.measure_zero()
    z = c.measure_get()
    assert z["ngz"].sum() == 0 and z["ngang"].sum() == 0 and z["calls_do"] == 0
    c.close()


def test_resident_profiles_accumulate(oracle):
    s, prm = configs.slab_water(nwat=128, cells=4, kmax=4, placement="lattice")
    c, d = _ctx(oracle, s, prm, force_hist=True, profiles=True)
    c.set_state(s)
    c.run(3)
    h = c.measure_get()
    assert h["calls_do"] == 3 and h["calls_force"] == 3
    assert h["ngz"].sum() == 3 * s.nmove
    c.measure_enable(False, False)
    c.run(2)
    assert c.measure_get()["calls_do"] == 3
    c.close()
