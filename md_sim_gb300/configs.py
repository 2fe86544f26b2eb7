"""Seeded synthetic systems with the shapes and parameters of the benchmark workloads.

There is no public dataset for this path; these generators stand in for it.  Each returns a
(System, RunParams) pair in the reference's units (A, fs, kJ/mol, e; masses in kg/mol in the
field file) and can be written out in the reference formats with system.write_fld/top/cfg.

  bulk_water(n_side, lattice)       rigid SPC/E-type water, cubic periodic box (fcc or sc lattice)
  slab_water(nwat, cells)           rigid water between two rocksalt (001) walls, slab semantics
  shake_water(nwat, cells)          3-site water as SHAKE-constrained surface molecules on walls
"""
from __future__ import annotations

import math
from typing import List, Optional, Tuple

import numpy as np

from . import system as S
from .abi import MDG_BULK, MDG_SLAB, RunParams

EV = 96.485  # kJ/mol per eV
Q_O, Q_H = -0.8476, 0.4238
M_O, M_H = 15.9994e-3, 1.008e-3
SIG_OO, EPS_OO = 3.166, 0.6502
HOH = 109.47
R_OH = 1.0
KB = S.PH_R / 1000.0  # kJ/mol/K


def _water_body() -> np.ndarray:
    """O, H, H in the principal-axis frame (symmetry axis y, molecule in the xy plane)."""
    h = math.radians(HOH / 2.0)
    return np.array([[0.0, 0.0, 0.0],
                     [R_OH * math.sin(h), R_OH * math.cos(h), 0.0],
                     [-R_OH * math.sin(h), R_OH * math.cos(h), 0.0]])


def _vdw_table(names, pairs):
    """pairs: {(i, j): ('LeJo', sig, eps) | ('Buck', A, rho, C)} with 1-based site-type ids."""
    out = []
    ijt = 0
    n = len(names)
    for i in range(1, n + 1):
        for j in range(i, n + 1):
            ijt += 1
            p = pairs.get((i, j)) or pairs.get((j, i))
            if p is None:
                out.append(S.VdwEntry(ijt, i, j, "zero", ()))
            else:
                out.append(S.VdwEntry(ijt, i, j, p[0], tuple(p[1:])))
    return out


def _random_quaternions(rng, n):
    """Uniform random unit quaternions (Shoemake 1992)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    q = np.stack([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)])
    return q


def _rigid_velocities(s: S.System, T: float, seed_v: int, seed_w: int):
    """Maxwell-Boltzmann COM velocities and body-frame angular velocities (per fs, dt = 1 fs so
    that internal mass units make kT/m an (A/fs)^2), net momentum removed; first quaternion
    derivatives consistent with the angular velocity (the relation move_correct drives them to,
    src/move.f90:285-288)."""
    kT = KB * T
    rng = np.random.default_rng(seed_v)
    v = rng.normal(0.0, math.sqrt(kT / s.mw), size=(3, s.nrig))
    v -= v.mean(axis=1, keepdims=True)
    s.c[1] = v
    rng = np.random.default_rng(seed_w)
    inert = (s.inxx, s.inyy, s.inzz)
    w = np.stack([rng.normal(0.0, math.sqrt(kT / inert[d]), size=s.nrig) for d in range(3)])
    s.w[0] = w
    q1, q2, q3, q4 = s.q[0]
    wx, wy, wz = w
    s.q[1, 0] = 0.5 * (-q3 * wx - q4 * wy + q2 * wz)
    s.q[1, 1] = 0.5 * (q4 * wx - q3 * wy - q1 * wz)
    s.q[1, 2] = 0.5 * (q1 * wx + q2 * wy + q4 * wz)
    s.q[1, 3] = 0.5 * (-q2 * wx + q1 * wy - q3 * wz)


def _water_moltype(kind="rigmol", nt=0) -> S.MolType:
    if kind == "rigmol":
        return S.MolType("spce", "rigmol", nt, ["O", "H"], [1, 2], [M_O, M_H], [Q_O, Q_H],
                         ns=3, geometry=_water_body())
    hh = 2.0 * R_OH * math.sin(math.radians(HOH / 2.0))
    return S.MolType("wat", "surfmol", nt, ["O", "H"], [1, 2], [M_O, M_H], [Q_O, Q_H], ns=3,
                     lengths=[R_OH, R_OH, round(hh, 3)], angles=[])


def _crystal(ns: int, a: float, lw: float, names=("Mg", "Ox"), q=(1.2, -1.2)) -> S.MolType:
    return S.MolType("oxide", "crystal", 1, list(names), [1, 1], [24.305e-3, 15.9994e-3], list(q),
                     ns=ns, cx=a / 2.0, cy=a / 2.0, cz=a / 2.0, lw=lw)


def _finish(s: S.System) -> S.System:
    s.config_init()
    s.rsx_after_predict()
    s.shake_init()
    return s


# ----------------------------------------------------------------------------------------------
def bulk_water(n_side: int = 4, lattice: str = "fcc", box: Optional[float] = None, T: float = 300.0,
               seeds=(1, 2, 3), rcut: float = 9.0, skin: float = 1.0, alpha: float = 0.30,
               kmax: int = 7) -> Tuple[S.System, RunParams]:
    """Rigid-water bulk box.  n_side=4, fcc, box 19.73: 256 waters (the 768-atom FP64 case);
    n_side=32, sc, box 99.3, alpha 0.32, rcut 10, kmax 24: 32,768 waters."""
    if lattice == "fcc":
        basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    else:
        basis = np.zeros((1, 3))
    nmol = n_side ** 3 * len(basis)
    L = box if box is not None else (19.73 if lattice == "fcc" and n_side == 4 else n_side * 3.103)
    a = L / n_side
    g = np.stack(np.meshgrid(*[np.arange(n_side)] * 3, indexing="ij"), -1).reshape(-1, 3)
    com = ((g[:, None, :] + basis[None, :, :]) * a).reshape(-1, 3) + 0.25 * a - 0.5 * L
    wat = _water_moltype("rigmol", nmol)
    crys = S.MolType("none", "crystal", 1, ["X1", "X2"], [1, 1], [1e-3, 1e-3], [0.0, 0.0], ns=0,
                     cx=L, cy=L, cz=L, lw=L)
    names = ["O", "H", "X1", "X2"]
    vdw = _vdw_table(names, {(1, 1): ("LeJo", SIG_OO, EPS_OO)})
    fld = S.FieldFile([wat, crys], vdw)
    top = S.TopFile([], [], [], [])
    s = S.System(fld, top, L, L, L, 1.0)
    s.c[0] = com.T
    s.q[0] = _random_quaternions(np.random.default_rng(seeds[0]), nmol)
    _rigid_velocities(s, T, seeds[1], seeds[2])
    s.temper = -1.0
    prm = RunParams(rcut=rcut, skin=skin, kmax=kmax, alpha=alpha, variant=MDG_BULK, pbc_z_list=1)
    return _finish(s), prm


def large_bulk_water(n_side: int = 32) -> Tuple[S.System, RunParams]:
    """32,768 rigid waters (98,304 atoms), 99.3 A box, alpha 0.32, rcut 10, kmax 24."""
    return bulk_water(n_side, "sc", box=n_side * 3.103, seeds=(5, 6, 7), rcut=10.0, skin=1.0,
                      alpha=0.32, kmax=24)


# ----------------------------------------------------------------------------------------------
def _rocksalt_walls(cells: int, a: float, lwh: float, layers: int = 4):
    """Two (001) rocksalt walls, surface layers at z = -lwh and +lwh, growing outward."""
    n = 2 * cells
    pos, typ = [], []
    for side in (-1, 1):
        for k in range(layers):
            z = side * (lwh + k * a / 2.0)
            for i in range(n):
                for j in range(n):
                    pos.append((i * a / 2.0, j * a / 2.0, z))
                    typ.append(1 if (i + j + k) % 2 == 0 else 2)
    return np.array(pos), np.array(typ, dtype=np.int64)


def _lattice_waters(rng, nwat, L, zlo, zhi, jitter=0.2):
    """nwat O positions on a random subset of a simple cubic lattice filling the film (x, y
    periodic), jittered: O-O >= spacing - 2 jitter.  Vectorised stand-in for random sequential
    placement when many systems are built."""
    h = zhi - zlo
    sp = (L * L * h / nwat) ** (1.0 / 3.0)
    while True:
        nx = max(1, int(L // sp))
        nz = max(1, int(h // sp) + 1)
        if nx * nx * nz >= nwat:
            break
        sp *= 0.98
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(nx), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
    pick = rng.choice(len(g), size=nwat, replace=False)
    dz = (h / max(nz - 1, 1)) if nz > 1 else 0.0
    pos = np.stack([g[pick, 0] * (L / nx), g[pick, 1] * (L / nx), zlo + g[pick, 2] * dz], 1)
    pos += rng.uniform(-jitter, jitter, size=pos.shape)
    pos[:, 2] = np.clip(pos[:, 2], zlo, zhi)
    return pos


def _place_waters(rng, nwat, L, zlo, zhi, walls, dmin_oo=2.5, dmin_ow=2.2, max_tries=200000):
    """Random sequential placement of O positions with overlap rejection (cell hashed)."""
    cs = 2.5
    ncx = max(1, int(L // cs))
    grid = {}
    out = []

    def key(p):
        return (int(p[0] / L * ncx) % ncx, int(p[1] / L * ncx) % ncx, int(math.floor(p[2] / cs)))

    wgrid = {}
    for w in walls:
        wgrid.setdefault(key(w), []).append(w)
    tries = 0
    while len(out) < nwat:
        tries += 1
        if tries > max_tries * 10:
            raise RuntimeError("water placement failed")
        p = np.array([rng.random() * L, rng.random() * L, zlo + rng.random() * (zhi - zlo)])
        kx, ky, kz = key(p)
        ok = True
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    kk = ((kx + dx) % ncx, (ky + dy) % ncx, kz + dz)
                    for src, dmin in ((grid, dmin_oo), (wgrid, dmin_ow)):
                        for q in src.get(kk, ()):
                            d = p - q
                            d[:2] -= L * np.round(d[:2] / L)
                            if d @ d < dmin * dmin:
                                ok = False
                                break
                        if not ok:
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if not ok:
                break
        if ok:
            out.append(p)
            grid.setdefault(key(p), []).append(p)
    return np.array(out)


def slab_water(nwat: int = 2048, cells: int = 10, a: float = 4.21, lz: Optional[float] = None,
               seed: int = 4, T: float = 300.0, rcut: float = 10.0, skin: float = 1.0,
               alpha: float = 0.30, kmax: int = 10, nvt: bool = False,
               placement: str = "rsa") -> Tuple[S.System, RunParams]:
    """Rigid waters between two rocksalt walls (4 layers, q +-1.2, Buckingham wall-O).
    NVE by default (T sets the initial velocities); nvt=True selects the reference's thermostat."""
    L = cells * a
    dens = 0.033427  # molecules / A^3 at 1 g/cm^3
    thick = nwat / (L * L * dens)
    lw = thick + 3.0
    lwh = 0.5 * lw
    lz = lz if lz is not None else 2.0 * L
    wpos, wtyp = _rocksalt_walls(cells, a, lwh)
    rng = np.random.default_rng(seed)
    if placement == "lattice":
        com = _lattice_waters(rng, nwat, L, -lwh + 2.2, lwh - 2.2)
    else:
        com = _place_waters(rng, nwat, L, -lwh + 1.4, lwh - 1.4, wpos)
    wat = _water_moltype("rigmol", nwat)
    crys = _crystal(len(wpos), a, lw)
    names = ["O", "H", "Mg", "Ox"]
    buck = ("Buck", 1000.0 * EV, 0.30, 10.0 * EV)
    vdw = _vdw_table(names, {(1, 1): ("LeJo", SIG_OO, EPS_OO), (1, 3): buck, (1, 4): buck})
    fld = S.FieldFile([wat, crys], vdw)
    top = S.TopFile([], [], [], [])
    s = S.System(fld, top, L, L, lz, 1.0)
    # COM positions: the O was placed; shift by the body-frame O offset is done via quaternions
    s.c[0] = com.T
    s.q[0] = _random_quaternions(np.random.default_rng(seed + 100), nwat)
    s.set_walls(wtyp, wpos)
    _rigid_velocities(s, T, seed + 200, seed + 300)
    s.temper = T if nvt else -1.0
    prm = RunParams(rcut=rcut, skin=skin, kmax=kmax, alpha=alpha, variant=MDG_SLAB)
    return _finish(s), prm


def slab_electrolyte(nwat: int = 384, npair: int = 12, cells: int = 6, a: float = 4.21, seed: int = 31,
                     T: float = 300.0, rcut: float = 9.0, skin: float = 1.0, alpha: float = 0.30,
                     kmax: int = 6) -> Tuple[S.System, RunParams]:
    """Rigid waters with npair Li+ / Cl- point ions (atmol site types 3 and 4, the numbering of the
    reference's y.fld) between two rocksalt walls: the case in which the force loops fill the
    ion field profiles (efipos, tefipos/nefipos).  Ions sit on free sites of the water lattice."""
    L = cells * a
    dens = 0.033427
    thick = (nwat + 2 * npair) / (L * L * dens)
    lw = thick + 3.0
    lwh = 0.5 * lw
    wpos, wtyp = _rocksalt_walls(cells, a, lwh)
    rng = np.random.default_rng(seed)
    pts = _lattice_waters(rng, nwat + 2 * npair, L, -lwh + 2.2, lwh - 2.2)
    com, ions = pts[:nwat], pts[nwat:]
    wat = _water_moltype("rigmol", nwat)
    li = S.MolType("Li", "atmol", npair, ["Li"], [1], [6.941e-3], [1.0], ns=1)
    cl = S.MolType("Cl", "atmol", npair, ["Cl"], [1], [35.453e-3], [-1.0], ns=1)
    crys = _crystal(len(wpos), a, lw)
    names = ["O", "H", "Li", "Cl", "Mg", "Ox"]
    buck = ("Buck", 1000.0 * EV, 0.30, 10.0 * EV)
    vdw = _vdw_table(names, {(1, 1): ("LeJo", SIG_OO, EPS_OO), (1, 3): ("LeJo", 2.34, 0.70),
                             (1, 4): ("LeJo", 3.78, 0.52), (3, 4): ("LeJo", 2.70, 0.35),
                             (3, 3): ("LeJo", 1.50, 0.70), (4, 4): ("LeJo", 4.40, 0.42),
                             (1, 5): buck, (1, 6): buck, (3, 6): buck, (4, 5): buck, (4, 6): buck})
    fld = S.FieldFile([wat, li, cl, crys], vdw)
    s = S.System(fld, S.TopFile([], [], [], []), L, L, 2.0 * L, 1.0)
    s.c[0] = com.T
    s.q[0] = _random_quaternions(np.random.default_rng(seed + 100), nwat)
    s.set_walls(wtyp, wpos)
    n0 = s.nriga
    s.x0[n0:n0 + 2 * npair], s.y0[n0:n0 + 2 * npair], s.z0[n0:n0 + 2 * npair] = ions.T
    _rigid_velocities(s, T, seed + 200, seed + 300)
    s.temper = -1.0
    prm = RunParams(rcut=rcut, skin=skin, kmax=kmax, alpha=alpha, variant=MDG_SLAB)
    return _finish(s), prm


# ----------------------------------------------------------------------------------------------
def replica_slabs(n: int = 64, seed: int = 8, nmin: int = 500, nmax: int = 4000, cmin: int = 7, cmax: int = 14,
                  a: float = 4.21) -> List[Tuple[S.System, RunParams]]:
    """Uneven interfacial replicas: water counts ~U{nmin..nmax} and wall cells ~U{cmin..cmax}
    (seeded), the slab-2048 walls and Buckingham parameters, alpha 0.30, rcut 10, kmax scaled to
    the box (nint(10 Lx / 42.1)).  A replica whose water film would be thicker than 95 A gets the
    smallest wider wall that brings it under (so that the z range of the reciprocal sum stays
    within the tensor-core tiles); Lz = max(2 Lx, film + 35 A)."""
    rng = np.random.default_rng(seed)
    nws = rng.integers(nmin, nmax + 1, size=n)
    cls = rng.integers(cmin, cmax + 1, size=n)
    dens = 0.033427
    out = []
    for i, (nw, cells) in enumerate(zip(nws.tolist(), cls.tolist())):
        while nw / ((cells * a) ** 2 * dens) > 95.0:
            cells += 1
        L = cells * a
        thick = nw / (L * L * dens)
        lz = max(2.0 * L, thick + 35.0)
        kmax = int(round(10.0 * L / 42.1))
        out.append(slab_water(nwat=nw, cells=cells, a=a, lz=lz, seed=seed * 1000 + i, kmax=kmax, placement="lattice"))
    return out


def shake_water(nwat: int = 8192, cells: int = 19, a: float = 4.21, seed: int = 9, T: float = 300.0,
                rcut: float = 10.0, skin: float = 1.0, alpha: float = 0.30,
                kmax: Optional[int] = None, tol2: float = 1e-10, maxit: int = 100,
                clean: bool = True) -> Tuple[S.System, RunParams]:
    """3-site waters as SHAKE-constrained surface molecules (O-H, O-H, H-H) between walls."""
    L = cells * a
    dens = 0.033427
    thick = nwat / (L * L * dens)
    lw = thick + 3.0
    lwh = 0.5 * lw
    lz = 2.0 * L
    wpos, wtyp = _rocksalt_walls(cells, a, lwh)
    rng = np.random.default_rng(seed)
    opos = _place_waters(rng, nwat, L, -lwh + 1.4, lwh - 1.4, wpos)
    wat = _water_moltype("surfmol", nwat)
    crys = _crystal(len(wpos), a, lw)
    names = ["O", "H", "Mg", "Ox"]
    buck = ("Buck", 1000.0 * EV, 0.30, 10.0 * EV)
    # H carries a bare charge; against the wall anions (-1.2 e) that is an unbounded attraction
    # which pulls the SHAKE-constrained molecule into the O-wall Buckingham collapse region within
    # a few hundred steps.  A short-range H-wall repulsion (A e^{-r/rho}, no dispersion) bounds it.
    hwall = ("Buck", 100.0 * EV, 0.25, 0.0)
    vdw = _vdw_table(names, {(1, 1): ("LeJo", SIG_OO, EPS_OO), (1, 3): buck, (1, 4): buck,
                             (2, 3): hwall, (2, 4): hwall})
    fld = S.FieldFile([wat, crys], vdw)
    constr = [[(3 * i + 1, 3 * i + 2), (3 * i + 1, 3 * i + 3), (3 * i + 2, 3 * i + 3)] for i in range(nwat)]
    top = S.TopFile(constr, [1] * nwat, [], [])
    s = S.System(fld, top, L, L, lz, 1.0)
    body = _water_body()
    hh = wat.lengths[2]
    # scale the H-H distance of the body to the constraint length exactly
    body[1, 0] = hh / 2.0
    body[2, 0] = -hh / 2.0
    body[1, 1] = body[2, 1] = math.sqrt(R_OH ** 2 - (hh / 2.0) ** 2)
    qrot = _random_quaternions(np.random.default_rng(seed + 1), nwat)
    qrot = _relax_orientations(np.random.default_rng(seed + 3), opos, qrot, body, L, lz, wpos)
    q1, q2, q3, q4 = qrot
    amat = np.empty((3, 3, nwat))
    amat[0, 0] = -q1 * q1 + q2 * q2 - q3 * q3 + q4 * q4
    amat[0, 1] = 2.0 * (q3 * q4 - q1 * q2)
    amat[0, 2] = 2.0 * (q2 * q3 + q1 * q4)
    amat[1, 0] = -2.0 * (q1 * q2 + q3 * q4)
    amat[1, 1] = q1 * q1 - q2 * q2 - q3 * q3 + q4 * q4
    amat[1, 2] = 2.0 * (q2 * q4 - q1 * q3)
    amat[2, 0] = 2.0 * (q2 * q3 - q1 * q4)
    amat[2, 1] = -2.0 * (q1 * q3 + q4 * q2)
    amat[2, 2] = -q1 * q1 - q2 * q2 + q3 * q3 + q4 * q4
    for j in range(3):
        for d in range(3):
            coords = opos[:, d] + amat[0, d] * body[j, 0] + amat[1, d] * body[j, 1] + amat[2, d] * body[j, 2]
            arr = (s.x0, s.y0, s.z0)[d]
            arr[np.arange(nwat) * 3 + j] = coords
    s.set_walls(wtyp, wpos)
    # previous positions: a thermal Verlet displacement per atom (dt = 1 fs), rigid-body consistent
    rngv = np.random.default_rng(seed + 2)
    v_unit = S.PH_A2m / (1.0 * S.f32(1.0e-15))
    kT = KB * T
    mtot = (M_O + 2 * M_H) * v_unit ** 2 / 1000.0
    vcom = rngv.normal(0.0, math.sqrt(kT / mtot), size=(nwat, 3))
    omega = rngv.normal(0.0, 0.012, size=(nwat, 3))  # ~ sqrt(kT / I) of water at 300 K, rad/fs
    nm = s.nmove
    xyz = np.stack([s.x0[:nm], s.y0[:nm], s.z0[:nm]], 1).reshape(nwat, 3, 3)
    ctr = xyz.mean(axis=1, keepdims=True)
    vel = vcom[:, None, :] + np.cross(omega[:, None, :], xyz - ctr)
    old = xyz - vel  # one fs earlier
    s.xold[:nm], s.yold[:nm], s.zold[:nm] = old.reshape(-1, 3).T
    nl = s.nliqa
    s.xold[nm:], s.yold[nm:], s.zold[nm:] = s.x0[nm:], s.y0[nm:], s.z0[nm:]
    del nl
    # surface molecules are integrated by the Verlet step of move_shake whatever the ensemble; the
    # thermostat of move_predict has no rigid or free atoms to act on here, so NVE is used
    s.temper = -1.0
    kmax = kmax if kmax is not None else int(round(10 * L / 42.1))
    prm = RunParams(rcut=rcut, skin=skin, kmax=kmax, alpha=alpha, variant=MDG_SLAB,
                    shake_tol2=tol2, shake_maxit=maxit,
                    quirks=1 if clean else 0)
    s.config_init()
    return s, prm


def _water_sites(opos, q, body):
    """(n, 3, 3) site positions of waters with head positions opos and quaternions q (the
    rotation of config_quatsite, src/config.f90:303-329)."""
    q1, q2, q3, q4 = q
    a = np.empty((3, 3, len(opos)))
    a[0, 0] = -q1 * q1 + q2 * q2 - q3 * q3 + q4 * q4
    a[0, 1] = 2.0 * (q3 * q4 - q1 * q2)
    a[0, 2] = 2.0 * (q2 * q3 + q1 * q4)
    a[1, 0] = -2.0 * (q1 * q2 + q3 * q4)
    a[1, 1] = q1 * q1 - q2 * q2 - q3 * q3 + q4 * q4
    a[1, 2] = 2.0 * (q2 * q4 - q1 * q3)
    a[2, 0] = 2.0 * (q2 * q3 - q1 * q4)
    a[2, 1] = -2.0 * (q1 * q3 + q4 * q2)
    a[2, 2] = -q1 * q1 - q2 * q2 + q3 * q3 + q4 * q4
    out = np.empty((len(opos), 3, 3))
    for j in range(3):
        for d in range(3):
            out[:, j, d] = opos[:, d] + a[0, d] * body[j, 0] + a[1, d] * body[j, 1] + a[2, d] * body[j, 2]
    return out


def _relax_orientations(rng, opos, q, body, L, lz, walls, dmin=1.7, iters=200):
    """Re-draws the orientation of every water with a site closer than dmin to a site of another
    molecule or to a wall atom (x, y periodic), until none is left: a random-orientation start
    with only O-O spacing enforced puts H atoms on top of neighbours, and the resulting forces
    break SHAKE in the first steps."""
    from scipy.spatial import cKDTree

    q = q.copy()
    n = len(opos)
    shift = np.array([0.0, 0.0, 4.0 * lz])
    box = np.array([L, L, 16.0 * lz])
    wtree = cKDTree(np.mod(np.asarray(walls) + shift, box), boxsize=box) if len(walls) else None
    for _ in range(iters):
        sites = np.mod(_water_sites(opos, q, body).reshape(-1, 3) + shift, box)
        tree = cKDTree(sites, boxsize=box)
        pairs = tree.query_pairs(dmin, output_type="ndarray")
        bad = set()
        if len(pairs):
            mi, mj = pairs[:, 0] // 3, pairs[:, 1] // 3
            sel = mi != mj
            bad.update(mi[sel].tolist())
            bad.update(mj[sel].tolist())
        if wtree is not None:
            for i, lst in enumerate(tree.query_ball_tree(wtree, dmin)):
                if lst:
                    bad.add(i // 3)
        if not bad:
            return q
        idx = np.array(sorted(bad))
        q[:, idx] = _random_quaternions(rng, len(idx))
    return q


def rescale_velocities(s: S.System, T: float) -> float:
    """Scales the velocity-like Gear derivatives of the rigid molecules and ions to temperature T
    (kinetic energy as in move_predict: ke = kp + kw, tempnow = ke*1000/(3 R (nfree + 2 nrig)),
    src/move.f90:69-102,379).  Returns the factor applied."""
    kp = float((s.mi[s.nriga:s.nliqa] * (s.xd[0, :, s.nriga:s.nliqa] ** 2).sum(0)).sum())
    if s.nrig:
        kp += s.mw * float((s.c[1] ** 2).sum())
        kw = s.inxx * float((s.w[0, 0] ** 2).sum()) + s.inyy * float((s.w[0, 1] ** 2).sum()) + \
            s.inzz * float((s.w[0, 2] ** 2).sum())
    else:
        kw = 0.0
    _rescale_shake_atoms(s, T)
    ndf = (s.nliqa - s.nriga) + 2 * s.nrig
    if ndf == 0 or kp + kw <= 0:
        return 1.0
    tnow = (kp + kw) * 1000.0 / (3.0 * S.PH_R * ndf)
    lam = math.sqrt(T / tnow)
    s.xd[:, :, s.nriga:s.nliqa] *= lam
    if s.nrig:
        s.c[1:] *= lam
        s.w *= lam
        s.q[1:] *= lam
    return lam


def _rescale_shake_atoms(s: S.System, T: float) -> float:
    """Verlet (SHAKE) atoms carry their velocity as the displacement x - xold: scale it to the
    temperature tkps = sum m d^2 1000 / (R nfreed) of move_shake (src/move.f90:416-439)."""
    lo, hi = s.nliqa, s.nmove
    if hi <= lo:
        return 1.0
    d = [s.x0[lo:hi] - s.xold[lo:hi], s.y0[lo:hi] - s.yold[lo:hi], s.z0[lo:hi] - s.zold[lo:hi]]
    d[0] -= s.lx * np.rint(d[0] / s.lx)
    d[1] -= s.ly * np.rint(d[1] / s.ly)
    k = float((s.mi[lo:hi] * (d[0] ** 2 + d[1] ** 2 + d[2] ** 2)).sum())
    nfreed = 3 * (hi - lo) - sum(int(s.nt[it]) * int(s.nconst[it]) for it in range(s.ntype) if s.moltypen[it] == 2)
    if nfreed <= 0 or k <= 0:
        return 1.0
    lam = math.sqrt(T / (k * 1000.0 / (S.PH_R * nfreed)))
    s.xold[lo:hi] = s.x0[lo:hi] - lam * d[0]
    s.yold[lo:hi] = s.y0[lo:hi] - lam * d[1]
    s.zold[lo:hi] = s.z0[lo:hi] - lam * d[2]
    return lam


def equilibrate(ctx, s: S.System, steps: int = 400, T: float = 300.0, every: int = 20) -> S.System:
    """Short MD with velocity rescaling every `every` steps through a resident-mode context
    (GPU or oracle), to take the synthetic lattice/placement starts to a stable state."""
    ctx.set_state(s)
    done = 0
    while done < steps:
        ctx.run(every)
        ctx.get_state(s)
        rescale_velocities(s, T)
        ctx.set_state(s)
        done += every
    return s


def ion_lattice(n_side: int = 6, spacing: float = 2.8, rcut: float = 2.0, alpha: float = 0.35,
                kmax: int = 6, seed: int = 21, jitter: float = 0.2,
                shuffle: bool = False) -> Tuple[S.System, RunParams]:
    """Rocksalt arrangement of +1/-1 point ions (two atmol types, no vdW) in a cubic periodic box,
    jittered; rcut below the closest approach so that the real-space sum is empty and the
    forces of force_get are the reciprocal-space forces alone.  shuffle=True deals the charges to
    the lattice sites at random (still neutral): the alternating crystal's reciprocal forces
    nearly cancel, the shuffled one's are of the order of the single terms."""
    n = n_side ** 3
    if n % 2:
        raise ValueError("n_side must be even")
    L = n_side * spacing
    g = np.stack(np.meshgrid(*[np.arange(n_side)] * 3, indexing="ij"), -1).reshape(-1, 3)
    par = g.sum(1) % 2
    rng = np.random.default_rng(seed)
    if shuffle:
        par = rng.permutation(par)
    pos = g * spacing + rng.uniform(-jitter, jitter, size=(n, 3)) - 0.5 * L
    cat = S.MolType("Na", "atmol", int((par == 0).sum()), ["Na"], [1], [22.99e-3], [1.0], ns=1)
    an = S.MolType("Cl", "atmol", int((par == 1).sum()), ["Cl"], [1], [35.45e-3], [-1.0], ns=1)
    crys = S.MolType("none", "crystal", 1, ["X1", "X2"], [1, 1], [1e-3, 1e-3], [0.0, 0.0], ns=0,
                     cx=L, cy=L, cz=L, lw=L)
    fld = S.FieldFile([cat, an, crys], _vdw_table(["Na", "Cl", "X1", "X2"], {}))
    s = S.System(fld, S.TopFile([], [], [], []), L, L, L, 1.0)
    order = np.concatenate([np.nonzero(par == 0)[0], np.nonzero(par == 1)[0]])
    s.x0[:n], s.y0[:n], s.z0[:n] = pos[order].T
    s.temper = -1.0
    prm = RunParams(rcut=rcut, skin=0.1, kmax=kmax, alpha=alpha, variant=MDG_BULK, pbc_z_list=1)
    return s, prm
