"""System description for the md_sim hot path: reference-format readers/writers and the
derived tables the force, neighbour-list and SHAKE routines read.

This is the caller side of the drop-in boundary.  In the reference the same tables are built by
  sysdef_input / sysdef_init   src/sysdef.f90:83-340, :356-457
  config_input / config_init   src/config.f90:174-242, :55-95 (+ config_quatsite :303-329)
and live in Fortran module globals.  Here they are numpy arrays held by `System`, laid out as the
Fortran modules hold them (1-based atom/type ids inside integer arrays, column-major 2-D tables),
so that `mdgpu.Context` can hand them to the C ABI unchanged.

Physical constants are single-precision literals stored in real*8 in the reference
(src/global.f90:18-24); `f32()` reproduces that rounding.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional

import numpy as np

SMX = 3


def f32(x: float) -> float:
    """Value of a default-real (single-precision) Fortran literal promoted to real*8."""
    return float(np.float32(x))


# src/global.f90:18-24
M_PI = f32(3.1415926535898)
PH_e = f32(1.6021892e-19)
PH_NA = f32(6.022045e23)
PH_R = f32(8.31441)
PH_eps0 = f32(8.85418782e-12)
PH_4epi = f32(8.987551784952e9)
PH_A2m = f32(1.0e-10)

MOLTYPEN = {"rigmol": 0, "atmol": 1, "surfmol": 2, "crystal": 3}


# ----------------------------------------------------------------------------------------------
# Fortran list-directed reading
# ----------------------------------------------------------------------------------------------
class _Records:
    """Record reader with Fortran list-directed semantics: every READ starts on a new record,
    takes blank-separated items across as many records as it needs (blank records carry no
    items) and drops the rest of the last record it touched."""

    def __init__(self, text: str):
        self.lines = text.splitlines()
        self.pos = 0

    def read(self, n: int) -> List[str]:
        items: List[str] = []
        while len(items) < n:
            if self.pos >= len(self.lines):
                raise EOFError("unexpected end of file")
            toks = self.lines[self.pos].replace(",", " ").split()
            self.pos += 1
            items.extend(toks)
        return items[:n]

    def skip(self) -> None:
        """READ with an empty list: skips exactly one record."""
        self.pos += 1


def _fnum(s: str) -> float:
    return float(s.replace("D", "E").replace("d", "e"))


def _inum(s: str) -> int:
    return int(float(s)) if ("." in s or "e" in s.lower()) else int(s)


# ----------------------------------------------------------------------------------------------
# Raw file contents
# ----------------------------------------------------------------------------------------------
@dataclasses.dataclass
class MolType:
    name: str
    kind: str  # rigmol / atmol / surfmol / crystal
    nt: int
    sitnam: List[str]
    nss: List[int]
    ms: List[float]  # site masses as read (kg/mol)
    qms: List[float]
    ns: int = 0
    geometry: Optional[np.ndarray] = None  # rigmol: (ns, 3)
    lengths: List[float] = dataclasses.field(default_factory=list)
    angles: List[tuple] = dataclasses.field(default_factory=list)  # (kt, theta_deg)
    cx: float = 0.0
    cy: float = 0.0
    cz: float = 0.0
    lw: float = 0.0
    qshift: List[float] = dataclasses.field(default_factory=list)


@dataclasses.dataclass
class VdwEntry:
    ijt: int
    ix: int
    jx: int
    kind: str  # zero / LeJo / Buck (12-6 is converted to LeJo on read)
    p: tuple


@dataclasses.dataclass
class FieldFile:
    moltypes: List[MolType]
    vdw: List[VdwEntry]


def parse_fld(text: str) -> FieldFile:
    """src/sysdef.f90:91-171."""
    r = _Records(text)
    r.read(1)
    ntype = _inum(r.read(1)[0])
    mts: List[MolType] = []
    for it in range(1, ntype + 1):
        r.read(1)
        ix, name, kind, nt = r.read(4)
        if _inum(ix) != it:
            raise ValueError("sysdef_input(): wrong molecule number!")
        r.read(1)
        nst = _inum(r.read(1)[0])
        sitnam, nss, ms, qms = [], [], [], []
        for _ in range(nst):
            a, b = r.read(2)
            sitnam.append(a)
            nss.append(_inum(b))
            m, q = r.read(2)
            ms.append(_fnum(m))
            qms.append(_fnum(q))
        mt = MolType(name, kind, _inum(nt), sitnam, nss, ms, qms, ns=sum(nss))
        if kind == "rigmol":
            r.read(1)
            g = [[_fnum(v) for v in r.read(3)] for _ in range(mt.ns)]
            mt.geometry = np.array(g, dtype=np.float64)
        elif kind == "atmol":
            pass
        elif kind == "surfmol":
            r.read(1)
            nc = _inum(r.read(1)[0])
            mt.lengths = [_fnum(r.read(1)[0]) for _ in range(nc)]
            r.read(1)
            na = _inum(r.read(1)[0])
            mt.angles = [tuple(_fnum(v) for v in r.read(2)) for _ in range(na)]
        elif kind == "crystal":
            mt.ns = _inum(r.read(1)[0])
            mt.cx, mt.cy, mt.cz = (_fnum(v) for v in r.read(3))
            mt.lw = _fnum(r.read(1)[0])
            nshift = _inum(r.read(1)[0])
            mt.qshift = [_fnum(r.read(1)[0]) for _ in range(nshift)]
        else:
            raise ValueError("sysdef_input(): Unknown moltype!")
        mts.append(mt)
    r.read(1)
    ntx = sum(len(m.nss) for m in mts)
    vdw: List[VdwEntry] = []
    for _ in range(ntx * (ntx + 1) // 2):
        ijt = _inum(r.read(1)[0])
        ix = _inum(r.read(3)[0])
        jx = _inum(r.read(3)[0])
        kind = r.read(1)[0]
        if kind == "zero":
            p: tuple = ()
        elif kind == "12-6":
            s, e = (_fnum(v) for v in r.read(2))
            six = (s / e) ** f32(1.0 / 6.0)
            epx = e**2 / (4.0 * s)
            kind, p = "LeJo", (six, epx)
        elif kind == "LeJo":
            p = tuple(_fnum(v) for v in r.read(2))
        elif kind == "Buck":
            p = tuple(_fnum(v) for v in r.read(3))
        else:
            raise ValueError("sysdef_input(): Unknown type of interaction!")
        vdw.append(VdwEntry(ijt, ix, jx, kind, p))
    return FieldFile(mts, vdw)


@dataclasses.dataclass
class TopFile:
    constr: List[List[tuple]]  # per constrained molecule: [(a, b), ...] 1-based
    ictype: List[int]
    angles: List[List[tuple]]  # per angle molecule: [(i, j, k), ...]
    iatype: List[int]


def parse_top(text: str, fld: FieldFile) -> TopFile:
    """src/sysdef.f90:174-219."""
    r = _Records(text)
    r.read(1)
    constr, ictype, angles, iatype = [], [], [], []
    for it, mt in enumerate(fld.moltypes, start=1):
        ix, mname, mtype, ntx = r.read(4)
        if _inum(ix) != it or mname != mt.name or mtype != mt.kind or _inum(ntx) != mt.nt:
            raise ValueError("sysdef_input(): Error in topofile!")
        if mtype == "rigmol":
            nsx = _inum(r.read(2)[1])
            if nsx != mt.ns:
                raise ValueError("sysdef_input(): Error in topofile (sites)!")
        elif mtype == "atmol":
            r.read(1)
        elif mtype == "surfmol":
            nsx = _inum(r.read(2)[1])
            if nsx != len(mt.lengths):
                raise ValueError("sysdef_input(): Error in topofile (nconst)!")
            for _ in range(mt.nt):
                constr.append([tuple(_inum(v) for v in r.read(2)) for _ in range(nsx)])
                ictype.append(it)
            nsx = _inum(r.read(2)[1])
            if nsx != len(mt.angles):
                raise ValueError("sysdef_input(): Error in topofile (nangt)!")
            if nsx > 0:
                for _ in range(mt.nt):
                    angles.append([tuple(_inum(v) for v in r.read(3)) for _ in range(nsx)])
                    iatype.append(it)
    return TopFile(constr, ictype, angles, iatype)


@dataclasses.dataclass
class InpFile:
    ensemble: str
    temper: float
    timeq: float
    timrun: float
    dt: float
    timprn: float
    rcut: float
    kmax: int
    skin: float
    rdel: float
    filname: str


def parse_inp(text: str) -> InpFile:
    """src/main.f90:121-155 (the optional analysis lines are skipped by their flags)."""
    r = _Records(text)
    ens = r.read(2)[1]
    temper = _fnum(r.read(2)[1]) if ens == "nvt" else -1.0
    _, timeq, timrun, dt = r.read(4)
    timprn = _fnum(r.read(2)[1])
    rcut = _fnum(r.read(2)[1])
    kmax = _inum(r.read(2)[1])
    skin = _fnum(r.read(2)[1])
    rdel = _fnum(r.read(2)[1])

    def flag() -> bool:
        return r.read(2)[1].upper().lstrip(".").startswith("T")

    l2d, lhb = flag(), flag()
    if l2d or lhb:
        r.read(3)
    if lhb:
        r.read(2)
    if flag():  # ldiff
        r.read(4)
    if flag():  # lcouett
        raise ValueError("Couette-pulled walls are outside this library")
    if flag():  # lfext
        r.read(4)
    if flag():  # lchempot
        r.read(2)
        r.read(5)
    filname = r.read(2)[1]
    return InpFile(ens, temper, _fnum(timeq), _fnum(timrun), _fnum(dt), timprn, rcut, kmax, skin,
                   rdel, filname)


# ----------------------------------------------------------------------------------------------
# Derived system (sysdef_init + config_init)
# ----------------------------------------------------------------------------------------------
class System:
    """Tables and state after sysdef_init/config_init, in the reference's layout.

    Integer arrays are int64 (the reference's integer*8) with 1-based ids; 2-D tables are
    column-major (Fortran order) flattened arrays."""

    def __init__(self, fld: FieldFile, top: TopFile, lx: float, ly: float, lz: float, dt: float):
        mts = fld.moltypes
        self.fld, self.top = fld, top
        self.ntype = len(mts)
        self.dt = float(dt)
        self.lx, self.ly, self.lz = float(lx), float(ly), float(lz)
        kinds = [m.kind for m in mts]
        self.moltypen = np.array([MOLTYPEN[k] for k in kinds], dtype=np.int64)
        nrtype = nltype = nstype = nwtype = 0
        for it, k in enumerate(kinds, start=1):
            if k == "rigmol":
                nrtype = nltype = it
            elif k == "atmol":
                nltype = it
            elif k == "surfmol":
                nstype = it
            elif k == "crystal":
                nwtype = it
        if nwtype != self.ntype:
            raise ValueError("the crystal must be the last molecule type")
        self.nrtype, self.nltype, self.nstype, self.nwtype = nrtype, nltype, nstype, nwtype
        nt = np.array([m.nt for m in mts], dtype=np.int64)
        ns = np.array([m.ns for m in mts], dtype=np.int64)
        nst = np.array([len(m.nss) for m in mts], dtype=np.int64)
        self.nt, self.ns, self.nst = nt, ns, nst
        if nt[nwtype - 1] > 1:
            raise ValueError("sysdef_init(): wrong number of crystals")
        # src/sysdef.f90:299-319
        self.nrig = int(nt[:nrtype].sum())
        self.nriga = int((ns[:nrtype] * nt[:nrtype]).sum())
        self.nliqa = int((ns[:nltype] * nt[:nltype]).sum())
        self.nsurf = int((ns[nltype:nstype] * nt[nltype:nstype]).sum()) if nstype > nltype else 0
        self.nmove = self.nliqa + self.nsurf
        self.nwall = int(ns[nwtype - 1] * nt[nwtype - 1])
        self.ngogo = self.nmove
        self.ntota = self.nmove + self.nwall
        self.nit = int(nst.sum())
        self.nijt = self.nit * (self.nit + 1) // 2
        self.ncons = len(top.constr)
        self.nang = len(top.angles)
        self.nconst = np.array([len(m.lengths) for m in mts], dtype=np.int64)
        self.nangt = np.array([len(m.angles) for m in mts], dtype=np.int64)
        crys = mts[nwtype - 1]
        self.nss_wall = np.array([crys.nss[0] if len(crys.nss) > 0 else 0,
                                  crys.nss[1] if len(crys.nss) > 1 else 0], dtype=np.int64)
        self.cx, self.cy, self.cz, self.lw = crys.cx, crys.cy, crys.cz, crys.lw
        self.lwh = 0.5 * self.lw

        # vdW tables (src/sysdef.f90:143-169, :321-335, :362-374)
        nit, nijt = self.nit, self.nijt
        ijtype = np.zeros((nit, nit), dtype=np.int64)
        ijt = 0
        for it in range(nit):
            for jt in range(it, nit):
                ijt += 1
                ijtype[it, jt] = ijt
                ijtype[jt, it] = ijt
        self.ijtype = ijtype.flatten(order="F")
        self.vdwnum = np.full(nijt, -1, dtype=np.int64)
        eps = np.zeros(nijt)
        sig = np.zeros(nijt)
        aa = np.zeros(nijt)
        rhoi = np.zeros(nijt)
        cc = np.zeros(nijt)
        for v in fld.vdw:
            k = v.ijt - 1
            if v.kind == "zero":
                self.vdwnum[k] = 0
            elif v.kind == "LeJo":
                self.vdwnum[k] = 1
                sig[k], eps[k] = v.p
            elif v.kind == "Buck":
                self.vdwnum[k] = 2
                aa[k], rhoi[k], cc[k] = v.p
        eps = 4.0 * eps
        sig = sig**6
        rhoi = np.where(rhoi != 0.0, 1.0 / np.where(rhoi != 0.0, rhoi, 1.0), 0.0)
        self.eps, self.sig, self.aa, self.rhoi, self.cc = eps, sig, aa, rhoi, cc

        # units: src/sysdef.f90:376-379
        v_unit = PH_A2m / (self.dt * f32(1.0e-15))
        ms = [[m_ * v_unit**2 / 1000.0 for m_ in m.ms] for m in mts]
        self.ms_internal = ms

        # per-atom tables: src/sysdef.f90:381-425
        ntota, nmove = self.ntota, self.nmove
        self.itype = np.zeros(ntota, dtype=np.int64)
        self.qs = np.zeros(ntota)
        self.mi = np.zeros(ntota)
        nsi = np.zeros(nit, dtype=np.int64)
        i = 0
        jjt = 0
        for it in range(max(nltype, nstype)):
            m = mts[it]
            for _ in range(m.nt):
                for ist in range(len(m.nss)):
                    iit = jjt + ist + 1
                    if self.moltypen[it] == 0:
                        nsi[iit - 1] = m.ns if ist == 0 else 0
                    else:
                        nsi[iit - 1] = 1
                    for _ in range(m.nss[ist]):
                        self.itype[i] = iit
                        self.mi[i] = ms[it][ist]
                        self.qs[i] = m.qms[ist]
                        i += 1
            jjt += len(m.nss)
        if i != nmove:
            raise ValueError("sysdef_init(): i /= nmove !")
        self.nsi = nsi
        self.jjt_wall = jjt
        self.mii = np.zeros(ntota)
        self.mii[:nmove] = 1.0 / self.mi[:nmove]

        # theta in radians (src/sysdef.f90:376)
        ntype = self.ntype
        self.length = np.zeros((ntype, SMX))
        self.kt = np.zeros((ntype, SMX))
        self.theta = np.zeros((ntype, SMX))
        for it, m in enumerate(mts):
            for s, L in enumerate(m.lengths):
                self.length[it, s] = L
            for s, (k_, th) in enumerate(m.angles):
                self.kt[it, s] = k_
                self.theta[it, s] = th * M_PI / 180.0
        self.constra = np.zeros((SMX, max(self.ncons, 1)), dtype=np.int64)
        self.constrb = np.zeros((SMX, max(self.ncons, 1)), dtype=np.int64)
        for ic, cl in enumerate(top.constr):
            for s, (a, b) in enumerate(cl):
                self.constra[s, ic] = a
                self.constrb[s, ic] = b
        self.ictype = np.array(top.ictype if top.ictype else [0], dtype=np.int64)
        self.ang = np.zeros((3, SMX, max(self.nang, 1)), dtype=np.int64)
        for ia, al in enumerate(top.angles):
            for s, (a, b, c) in enumerate(al):
                self.ang[:, s, ia] = (a, b, c)
        self.iatype = np.array(top.iatype if top.iatype else [0], dtype=np.int64)

        # rigid water geometry: src/sysdef.f90:427-452
        self.xbody = np.zeros(SMX)
        self.ybody = np.zeros(SMX)
        self.zbody = np.zeros(SMX)
        self.mw = 0.0
        self.inxx = self.inyy = self.inzz = 0.0
        if mts[0].kind == "rigmol":
            m = mts[0]
            g = m.geometry.copy()
            mm = self.mi[0:m.ns]
            for d in range(3):
                g[:, d] = g[:, d] - (g[:, d] * mm).sum() / mm.sum()
            self.inxx = float((mm * (g[:, 1] ** 2 + g[:, 2] ** 2)).sum())
            self.inyy = float((mm * (g[:, 2] ** 2 + g[:, 0] ** 2)).sum())
            self.inzz = float((mm * (g[:, 0] ** 2 + g[:, 1] ** 2)).sum())
            self.mw = float(sum(n_ * w for n_, w in zip(m.nss, ms[0])))
            self.xbody[:m.ns] = g[:, 0]
            self.ybody[:m.ns] = g[:, 1]
            self.zbody[:m.ns] = g[:, 2]

        # state arrays (src/config.f90:20-51)
        self.x0 = np.zeros(ntota)
        self.y0 = np.zeros(ntota)
        self.z0 = np.zeros(ntota)
        self.xd = np.zeros((4, 3, ntota))  # x1..x4, y1..y4, z1..z4 of flexible atoms
        nrig = self.nrig
        self.c = np.zeros((5, 3, nrig))  # cx0..cx4
        self.q = np.zeros((5, 4, nrig))  # q10..q44 : [deriv, component]
        self.w = np.zeros((5, 3, nrig))  # wx0..wx4
        self.xold = np.zeros(ntota)
        self.yold = np.zeros(ntota)
        self.zold = np.zeros(ntota)
        self.rsx = np.zeros(nmove)
        self.rsy = np.zeros(nmove)
        self.rsz = np.zeros(nmove)
        self.s = np.zeros(5)
        self.rs = np.zeros(5)
        self.temper = -1.0

    # ------------------------------------------------------------------ config handling
    def set_walls(self, wtype: np.ndarray, pos: np.ndarray) -> None:
        """Crystal sites: src/config.f90:460-471 + type remap src/sysdef.f90:406-419."""
        crys = self.fld.moltypes[self.nwtype - 1]
        nmove = self.nmove
        for k in range(self.nwall):
            i = nmove + k
            is_ = int(wtype[k])
            if is_ > 0:
                self.qs[i] = crys.qms[is_ - 1]
            else:
                self.qs[i] = crys.qshift[-is_ - 1]
                is_ = 1 if -is_ <= crys.nss[0] else 2
            self.itype[i] = self.jjt_wall + is_
        self.walltype = np.asarray(wtype, dtype=np.int64).copy()
        self.x0[nmove:] = pos[:, 0]
        self.y0[nmove:] = pos[:, 1]
        self.z0[nmove:] = pos[:, 2]

    def quatsite(self) -> None:
        """config_quatsite, src/config.f90:303-329 (rotation matrix + site positions)."""
        q1, q2, q3, q4 = self.q[0]
        a = np.empty((3, 3, self.nrig))
        a[0, 0] = -q1 * q1 + q2 * q2 - q3 * q3 + q4 * q4
        a[0, 1] = 2.0 * (q3 * q4 - q1 * q2)
        a[0, 2] = 2.0 * (q2 * q3 + q1 * q4)
        a[1, 0] = -2.0 * (q1 * q2 + q3 * q4)
        a[1, 1] = q1 * q1 - q2 * q2 - q3 * q3 + q4 * q4
        a[1, 2] = 2.0 * (q2 * q4 - q1 * q3)
        a[2, 0] = 2.0 * (q2 * q3 - q1 * q4)
        a[2, 1] = -2.0 * (q1 * q3 + q4 * q2)
        a[2, 2] = -q1 * q1 - q2 * q2 + q3 * q3 + q4 * q4
        self.amat = a
        for j in range(3):
            idx = np.arange(self.nrig) * 3 + j
            self.x0[idx] = self.c[0, 0] + a[0, 0] * self.xbody[j] + a[1, 0] * self.ybody[j] + a[2, 0] * self.zbody[j]
            self.y0[idx] = self.c[0, 1] + a[0, 1] * self.xbody[j] + a[1, 1] * self.ybody[j] + a[2, 1] * self.zbody[j]
            self.z0[idx] = self.c[0, 2] + a[0, 2] * self.xbody[j] + a[1, 2] * self.ybody[j] + a[2, 2] * self.zbody[j]

    def config_init(self) -> None:
        """src/config.f90:55-95: derivatives from 1 fs units to time-step units, then sites."""
        dt = self.dt
        for k in range(4):
            self.xd[k] *= dt ** (k + 1)
            self.c[k + 1] *= dt ** (k + 1)
        for k in range(5):
            self.w[k] *= dt ** (k + 1)
        if self.nrig:
            self.quatsite()

    def rsx_after_predict(self) -> None:
        """Site offsets move_predict writes (src/move.f90:157-161): H sites relative to O."""
        for j in (1, 2):
            idx = np.arange(self.nrig) * 3 + j
            self.rsx[idx] = self.x0[idx] - self.x0[idx - j]
            self.rsy[idx] = self.y0[idx] - self.y0[idx - j]
            self.rsz[idx] = self.z0[idx] - self.z0[idx - j]

    def shake_init(self) -> None:
        """move_shake_init, src/move.f90:394-396: previous positions of the surface and wall
        atoms start equal to the current ones (the values read from the .cfg are dropped)."""
        nl = self.nliqa
        self.xold[nl:] = self.x0[nl:]
        self.yold[nl:] = self.y0[nl:]
        self.zold[nl:] = self.z0[nl:]

    def copy(self) -> "System":
        other = System.__new__(System)
        for k, v in self.__dict__.items():
            setattr(other, k, v.copy() if isinstance(v, np.ndarray) else v)
        return other

    # ------------------------------------------------------------------ summaries
    @property
    def heads(self) -> np.ndarray:
        """0-based indices of moving atoms that carry a molecule (nsi /= 0)."""
        t = self.itype[: self.nmove] - 1
        return np.nonzero(self.nsi[t] != 0)[0]

    def describe(self) -> Dict[str, int]:
        return dict(nrig=self.nrig, nriga=self.nriga, nliqa=self.nliqa, nsurf=self.nsurf,
                    nmove=self.nmove, nwall=self.nwall, ntota=self.ntota, nit=self.nit,
                    ncons=self.ncons, nang=self.nang)


def parse_cfg(text: str, fld: FieldFile, top: TopFile, dt: float) -> System:
    """config_input, src/config.f90:174-242, then sysdef_init + config_init."""
    r = _Records(text)
    r.read(1)
    lx, ly, lz = (_fnum(v) for v in r.read(3))
    r.skip()
    r.read(1)
    if _inum(r.read(1)[0]) != len(fld.moltypes):
        raise ValueError("config_input(): wrong number of types!")
    r.skip()
    r.read(1)
    sys_ = System(fld, top, lx, ly, lz, dt)
    wtype = np.zeros(sys_.nwall, dtype=np.int64)
    wpos = np.zeros((sys_.nwall, 3))
    for it, m in enumerate(fld.moltypes):
        mname, mtype, ntx = r.read(3)
        if mname != m.name or mtype != m.kind or _inum(ntx) != m.nt:
            raise ValueError("config_input(): Error in configfile!")
        if m.kind == "rigmol":
            for _ in range(m.nt):
                i = _inum(r.read(1 + m.ns)[0]) - 1
                for k in range(5):
                    sys_.c[k, :, i] = [_fnum(v) for v in r.read(3)]
                for k in range(5):
                    sys_.q[k, :, i] = [_fnum(v) for v in r.read(4)]
                for k in range(5):
                    sys_.w[k, :, i] = [_fnum(v) for v in r.read(3)]
        elif m.kind == "atmol":
            for _ in range(m.nt * m.ns):
                i = _inum(r.read(2)[0]) - 1
                sys_.x0[i], sys_.y0[i], sys_.z0[i] = (_fnum(v) for v in r.read(3))
                for k in range(4):
                    sys_.xd[k, :, i] = [_fnum(v) for v in r.read(3)]
        elif m.kind == "surfmol":
            for _ in range(m.nt * m.ns):
                i = _inum(r.read(2)[0]) - 1
                x, y, z = (_fnum(v) for v in r.read(3))
                sys_.x0[i], sys_.y0[i], sys_.z0[i] = x, y, z
                xo, yo, zo = (_fnum(v) for v in r.read(3))
                sys_.xold[i] = x + (xo - x) * dt
                sys_.yold[i] = y + (yo - y) * dt
                sys_.zold[i] = z + (zo - z) * dt
        elif m.kind == "crystal":
            for _ in range(m.nt * m.ns):
                a, b = r.read(2)
                k = _inum(a) - 1 - sys_.nmove
                wtype[k] = _inum(b)
                wpos[k] = [_fnum(v) for v in r.read(3)]
        r.skip()
    r.read(1)
    sys_.s[:] = [_fnum(v) for v in r.read(5)]
    sys_.rs[:] = [_fnum(v) for v in r.read(5)]
    if sys_.nwall:
        sys_.set_walls(wtype, wpos)
    sys_.config_init()
    return sys_


def load_reference_case(directory: str, base: str = "y"):
    """Reads <base>.inp/.fld/.top/.cfg of a reference case directory."""
    import os

    with open(os.path.join(directory, base + ".inp")) as fh:
        inp = parse_inp(fh.read())
    with open(os.path.join(directory, base + ".fld")) as fh:
        fld = parse_fld(fh.read())
    with open(os.path.join(directory, base + ".top")) as fh:
        top = parse_top(fh.read(), fld)
    with open(os.path.join(directory, base + ".cfg")) as fh:
        sys_ = parse_cfg(fh.read(), fld, top, inp.dt)
    sys_.temper = inp.temper
    return inp, sys_


# ----------------------------------------------------------------------------------------------
# Writers (reference formats) -- used to hand the synthetic configs to a Fortran build
# ----------------------------------------------------------------------------------------------
def write_fld(fld: FieldFile) -> str:
    out = ["# MOLECULES", f"  {len(fld.moltypes)}"]
    for it, m in enumerate(fld.moltypes, start=1):
        out += [" # Molecule", f" {it} {m.name} {m.kind} {m.nt}", " # sites", f"  {len(m.nss)}"]
        for s, n, mm, q in zip(m.sitnam, m.nss, m.ms, m.qms):
            out += [f"{s} {n}", f" {mm!r} {q!r}"]
        if m.kind == "rigmol":
            out.append(" # geometry")
            out += [" " + " ".join(repr(float(v)) for v in row) for row in m.geometry]
        elif m.kind == "surfmol":
            out += [" # constraints", f"  {len(m.lengths)}"] + [f"  {L!r}" for L in m.lengths]
            out += [" # angles", f"  {len(m.angles)}"] + [f"  {a!r} {b!r}" for a, b in m.angles]
        elif m.kind == "crystal":
            out += [f"  {m.ns}", f" {m.cx!r} {m.cy!r} {m.cz!r}", f" {m.lw!r}", f"  {len(m.qshift)}"]
            out += [f" {q!r}" for q in m.qshift]
    out.append(" # VDW INTERACTIONS")
    names = [(m.name, s) for m in fld.moltypes for s in m.sitnam]
    for v in fld.vdw:
        out += [f"  {v.ijt}", f"  {v.ix} {names[v.ix-1][0]} {names[v.ix-1][1]}",
                f"  {v.jx} {names[v.jx-1][0]} {names[v.jx-1][1]}", v.kind]
        if v.p:
            out.append(" " + " ".join(repr(float(x)) for x in v.p))
        out.append(" ")
    return "\n".join(out) + "\n"


def write_top(fld: FieldFile, top: TopFile) -> str:
    out = [" # Atom connections, specific interactions"]
    ic = ia = 0
    for it, m in enumerate(fld.moltypes, start=1):
        out.append(f" {it} {m.name} {m.kind} {m.nt}")
        if m.kind == "rigmol":
            out.append(f" sites: {m.ns}")
        elif m.kind == "atmol":
            out.append(" no connections")
        elif m.kind == "surfmol":
            out.append(f" constraints: {len(m.lengths)}")
            for _ in range(m.nt):
                out += [f" {a} {b}" for a, b in top.constr[ic]]
                ic += 1
            out.append(f" angles: {len(m.angles)}")
            if m.angles:
                for _ in range(m.nt):
                    out += [f" {a} {b} {c}" for a, b, c in top.angles[ia]]
                    ia += 1
    return "\n".join(out) + "\n"


def write_cfg(s: System) -> str:
    """Text configuration in the layout config_input reads (full precision, 1 fs units)."""
    dt = s.dt
    out = [" # SIMULATION BOX SIZE", f" {s.lx!r} {s.ly!r} {s.lz!r}", " ",
           " # NUMBER OF PARTICLE TYPES", f" {s.ntype}", " ", " # PARTICLE COORDINATES"]

    def row(v):
        return " " + " ".join(repr(float(x)) for x in v)

    atom = 0
    for m in s.fld.moltypes:
        out.append(f" {m.name} {m.kind} {m.nt}")
        if m.kind == "rigmol":
            for i in range(m.nt):
                out.append(f" {i+1} " + " ".join(str(int(t)) for t in s.itype[3*i:3*i+m.ns]))
                out.append(row(s.c[0, :, i]))
                for k in range(1, 5):
                    out.append(row(s.c[k, :, i] / dt**k))
                for k in range(5):
                    out.append(row(s.q[k, :, i]))
                for k in range(5):
                    out.append(row(s.w[k, :, i] / dt ** (k + 1)))
            atom += m.nt * m.ns
        elif m.kind == "atmol":
            first = s.itype[atom] - 1 if m.nt else 0
            for i in range(atom, atom + m.nt * m.ns):
                out.append(f" {i+1} {int(s.itype[i] - first)}")
                out.append(row([s.x0[i], s.y0[i], s.z0[i]]))
                for k in range(4):
                    out.append(row(s.xd[k, :, i] / dt ** (k + 1)))
            atom += m.nt * m.ns
        elif m.kind == "surfmol":
            first = s.itype[atom] - 1 if m.nt else 0
            for i in range(atom, atom + m.nt * m.ns):
                out.append(f" {i+1} {int(s.itype[i] - first)}")
                out.append(row([s.x0[i], s.y0[i], s.z0[i]]))
                out.append(row([s.x0[i] + (s.xold[i] - s.x0[i]) / dt,
                                s.y0[i] + (s.yold[i] - s.y0[i]) / dt,
                                s.z0[i] + (s.zold[i] - s.z0[i]) / dt]))
            atom += m.nt * m.ns
        elif m.kind == "crystal":
            for k in range(s.nwall):
                i = s.nmove + k
                out.append(f" {i+1} {int(s.walltype[k])}")
                out.append(row([s.x0[i], s.y0[i], s.z0[i]]))
        out.append(" ")
    out += [" # THERMOSTAT", row(s.s), row(s.rs)]
    return "\n".join(out) + "\n"
