"""ctypes mirror of include/mdgpu.h and a thin host-side wrapper around one context.

`Context` plays the role of the Fortran caller: it owns the host arrays the reference keeps in
module globals (positions, site offsets, forces, SHAKE old positions) and passes them to
  mdg_create      <- force_init + nnlist_init + move_shake_init  (src/forcem.f90:54-81)
  mdg_force_get   <- force_get                                   (src/forcem.f90:93-129)
  mdg_nnlist_make <- nnlist_make                                 (src/nnlist.f90:92-165)
  mdg_shake       <- move_shake                                  (src/move.f90:408-529)
The same wrapper drives any library exporting these entry points under another prefix.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import weakref
from typing import Dict, Optional

import numpy as np

from .system import System

I64P = C.POINTER(C.c_int64)
DP = C.POINTER(C.c_double)

MDG_OK = 0
MDG_SLAB, MDG_BULK = 0, 1
MDG_FP64, MDG_MIXED = 0, 1
MDG_BATCH_GRAPHS, MDG_BATCH_PHASES = 0, 1
MDG_QUIRK_CLEAN_SHAKE_DONE = 1

ERRORS = {
    -1: "MDG_E_ARG", -2: "MDG_E_CUDA", -3: "MDG_E_LIST_OVERFLOW", -4: "MDG_E_SHAKE_MAXIT",
    -5: "MDG_E_SHAKE_RPTOL", -6: "MDG_E_NAN", -7: "MDG_E_UNSUPPORTED",
}


class MdgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class SysDesc(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "ntype", "nrig", "nriga", "nliqa", "nsurf", "nmove", "nwall", "ntota", "ngogo",
        "nit", "nijt", "nltype", "ncons", "nang")] + [
        ("moltypen", I64P), ("nt", I64P), ("ns", I64P), ("nst", I64P), ("nconst", I64P),
        ("nangt", I64P), ("nss_wall", I64P), ("nsi", I64P), ("ijtype", I64P), ("vdwnum", I64P),
        ("eps", DP), ("sig", DP), ("aa", DP), ("rhoi", DP), ("cc", DP),
        ("itype", I64P), ("qs", DP), ("mi", DP), ("mii", DP),
        ("ictype", I64P), ("constra", I64P), ("constrb", I64P), ("length", DP),
        ("iatype", I64P), ("ang1", I64P), ("ang2", I64P), ("ang3", I64P), ("kt", DP),
        ("theta", DP),
        ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
        ("cx", C.c_double), ("cy", C.c_double), ("cz", C.c_double), ("lw", C.c_double),
        ("dt", C.c_double)]


class Params(C.Structure):
    _fields_ = [
        ("rcut", C.c_double), ("skin", C.c_double), ("alpha", C.c_double), ("kmax", C.c_int64),
        ("dshsq", C.c_double), ("variant", C.c_int32), ("pbc_z_list", C.c_int32),
        ("precision", C.c_int32), ("quirks", C.c_uint32), ("list_capacity", C.c_int64),
        ("wlist_capacity", C.c_int64), ("shake_maxit", C.c_int32), ("shake_tol2", C.c_double),
        ("shake_rptol", C.c_double)]


class Energies(C.Structure):
    _fields_ = [("elj", DP), ("eqq", DP)] + [(n, C.c_double) for n in (
        "uewa", "urf", "ulr", "uself", "uconf", "uavex", "press", "vir", "ewqLL", "ewqWL",
        "ewqWW")] + [("fwsx", C.c_double * 3), ("fwsy", C.c_double * 3), ("fwsz", C.c_double * 3)]


class State(C.Structure):
    _fields_ = [("x0", DP), ("y0", DP), ("z0", DP), ("xd", DP * 4), ("yd", DP * 4), ("zd", DP * 4),
                ("cx", DP * 5), ("cy", DP * 5), ("cz", DP * 5), ("q", (DP * 5) * 4),
                ("wx", DP * 5), ("wy", DP * 5), ("wz", DP * 5), ("xold", DP), ("yold", DP),
                ("zold", DP), ("rsx", DP), ("rsy", DP), ("rsz", DP), ("s", C.c_double * 5),
                ("rs", C.c_double * 5)]


class Rigid(C.Structure):
    _fields_ = [("xbody", C.c_double * 3), ("ybody", C.c_double * 3), ("zbody", C.c_double * 3),
                ("mw", C.c_double), ("inxx", C.c_double), ("inyy", C.c_double), ("inzz", C.c_double),
                ("temper", C.c_double)]


class Report(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("kp", "kw", "ke", "htot", "tempnow", "uconf", "tkps", "press")] + [
        ("steps", C.c_int64), ("rebuilds", C.c_int64), ("last_sweeps", C.c_int32)]


@dataclasses.dataclass
class RunParams:
    rcut: float
    skin: float
    kmax: int
    alpha: float = 0.0
    variant: int = MDG_SLAB
    pbc_z_list: int = 0
    precision: int = MDG_FP64
    quirks: int = 0
    dshsq: float = 0.0
    list_capacity: int = 0
    wlist_capacity: int = 0
    shake_maxit: int = 0
    shake_tol2: float = 0.0
    shake_rptol: float = 0.0

    def to_c(self) -> Params:
        return Params(self.rcut, self.skin, self.alpha, self.kmax, self.dshsq, self.variant,
                      self.pbc_z_list, self.precision, self.quirks, self.list_capacity,
                      self.wlist_capacity, self.shake_maxit, self.shake_tol2, self.shake_rptol)


def _p(a: np.ndarray, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def make_sysdesc(s: System):
    """Builds the C description; returns (struct, keep-alive list)."""
    keep = []

    def i64(a):
        a = np.ascontiguousarray(np.asarray(a, dtype=np.int64))
        keep.append(a)
        return _p(a, C.c_int64)

    def f64(a):
        a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
        keep.append(a)
        return _p(a, C.c_double)

    nstw = int(s.nst[s.ntype - 1])
    crys = s.fld.moltypes[s.ntype - 1]
    nss_wall = list(crys.nss) + [0] * max(0, 2 - len(crys.nss))
    d = SysDesc(
        s.ntype, s.nrig, s.nriga, s.nliqa, s.nsurf, s.nmove, s.nwall, s.ntota, s.ngogo,
        s.nit, s.nijt, s.nltype, s.ncons, s.nang,
        i64(s.moltypen), i64(s.nt), i64(s.ns), i64(s.nst), i64(s.nconst), i64(s.nangt),
        i64(nss_wall[:max(2, nstw)]), i64(s.nsi), i64(s.ijtype), i64(s.vdwnum),
        f64(s.eps), f64(s.sig), f64(s.aa), f64(s.rhoi), f64(s.cc),
        i64(s.itype), f64(s.qs), f64(s.mi), f64(s.mii),
        i64(s.ictype), i64(s.constra.flatten(order="F")), i64(s.constrb.flatten(order="F")),
        f64(s.length.flatten(order="F")),
        i64(s.iatype), i64(s.ang[0].flatten(order="F")), i64(s.ang[1].flatten(order="F")),
        i64(s.ang[2].flatten(order="F")), f64(s.kt.flatten(order="F")),
        f64(s.theta.flatten(order="F")),
        s.lx, s.ly, s.lz, s.cx, s.cy, s.cz, s.lw, s.dt)
    return d, keep


class MeasureParams(C.Structure):
    _fields_ = [("rdel", C.c_double), ("force_hist", C.c_int32), ("profiles", C.c_int32), ("l2d", C.c_int32),
                ("pad", C.c_int32), ("rfrst", C.c_double), ("rscnd", C.c_double)]


class MeasureDims(C.Structure):
    _fields_ = [("lmax", C.c_int64), ("nijt", C.c_int64), ("ntz", C.c_int64), ("langmax", C.c_int64),
                ("lgxmax", C.c_int64), ("lgymax", C.c_int64)]


class MeasureOut(C.Structure):
    _fields_ = [("ngc", I64P), ("efipos", DP), ("tefipos", DP), ("nefipos", I64P), ("ngang", I64P),
                ("ngz", I64P), ("ndipx", DP), ("ndipy", DP), ("ndipz", DP), ("ndipsq", DP),
                ("ng2d1", I64P), ("ng2d2", I64P), ("ftot", (C.c_double * 3) * 3), ("calls_force", C.c_int64),
                ("calls_do", C.c_int64), ("out_of_range", C.c_int64)]


MDG_WIDOM_SKIP_OVERLAP = 1
MDG_WIDOM_EW3DC = 2


class WidomParams(C.Structure):
    _fields_ = [("ichmax", C.c_int64), ("lwmin", C.c_double), ("lwmax", C.c_double), ("lchmax", C.c_int64),
                ("ilmid", C.c_int64), ("temper", C.c_double), ("flags", C.c_uint32), ("pad", C.c_int32)]


class Lib:
    """Binds the entry points of one shared library (`prefix` = 'mdg_' for the product)."""

    def __init__(self, path: str, prefix: str = "mdg_"):
        self.path = path
        self.prefix = prefix
        self.so = C.CDLL(path)
        g = self.fn
        g("create", C.c_int, [C.POINTER(SysDesc), C.POINTER(Params)] + [DP] * 6 + [C.POINTER(C.c_void_p)])
        g("destroy", None, [C.c_void_p])
        g("last_error", C.c_char_p, [C.c_void_p])
        g("nnlist_make", C.c_int, [C.c_void_p] + [DP] * 6 + [I64P, I64P])
        g("get_lists", C.c_int, [C.c_void_p, I64P, I64P, C.c_int64, I64P, I64P, C.c_int64, I64P, I64P])
        g("force_get", C.c_int, [C.c_void_p] + [DP] * 21 + [C.POINTER(Energies)])
        if self.has("kvectors"):
            I32P = C.POINTER(C.c_int32)
            g("kvectors", C.c_int64, [C.c_void_p, I32P, I32P, I32P, DP, C.c_int64])
        g("shake", C.c_int, [C.c_void_p] + [DP] * 10 + [C.POINTER(C.c_double), C.POINTER(C.c_int32)])
        if self.has("sysdef_load"):
            g("sysdef_load", C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_double, C.POINTER(C.c_void_p)])
            g("sysdef_desc", C.POINTER(SysDesc), [C.c_void_p])
            g("sysdef_rigid", C.POINTER(Rigid), [C.c_void_p])
            g("sysdef_state", C.POINTER(State), [C.c_void_p])
            g("sysdef_free", None, [C.c_void_p])
        if self.has("pin_host"):
            g("pin_host", C.c_int, [C.c_void_p, C.c_int64])
            g("unpin_host", C.c_int, [C.c_void_p])
        if self.has("set_stream"):
            g("set_stream", C.c_int, [C.c_void_p, C.c_void_p])
            g("phase_times", C.c_int, [C.c_void_p, C.c_int, DP])
        if self.has("run_async"):
            g("run_async", C.c_int, [C.c_void_p, C.c_int64])
            g("check", C.c_int, [C.c_void_p, C.POINTER(Report)])
            g("kernels_per_step", C.c_int64, [C.c_void_p])
        if self.has("mlp_nw"):
            FP = C.POINTER(C.c_float)
            g("mlp_nw", C.c_int, [])
            g("shake_set_model", C.c_int, [C.c_void_p, FP, C.c_int64])
            g("shake_record", C.c_int, [C.c_void_p, C.c_int])
            g("shake_samples", C.c_int, [C.c_void_p, FP])
            g("mlp_forward", C.c_int, [FP, FP, C.c_int64, FP])
            g("mlp_grad", C.c_int, [FP, FP, FP, C.c_int64, FP, FP])
            g("mlp_train", C.c_int, [FP, FP, C.c_int64, C.c_int, C.c_int, C.c_float, C.c_uint64, FP, FP])
        if self.has("autotune"):
            g("autotune", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p])
        if self.has("batch_create"):
            g("batch_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p)])
            g("batch_destroy", None, [C.c_void_p])
            g("batch_last_error", C.c_char_p, [C.c_void_p])
            g("batch_set_stream", C.c_int, [C.c_void_p, C.c_void_p])
            g("batch_run", C.c_int, [C.c_void_p, C.c_int64, C.c_void_p])
            g("batch_run_async", C.c_int, [C.c_void_p, C.c_int64])
        if self.has("batch_set_mode"):
            g("batch_set_mode", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int])
            g("batch_phased", C.c_int, [C.c_void_p])
        if self.has("measure_init"):
            g("measure_init", C.c_int, [C.c_void_p, C.POINTER(MeasureParams), C.POINTER(MeasureDims)])
            g("measure_enable", C.c_int, [C.c_void_p, C.c_int, C.c_int])
            g("measure_zero", C.c_int, [C.c_void_p])
            g("measure_do", C.c_int, [C.c_void_p, DP, DP, DP])
            g("measure_get", C.c_int, [C.c_void_p, C.POINTER(MeasureOut)])
        if self.has("write_cfg"):
            CPP = C.POINTER(C.c_char_p)
            g("write_cfg", C.c_int, [C.c_void_p, C.c_char_p, CPP, C.c_int])
            g("read_cfg", C.c_int, [C.c_void_p, C.c_char_p, CPP, C.POINTER(Rigid)])
            g("checkpoint_save", C.c_int, [C.c_void_p, C.c_char_p])
            g("checkpoint_load", C.c_int, [C.c_void_p, C.c_char_p])
        if self.has("widom"):
            g("widom", C.c_int, [C.c_void_p, C.POINTER(WidomParams), DP, DP, I64P, I64P])
        if self.has("host_gear_create"):
            g("host_gear_create", C.c_int, [C.POINTER(SysDesc), C.POINTER(Rigid), C.POINTER(C.c_void_p)])
            g("host_gear_destroy", None, [C.c_void_p])
            g("host_predict", C.c_int, [C.c_void_p, C.POINTER(State)])
            g("host_correct", C.c_int, [C.c_void_p, C.POINTER(State)] + [DP] * 9 + [C.c_double])
            g("host_report", C.c_int, [C.c_void_p, C.POINTER(Report)])
        if self.has("run"):
            g("set_state", C.c_int, [C.c_void_p, C.POINTER(Rigid), C.POINTER(State)])
            g("get_state", C.c_int, [C.c_void_p, C.POINTER(State)])
            g("run", C.c_int, [C.c_void_p, C.c_int64, C.POINTER(Report)])

    def fn(self, name, restype, argtypes):
        f = getattr(self.so, self.prefix + name)
        f.restype = restype
        f.argtypes = argtypes
        setattr(self, name, f)
        return f

    def has(self, name: str) -> bool:
        return hasattr(self.so, self.prefix + name)


def _dp(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(DP)


class Context:
    """One system on one library context; numpy in, numpy out."""

    def __init__(self, lib: Lib, s: System, prm: RunParams):
        self.lib, self.sys, self.prm = lib, s, prm
        self._desc, self._keep = make_sysdesc(s)
        self._cprm = prm.to_c()
        h = C.c_void_p()
        cx = np.ascontiguousarray(s.c[0, 0]) if s.nrig else np.zeros(1)
        cy = np.ascontiguousarray(s.c[0, 1]) if s.nrig else np.zeros(1)
        cz = np.ascontiguousarray(s.c[0, 2]) if s.nrig else np.zeros(1)
        rc = lib.create(C.byref(self._desc), C.byref(self._cprm), _dp(s.x0), _dp(s.y0), _dp(s.z0),
                        _dp(cx), _dp(cy), _dp(cz), C.byref(h))
        if rc != MDG_OK:
            raise MdgError(rc, (lib.last_error(None) or b"").decode())
        self.h = h
        n = s.nijt
        self.elj = np.zeros(n)
        self.eqq = np.zeros(n)

    def close(self):
        # a batch over this context goes first (mdg_batch_destroy restores its replicas' plans)
        for b in list(getattr(self, "_batches", ())):
            b.close()
        if getattr(self, "h", None):
            self.lib.destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != MDG_OK:
            raise MdgError(rc, (self.lib.last_error(self.h) or b"").decode())

    @staticmethod
    def _com(s: System):
        if s.nrig:
            return [np.ascontiguousarray(s.c[0, d]) for d in range(3)]
        return [np.zeros(1)] * 3

    def nnlist_make(self, s: Optional[System] = None):
        s = s or self.sys
        cx, cy, cz = self._com(s)
        ip, wp = C.c_int64(), C.c_int64()
        self._check(self.lib.nnlist_make(self.h, _dp(s.x0), _dp(s.y0), _dp(s.z0), _dp(cx), _dp(cy),
                                         _dp(cz), C.byref(ip), C.byref(wp)))
        return ip.value, wp.value

    def get_lists(self):
        ip, wp = C.c_int64(), C.c_int64()
        self._check(self.lib.get_lists(self.h, None, None, 0, None, None, 0, C.byref(ip), C.byref(wp)))
        n, nw = ip.value, wp.value
        li, lj = np.zeros(max(n, 1), np.int64), np.zeros(max(n, 1), np.int64)
        wi, wj = np.zeros(max(nw, 1), np.int64), np.zeros(max(nw, 1), np.int64)
        self._check(self.lib.get_lists(self.h, _p(li, C.c_int64), _p(lj, C.c_int64), n,
                                       _p(wi, C.c_int64), _p(wj, C.c_int64), nw, C.byref(ip), C.byref(wp)))
        return (li[:n], lj[:n]), (wi[:nw], wj[:nw])

    def kvectors(self):
        """The context's k set: (kl, km, kn) int32 arrays in the reference's order and Ak."""
        n = int(self.lib.kvectors(self.h, None, None, None, None, 0))
        if n < 0:
            self._check(n)
        kl, km, kn = (np.zeros(max(n, 1), np.int32) for _ in range(3))
        ak = np.zeros(max(n, 1))
        self.lib.kvectors(self.h, _p(kl, C.c_int32), _p(km, C.c_int32), _p(kn, C.c_int32), _dp(ak), n)
        return kl[:n], km[:n], kn[:n], ak[:n]

    def force_get(self, s: Optional[System] = None, want_sites: bool = True) -> Dict[str, object]:
        """One force evaluation; updates s.rsx[0:3] as force_sum does."""
        s = s or self.sys
        nm, nr = s.nmove, s.nriga
        nrig = max(s.nrig, 1)
        ft = [np.zeros(max(nm - nr, 1)) for _ in range(3)]
        fc = [np.zeros(nrig) for _ in range(3)]
        tq = [np.zeros(nrig) for _ in range(3)]
        fs = [np.zeros(nm) for _ in range(3)] if want_sites else [None] * 3
        cx, cy, cz = self._com(s)
        e = Energies()
        e.elj = _dp(self.elj)
        e.eqq = _dp(self.eqq)
        self._check(self.lib.force_get(
            self.h, _dp(s.x0), _dp(s.y0), _dp(s.z0), _dp(cx), _dp(cy), _dp(cz),
            _dp(s.rsx), _dp(s.rsy), _dp(s.rsz), *[_dp(a) for a in ft], *[_dp(a) for a in fc],
            *[_dp(a) for a in tq], *[_dp(a) for a in fs], C.byref(e)))
        out: Dict[str, object] = {
            "ft": np.stack(ft)[:, : nm - nr], "fc": np.stack(fc)[:, : s.nrig],
            "torque": np.stack(tq)[:, : s.nrig], "elj": self.elj.copy(), "eqq": self.eqq.copy(),
        }
        if want_sites:
            out["f"] = np.stack(fs)
        for k in ("uewa", "urf", "ulr", "uself", "uconf", "uavex", "press", "vir", "ewqLL",
                  "ewqWL", "ewqWW"):
            out[k] = getattr(e, k)
        out["fws"] = np.array([list(e.fwsx), list(e.fwsy), list(e.fwsz)])
        return out

    def shake(self, s: System, ft: np.ndarray):
        """Verlet + SHAKE on s in place (x0.., xold..); ft: (3, nmove-nriga)."""
        nl = s.nliqa
        xo = np.ascontiguousarray(s.xold[nl:])
        yo = np.ascontiguousarray(s.yold[nl:])
        zo = np.ascontiguousarray(s.zold[nl:])
        f = [np.ascontiguousarray(ft[d]) for d in range(3)]
        kps = np.zeros(s.nit)
        tk = C.c_double()
        sw = C.c_int32()
        rc = self.lib.shake(self.h, _dp(s.x0), _dp(s.y0), _dp(s.z0), _dp(xo), _dp(yo), _dp(zo),
                            _dp(f[0]), _dp(f[1]), _dp(f[2]), _dp(kps), C.byref(tk), C.byref(sw))
        s.xold[nl:], s.yold[nl:], s.zold[nl:] = xo, yo, zo
        self._check(rc)
        return {"kps": kps, "tkps": tk.value, "sweeps": sw.value}


class _StateArrays:
    """Contiguous copies of a System's integrator state, bound into an mdg_state struct."""

    def __init__(self, s: System, alloc=None):
        """alloc(n) -> an empty float64 array of n elements (e.g. pinned host memory); numpy's
        allocator by default."""
        nl, nr = s.nliqa, max(s.nrig, 1)
        if alloc is None:
            c = np.ascontiguousarray
        else:
            def c(a):
                out = alloc(len(a))
                out[:] = a
                return out
        self.x = [c(s.x0), c(s.y0), c(s.z0)]
        self.xd = [[c(s.xd[k, d]) for d in range(3)] for k in range(4)]
        self.c = [[c(s.c[k, d]) if s.nrig else np.zeros(nr) for d in range(3)] for k in range(5)]
        self.q = [[c(s.q[k, cc]) if s.nrig else np.zeros(nr) for k in range(5)] for cc in range(4)]
        self.w = [[c(s.w[k, d]) if s.nrig else np.zeros(nr) for d in range(3)] for k in range(5)]
        self.old = [c(s.xold[nl:]), c(s.yold[nl:]), c(s.zold[nl:])]
        self.rs = [c(s.rsx), c(s.rsy), c(s.rsz)]
        st = State()
        st.x0, st.y0, st.z0 = (_dp(a) for a in self.x)
        for k in range(4):
            st.xd[k], st.yd[k], st.zd[k] = (_dp(a) for a in self.xd[k])
        for k in range(5):
            st.cx[k], st.cy[k], st.cz[k] = (_dp(a) for a in self.c[k])
            st.wx[k], st.wy[k], st.wz[k] = (_dp(a) for a in self.w[k])
            for cc in range(4):
                st.q[cc][k] = _dp(self.q[cc][k])
        st.xold, st.yold, st.zold = (_dp(a) for a in self.old)
        st.rsx, st.rsy, st.rsz = (_dp(a) for a in self.rs)
        for k in range(5):
            st.s[k] = s.s[k]
            st.rs[k] = s.rs[k]
        self.st = st

    def write_back(self, s: System):
        nl = s.nliqa
        s.x0[:], s.y0[:], s.z0[:] = self.x
        for k in range(4):
            for d in range(3):
                s.xd[k, d] = self.xd[k][d]
        if s.nrig:
            for k in range(5):
                for d in range(3):
                    s.c[k, d] = self.c[k][d]
                    s.w[k, d] = self.w[k][d]
                for cc in range(4):
                    s.q[k, cc] = self.q[cc][k]
        s.xold[nl:], s.yold[nl:], s.zold[nl:] = self.old
        s.rsx[:], s.rsy[:], s.rsz[:] = self.rs
        s.s[:] = list(self.st.s)
        s.rs[:] = list(self.st.rs)


def rigid_of(s: System) -> Rigid:
    r = Rigid()
    for j in range(3):
        r.xbody[j], r.ybody[j], r.zbody[j] = s.xbody[j], s.ybody[j], s.zbody[j]
    r.mw, r.inxx, r.inyy, r.inzz = s.mw, s.inxx or 1.0, s.inyy or 1.0, s.inzz or 1.0
    r.temper = s.temper
    return r


def _ctx_set_state(self, s: Optional[System] = None):
    s = s or self.sys
    self._state = _StateArrays(s)
    self._rigid = rigid_of(s)
    self._check(self.lib.set_state(self.h, C.byref(self._rigid), C.byref(self._state.st)))


def _ctx_get_state(self, s: Optional[System] = None):
    s = s or self.sys
    arr = _StateArrays(s)
    self._check(self.lib.get_state(self.h, C.byref(arr.st)))
    arr.write_back(s)
    return s


def _ctx_run(self, nsteps: int) -> Dict[str, float]:
    rep = Report()
    self._check(self.lib.run(self.h, int(nsteps), C.byref(rep)))
    return {f: getattr(rep, f) for f, _ in Report._fields_}


class HostGear:
    """The drop-in MD step of a caller that keeps the integrator on the host (mdg_host_*):
    predict on the host arrays, one force call of `ctx` (the GPU library or the oracle) on them,
    correct, and SHAKE through `ctx` when the system has surface atoms (src/main.f90:58-68).
    The state lives in contiguous copies of the System's arrays until write_back()."""

    def __init__(self, lib: Lib, s: System, alloc=None):
        """alloc(n): allocator of the host arrays (state, forces), e.g. pinned memory."""
        self.lib, self.sys = lib, s
        self._desc, self._keep = make_sysdesc(s)
        self._rigid = rigid_of(s)
        alloc = alloc or (lambda n: np.zeros(n))
        h = C.c_void_p()
        rc = lib.host_gear_create(C.byref(self._desc), C.byref(self._rigid), C.byref(h))
        if rc != MDG_OK:
            raise MdgError(rc, "mdg_host_gear_create failed")
        self.h = h
        self.arr = _StateArrays(s, alloc)
        nflex, nrig = max(s.nmove - s.nriga, 1), max(s.nrig, 1)

        def zeros(n):
            a = alloc(n)
            a[:] = 0.0
            return a

        self.ft = [zeros(nflex) for _ in range(3)]
        self.fc = [zeros(nrig) for _ in range(3)]
        self.tq = [zeros(nrig) for _ in range(3)]
        self.elj, self.eqq = zeros(s.nijt), zeros(s.nijt)
        self.e = Energies()
        self.e.elj, self.e.eqq = _dp(self.elj), _dp(self.eqq)
        self.shake = s.nmove > s.nliqa
        self.sweeps, self.tk = C.c_int32(), C.c_double()

    def predict(self):
        rc = self.lib.host_predict(self.h, C.byref(self.arr.st))
        if rc != MDG_OK:
            raise MdgError(rc, "mdg_host_predict failed")

    def correct(self, uconf: float):
        rc = self.lib.host_correct(self.h, C.byref(self.arr.st), *[_dp(a) for a in self.ft + self.fc + self.tq],
                                   float(uconf))
        if rc != MDG_OK:
            raise MdgError(rc, "mdg_host_correct failed")

    def step(self, ctx: "Context", nsteps: int = 1):
        a = self.arr
        cx0 = [_dp(x) for x in a.c[0]]
        for _ in range(nsteps):
            self.predict()
            ctx._check(ctx.lib.force_get(ctx.h, *[_dp(x) for x in a.x], *cx0, *[_dp(x) for x in a.rs],
                                         *[_dp(x) for x in self.ft + self.fc + self.tq], None, None, None,
                                         C.byref(self.e)))
            self.correct(self.e.uconf)
            if self.shake:
                ctx._check(ctx.lib.shake(ctx.h, *[_dp(x) for x in a.x], *[_dp(x) for x in a.old],
                                         *[_dp(x) for x in self.ft], None, C.byref(self.tk), C.byref(self.sweeps)))

    def report(self) -> Dict[str, float]:
        rep = Report()
        self.lib.host_report(self.h, C.byref(rep))
        return {"kp": rep.kp, "kw": rep.kw, "ke": rep.ke, "htot": rep.htot, "tempnow": rep.tempnow,
                "uconf": rep.uconf}

    def write_back(self, s: Optional[System] = None) -> System:
        s = s or self.sys
        self.arr.write_back(s)
        return s

    def close(self):
        if getattr(self, "h", None):
            self.lib.host_gear_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


Context.set_state = _ctx_set_state
Context.get_state = _ctx_get_state
Context.run = _ctx_run


PHASES = ("list", "pairs", "walls", "reciprocal", "other", "integrator", "shake")


def _ctx_set_stream(self, stream_handle: int):
    self._check(self.lib.set_stream(self.h, C.c_void_p(stream_handle)))


def _ctx_phase_times(self, reps: int = 5) -> Dict[str, float]:
    out = np.zeros(len(PHASES))
    self._check(self.lib.phase_times(self.h, int(reps), _dp(out)))
    return dict(zip(PHASES, out.tolist()))


Context.set_stream = _ctx_set_stream
Context.phase_times = _ctx_phase_times


def _ctx_run_async(self, nsteps: int):
    self._check(self.lib.run_async(self.h, int(nsteps)))


def _ctx_check(self) -> Dict[str, float]:
    rep = Report()
    self._check(self.lib.check(self.h, C.byref(rep)))
    return {f: getattr(rep, f) for f, _ in Report._fields_}


def _ctx_kernels_per_step(self) -> int:
    return int(self.lib.kernels_per_step(self.h))


Context.run_async = _ctx_run_async
Context.check = _ctx_check
Context.kernels_per_step = _ctx_kernels_per_step


def _fp(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def _ctx_set_shake_model(self, w: Optional[np.ndarray]):
    """Seed SHAKE with the network blob w (float32, mdg_mlp_nw() values); None stops seeding."""
    if w is None:
        self._check(self.lib.shake_set_model(self.h, None, 0))
        return
    self._mlpw = np.ascontiguousarray(w, dtype=np.float32)
    self._check(self.lib.shake_set_model(self.h, _fp(self._mlpw), self._mlpw.size))


def _ctx_shake_record(self, enable: bool = True):
    self._check(self.lib.shake_record(self.h, 1 if enable else 0))


def _ctx_shake_samples(self) -> np.ndarray:
    """(ncons, 16) float32: features[9], multipliers[3], sweeps, 0, 0, 0 of the last SHAKE step."""
    out = np.zeros((max(self.sys.ncons, 1), 16), np.float32)
    self._check(self.lib.shake_samples(self.h, _fp(out)))
    return out[: self.sys.ncons]


Context.set_shake_model = _ctx_set_shake_model
Context.shake_record = _ctx_shake_record
Context.shake_samples = _ctx_shake_samples


class Batch:
    """Replica batch over resident contexts (mdg_batch_*): one graph launch steps all of them."""

    def __init__(self, lib: Lib, ctxs):
        self.lib, self.ctxs = lib, list(ctxs)
        arr = (C.c_void_p * len(self.ctxs))(*[c.h.value if hasattr(c.h, "value") else c.h for c in self.ctxs])
        h = C.c_void_p()
        rc = lib.batch_create(arr, len(self.ctxs), C.byref(h))
        if rc != MDG_OK:
            raise MdgError(rc, (lib.batch_last_error(None) or b"").decode())
        self.h = h
        for c in self.ctxs:  # closing a context closes this batch first
            if not hasattr(c, "_batches"):
                c._batches = weakref.WeakSet()
            c._batches.add(self)

    def _check(self, rc):
        if rc != MDG_OK:
            raise MdgError(rc, (self.lib.batch_last_error(self.h) or b"").decode())

    def set_stream(self, stream_handle: int):
        self._check(self.lib.batch_set_stream(self.h, C.c_void_p(stream_handle)))

    def run(self, nsteps: int):
        reps = (Report * len(self.ctxs))()
        self._check(self.lib.batch_run(self.h, int(nsteps), C.cast(reps, C.c_void_p)))
        return [{f: getattr(r, f) for f, _ in Report._fields_} for r in reps]

    def run_async(self, nsteps: int):
        self._check(self.lib.batch_run_async(self.h, int(nsteps)))

    def set_mode(self, mode: int, pair_blocks: int = 0, wall_blocks: int = 0):
        """MDG_BATCH_PHASES (the replicas' real-space loops in one kernel each) or MDG_BATCH_GRAPHS
        (every replica's own step graph as a child graph); takes effect at the next run."""
        self._check(self.lib.batch_set_mode(self.h, int(mode), int(pair_blocks), int(wall_blocks)))

    def phased(self) -> int:
        """Replicas whose real-space loops ran in the batch's kernels at the last graph build."""
        return int(self.lib.batch_phased(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Tuning(C.Structure):
    _fields_ = [("pair_blocks", C.c_int32), ("tc_rows_per_cta", C.c_int32), ("tc_atom_splits", C.c_int32),
                ("ms_before", C.c_float), ("ms_after", C.c_float)]


def _ctx_autotune(self, reps: int = 5) -> Dict[str, float]:
    """mdg_autotune: pick launch parameters for this system; returns the choice and the force
    evaluation time before and after (ms)."""
    t = Tuning()
    self._check(self.lib.autotune(self.h, int(reps), C.byref(t)))
    return {f: getattr(t, f) for f, _ in Tuning._fields_}


Context.autotune = _ctx_autotune


# ---------------------------------------------------------------------------------------------
# Measurement histograms (mdg_measure_*): measure_init / measure_zero / measure_do and the
# force-loop side outputs, src/measure.f90:66-454 and src/forcem.f90:347-354,388-395,486-495,
# 617-625,930-934,1094-1098.  Arrays come back column-major as the Fortran module holds them,
# reshaped to (rows, bins) numpy arrays.
# ---------------------------------------------------------------------------------------------
def _ctx_measure_init(self, rdel: float, force_hist: bool = True, profiles: bool = False, l2d: bool = False,
                      rfrst: float = 0.0, rscnd: float = 0.0) -> Dict[str, int]:
    p = MeasureParams(float(rdel), int(force_hist), int(profiles), int(l2d), 0, float(rfrst), float(rscnd))
    d = MeasureDims()
    self._check(self.lib.measure_init(self.h, C.byref(p), C.byref(d)))
    self._mdims = {f: int(getattr(d, f)) for f, _ in MeasureDims._fields_}
    return dict(self._mdims)


def _ctx_measure_enable(self, force_hist: bool, profiles: bool) -> None:
    self._check(self.lib.measure_enable(self.h, int(force_hist), int(profiles)))


def _ctx_measure_zero(self) -> None:
    self._check(self.lib.measure_zero(self.h))


def _ctx_measure_do(self, s: Optional[System] = None) -> None:
    """measure_do on the moving atoms of s, or on the resident state when s is None."""
    if s is None:
        self._check(self.lib.measure_do(self.h, None, None, None))
    else:
        n = s.nmove
        xs = [np.ascontiguousarray(a[:n]) for a in (s.x0, s.y0, s.z0)]
        self._check(self.lib.measure_do(self.h, *[_dp(a) for a in xs]))


def _ctx_measure_get(self) -> Dict[str, object]:
    d = self._mdims
    L, nijt, ntz, la = d["lmax"] + 1, d["nijt"], d["ntz"], d["langmax"] + 1
    g2 = ntz * (d["lgxmax"] + 1) * (d["lgymax"] + 1)
    arrs = {"ngc": np.zeros(nijt * L, np.int64), "efipos": np.zeros(2 * L), "tefipos": np.zeros(2 * L),
            "nefipos": np.zeros(2 * L, np.int64), "ngang": np.zeros(ntz * la, np.int64),
            "ngz": np.zeros(ntz * L, np.int64), "ndipx": np.zeros(L), "ndipy": np.zeros(L), "ndipz": np.zeros(L),
            "ndipsq": np.zeros(L), "ng2d1": np.zeros(g2, np.int64), "ng2d2": np.zeros(g2, np.int64)}
    o = MeasureOut()
    for k, a in arrs.items():
        setattr(o, k, a.ctypes.data_as(I64P if a.dtype == np.int64 else DP))
    self._check(self.lib.measure_get(self.h, C.byref(o)))
    shape = {"ngc": (nijt, L), "efipos": (2, L), "tefipos": (2, L), "nefipos": (2, L), "ngang": (ntz, la),
             "ngz": (ntz, L), "ng2d1": (ntz, d["lgxmax"] + 1, d["lgymax"] + 1),
             "ng2d2": (ntz, d["lgxmax"] + 1, d["lgymax"] + 1)}
    out: Dict[str, object] = {k: (a.reshape(shape[k], order="F") if k in shape else a) for k, a in arrs.items()}
    out["ftot"] = np.array([[o.ftot[c][k] for k in range(3)] for c in range(3)])
    out["calls_force"], out["calls_do"], out["out_of_range"] = o.calls_force, o.calls_do, o.out_of_range
    return out


Context.measure_init = _ctx_measure_init
Context.measure_enable = _ctx_measure_enable
Context.measure_zero = _ctx_measure_zero
Context.measure_do = _ctx_measure_do
Context.measure_get = _ctx_measure_get


# ---------------------------------------------------------------------------------------------
# Widom insertion (mdg_widom): chempot, src/forcem.f90:1226-1507.
# ---------------------------------------------------------------------------------------------
def _ctx_widom(self, ichmax: int, lwmin: float, lwmax: float, lchmax: int, ilmid: int, seed: float,
               temper: float = 0.0, flags: int = 0, pave: Optional[np.ndarray] = None,
               inave: Optional[np.ndarray] = None) -> Dict[str, object]:
    """One chempot call on the last force evaluation; pave/inave accumulate (new zero arrays when
    not given).  Returns the arrays, the generator state after the call and the positions tried."""
    p = WidomParams(int(ichmax), float(lwmin), float(lwmax), int(lchmax), int(ilmid), float(temper), int(flags), 0)
    pave = np.zeros(lchmax) if pave is None else pave
    inave = np.zeros(lchmax, np.int64) if inave is None else inave
    sd = C.c_double(float(seed))
    done = C.c_int64(0)
    self._check(self.lib.widom(self.h, C.byref(p), C.byref(sd), _dp(pave), inave.ctypes.data_as(I64P),
                               C.byref(done)))
    return {"pave": pave, "inave": inave, "seed": sd.value, "done": int(done.value)}


Context.widom = _ctx_widom


# ---------------------------------------------------------------------------------------------
# Configuration files and checkpoints (mdg_write_cfg / mdg_read_cfg / mdg_checkpoint_*).
# ---------------------------------------------------------------------------------------------
def _molnames(s: System):
    names = [m.name.encode() for m in s.fld.moltypes]
    return (C.c_char_p * len(names))(*names)


def _ctx_write_cfg(self, path: str, full_precision: bool = False) -> None:
    """config_output of the resident state (E15.8 fields, or 17 digits with full_precision)."""
    self._check(self.lib.write_cfg(self.h, path.encode(), _molnames(self.sys), int(full_precision)))


def _ctx_read_cfg(self, path: str, s: Optional[System] = None) -> None:
    """config_input + config_init of a .cfg file, installed as the resident state."""
    s = s or self.sys
    self._rigid = rigid_of(s)
    self._check(self.lib.read_cfg(self.h, path.encode(), _molnames(s), C.byref(self._rigid)))


def _ctx_checkpoint_save(self, path: str) -> None:
    self._check(self.lib.checkpoint_save(self.h, path.encode()))


def _ctx_checkpoint_load(self, path: str) -> None:
    self._check(self.lib.checkpoint_load(self.h, path.encode()))


Context.write_cfg = _ctx_write_cfg
Context.read_cfg = _ctx_read_cfg
Context.checkpoint_save = _ctx_checkpoint_save
Context.checkpoint_load = _ctx_checkpoint_load
