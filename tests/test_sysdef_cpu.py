"""The C++ readers of the reference's input files (mdg_sysdef_load: sysdef_input / sysdef_init,
src/sysdef.f90:83-340, :356-457; config_input / config_init, src/config.f90:174-242, :55-95)
against the Python readers of this package on the same .fld/.top/.cfg texts: every table of
mdg_sysdesc, the rigid-water body and the state must agree bit for bit.  Cases: the reference's
own interfacial sample (its .fld/.top, the committed state written as a .cfg) and synthetic
systems covering rigid waters, flexible ions, SHAKE molecules with angles and crystal walls with
charge-shifted sites.  Runs on the CPU (host code only)."""
import ctypes as C
import os

import numpy as np
import pytest

from md_sim_gb300 import abi, configs
from md_sim_gb300 import system as S


def _golden():
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import fixture

    s, _, z = fixture.y_n_case()
    return s, str(z["fld"]), str(z["top"])


CASES = {
    "reference y_n": _golden,
    "slab512": lambda: configs.slab_water(nwat=512, cells=6)[0],
    "electrolyte": lambda: configs.slab_electrolyte()[0],
    "shake256": lambda: configs.shake_water(nwat=256, cells=6)[0],
    "bulk256": lambda: configs.bulk_water()[0],
}


def _arr(p, n, ct=C.c_double):
    return np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), shape=(n,)).copy() if n > 0 else np.zeros(0)


@pytest.mark.parametrize("name", list(CASES))
def test_cpp_readers_match_python(name, gpulib, tmp_path):
    if not gpulib.has("sysdef_load"):
        pytest.skip("library without the readers")
    got = CASES[name]()
    if isinstance(got, tuple):
        s0, fld_t, top_t = got
    else:
        s0 = got
        fld_t, top_t = S.write_fld(s0.fld), S.write_top(s0.fld, s0.top)
    cfg_t = S.write_cfg(s0)
    paths = {}
    for ext, text in (("fld", fld_t), ("top", top_t), ("cfg", cfg_t)):
        paths[ext] = str(tmp_path / f"case.{ext}")
        open(paths[ext], "w").write(text)
    # Python readers
    fld = S.parse_fld(fld_t)
    top = S.parse_top(top_t, fld)
    s = S.parse_cfg(cfg_t, fld, top, s0.dt)
    ref, _keep = abi.make_sysdesc(s)
    # C++ readers
    h = C.c_void_p()
    rc = gpulib.sysdef_load(paths["fld"].encode(), paths["top"].encode(), paths["cfg"].encode(), s0.dt, C.byref(h))
    assert rc == 0, gpulib.last_error(None)
    try:
        d = gpulib.sysdef_desc(h).contents
        for f, _ in abi.SysDesc._fields_:
            a, b = getattr(ref, f), getattr(d, f)
            if isinstance(a, (int, float)):
                assert a == b, f
        n_of = {"moltypen": s.ntype, "nt": s.ntype, "ns": s.ntype, "nst": s.ntype, "nconst": s.ntype,
                "nangt": s.ntype, "nss_wall": max(2, int(s.nst[s.ntype - 1])), "nsi": s.nit,
                "ijtype": s.nit * s.nit, "vdwnum": s.nijt, "itype": s.ntota, "ictype": max(s.ncons, 1),
                "constra": S.SMX * max(s.ncons, 1), "constrb": S.SMX * max(s.ncons, 1),
                "iatype": max(s.nang, 1), "ang1": S.SMX * max(s.nang, 1), "ang2": S.SMX * max(s.nang, 1),
                "ang3": S.SMX * max(s.nang, 1)}
        for f, n in n_of.items():
            np.testing.assert_array_equal(_arr(getattr(d, f), n, C.c_int64), _arr(getattr(ref, f), n, C.c_int64), err_msg=f)
        nf = {"eps": s.nijt, "sig": s.nijt, "aa": s.nijt, "rhoi": s.nijt, "cc": s.nijt, "qs": s.ntota,
              "mi": s.ntota, "mii": s.ntota, "length": s.ntype * S.SMX, "kt": s.ntype * S.SMX,
              "theta": s.ntype * S.SMX}
        for f, n in nf.items():
            np.testing.assert_array_equal(_arr(getattr(d, f), n), _arr(getattr(ref, f), n), err_msg=f)
        b = gpulib.sysdef_rigid(h).contents
        np.testing.assert_array_equal(np.array(b.xbody[:]), s.xbody)
        np.testing.assert_array_equal(np.array(b.ybody[:]), s.ybody)
        np.testing.assert_array_equal(np.array(b.zbody[:]), s.zbody)
        assert (b.mw, b.inxx, b.inyy, b.inzz) == (s.mw, s.inxx, s.inyy, s.inzz)
        st = gpulib.sysdef_state(h).contents
        nt, nr, nl = s.ntota, s.nrig, s.nliqa
        np.testing.assert_array_equal(_arr(st.x0, nt), s.x0)
        np.testing.assert_array_equal(_arr(st.y0, nt), s.y0)
        np.testing.assert_array_equal(_arr(st.z0, nt), s.z0)
        for k in range(4):
            np.testing.assert_array_equal(_arr(st.xd[k], nt), s.xd[k, 0])
            np.testing.assert_array_equal(_arr(st.zd[k], nt), s.xd[k, 2])
        for k in range(5):
            np.testing.assert_array_equal(_arr(st.cx[k], nr), s.c[k, 0])
            np.testing.assert_array_equal(_arr(st.cz[k], nr), s.c[k, 2])
            np.testing.assert_array_equal(_arr(st.wy[k], nr), s.w[k, 1])
            for cc in range(4):
                np.testing.assert_array_equal(_arr(st.q[cc][k], nr), s.q[k, cc])
        np.testing.assert_array_equal(_arr(st.xold, nt - nl), s.xold[nl:])
        np.testing.assert_array_equal(_arr(st.zold, nt - nl), s.zold[nl:])
        np.testing.assert_array_equal(np.array(st.s[:]), s.s)
        np.testing.assert_array_equal(np.array(st.rs[:]), s.rs)
    finally:
        gpulib.sysdef_free(h)


def test_cpp_readers_report_format_errors(gpulib, tmp_path):
    if not gpulib.has("sysdef_load"):
        pytest.skip("library without the readers")
    s = configs.slab_water(nwat=512, cells=6)[0]
    fld_t = S.write_fld(s.fld)
    top_t = S.write_top(s.fld, s.top).replace(" 1 ", " 7 ", 1)  # wrong molecule number in the topology
    for ext, text in (("fld", fld_t), ("top", top_t), ("cfg", S.write_cfg(s))):
        open(tmp_path / f"bad.{ext}", "w").write(text)
    h = C.c_void_p()
    rc = gpulib.sysdef_load(str(tmp_path / "bad.fld").encode(), str(tmp_path / "bad.top").encode(),
                            str(tmp_path / "bad.cfg").encode(), s.dt, C.byref(h))
    assert rc == -1  # MDG_E_ARG
    assert b"topofile" in gpulib.last_error(None)
    rc = gpulib.sysdef_load(b"/nonexistent.fld", b"x", b"y", 1.0, C.byref(h))
    assert rc == -1  # MDG_E_ARG
