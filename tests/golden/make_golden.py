"""Regenerates tests/golden/*.npz from the reference's fixture directory src/sim.

Usage: python tests/golden/make_golden.py <reference checkout>/src/sim
(or set MDSIM_REF_SIM to that directory).

y_n_case.npz: the reference's interfacial sample (src/sim/y.fld, y.top, y.inp and the evolved
state y_n.cfg: 258 rigid waters, 54 surface OH bound to a 3189-site rutile slab, angles and
wall-bound constraints).  Stored as the field/topology texts plus the parsed state arrays, so the
GPU tests can rebuild the System without the reference tree, and with the oracle's results for
that state (a regression record of the oracle itself; the reference ships no results for it).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MDSIM_REF_SIM")
    if not ref or not os.path.isdir(ref):
        raise SystemExit("usage: make_golden.py <reference>/src/sim (or MDSIM_REF_SIM=<dir>)")
    import build as oracle_build
    from md_sim_gb300 import abi
    from md_sim_gb300 import system as S

    inp = S.parse_inp(open(os.path.join(ref, "y.inp")).read())
    fld_t = open(os.path.join(ref, "y.fld")).read()
    top_t = open(os.path.join(ref, "y.top")).read()
    fld = S.parse_fld(fld_t)
    top = S.parse_top(top_t, fld)
    s = S.parse_cfg(open(os.path.join(ref, "y_n.cfg")).read(), fld, top, inp.dt)
    s.rsx_after_predict()
    s.shake_init()
    oracle_build.build()
    lib = abi.Lib(oracle_build.path(), "ref_")
    prm = abi.RunParams(rcut=inp.rcut, skin=inp.skin, kmax=inp.kmax)
    ctx = abi.Context(lib, s.copy(), prm)
    out = ctx.force_get()
    np.savez_compressed(
        os.path.join(HERE, "y_n_case.npz"), fld=fld_t, top=top_t, lx=s.lx, ly=s.ly, lz=s.lz,
        dt=s.dt, rcut=inp.rcut, skin=inp.skin, kmax=inp.kmax, x0=s.x0, y0=s.y0, z0=s.z0,
        c=s.c, q=s.q, w=s.w, walltype=s.walltype, xold=s.xold, yold=s.yold, zold=s.zold,
        ref_f=out["f"], ref_elj=out["elj"], ref_eqq=out["eqq"], ref_uewa=out["uewa"],
        ref_urf=out["urf"], ref_ulr=out["ulr"], ref_uconf=out["uconf"], ref_fws=out["fws"])
    print("wrote", os.path.join(HERE, "y_n_case.npz"))


if __name__ == "__main__":
    main()
