"""Loads the committed golden cases into md_sim_gb300 System objects (no reference tree needed)."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def y_n_case():
    from md_sim_gb300 import abi
    from md_sim_gb300 import system as S

    z = np.load(os.path.join(HERE, "y_n_case.npz"))
    fld = S.parse_fld(str(z["fld"]))
    top = S.parse_top(str(z["top"]), fld)
    s = S.System(fld, top, float(z["lx"]), float(z["ly"]), float(z["lz"]), float(z["dt"]))
    nm = s.nmove
    s.set_walls(z["walltype"], np.stack([z["x0"][nm:], z["y0"][nm:], z["z0"][nm:]], 1))
    s.x0[:], s.y0[:], s.z0[:] = z["x0"], z["y0"], z["z0"]
    s.c[:], s.q[:], s.w[:] = z["c"], z["q"], z["w"]
    s.xold[:], s.yold[:], s.zold[:] = z["xold"], z["yold"], z["zold"]
    s.quatsite()
    s.rsx_after_predict()
    prm = abi.RunParams(rcut=float(z["rcut"]), skin=float(z["skin"]), kmax=int(z["kmax"]))
    return s, prm, z
