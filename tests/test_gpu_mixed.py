"""Mixed precision (FP32 pair arithmetic with compensated sums, FP64 accumulation) against the
FP64 path of the same library and against the FP64 oracle directly, on the same inputs: force
rel-RMS <= 1e-5, energies within 1e-5 of the energy scale."""
import numpy as np
import pytest

from md_sim_gb300 import abi, configs
from tests.golden.fixture import y_n_case

pytestmark = pytest.mark.gpu

MIXED_FORCE_RTOL = 1e-5


CASES = {
    "bulk256": lambda: configs.bulk_water(),
    "slab512": lambda: configs.slab_water(nwat=512, cells=6),
    "shake256": lambda: configs.shake_water(nwat=256, cells=6),
    "y_n": lambda: y_n_case()[:2],
    "electrolyte": lambda: configs.slab_electrolyte(),
}


@pytest.mark.parametrize("name", list(CASES))
def test_mixed_forces_vs_fp64(name, gpulib, oracle):
    s, prm = CASES[name]()
    s64, s32, so = s.copy(), s.copy(), s.copy()
    p64 = abi.RunParams(**{**prm.__dict__, "precision": abi.MDG_FP64})
    p32 = abi.RunParams(**{**prm.__dict__, "precision": abi.MDG_MIXED})
    a = abi.Context(gpulib, s64, p64).force_get(s64)
    b = abi.Context(gpulib, s32, p32).force_get(s32)
    r = abi.Context(oracle, so, p64).force_get(so)
    scale = np.abs(a["elj"]).sum() + np.abs(a["eqq"]).sum() + abs(a["uewa"]) + 1.0
    for ref in (a, r):  # the library's FP64 form, then the oracle
        rel = np.linalg.norm(b["f"] - ref["f"]) / np.linalg.norm(ref["f"])
        assert rel <= MIXED_FORCE_RTOL, rel
        assert abs(b["uconf"] - ref["uconf"]) <= 1e-5 * scale


@pytest.mark.parametrize("name", ["slab512", "bulk256"])
def test_autotune_keeps_forces(name, gpulib):
    """mdg_autotune only changes launch shapes: the chosen grid and structure-factor split give
    the same forces (mixed tolerance against FP64) as the defaults."""
    s, prm = CASES[name]()
    s64, s32 = s.copy(), s.copy()
    p64 = abi.RunParams(**{**prm.__dict__, "precision": abi.MDG_FP64})
    p32 = abi.RunParams(**{**prm.__dict__, "precision": abi.MDG_MIXED})
    a = abi.Context(gpulib, s64, p64).force_get(s64)
    ctx = abi.Context(gpulib, s32, p32)
    ctx.set_state(s32)
    t = ctx.autotune(2)
    assert t["pair_blocks"] in (0, 304, 608, 1216)
    assert t["tc_rows_per_cta"] in (256, 512)
    assert t["tc_atom_splits"] >= 1
    assert t["ms_after"] > 0 and t["ms_before"] > 0
    b = ctx.force_get(s32)
    rel = np.linalg.norm(b["f"] - a["f"]) / np.linalg.norm(a["f"])
    assert rel <= MIXED_FORCE_RTOL, rel
    rep = ctx.run(5)
    assert np.isfinite(rep["htot"])
