"""tcgen05 tensor-core path: the UMMA operand layout against numpy, and the BF16 hi/lo reciprocal
sum against the FP64 reciprocal sum of the same library."""
import ctypes as C

import numpy as np
import pytest

from md_sim_gb300 import abi, configs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,k", [(16, 16), (64, 32), (112, 48), (128, 64), (256, 16)])
def test_umma_selftest_matches_numpy(n, k, gpulib):
    f = gpulib.so.mdg_selftest_umma
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    rng = np.random.default_rng(n * 1000 + k)
    # BF16-representable operands: products are exact in FP32 up to accumulation order
    a = (rng.integers(-64, 64, size=(128, k)) / 64.0).astype(np.float32)
    b = (rng.integers(-64, 64, size=(n, k)) / 64.0).astype(np.float32)
    d = np.zeros((128, n), dtype=np.float32)
    rc = f(n, k, a.ctypes.data, b.ctypes.data, d.ctypes.data)
    assert rc == 0, gpulib.last_error(None)
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    np.testing.assert_allclose(d, ref, rtol=1e-6, atol=1e-5)


def test_tensor_reciprocal_vs_fp64(gpulib):
    """Ion lattice: the real-space sum is empty, so the forces are the reciprocal forces alone."""
    s, prm = configs.ion_lattice(n_side=8, kmax=8)
    s64, s32 = s.copy(), s.copy()
    a = abi.Context(gpulib, s64, abi.RunParams(**{**prm.__dict__, "precision": abi.MDG_FP64})).force_get(s64)
    b = abi.Context(gpulib, s32, abi.RunParams(**{**prm.__dict__, "precision": abi.MDG_MIXED})).force_get(s32)
    rel = np.linalg.norm(b["f"] - a["f"]) / np.linalg.norm(a["f"])
    assert rel < 1e-5, rel
    assert abs(b["uewa"] - a["uewa"]) < 1e-5 * abs(a["uewa"])


@pytest.mark.parametrize("make", [
    lambda: configs.slab_water(),
    lambda: configs.bulk_water(8, "sc", box=8 * 3.103, seeds=(5, 6, 7), rcut=10.0, alpha=0.32, kmax=12),
])
def test_mixed_step_force_error(make, gpulib):
    """Force rel-RMS of the full mixed evaluation against FP64 on the benchmark-type systems."""
    s, prm = make()
    s64, s32 = s.copy(), s.copy()
    a = abi.Context(gpulib, s64, abi.RunParams(**{**prm.__dict__, "precision": abi.MDG_FP64})).force_get(s64)
    b = abi.Context(gpulib, s32, abi.RunParams(**{**prm.__dict__, "precision": abi.MDG_MIXED})).force_get(s32)
    rel = np.linalg.norm(b["f"] - a["f"]) / np.linalg.norm(a["f"])
    assert rel < 1e-5, rel
    for key in ("fc", "torque"):
        if a[key].size:
            e = np.linalg.norm(b[key] - a[key]) / np.linalg.norm(a[key])
            assert e < 1e-5, (key, e)
