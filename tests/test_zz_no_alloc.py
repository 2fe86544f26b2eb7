"""The allocation-free reciprocal sum, through the C ABI, against mdg_force_get.

mdg_recip_forces_noalloc exists for callers that must not allocate device memory while they run
(a host that sized its device memory once at start-up, a framework whose caching allocator owns
all of the device memory).  It keeps its scratch in a static device
array, so this test checks that two calls in a row, sharing that array, both reproduce the
reciprocal forces and energy that mdg_force_get computes for the same charges, within the FP64
tolerance of the other parity tests.  The system is a lattice of point ions whose real-space sum
is empty (closest approach above the cutoff), so mdg_force_get's forces are its reciprocal
forces.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from md_sim_gb300 import abi, configs

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-12


def _bind(lib):
    f = lib.so.mdg_recip_forces_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p] * 4 + [C.c_int64] + [C.c_double] * 4 + [C.c_int64] + [C.c_void_p] * 5
    return f


def test_noalloc_matches_force_get_twice(gpulib):
    torch = pytest.importorskip("torch")
    s, prm = configs.ion_lattice()
    n = s.nmove
    # no pair inside the cutoff: the real-space part of force_get is empty
    xyz = np.stack([s.x0[:n], s.y0[:n], s.z0[:n]], 1)
    d = xyz[:, None, :] - xyz[None, :, :]
    d -= s.lx * np.round(d / s.lx)
    r2 = (d ** 2).sum(-1) + np.eye(n) * 1e9
    assert r2.min() > prm.rcut ** 2
    ctx = abi.Context(gpulib, s, prm)
    ref = ctx.force_get(s)
    fref = ref["f"]
    fn = _bind(gpulib)
    dev = torch.device("cuda:0")
    x, y, z = (torch.tensor(a, dtype=torch.float64, device=dev) for a in (s.x0[:n], s.y0[:n], s.z0[:n]))
    q = torch.tensor(s.qs[:n], dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        fx, fy, fz = (torch.full((n,), 7.0, dtype=torch.float64, device=dev) for _ in range(3))
        u = torch.zeros(1, dtype=torch.float64, device=dev)
        rc = fn(x.data_ptr(), y.data_ptr(), z.data_ptr(), q.data_ptr(), n, s.lx, s.ly, s.lz, prm.alpha,
                prm.kmax, fx.data_ptr(), fy.data_ptr(), fz.data_ptr(), u.data_ptr(), stream.cuda_stream)
        assert rc == 0, gpulib.last_error(None)
        torch.cuda.synchronize()
        f = np.stack([fx.cpu().numpy(), fy.cpu().numpy(), fz.cpu().numpy()])
        err = np.linalg.norm(f - fref) / np.linalg.norm(fref)
        assert err < FORCE_RTOL, (call, err)
        assert abs(u.item() - ref["uewa"]) <= 1e-12 * abs(ref["uewa"]), (call, u.item(), ref["uewa"])


def test_noalloc_rejects_oversized_k_set(gpulib):
    torch = pytest.importorskip("torch")
    fn = _bind(gpulib)
    dev = torch.device("cuda:0")
    a = torch.zeros(8, dtype=torch.float64, device=dev)
    rc = fn(a.data_ptr(), a.data_ptr(), a.data_ptr(), a.data_ptr(), 8, 30.0, 30.0, 30.0, 0.3, 40,
            a.data_ptr(), a.data_ptr(), a.data_ptr(), None, None)
    assert rc == -7
    assert b"MDG_NOALLOC_MAX_K" in gpulib.last_error(None)
