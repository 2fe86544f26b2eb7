"""Drop-in calls with pinned host arrays.

mdg_force_get and mdg_shake move the arrays whose host side is pinned through the GPU's mapping
of pinned memory (one gather and one scatter kernel per call) and the others by driver copies.
The results must not depend on which way an array travelled: the same call with pageable,
pinned and mixed arrays gives the same numbers (bit-exact for SHAKE, whose kernels sum in a fixed
order; within the run-to-run spread of the atomics' summation order for forces).
"""
import ctypes as C
import mmap

import numpy as np
import pytest

from md_sim_gb300 import abi, configs

pytestmark = pytest.mark.gpu

_keep = []  # pinned tensors backing the numpy views handed to the library


def _pageable(a):
    return np.array(a, dtype=np.float64, copy=True)


def _pinned(a):
    torch = pytest.importorskip("torch")
    a = np.asarray(a, dtype=np.float64)
    t = torch.zeros(max(a.size, 1), dtype=torch.float64).pin_memory()
    _keep.append(t)
    v = t.numpy()[: a.size]
    v[:] = a
    return v


def _force_get(lib, ctx, s, mk_in, mk_out):
    nm, nr = s.nmove, s.nriga
    nrig = max(s.nrig, 1)
    cx, cy, cz = abi.Context._com(s)
    ins = [mk_in(a) for a in (s.x0, s.y0, s.z0, cx, cy, cz, s.rsx, s.rsy, s.rsz)]
    outs = ([mk_out(np.zeros(max(nm - nr, 1))) for _ in range(3)] + [mk_out(np.zeros(nrig)) for _ in range(6)]
            + [mk_out(np.zeros(nm)) for _ in range(3)])
    e = abi.Energies()
    elj, eqq = np.zeros(s.nijt), np.zeros(s.nijt)
    e.elj, e.eqq = abi._dp(elj), abi._dp(eqq)
    rc = lib.force_get(ctx.h, *[abi._dp(a) for a in ins], *[abi._dp(a) for a in outs], C.byref(e))
    assert rc == 0, lib.last_error(ctx.h)
    res = {"ft": np.stack(outs[0:3]), "fc": np.stack(outs[3:6]), "tq": np.stack(outs[6:9]),
           "f": np.stack(outs[9:12]), "rs": np.stack([np.array(a) for a in ins[6:9]]),
           "elj": elj, "eqq": eqq}
    for k in ("uewa", "urf", "ulr", "uconf", "ewqLL", "press"):
        res[k] = np.array([getattr(e, k)])
    return res


def _close(a, b, rtol):
    for k in a:
        scale = max(np.abs(b[k]).max(), 1e-300)
        assert np.abs(a[k] - b[k]).max() <= rtol * scale, (k, np.abs(a[k] - b[k]).max(), scale)


@pytest.mark.parametrize("precision", [abi.MDG_FP64, abi.MDG_MIXED])
def test_force_get_pinned_equals_pageable(precision, gpulib):
    s, prm = configs.slab_water(nwat=512, cells=6)
    prm.precision = precision
    ctx = abi.Context(gpulib, s.copy(), prm)
    try:
        ref = _force_get(gpulib, ctx, s.copy(), _pageable, _pageable)
        rtol = 1e-13 if precision == abi.MDG_FP64 else 1e-5
        for mk_in, mk_out in ((_pinned, _pinned), (_pinned, _pageable), (_pageable, _pinned)):
            got = _force_get(gpulib, ctx, s.copy(), mk_in, mk_out)
            _close(got, ref, rtol)
            # the stale offsets written back (force_sum's rsx(1:3)) arrive either way
            assert np.array_equal(got["rs"], ref["rs"])
    finally:
        ctx.close()


def test_pin_host_arrays(gpulib):
    """Arrays pinned in place by mdg_pin_host (as a Fortran host would pin its module arrays)."""
    s, prm = configs.slab_water(nwat=512, cells=6)
    prm.precision = abi.MDG_MIXED
    ctx = abi.Context(gpulib, s.copy(), prm)
    pinned = []

    def pin(a):
        # its own whole pages (64 KB covers the Arm hosts' page size): ranges that share a page
        # cannot be registered twice
        a = np.asarray(a, dtype=np.float64)
        mm = mmap.mmap(-1, -(-max(a.nbytes, 8) // 65536) * 65536)
        b = np.frombuffer(mm, dtype=np.float64, count=a.size)
        b[:] = a
        assert gpulib.pin_host(b.ctypes.data, b.nbytes) == 0, gpulib.last_error(None)
        pinned.append((mm, b))
        return b

    try:
        ref = _force_get(gpulib, ctx, s.copy(), _pageable, _pageable)
        got = _force_get(gpulib, ctx, s.copy(), pin, pin)
        _close(got, ref, 1e-5)
        assert np.array_equal(got["rs"], ref["rs"])
    finally:
        ctx.close()
        for mm, b in pinned:
            assert gpulib.unpin_host(b.ctypes.data) == 0
    assert gpulib.pin_host(None, 8) != 0  # a null range is refused, not pinned


def test_shake_pinned_equals_pageable(gpulib):
    s, prm = configs.shake_water(nwat=256, cells=6)
    prm.shake_maxit = 100
    ctx = abi.Context(gpulib, s.copy(), prm)
    try:
        ft = ctx.force_get(s.copy())["ft"]
        nl = s.nliqa
        out = []
        for mk in (_pageable, _pinned):
            x, y, z = mk(s.x0), mk(s.y0), mk(s.z0)
            xo, yo, zo = mk(s.xold[nl:]), mk(s.yold[nl:]), mk(s.zold[nl:])
            f = [mk(ft[d]) for d in range(3)]
            kps = mk(np.zeros(s.nit))
            tk, sw = C.c_double(), C.c_int32()
            rc = gpulib.shake(ctx.h, *[abi._dp(a) for a in (x, y, z, xo, yo, zo, *f, kps)], C.byref(tk), C.byref(sw))
            assert rc == 0, gpulib.last_error(ctx.h)
            out.append((np.array(x), np.array(y), np.array(z), np.array(xo), np.array(kps), tk.value, sw.value))
        a, b = out
        for u, w in zip(a[:4], b[:4]):
            assert np.array_equal(u, w)
        np.testing.assert_allclose(a[4], b[4], rtol=1e-13, atol=0)
        assert a[6] == b[6] and a[6] > 0
        assert abs(a[5] - b[5]) <= 1e-13 * abs(b[5])
    finally:
        ctx.close()
