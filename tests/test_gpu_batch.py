"""Replica batches (mdg_batch_*): independent systems stepped by one graph launch give the same
trajectories as the same systems stepped one by one, including a replica whose neighbour list
has to grow mid-run."""
import numpy as np
import pytest

from md_sim_gb300 import abi, configs

pytestmark = pytest.mark.gpu


def _systems():
    return [configs.slab_water(nwat=256 + 64 * i, cells=6 + (i % 2), seed=40 + i, kmax=6, placement="lattice")
            for i in range(3)]


def test_batch_matches_individual_runs(gpulib):
    a_sys, b_sys = _systems(), _systems()
    a_ctx, b_ctx = [], []
    for (s, p), (s2, p2) in zip(a_sys, b_sys):
        ca, cb = abi.Context(gpulib, s, p), abi.Context(gpulib, s2, p2)
        ca.set_state(s)
        cb.set_state(s2)
        a_ctx.append(ca)
        b_ctx.append(cb)
    batch = abi.Batch(gpulib, a_ctx)
    reps = batch.run(12)
    assert len(reps) == 3
    for c in b_ctx:
        c.run(12)
    for (sa, _), (sb, _), ca, cb in zip(a_sys, b_sys, a_ctx, b_ctx):
        ca.get_state(sa)
        cb.get_state(sb)
        for u, w in ((sa.x0, sb.x0), (sa.y0, sb.y0), (sa.z0, sb.z0)):
            assert np.abs(u - w).max() < 1e-9 * sa.lx
    batch.close()


def test_batch_list_regrowth(gpulib):
    """A replica created with a tight list capacity overflows inside the batch and is redone."""
    systems = _systems()
    ctxs = []
    for i, (s, p) in enumerate(systems):
        if i == 1:
            p.list_capacity = 1   # grown at create to fit, with no margin left
        c = abi.Context(gpulib, s, p)
        c.set_state(s)
        ctxs.append(c)
    batch = abi.Batch(gpulib, ctxs)
    reps = batch.run(200)
    assert all(np.isfinite(r["htot"]) for r in reps)
    batch.close()


def test_batch_leaves_caller_stream(gpulib):
    """A batch launched on a caller's stream destroys only its own stream when closed."""
    import torch

    s, p = _systems()[0]
    c = abi.Context(gpulib, s, p)
    c.set_state(s)
    st = torch.cuda.Stream()
    b = abi.Batch(gpulib, [c])
    b.set_stream(st.cuda_stream)
    b.run(3)
    b.close()
    with torch.cuda.stream(st):
        x = torch.ones(1024, device="cuda") * 2
    st.synchronize()
    assert float(x.sum()) == 2048.0
    c.set_stream(st.cuda_stream)
    c.run(2)
    c.close()
    st.synchronize()
