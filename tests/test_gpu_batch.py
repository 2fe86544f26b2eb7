"""Replica batches (mdg_batch_*): independent systems stepped by one graph launch give the same
trajectories as the same systems stepped one by one, including a replica whose neighbour list
has to grow mid-run, in both graph forms (every replica's own step graph as a child graph, and
phase order with the real-space loops of all replicas in one kernel each)."""
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


def _mixed(systems):
    for _, p in systems:
        p.precision = abi.MDG_MIXED
    return systems


@pytest.mark.parametrize("blocks", [(0, 0), (2, 3)])
def test_batch_phases_match_individual_runs(gpulib, blocks):
    """Phase order: the head-head and head-wall loops of the three mixed-precision slabs run as
    one kernel each over all their heads (with 2 and 3 blocks every block walks items of several
    replicas); a bulk box without walls in the same batch keeps its own loops.  Trajectories
    and energies against the same systems stepped one by one with their own graphs."""
    def build():
        sy = _mixed(_systems())
        sy.append(_mixed([configs.bulk_water()])[0])
        return sy

    a_sys, b_sys = build(), build()
    a_ctx, b_ctx = [], []
    for (s, p), (s2, p2) in zip(a_sys, b_sys):
        ca, cb = abi.Context(gpulib, s, p), abi.Context(gpulib, s2, p2)
        ca.set_state(s)
        cb.set_state(s2)
        a_ctx.append(ca)
        b_ctx.append(cb)
    batch = abi.Batch(gpulib, a_ctx)
    batch.set_mode(abi.MDG_BATCH_PHASES, *blocks)
    reps = batch.run(12)
    assert batch.phased() == 3
    one = [c.run(12) for c in b_ctx]
    for (sa, _), (sb, _), ca, cb, ra, rb in zip(a_sys, b_sys, a_ctx, b_ctx, reps, one):
        ca.get_state(sa)
        cb.get_state(sb)
        # FP32 force sums (vector reductions) in another order: positions differ at FP32
        # rounding, energies by the mixed form's run-to-run spread (measured: up to 1.5e-6 of
        # uconf after 12 steps, batched or not), far below what a missing or doubled term gives
        for u, w in ((sa.x0, sb.x0), (sa.y0, sb.y0), (sa.z0, sb.z0)):
            assert np.abs(u - w).max() < 1e-7 * sa.lx
        assert abs(ra["htot"] - rb["htot"]) <= 1e-5 * abs(rb["htot"])
        assert abs(ra["uconf"] - rb["uconf"]) <= 1e-5 * abs(rb["uconf"])
    batch.set_mode(abi.MDG_BATCH_GRAPHS)
    batch.run(2)
    assert batch.phased() == 0
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


def test_batch_phases_list_regrowth(gpulib):
    """The same in phase order (mixed precision): the overflowing replica redoes its chunk alone,
    the batch's kernels are rebuilt on the grown lists, and every replica's energies agree with
    the same system stepped alone."""
    systems, alone = _mixed(_systems()), _mixed(_systems())
    ctxs, solo = [], []
    for i, ((s, p), (s2, p2)) in enumerate(zip(systems, alone)):
        if i == 1:
            p.list_capacity = 1
        c = abi.Context(gpulib, s, p)
        c.set_state(s)
        ctxs.append(c)
        c2 = abi.Context(gpulib, s2, p2)
        c2.set_state(s2)
        solo.append(c2)
    batch = abi.Batch(gpulib, ctxs)
    reps = batch.run(150)
    assert batch.phased() == 3
    for r, c2 in zip(reps, solo):
        r2 = c2.run(150)
        assert np.isfinite(r["htot"])
        assert abs(r["htot"] - r2["htot"]) <= 1e-4 * abs(r2["htot"])
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
