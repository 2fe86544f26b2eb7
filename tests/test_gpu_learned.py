"""The learned SHAKE seed on the GPU: network forward and gradient kernels against the CPU
restatement (oracle/mlp.py), training through mdg_mlp_train, and SHAKE seeded by the trained
network converging to the same tolerance in fewer sweeps."""
import numpy as np
import pytest

import mlp as M
from md_sim_gb300 import abi, configs, learned

pytestmark = pytest.mark.gpu


def _blob(rng):
    b = np.zeros(M.NW, np.float32)
    b[M.OW1:M.OB1] = rng.normal(0, np.sqrt(2 / 9), M.NH * M.NI)
    b[M.OW2:M.OB2] = rng.normal(0, np.sqrt(2 / 64), M.NH * M.NH)
    b[M.OW3:M.OB3] = 0.3 * rng.normal(0, np.sqrt(2 / 64), M.NO * M.NH)
    b[M.OB1:M.OW2] = rng.normal(0, 0.1, M.NH)
    b[M.OB2:M.OW3] = rng.normal(0, 0.1, M.NH)
    b[M.OB3:M.NPARAM] = rng.normal(0, 0.1, M.NO)
    b[M.OXM:M.OXS] = rng.normal(0, 1, 9)
    b[M.OXS:M.OYM] = rng.uniform(0.5, 2, 9)
    b[M.OYM:M.OYS] = rng.normal(0, 1, 3)
    b[M.OYS:M.NW] = rng.uniform(0.5, 2, 3)
    return b


def test_nw(gpulib):
    assert learned.nw(gpulib) == M.NW


def test_forward_matches_oracle(gpulib):
    rng = np.random.default_rng(11)
    b = _blob(rng)
    X = rng.normal(0, 1.5, (1000, 9)).astype(np.float32)
    y_gpu = learned.forward(gpulib, b, X)
    y_ref = M.forward(b, X)
    # FP32 accumulation and the fast exponential against float64: ~1e-6 relative
    assert np.abs(y_gpu - y_ref).max() <= 2e-5 * (np.abs(y_ref).max() + 1)


def test_gradient_matches_oracle(gpulib):
    rng = np.random.default_rng(12)
    b = _blob(rng)
    X = rng.normal(0, 1.5, (700, 9)).astype(np.float32)   # not a multiple of the 128-sample block
    T = rng.normal(0, 1.0, (700, 3)).astype(np.float32)
    loss_g, g_gpu = learned.grad(gpulib, b, X, T)
    loss_r, g_ref = M.loss_grad(b, X, T)
    assert abs(loss_g - loss_r) <= 1e-4 * loss_r
    err = np.linalg.norm(g_gpu - g_ref) / np.linalg.norm(g_ref)
    assert err < 1e-4, err
    # every parameter block individually
    for a, z in ((M.OW1, M.OB1), (M.OB1, M.OW2), (M.OW2, M.OB2), (M.OB2, M.OW3), (M.OW3, M.OB3),
                 (M.OB3, M.NPARAM)):
        e = np.linalg.norm(g_gpu[a:z] - g_ref[a:z]) / (np.linalg.norm(g_ref[a:z]) + 1e-30)
        assert e < 1e-3, (a, z, e)


def test_training_fits_a_smooth_map(gpulib):
    rng = np.random.default_rng(13)
    X = rng.normal(0, 1, (20000, 9)).astype(np.float32)
    Y = np.stack([np.sin(X[:, 0]) + 0.5 * X[:, 1] * X[:, 2], X[:, 3] ** 2 - X[:, 4],
                  np.tanh(X[:, 5] + X[:, 6] - X[:, 7] * X[:, 8])], 1).astype(np.float32)
    w, losses = learned.train(gpulib, X, Y, epochs=30, batch=1024, lr=3e-3, seed=1)
    assert losses[-1] < 0.1 * losses[0]
    assert losses[-1] < 0.1
    # the blob carries its normalisation: the forward pass reproduces the targets
    pred = learned.forward(gpulib, w, X[:2000])
    rel = np.sqrt(np.mean((pred - Y[:2000]) ** 2, 0)) / Y[:2000].std(0)
    assert np.all(rel < 0.35), rel


def _worst_bond(s):
    """max over constraints of |l^2 - d^2| / l^2 (minimum image on every axis, as move_shake)."""
    x = np.stack([s.x0, s.y0, s.z0], 1)
    box = np.array([s.lx, s.ly, s.lz])
    worst = 0.0
    for c in range(s.ncons):
        for k in range(3):
            a, b = int(s.constra[k, c]), int(s.constrb[k, c])
            if a <= 0:
                continue
            d = x[a - 1] - x[b - 1]
            d -= box * np.rint(d / box)
            l2 = s.length[s.ictype[c] - 1, k] ** 2
            worst = max(worst, abs(l2 - d @ d) / l2)
    return worst


def test_seeded_shake_converges_in_fewer_sweeps(gpulib):
    s, prm = configs.shake_water(nwat=1024, cells=7)
    ctx = abi.Context(gpulib, s, prm)
    ctx.set_state(s)
    X, Y, sw = learned.collect(ctx, steps=40)
    assert X.shape == (40 * s.ncons, 9) and np.all(np.isfinite(X)) and np.all(np.isfinite(Y))
    assert sw.min() >= 2
    w, losses = learned.train(gpulib, X, Y, epochs=40, batch=2048, lr=2e-3, seed=0)
    assert losses[-1] < 0.2 * losses[0]
    ev = learned.evaluate(ctx, w, steps=20, phase_reps=5)
    assert ev["sweeps_seeded"] < ev["sweeps_plain"], ev
    # same tolerance: after seeded steps the constraints still hold to tol2
    ctx.set_shake_model(w)
    ctx.run(5)
    ctx.get_state(s)
    assert _worst_bond(s) <= prm.shake_tol2 * 1.0001


def test_seed_off_restores_plain_shake(gpulib):
    """Setting and clearing a model returns to the plain SHAKE path (two contexts agree to the
    run-to-run spread of FP64 atomic summation order)."""
    s, prm = configs.shake_water(nwat=256, cells=6)
    s1, s2 = s.copy(), s.copy()
    a, b = abi.Context(gpulib, s1, prm), abi.Context(gpulib, s2, prm)
    a.set_state(s1)
    b.set_state(s2)
    b.set_shake_model(_blob(np.random.default_rng(1)))
    b.set_shake_model(None)
    a.run(4)
    b.run(4)
    a.get_state(s1)
    b.get_state(s2)
    for u, w in ((s1.x0, s2.x0), (s1.y0, s2.y0), (s1.z0, s2.z0)):
        assert np.abs(u - w).max() < 1e-9 * s.lx
