"""CPU checks of the SHAKE-seed restatement (oracle/mlp.py): its gradient against finite
differences, BF16 rounding, feature invariance, and the seed algebra (an exact multiplier
prediction leaves SHAKE a single checking sweep)."""
import numpy as np
import pytest

import mlp as M


def _blob(rng):
    b = np.zeros(M.NW, np.float32)
    b[M.OW1:M.OB1] = rng.normal(0, np.sqrt(2 / 9), M.NH * M.NI)
    b[M.OW2:M.OB2] = rng.normal(0, np.sqrt(2 / 64), M.NH * M.NH)
    b[M.OW3:M.OB3] = 0.1 * rng.normal(0, np.sqrt(2 / 64), M.NO * M.NH)
    b[M.OB1:M.OW2] = rng.normal(0, 0.1, M.NH)
    b[M.OXM:M.OXS] = rng.normal(0, 1, 9)
    b[M.OXS:M.OYM] = rng.uniform(0.5, 2, 9)
    b[M.OYM:M.OYS] = rng.normal(0, 1, 3)
    b[M.OYS:M.NW] = rng.uniform(0.5, 2, 3)
    return b


def test_layout():
    assert M.NPARAM == 4995 and M.NW == 5019


def test_bf16_round_known_values():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -3.140625, 1.00390625], np.float32)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: nearest even -> 1.0
    assert M.bf16_round(x).tolist() == [1.0, 1.0, 1.0 + 2 ** -7, -3.140625, 1.0]


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    b = _blob(rng)
    X = rng.normal(0, 1, (40, 9))
    T = rng.normal(0, 1, (40, 3))
    # evaluate at BF16-representable weights so the rounding inside unpack() is the identity
    b[:M.NPARAM] = M.bf16_round(b[:M.NPARAM])
    loss, g = M.loss_grad(b, X, T)
    assert loss > 0
    p = M.unpack(b)

    def loss_at(theta):
        W1 = theta[M.OW1:M.OB1].reshape(64, 9); b1 = theta[M.OB1:M.OW2]
        W2 = theta[M.OW2:M.OB2].reshape(64, 64); b2 = theta[M.OB2:M.OW3]
        W3 = theta[M.OW3:M.OB3].reshape(3, 64); b3 = theta[M.OB3:M.NPARAM]
        x = (X - p["xm"]) * p["xs"]
        y = M.silu(M.silu(x @ W1.T + b1) @ W2.T + b2) @ W3.T + b3
        e = y - (T - p["ym"]) / p["ys"]
        return (e * e).sum() / X.shape[0]

    theta = b[:M.NPARAM].astype(np.float64)
    assert abs(loss_at(theta) - loss) < 1e-12 * max(1, loss)
    for k in list(rng.choice(M.NPARAM, 60, replace=False)) + [M.OB3, M.OB1 + 3, M.OW3 + 7]:
        h = 1e-6
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        fd = (loss_at(tp) - loss_at(tm)) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, g[k])


def _rot(rng):
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    return q


def _molecule(rng):
    """A water-like molecule: previous positions on the constraints, unconstrained = moved."""
    l = np.array([1.0, 1.0, 1.633])
    old = np.array([[0.0, 0.0, 0.0], [0.8165, 0.5773, 0.0], [-0.8165, 0.5773, 0.0]])
    pairs = [(0, 1), (0, 2), (1, 2)]
    l2 = np.array([np.sum((old[a] - old[b]) ** 2) for a, b in pairs])
    pos = old + rng.normal(0, 0.02, old.shape) + np.array([0.1, 0.0, 0.0])
    return pos, old, pairs, l2


def test_features_are_rotation_and_translation_invariant():
    rng = np.random.default_rng(5)
    pos, old, pairs, l2 = _molecule(rng)
    f0 = M.features(np.array([pos[a] - pos[b] for a, b in pairs]),
                    np.array([old[a] - old[b] for a, b in pairs]), l2)
    R = _rot(rng)
    t = rng.normal(size=3) * 10
    p2, o2 = pos @ R.T + t, old @ R.T + t
    f1 = M.features(np.array([p2[a] - p2[b] for a, b in pairs]),
                    np.array([o2[a] - o2[b] for a, b in pairs]), l2)
    assert np.allclose(f0, f1, atol=1e-12)


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_exact_seed_leaves_one_checking_sweep(seed):
    rng = np.random.default_rng(seed)
    pos, old, pairs, l2 = _molecule(rng)
    mii = np.array([1 / 15.9994, 1 / 1.008, 1 / 1.008])
    x1, sw1, y = M.shake_molecule(pos, old, pairs, l2, mii, 1e-10, 100)
    assert sw1 > 2
    x2, sw2, y2 = M.shake_molecule(pos, old, pairs, l2, mii, 1e-10, 100, seed_y=y)
    assert sw2 == 1
    assert np.abs(x2 - x1).max() < 1e-12
    # a 1 % error in the prediction still converges, in fewer sweeps than no seed
    x3, sw3, _ = M.shake_molecule(pos, old, pairs, l2, mii, 1e-10, 100, seed_y=y * 1.01)
    assert sw3 < sw1
    for c, (a, b) in enumerate(pairs):
        d = x3[a] - x3[b]
        assert abs(l2[c] - d @ d) <= l2[c] * 1e-10
