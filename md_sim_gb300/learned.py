"""Learned SHAKE seed: sample collection, training and evaluation on the GPU.

SHAKE (src/move.f90:441-515) moves the two atoms of each constraint c along the constraint's
previous bond vector r_c by multiples of their inverse masses, so after any number of sweeps a
molecule's positions are the unconstrained positions plus sum_c G_c (mii_a r_c, -mii_b r_c) with
G_c the multiplier accumulated over the sweeps.  The network (9 -> 64 -> 64 -> 3, SiLU; BF16
weights, FP32 accumulation, kernels in csrc/mlp.cu) predicts y_c = G_c (mii_a + mii_b) from nine
rotation-invariant features of the unconstrained and previous bonds; the library applies the
prediction as one SHAKE-type update before the sweeps, which then iterate to the unchanged
tolerance.  A perfect prediction leaves one checking sweep; a poor one costs nothing but the
forward pass, since convergence is still tested by SHAKE itself.

All arrays cross the C ABI (mdg_mlp_*, mdg_shake_set_model / _record / _samples).
"""
from __future__ import annotations

import ctypes as C
import os
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from .abi import Context, Lib, MdgError, MDG_OK

NI, NO = 9, 3


def _fp(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def _check(lib: Lib, rc: int):
    if rc != MDG_OK:
        raise MdgError(rc, (lib.last_error(None) or b"").decode())


def nw(lib: Lib) -> int:
    return int(lib.mlp_nw())


def forward(lib: Lib, w: np.ndarray, X: np.ndarray) -> np.ndarray:
    """Network outputs (n, 3) for features X (n, 9), on the GPU."""
    X = np.ascontiguousarray(X, np.float32)
    w = np.ascontiguousarray(w, np.float32)
    Y = np.zeros((X.shape[0], NO), np.float32)
    _check(lib, lib.mlp_forward(_fp(w), _fp(X), X.shape[0], _fp(Y)))
    return Y


def grad(lib: Lib, w: np.ndarray, X: np.ndarray, Y: np.ndarray):
    """(loss, gradient over the trained parameters) of the mean normalised squared error."""
    X = np.ascontiguousarray(X, np.float32)
    Y = np.ascontiguousarray(Y, np.float32)
    w = np.ascontiguousarray(w, np.float32)
    g = np.zeros(nw(lib) - 24, np.float32)
    loss = C.c_float()
    _check(lib, lib.mlp_grad(_fp(w), _fp(X), _fp(Y), X.shape[0], _fp(g), C.byref(loss)))
    return float(loss.value), g


def train(lib: Lib, X: np.ndarray, Y: np.ndarray, epochs: int = 40, batch: int = 2048, lr: float = 2e-3,
          seed: int = 0):
    """Adam with cosine decay from a seeded start; returns (blob, per-epoch mean loss)."""
    X = np.ascontiguousarray(X, np.float32)
    Y = np.ascontiguousarray(Y, np.float32)
    w = np.zeros(nw(lib), np.float32)
    losses = np.zeros(epochs, np.float32)
    _check(lib, lib.mlp_train(_fp(X), _fp(Y), X.shape[0], int(epochs), int(batch), float(lr), int(seed),
                              _fp(w), _fp(losses)))
    return w, losses


def collect(ctx: Context, steps: int, every: int = 1):
    """Runs `steps` resident MD steps recording SHAKE; returns features (n, 9), targets (n, 3)
    and the sweeps each molecule took (n,), from every `every`-th step."""
    ctx.shake_record(True)
    xs: List[np.ndarray] = []
    try:
        for k in range(steps):
            ctx.run(1)
            if k % every == 0:
                xs.append(ctx.shake_samples().copy())
    finally:
        ctx.shake_record(False)
    r = np.concatenate(xs, 0)
    return r[:, :NI], r[:, NI:NI + NO], r[:, 12]


@dataclass
class SweepStats:
    steps: int
    mean_sweeps: float          # per molecule and step
    max_sweeps: float
    step_ms: float              # wall time per resident step (host clock around run())
    per_step_mean: List[float] = field(default_factory=list)


def sweep_stats(ctx: Context, steps: int) -> SweepStats:
    ctx.shake_record(True)
    means, mx = [], 0.0
    t_total = 0.0
    try:
        for _ in range(steps):
            t0 = time.perf_counter()
            ctx.run(1)
            t_total += time.perf_counter() - t0
            r = ctx.shake_samples()
            means.append(float(r[:, 12].mean()))
            mx = max(mx, float(r[:, 12].max()))
    finally:
        ctx.shake_record(False)
    return SweepStats(steps, float(np.mean(means)), mx, 1e3 * t_total / max(steps, 1), means)


def evaluate(ctx: Context, w: np.ndarray, steps: int = 50, phase_reps: int = 20) -> Dict[str, float]:
    """Same starting state, SHAKE plain then seeded: sweeps per molecule and the SHAKE phase time
    (CUDA events around the SHAKE kernels of a full step, mdg_phase_times)."""
    s0 = ctx.get_state(ctx.sys.copy())
    ctx.set_shake_model(None)
    plain = sweep_stats(ctx, steps)
    t_plain = ctx.phase_times(phase_reps)["shake"]
    ctx.set_state(s0)
    ctx.set_shake_model(w)
    seeded = sweep_stats(ctx, steps)
    t_seed = ctx.phase_times(phase_reps)["shake"]
    ctx.set_shake_model(None)
    return {
        "steps": steps,
        "sweeps_plain": plain.mean_sweeps, "sweeps_seeded": seeded.mean_sweeps,
        "max_sweeps_plain": plain.max_sweeps, "max_sweeps_seeded": seeded.max_sweeps,
        "sweeps_saved_frac": 1.0 - seeded.mean_sweeps / max(plain.mean_sweeps, 1e-30),
        "shake_ms_plain": t_plain, "shake_ms_seeded": t_seed,
        "shake_ms_saved": t_plain - t_seed,
    }


DEFAULT_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "shake_seed.npy")


def load_or_train(lib: Lib, ctx: Context, s_start, path: str = DEFAULT_MODEL, steps: int = 30, epochs: int = 20):
    """The stored seed network if it exists (and matches this build's parameter count), else a
    quick one trained on `steps` plain SHAKE steps from s_start.  Returns (blob, description)."""
    if os.path.exists(path):
        w = np.load(path).astype(np.float32)
        if w.size == nw(lib):
            return w, f"stored ({os.path.basename(path)})"
    ctx.set_state(s_start.copy())
    X, Y, _ = collect(ctx, steps)
    w, losses = train(lib, X, Y, epochs=epochs, batch=4096, lr=2e-3, seed=9)
    return w, f"trained here on {X.shape[0]} samples, {epochs} epochs, loss {losses[0]:.3g} -> {losses[-1]:.3g}"


def main(argv=None):
    """Collect multipliers from plain SHAKE on the 8192-water SHAKE config, train the seed network
    on the GPU, evaluate it from a fresh start and save the parameter blob (float32 .npy)."""
    import argparse
    import json

    import md_sim_gb300
    from . import configs
    from .abi import MDG_MIXED

    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--nwat", type=int, default=8192)
    ap.add_argument("--cells", type=int, default=19)
    ap.add_argument("--samples", type=int, default=1_000_000)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=9)
    ap.add_argument("--eval-steps", type=int, default=100)
    ap.add_argument("--equil", type=int, default=300)
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                                                  "shake_seed.npy"))
    args = ap.parse_args(argv)
    lib = md_sim_gb300.load()
    s, prm = configs.shake_water(nwat=args.nwat, cells=args.cells)
    prm.precision = MDG_MIXED
    ctx = Context(lib, s, prm)
    configs.equilibrate(ctx, s, steps=args.equil, every=10)   # leave the start-up transient at 300 K
    ctx.set_state(s)
    steps = max(1, (args.samples + s.ncons - 1) // s.ncons)
    t0 = time.perf_counter()
    X, Y, sw = collect(ctx, steps)
    t_collect = time.perf_counter() - t0
    t0 = time.perf_counter()
    w, losses = train(lib, X, Y, epochs=args.epochs, batch=args.batch, lr=args.lr, seed=args.seed)
    t_train = time.perf_counter() - t0
    ev = evaluate(ctx, w, steps=args.eval_steps)
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    np.save(args.out, w)
    rep = {"samples": int(X.shape[0]), "collect_s": t_collect, "train_s": t_train, "epochs": args.epochs,
           "loss_first": float(losses[0]), "loss_last": float(losses[-1]), "plain_sweeps_in_data": float(sw.mean()),
           **ev, "out": args.out}
    print(json.dumps(rep))
    return rep


if __name__ == "__main__":
    main()
