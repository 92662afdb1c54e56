"""Learned warm start: the model file, sample collection and GPU training.

Contact points that miss the manifold cache start the solve from zero impulses in the reference
(PhysicsWorld.cpp:518-529).  Here an MLP (24 features -> 64 -> 64 -> 3) can predict their
impulses instead; everything runs in libkzg (kzg_mlp_* in include/kzg.h):

* ``collect`` steps a scene with many velocity iterations (so the impulses are converged) and logs
  every cache-missing point: its 24 features before the solve and impulse / effective mass after;
* ``train`` fits the network on the GPU with the library's own forward and backward kernels
  (Adam, mini-batches, deterministic per-batch gradients);
* ``WarmStartModel`` holds the parameters with the feature standardisation and reads/writes the
  ``.npz`` model file that ``World.mlp_set_params`` loads.

    python -m kizuriphysics3d_gb300.learned --out kizuriphysics3d_gb300/data/warmstart_mlp.npz
"""
from __future__ import annotations

import argparse
import json
import os
import time
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from . import capi, scenes
from .world import World

HERE = os.path.dirname(os.path.abspath(__file__))
MODEL_PATH = os.path.join(HERE, "data", "warmstart_mlp.npz")
F, H, O = capi.MLP_FEATURES, 64, 3
TARGET_SCALE = 0.05  # the network regresses asinh(y / TARGET_SCALE); kzg_mlp.cu maps back with sinh


def to_network_targets(samples: np.ndarray) -> np.ndarray:
    """Logged samples (targets y = impulse / effective mass, m/s) -> training samples."""
    s = np.array(samples, np.float32, copy=True)
    s[:, F:F + O] = np.arcsinh(s[:, F:F + O] / TARGET_SCALE)
    return s


@dataclass
class WarmStartModel:
    theta: np.ndarray  # MLP_PARAMS float32
    mean: np.ndarray   # 24
    std: np.ndarray    # 24

    @staticmethod
    def init(mean: np.ndarray, std: np.ndarray, seed: int = 0) -> "WarmStartModel":
        """He-initialised weights, zero biases."""
        rng = np.random.default_rng(seed)
        W1 = rng.standard_normal((H, F)) * np.sqrt(2.0 / F)
        W2 = rng.standard_normal((H, H)) * np.sqrt(2.0 / H)
        W3 = rng.standard_normal((O, H)) * np.sqrt(1.0 / H)
        theta = np.concatenate([W1.ravel(), np.zeros(H), W2.ravel(), np.zeros(H), W3.ravel(), np.zeros(O)])
        return WarmStartModel(theta.astype(np.float32), np.asarray(mean, np.float32), np.asarray(std, np.float32))

    def save(self, path: str, meta: Optional[dict] = None):
        np.savez(path, theta=self.theta, mean=self.mean, std=self.std,
                 meta=json.dumps(meta or {}))

    @staticmethod
    def load(path: str = MODEL_PATH) -> "WarmStartModel":
        with np.load(path) as z:
            return WarmStartModel(z["theta"].astype(np.float32), z["mean"].astype(np.float32),
                                  z["std"].astype(np.float32))

    def apply(self, world: World, enable: bool = True):
        world.mlp_set_params(self.theta, self.mean, self.std)
        world.mlp_enable(enable)


def feature_stats(samples: np.ndarray):
    x = samples[:, :F].astype(np.float64)
    return x.mean(0).astype(np.float32), np.maximum(x.std(0), 1e-3).astype(np.float32)


def collect(scene: scenes.Scene, steps: int, skip: int = 0, iterations: int = 64, capacity: int = 2_000_000,
            max_pairs: Optional[int] = None) -> np.ndarray:
    """Log (features, converged impulse / effective mass, masks) of every cache-missing contact point
    over `steps` steps after `skip` unlogged steps, solving with `iterations` velocity iterations."""
    with World(scene, max_pairs=max_pairs) as w:
        w.set_solver(velocity_iterations=int(iterations))
        if skip:
            w.step_fixed(n=skip)
        w.mlp_log_begin(capacity)
        w.step_fixed(n=steps)
        return w.mlp_log_fetch()


def train(samples: np.ndarray, model: WarmStartModel, epochs: int = 20, batch: int = 4096, lr: float = 1e-3,
          seed: int = 0, world: Optional[World] = None, log=None) -> List[float]:
    """Adam on the mean-squared error of the valid targets, on the GPU.  Returns the epoch losses."""
    own = world is None
    if own:
        world = World(scenes.pyramid(1))
    try:
        rng = np.random.default_rng(seed)
        order = rng.permutation(samples.shape[0])
        world.mlp_set_params(model.theta, model.mean, model.std)
        world.mlp_set_dataset(to_network_targets(samples[order]))
        n = samples.shape[0]
        losses = []
        for ep in range(epochs):
            tot, cnt = 0.0, 0
            for first in range(0, n, batch):
                cnt_b = min(batch, n - first)
                tot += world.mlp_train_step(first, cnt_b, lr) * cnt_b
                cnt += cnt_b
            losses.append(tot / max(cnt, 1))
            if log:
                log(f"epoch {ep}: loss {losses[-1]:.6f}")
        model.theta = world.mlp_get_params()[0]
        return losses
    finally:
        if own:
            world.close()


def evaluate(scene: scenes.Scene, model: Optional[WarmStartModel], steps: int, skip: int = 0, tol: float = 1e-4,
             cap: int = 64, max_pairs: Optional[int] = None) -> dict:
    """Step a scene with residual-terminated velocity iterations, with or without the learned warm
    start, and sum the solver work (batched points x iterations) and the final residuals."""
    with World(scene, max_pairs=max_pairs) as w:
        if skip:
            w.step_fixed(n=skip)
        w.set_residual(tol, cap)
        if model is not None:
            model.apply(w)
        pt_iters, res, iters, ms = 0, [], [], 0.0
        for _ in range(steps):
            w.step_fixed()
            st = w.get_stats()
            pt_iters += st["point_velocity_iterations"]
            res.append(st["final_residual"])
            iters.append(st["max_velocity_iterations_used"])
            ms += st["step_ms"]
        return {"point_iterations": int(pt_iters), "mean_final_residual": float(np.mean(res)),
                "mean_max_iterations": float(np.mean(iters)), "step_ms": ms / max(steps, 1)}


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--out", default=MODEL_PATH)
    ap.add_argument("--pile-steps", type=int, default=240)
    ap.add_argument("--pile-skip", type=int, default=120)
    ap.add_argument("--field-steps", type=int, default=6)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--save-samples", default=None, help="also write the collected samples (.npz)")
    args = ap.parse_args()
    t0 = time.time()
    log = lambda m: print(f"[{time.time() - t0:7.1f} s] {m}", flush=True)
    pile = scenes.pile(20000, seed=1234)
    s1 = collect(pile, args.pile_steps, args.pile_skip, max_pairs=48 * 20001)
    log(f"random convex pile (seed 1234): {s1.shape[0]} samples")
    field = scenes.stacks(20, 20, 500)
    s2 = collect(field, args.field_steps, 0, max_pairs=4 * 200_401)
    keep = np.random.default_rng(7).permutation(s2.shape[0])[:s1.shape[0]]  # as many as the pile gave
    s2 = s2[np.sort(keep)]
    log(f"large box field (seed 7): {s2.shape[0]} samples")
    samples = np.concatenate([s1, s2])
    if args.save_samples:  # a 100k subsample of each source, for inspection
        sub = lambda a: a[np.sort(np.random.default_rng(0).permutation(a.shape[0])[:100000])]
        np.savez_compressed(args.save_samples, pile=sub(s1), field=sub(s2))
    mean, std = feature_stats(samples)
    model = WarmStartModel.init(mean, std, seed=0)
    losses = train(samples, model, epochs=args.epochs, lr=args.lr, log=log)
    model.save(args.out, {"samples": int(samples.shape[0]), "losses": losses, "pile_steps": args.pile_steps,
                          "pile_skip": args.pile_skip, "field_steps": args.field_steps, "epochs": args.epochs})
    log(f"saved {args.out}")


if __name__ == "__main__":
    main()
