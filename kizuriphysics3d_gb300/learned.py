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
    blend: float = 1.0          # fraction of the normal prediction used (chosen on held-out scenes)
    blend_tangent: float = 0.0  # fraction of the tangent predictions used

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
        np.savez(path, theta=self.theta, mean=self.mean, std=self.std, blend=np.float32(self.blend),
                 blend_tangent=np.float32(self.blend_tangent), meta=json.dumps(meta or {}))

    @staticmethod
    def load(path: str = MODEL_PATH) -> "WarmStartModel":
        with np.load(path) as z:
            blend = float(z["blend"]) if "blend" in z.files else 1.0
            bt = float(z["blend_tangent"]) if "blend_tangent" in z.files else 0.0
            return WarmStartModel(z["theta"].astype(np.float32), z["mean"].astype(np.float32),
                                  z["std"].astype(np.float32), blend, bt)

    def apply(self, world: World, enable: bool = True):
        world.mlp_set_params(self.theta, self.mean, self.std)
        world.mlp_set_blend(self.blend, self.blend_tangent)
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
          seed: int = 0, world: Optional[World] = None, log=None, quantile: float = 0.0) -> List[float]:
    """Adam on the valid targets, on the GPU: squared error, or with 0 < quantile < 1 the pinball
    loss of that quantile.  Returns the epoch losses."""
    own = world is None
    if own:
        world = World(scenes.pyramid(1))
    try:
        rng = np.random.default_rng(seed)
        order = rng.permutation(samples.shape[0])
        world.mlp_set_params(model.theta, model.mean, model.std)
        world.mlp_set_quantile(quantile)
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
    ap.add_argument("--per-source", type=int, default=60000, help="samples kept from each source")
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--save-samples", default=None, help="also write the training samples (.npz)")
    args = ap.parse_args()
    t0 = time.time()
    log = lambda m: print(f"[{time.time() - t0:7.1f} s] {m}", flush=True)
    rng = np.random.default_rng(0)
    keep = lambda a: a[np.sort(rng.permutation(a.shape[0])[:args.per_source])]
    pile = scenes.pile(20000, seed=1234)
    falling = keep(collect(pile, 200, 150, max_pairs=48 * 20001))
    snap = os.path.join(HERE, "data", "pile20000_step600.npz")
    with np.load(snap) as z:
        state = z["state"]
    settled_scene = scenes.pile(20000, seed=1234)
    for b, st in zip(settled_scene.bodies, state):
        b.pos, b.rot, b.vel, b.ang = tuple(st[0:3]), tuple(st[3:7]), tuple(st[7:10]), tuple(st[10:13])
    settled = keep(collect(settled_scene, 40, 5, max_pairs=48 * 20001))
    field = keep(collect(scenes.stacks(20, 20, 500), 4, 0, max_pairs=4 * 200_401))
    log(f"samples: pile falling {falling.shape[0]}, pile settled {settled.shape[0]}, box field {field.shape[0]}")
    samples = np.concatenate([falling, settled, field])
    if args.save_samples:
        np.savez_compressed(args.save_samples, pile=falling, settled=settled, field=field)
    mean, std = feature_stats(samples)
    model = WarmStartModel.init(mean, std, seed=0)
    losses = train(samples, model, epochs=args.epochs, batch=2048, lr=args.lr, log=log)
    model.blend, model.blend_tangent = 1.0, 0.0  # normal impulse only: tangent predictions hurt
    model.save(args.out, {"samples": int(samples.shape[0]), "losses": losses, "epochs": args.epochs})
    log(f"saved {args.out}")


if __name__ == "__main__":
    main()
