"""Learned warm start on the GPU (libkzg kzg_mlp_*): forward and backward kernels against the CPU
restatement (oracle/mlp_ref.py), training, logging inside the step, and what the trained network
gains over the plain warm start."""
import os

import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def _problem(n, seed):
    rng = np.random.default_rng(seed)
    theta = (rng.standard_normal(mlp_ref.P) * 0.25).astype(np.float32)
    s = np.zeros((n, mlp_ref.LOG_FLOATS), np.float32)
    s[:, :24] = rng.standard_normal((n, 24)) * rng.uniform(0.1, 5.0, 24) + rng.uniform(-3, 3, 24)
    s[:, 24:27] = rng.standard_normal((n, 3)) * 0.2
    s[:, 27:30] = rng.random((n, 3)) > 0.15
    mean = s[:, :24].mean(0).astype(np.float32)
    std = s[:, :24].std(0).astype(np.float32)
    return theta, mean, std, s


def _ctx():
    from kizuriphysics3d_gb300 import World, scenes
    return World(scenes.pyramid(1))


def _split(v):
    return mlp_ref.unpack(v)


@pytest.mark.parametrize("first,count,tau", [(0, 300, 0.0), (37, 150, 0.0), (5, 1, 0.0), (11, 250, 0.2)])
def test_gradient_matches_cpu_oracle(first, count, tau):
    theta, mean, std, s = _problem(400, seed=11)
    with _ctx() as w:
        w.mlp_set_params(theta, mean, std)
        w.mlp_set_quantile(tau)
        w.mlp_set_dataset(s)
        g, loss = w.mlp_gradient(first, count)
    ref_loss, ref = mlp_ref.loss_and_grad(theta, mean, std, s[first:first + count], bf=True, tau=tau)
    assert abs(loss - ref_loss) <= 1e-3 * abs(ref_loss) + 1e-7
    for name, a, b in zip(("W1", "b1", "W2", "b2", "W3", "b3"), _split(g), _split(ref)):
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
        assert err < 2e-2, (name, err)


def test_forward_matches_cpu_oracle():
    theta, mean, std, s = _problem(333, seed=5)
    with _ctx() as w:
        w.mlp_set_params(theta, mean, std)
        w.mlp_set_dataset(s)
        y = w.mlp_predict(0, 333)
    ref = mlp_ref.forward(theta, mean, std, s[:, :24])["Y"]
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-2


def test_training_reduces_loss_and_is_deterministic():
    from kizuriphysics3d_gb300.learned import WarmStartModel, train
    rng = np.random.default_rng(2)
    n = 6000
    s = np.zeros((n, mlp_ref.LOG_FLOATS), np.float32)
    s[:, :24] = rng.standard_normal((n, 24))
    s[:, 24] = np.tanh(s[:, 0] - 0.5 * s[:, 3])        # smooth targets of the features
    s[:, 25] = 0.3 * s[:, 5] * (s[:, 6] > 0)
    s[:, 26] = np.sin(s[:, 7])
    s[:, 27:30] = 1.0
    mean, std = s[:, :24].mean(0), s[:, :24].std(0)
    runs = []
    for _ in range(2):
        m = WarmStartModel.init(mean, std, seed=4)
        losses = train(s, m, epochs=25, batch=1024, lr=3e-3, seed=1)
        runs.append((losses, m.theta.copy()))
    assert runs[0][0][-1] < 0.2 * runs[0][0][0]
    assert np.array_equal(runs[0][1], runs[1][1])  # fixed-order gradient sums: identical runs


def test_step_logs_cache_misses():
    from kizuriphysics3d_gb300 import World, scenes
    sc = scenes.pile(300, seed=21, extent=3.0, y_range=(1.0, 10.0))
    with World(sc) as w:
        w.step_fixed(n=30)
        w.mlp_log_begin(100000)
        w.step_fixed(n=40)
        log = w.mlp_log_fetch()
    assert log.shape[0] > 100
    assert np.all(np.isfinite(log))
    assert set(np.unique(log[:, 27:30])) <= {0.0, 1.0}
    assert log[:, 27].mean() > 0.9  # normal rows have a positive effective mass


def test_zero_prediction_equals_plain_warm_start():
    """A model that predicts zero leaves every cache-missing point at the reference's zero warm
    start, so the learned path reproduces the plain path bit for bit (the prediction touches
    nothing else)."""
    from kizuriphysics3d_gb300 import World, scenes
    from kizuriphysics3d_gb300.learned import WarmStartModel
    _, mean, std, _ = _problem(10, seed=1)
    sc = scenes.pile(300, seed=23, extent=3.0, y_range=(1.0, 10.0))
    hashes = []
    for learned in (False, True):
        with World(sc) as w:
            if learned:
                WarmStartModel(np.zeros(mlp_ref.P, np.float32), mean, std).apply(w)
            w.step_fixed(n=60)
            hashes.append(w.compute_state_hash())
    assert hashes[0] == hashes[1]


def test_learned_warm_start_keeps_determinism():
    from kizuriphysics3d_gb300 import World, scenes
    from kizuriphysics3d_gb300.learned import WarmStartModel
    theta, mean, std, _ = _problem(10, seed=1)
    sc = scenes.pile(300, seed=22, extent=3.0, y_range=(1.0, 10.0))
    hashes = []
    for _ in range(2):
        with World(sc) as w:
            WarmStartModel(theta * 0.1, mean, std).apply(w)
            w.set_residual(1e-4, 64)
            w.step_fixed(n=80)
            hashes.append(w.compute_state_hash())
    assert hashes[0] == hashes[1]


def test_learned_warm_start_on_held_out_pile_at_the_metric_tolerance():
    """The committed model on data it was not trained on: the 20,000-body pile of a fresh seed (98765)
    after 600 steps (committed snapshot), relative impulse change <= 1e-4 with the cap raised to
    1,024 so that the tolerance is actually reached.  Both warm starts converge to it (the solver's
    own residual judges the prediction).  Measured on GB300 (6 steps after 2): plain 357,304,682
    point-iterations (~598 iterations on the giant island), learned 363,093,274 (+1.6%): at this
    tolerance the learned warm start costs iterations; at 1e-3 it saves 1.0% and at 3e-3 0.35%.
    The test holds the convergence and bounds the cost."""
    from kizuriphysics3d_gb300 import scenes
    from kizuriphysics3d_gb300.learned import MODEL_PATH, WarmStartModel, evaluate
    model = WarmStartModel.load(MODEL_PATH)
    snap = os.path.join(os.path.dirname(__file__), "..", "kizuriphysics3d_gb300", "data",
                        "pile20000_s98765_step600.npz")
    sc = scenes.pile(20000, seed=98765)
    with np.load(snap) as z:
        state = z["state"]
    for b, st in zip(sc.bodies, state):
        b.pos, b.rot, b.vel, b.ang = tuple(st[0:3]), tuple(st[3:7]), tuple(st[7:10]), tuple(st[10:13])
    kw = dict(steps=4, skip=2, tol=1e-4, cap=1024, max_pairs=48 * 20001)
    plain = evaluate(sc, None, **kw)
    learned = evaluate(sc, model, **kw)
    for r in (plain, learned):
        assert r["mean_max_iterations"] < 1024  # reached the tolerance before the cap
        assert r["mean_final_residual"] <= 1.01e-4
    assert learned["point_iterations"] <= 1.05 * plain["point_iterations"], (plain, learned)
