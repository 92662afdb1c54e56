"""The CPU restatement of the learned warm-start MLP (no GPU): its backward pass against finite
differences of its own float64 forward pass, and the BF16 rounding helper."""
import numpy as np

from oracle import mlp_ref


def _problem(n=40, seed=3):
    rng = np.random.default_rng(seed)
    theta = rng.standard_normal(mlp_ref.P) * 0.3
    samples = np.zeros((n, mlp_ref.LOG_FLOATS))
    samples[:, :24] = rng.standard_normal((n, 24)) * 2.0 + 1.0
    samples[:, 24:27] = rng.standard_normal((n, 3))
    samples[:, 27:30] = (rng.random((n, 3)) > 0.2).astype(np.float64)
    mean = samples[:, :24].mean(0)
    std = samples[:, :24].std(0)
    return theta, mean, std, samples


def test_backward_matches_finite_differences():
    theta, mean, std, samples = _problem()
    loss, grad = mlp_ref.loss_and_grad(theta, mean, std, samples, bf=False)
    rng = np.random.default_rng(0)
    idx = rng.choice(mlp_ref.P, 60, replace=False)
    h = 1e-6
    for i in idx:
        tp = theta.copy(); tp[i] += h
        tm = theta.copy(); tm[i] -= h
        fd = (mlp_ref.loss_and_grad(tp, mean, std, samples, bf=False)[0] -
              mlp_ref.loss_and_grad(tm, mean, std, samples, bf=False)[0]) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, grad[i])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -3.14159, 65504.0, 1e-30], np.float32)
    r = mlp_ref.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                    # halfway 1 + 2^-8 rounds to even (1.0)
    assert r[2] == 1.0078125              # above halfway rounds up
    assert r[3] == 1.0078125              # representable
    assert abs(r[4] + 3.140625) < 1e-12
    assert np.all(np.isfinite(r))
