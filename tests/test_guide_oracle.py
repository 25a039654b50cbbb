"""The guiding network's FP64 restatement (oracle): mixture density
normalisation and the loss gradient of the output layer against finite
differences (CPU)."""
from __future__ import annotations

import numpy as np
import pytest


def _sphere_dirs(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def _random_y(seed, kappa_scale=3.0):
    rng = np.random.default_rng(seed)
    y = rng.normal(size=48).astype(np.float32)
    y[1:40:5] = rng.uniform(-3, kappa_scale, 8)   # log-concentrations
    return y


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_mixture_density_integrates_to_one(oracle, seed):
    y = _random_y(seed)
    w = _sphere_dirs(200000, seed + 10)
    lp = np.array([oracle.vmf_mixture_log_pdf(y, d) for d in w[:20000]])
    # Monte Carlo over uniform directions: E[q] * 4 pi = 1
    est = np.exp(lp).mean() * 4 * np.pi
    assert abs(est - 1.0) < 0.05


def test_output_bias_gradient_matches_finite_differences(oracle):
    rng = np.random.default_rng(3)
    n = 32
    params = (rng.normal(size=oracle.mlp_num_params()) * 0.2).astype(np.float32)
    inputs = rng.uniform(-1, 1, (n, 80)).astype(np.float32)
    inputs[:, 75:] = 0
    dirs = _sphere_dirs(n, 4)
    w = rng.uniform(0.1, 2.0, n).astype(np.float32)
    loss, grad = oracle.mlp_loss_grad(params, inputs, dirs, w)
    assert np.isfinite(loss)
    nb = oracle.mlp_num_params()
    b4 = nb - 48
    for j in [0, 1, 2, 5, 7, 13, 21, 39]:
        h = 1e-2
        p1, p2 = params.copy(), params.copy()
        p1[b4 + j] += h
        p2[b4 + j] -= h
        fd = (oracle.mlp_loss_grad(p1, inputs, dirs, w)[0] - oracle.mlp_loss_grad(p2, inputs, dirs, w)[0]) / (2 * h)
        assert abs(fd - grad[b4 + j]) <= 2e-3 * max(1.0, abs(fd)), (j, fd, grad[b4 + j])
    assert np.all(grad[b4 + 40:] == 0)   # unused outputs


def test_adam_step_matches_formula(oracle):
    rng = np.random.default_rng(5)
    n = 100
    p, m, v, g = (rng.normal(size=n).astype(np.float32) for _ in range(4))
    v = np.abs(v)
    p2, m2, v2 = oracle.adam_step(p, m, v, g, t=3)
    mm = 0.9 * m + 0.1 * g
    vv = 0.999 * v + 0.001 * g * g
    want = p - 1e-3 * (mm / (1 - 0.9 ** 3)) / (np.sqrt(vv / (1 - 0.999 ** 3)) + 1e-8)
    assert np.allclose(p2, want, rtol=1e-5, atol=1e-7)
