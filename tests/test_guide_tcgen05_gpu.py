"""The guiding network's tcgen05 inference kernel (tensor-memory
accumulators, shared-memory descriptors) against the warp-level mma.sync
kernel: the same BF16 products summed in FP32, so the outputs agree to FP32
summation-order differences (and the rare activation that then rounds to the
neighbouring BF16 value)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("n", [1, 128, 129, 5000, 100000])
def test_tcgen05_matches_mma_sync(native, ctx, n):
    rng = np.random.default_rng(n)
    tc = native.Guide(ctx, seed=4, center=(0.0, 0.0, 0.0), half_extent=10.0, infer_kernel=0)
    ms = native.Guide(ctx, seed=4, center=(0.0, 0.0, 0.0), half_extent=10.0, infer_kernel=1)
    p = tc.params()
    p[-48:] = rng.normal(0, 0.3, 48)   # nonzero output biases
    tc.set_params(p)
    ms.set_params(p)
    pos = torch.from_numpy(rng.uniform(-10, 10, (n, 3)).astype(np.float32)).cuda()
    d = rng.normal(size=(n, 3))
    nrm = torch.from_numpy((d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)).cuda()
    y_tc = torch.full((n, 40), float("nan"), dtype=torch.float32, device="cuda")
    y_ms = torch.full((n, 40), float("nan"), dtype=torch.float32, device="cuda")
    tc.infer(pos, nrm, n, y_tc)
    ms.infer(pos, nrm, n, y_ms)
    torch.cuda.synchronize()
    ctx.check()
    a, b = y_tc.cpu().numpy(), y_ms.cpu().numpy()
    assert np.all(np.isfinite(a))
    err = np.abs(a - b)
    scale = np.abs(b).max() + 1e-6
    assert np.median(err) <= 1e-6 * scale + 1e-7 and err.max() <= 2e-2 * scale, (np.median(err), err.max(), scale)


@pytest.mark.parametrize("n", [300, 50000])
def test_tcgen05_training_matches_mma_sync(native, ctx, n):
    """Gradients of the tcgen05 training kernel against the mma.sync one on the
    same batch (50,000 rows: more 128-row tiles than resident CTAs)."""
    rng = np.random.default_rng(n + 1)
    tc = native.Guide(ctx, seed=5, center=(0.0, 0.0, 0.0), half_extent=10.0, infer_kernel=0)
    ms = native.Guide(ctx, seed=5, center=(0.0, 0.0, 0.0), half_extent=10.0, infer_kernel=1)
    p = tc.params()
    p[-48:] = rng.normal(0, 0.3, 48)
    tc.set_params(p)
    ms.set_params(p)

    def unit(k):
        d = rng.normal(size=(k, 3))
        return torch.from_numpy((d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)).cuda()

    pos = torch.from_numpy(rng.uniform(-10, 10, (n, 3)).astype(np.float32)).cuda()
    nrm, sdir = unit(n), unit(n)
    w = torch.from_numpy(rng.lognormal(0.0, 1.0, n).astype(np.float32)).cuda()
    l_tc, g_tc = tc.gradients(pos, nrm, sdir, w, n)
    l_ms, g_ms = ms.gradients(pos, nrm, sdir, w, n)
    ctx.check()
    assert np.all(np.isfinite(g_tc))
    assert abs(l_tc - l_ms) <= 1e-4 * abs(l_ms)
    a, b = g_tc.astype(np.float64), g_ms.astype(np.float64)
    rel = np.linalg.norm(a - b) / np.linalg.norm(b)
    assert rel <= 1e-2, rel
