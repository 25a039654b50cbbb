"""What the trained guiding network gains.

The guided configuration's scene (the many-light geometry with its 65,536
emitters above a slab that spans the room but for a gap along one wall, so
most light reaches the camera's region indirectly) is rendered at 192x108,
depth 16, by the plain MIS tracer and by the guided tracer, whose network
starts untrained and is trained online on the tracer's own samples (16 Adam
steps of 65,536 samples after every 16-spp wave, the first 3 bounces guided,
alpha 0.75: the benchmark's schedule). At equal samples per pixel the guided
renders' mean squared error against a converged render is lower than the
plain renders', over 3 seeds each. The converged render is the plain tracer's
with 32,768 spp accumulated in FP64 (the guided estimator's unbiasedness is
tested in test_guided_render_gpu.py).
"""
from __future__ import annotations

import numpy as np
import pytest

from devilray_gb300 import scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

W, H, SPP, DEPTH, SEEDS = 192, 108, 512, 16, 3


@pytest.fixture(scope="module")
def setup(native, ctx):
    spec = scenes.occluded_light(slab_gap=0.15)
    scene = native.Scene.from_spec(ctx, spec)
    cam = scenes.lower_camera(W, H)
    n = W * H
    acc = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    ref = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    for off in range(0, 32768, 4096):
        acc.zero_()
        scene.render(cam, acc, spp=4096, max_depth=DEPTH, sample_offset=off, seed=4321)
        torch.cuda.synchronize()
        ref += acc[:, :3].double()
    pos = spec.positions.reshape(-1, 3)
    lo, hi = pos.min(0), pos.max(0)
    return spec, scene, cam, (ref / 32768.0), tuple(float(x) for x in (lo + hi) / 2), float((hi - lo).max() / 2)


def _mse(acc, ref):
    img = acc[:, :3].double() / acc[:, 3:4].double()
    return float(torch.mean((img - ref) ** 2).item())


def test_trained_guide_lowers_error_at_equal_samples(native, ctx, setup):
    spec, scene, cam, ref, center, half = setup
    n = W * H
    acc = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    plain, guided = [], []
    for sd in range(SEEDS):
        acc.zero_()
        scene.render(cam, acc, spp=SPP, max_depth=DEPTH, seed=100 + sd, wave_paths=16 * n)
        torch.cuda.synchronize()
        plain.append(_mse(acc, ref))
        g = native.Guide(ctx, seed=1 + sd, center=center, half_extent=half)
        acc.zero_()
        scene.render_guided(g, cam, acc, spp=SPP, max_depth=DEPTH, seed=200 + sd, alpha=0.75, train=True,
                            train_batch=65536, train_steps=16, train_budget=512, bounces=3, wave_paths=16 * n)
        torch.cuda.synchronize()
        guided.append(_mse(acc, ref))
        assert np.isfinite(g.last_loss())
        g.close()
    ratio = float(np.mean(plain) / np.mean(guided))
    print(f"plain mse {plain}, guided mse {guided}, rmse ratio {ratio ** 0.5:.3f}")
    assert ratio ** 0.5 >= 1.08, (plain, guided)
