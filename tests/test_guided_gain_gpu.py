"""What the trained guiding network gains.

The guided configuration's scene (the many-light geometry with its 65,536
emitters above a slab that spans the room but for a gap along one wall, so
most light reaches the camera's region indirectly) is rendered at 320x180,
depth 16. For each of 4 seeds a fresh network is trained online on the
tracer's own samples (512 spp in 16-spp waves, 16 Adam steps of 65,536 samples
after each, 512 steps in all; the first 3 bounces guided, alpha 0.75: the
benchmark's schedule) and then frozen. At equal samples (256 spp) the frozen
guided renders' mean squared error against a converged render is compared
with the plain MIS tracer's. The converged render is the plain tracer's with
16,384 spp accumulated in FP64 in two halves; its own variance (a quarter of
the mean squared difference of the halves) is subtracted from every squared
error. The guided estimator's unbiasedness is tested in
test_guided_render_gpu.py.

Single renders of this scene differ by tens of percent in squared error (1 %
of the pixels, next to the slab's gap, holds about 80 % of it), so the test
averages the seeds and asks for a ratio well inside what the benchmark
measures at 480x270 (1.43-1.51x in RMSE).
"""
from __future__ import annotations

import numpy as np
import pytest

from devilray_gb300 import scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

W, H, SPP, DEPTH, SEEDS, REF = 320, 180, 256, 16, 4, 16384


@pytest.fixture(scope="module")
def setup(native, ctx):
    spec = scenes.occluded_light(slab_gap=0.15)
    scene = native.Scene.from_spec(ctx, spec)
    cam = scenes.lower_camera(W, H)
    n = W * H
    acc = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    halves = []
    for h in range(2):
        ref = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
        for off in range(0, REF // 2, 4096):
            acc.zero_()
            scene.render(cam, acc, spp=4096, max_depth=DEPTH, sample_offset=h * (REF // 2) + off, seed=4321)
            torch.cuda.synchronize()
            ref += acc[:, :3].double()
        halves.append(ref / (REF // 2))
    var_ref = float(torch.mean((halves[0] - halves[1]) ** 2).item()) / 4.0
    pos = spec.positions.reshape(-1, 3)
    lo, hi = pos.min(0), pos.max(0)
    return scene, cam, 0.5 * (halves[0] + halves[1]), var_ref, tuple(float(x) for x in (lo + hi) / 2), \
        float((hi - lo).max() / 2)


def _mse(acc, ref, var_ref):
    img = acc[:, :3].double() / acc[:, 3:4].double()
    return float(torch.mean((img - ref) ** 2).item()) - var_ref


def test_trained_guide_lowers_error_at_equal_samples(native, ctx, setup):
    scene, cam, ref, var_ref, center, half = setup
    n = W * H
    wave = 16 * n
    acc = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    plain, guided = [], []
    for sd in range(SEEDS):
        acc.zero_()
        scene.render(cam, acc, spp=SPP, max_depth=DEPTH, seed=100 + sd, wave_paths=wave)
        torch.cuda.synchronize()
        plain.append(_mse(acc, ref, var_ref))
        g = native.Guide(ctx, seed=1 + sd, center=center, half_extent=half)
        acc.zero_()
        scene.render_guided(g, cam, acc, spp=512, max_depth=DEPTH, seed=200 + sd, alpha=0.75, train=True,
                            train_batch=65536, train_steps=16, train_budget=512, bounces=3, wave_paths=wave)
        torch.cuda.synchronize()
        assert np.isfinite(g.last_loss())
        acc.zero_()
        scene.render_guided(g, cam, acc, spp=SPP, max_depth=DEPTH, seed=300 + sd, alpha=0.75, train=False,
                            bounces=3, wave_paths=wave)
        torch.cuda.synchronize()
        guided.append(_mse(acc, ref, var_ref))
        g.close()
    ratio = float(np.mean(plain) / np.mean(guided)) ** 0.5
    print(f"plain mse {plain}, trained-guide mse {guided}, rmse ratio {ratio:.3f}")
    assert ratio >= 1.15, (plain, guided)
