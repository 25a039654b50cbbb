"""Guided rendering (dr_render_guided).

The guided estimator divides by the density of the one-sample mixture
(alpha x network mixture + (1 - alpha) x cosine lobe), so for any network the
image converges to the plain tracer's: with alpha = 0 it reproduces the plain
image up to FP32 rounding, and with an untrained (random) network its mean
agrees with independent plain renders within their noise.
"""
from __future__ import annotations

import numpy as np
import pytest

from devilray_gb300 import scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _render(native, scene, cam, spp, depth, seed, guide=None, **kw):
    n = cam["width"] * cam["height"]
    acc = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    casts = torch.zeros(n, dtype=torch.int32, device="cuda")
    if guide is None:
        scene.render(cam, acc, casts, spp=spp, max_depth=depth, seed=seed)
    else:
        scene.render_guided(guide, cam, acc, casts, spp=spp, max_depth=depth, seed=seed, **kw)
    torch.cuda.synchronize()
    a = acc.cpu().numpy().astype(np.float64)
    return a[:, :3] / a[:, 3:4], a


def _guide_for(native, ctx, spec, seed=7, kernel=0):
    pos = spec.positions.reshape(-1, 3)
    lo, hi = pos.min(0), pos.max(0)
    return native.Guide(ctx, seed=seed, center=tuple((lo + hi) / 2), half_extent=float((hi - lo).max() / 2),
                        infer_kernel=kernel)


def test_alpha_zero_reproduces_the_plain_image(native, ctx):
    spec = scenes.box_room(sphere_level=2)
    scene = native.Scene.from_spec(ctx, spec)
    cam = scenes.camera(40, 30)
    g = _guide_for(native, ctx, spec)
    plain, pa = _render(native, scene, cam, 16, 8, 3)
    guided, ga = _render(native, scene, cam, 16, 8, 3, guide=g, alpha=0.0, train=False)
    assert np.array_equal(pa[:, 3], ga[:, 3])
    # the same paths; only the rounding of f cos / pdf and of the stored pdf differs
    rel = np.abs(guided - plain) / (np.abs(plain) + 1e-3)
    assert np.median(rel) < 1e-5 and rel.max() < 2e-3, (np.median(rel), rel.max())


@pytest.mark.parametrize("bounces,kernel", [(0, 0), (1, 0), (0, 1)])
def test_untrained_guide_is_unbiased(native, ctx, bounces, kernel):
    """kernel 1: the mma.sync inference, whose rows the renderer decodes in a
    separate pass (the tcgen05 inference decodes in its epilogue)."""
    spec = scenes.box_room(sphere_level=2)
    scene = native.Scene.from_spec(ctx, spec)
    cam = scenes.camera(24, 18)
    g = _guide_for(native, ctx, spec, seed=11, kernel=kernel)
    a, _ = _render(native, scene, cam, 2048, 6, 1)
    b, _ = _render(native, scene, cam, 2048, 6, 2)
    gi, _ = _render(native, scene, cam, 2048, 6, 3, guide=g, alpha=0.5, train=False, bounces=bounces)
    noise = np.sqrt(np.mean((a - b) ** 2))
    assert np.sqrt(np.mean((gi - a) ** 2)) < 3.0 * noise
    ma, mb, mg = a.mean(), b.mean(), gi.mean()
    assert abs(mg - ma) < max(4 * abs(ma - mb), 0.01 * ma), (ma, mb, mg)


def test_online_training_changes_the_network_and_keeps_the_image(native, ctx):
    spec = scenes.occluded_light(24 * 1280, 3000, seed=2, half=12.0)
    scene = native.Scene.from_spec(ctx, spec)
    cam = scenes.lower_camera(64, 48, distance=36.0, half=12.0)
    assert spec.positions.shape[0] > 24 * 1280
    g = _guide_for(native, ctx, spec, seed=5)
    p0 = g.params()
    guided, _ = _render(native, scene, cam, 256, 12, 4, guide=g, alpha=0.5, train=True, train_batch=4096,
                        train_steps=4, wave_paths=64 * 48 * 4)
    p1 = g.params()
    assert not np.array_equal(p0, p1) and np.all(np.isfinite(p1))
    assert np.isfinite(g.last_loss())
    assert np.all(np.isfinite(guided))
    # two independent plain renders of the same size give the noise of a mean
    a, _ = _render(native, scene, cam, 256, 12, 9)
    b, _ = _render(native, scene, cam, 256, 12, 10)
    ref, noise = 0.5 * (a.mean() + b.mean()), abs(a.mean() - b.mean())
    assert abs(guided.mean() - ref) < max(6.0 * noise, 0.05 * ref), (guided.mean(), a.mean(), b.mean())


def test_alpha_ramp_and_step_budget(native, ctx):
    """With alpha rising over the network's first steps the image still
    converges to the plain tracer's; once the step budget is spent, further
    training renders leave the network unchanged (no records, no steps)."""
    spec = scenes.occluded_light(24 * 1280, 3000, seed=2, half=12.0)
    scene = native.Scene.from_spec(ctx, spec)
    cam = scenes.lower_camera(64, 48, distance=36.0, half=12.0)
    g = _guide_for(native, ctx, spec, seed=6)
    wave = 64 * 48 * 4
    guided, _ = _render(native, scene, cam, 256, 12, 4, guide=g, alpha=0.5, train=True, train_batch=4096,
                        train_steps=4, train_budget=32, alpha_ramp=24, wave_paths=wave)
    assert np.all(np.isfinite(guided))
    p_spent = g.params()
    _render(native, scene, cam, 64, 12, 5, guide=g, alpha=0.5, train=True, train_batch=4096, train_steps=4,
            train_budget=32, wave_paths=wave)
    assert np.array_equal(p_spent, g.params())
    a, _ = _render(native, scene, cam, 256, 12, 9)
    b, _ = _render(native, scene, cam, 256, 12, 10)
    ref, noise = 0.5 * (a.mean() + b.mean()), abs(a.mean() - b.mean())
    assert abs(guided.mean() - ref) < max(6.0 * noise, 0.05 * ref), (guided.mean(), a.mean(), b.mean())
