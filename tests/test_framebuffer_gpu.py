"""Framebuffer (Buffers) and device tonemapping (Renderer::createPixels).

The device conversion must give the same RGBA8 words as the oracle's
restatement of createPixels (src/Renderer.cpp:51-90): averages, sRGB or linear
encoding, 8-bit rounding, alpha 255 and the vertical flip.
"""
from __future__ import annotations

import numpy as np
import pytest

from devilray_gb300 import scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _accum(w, h, seed):
    rng = np.random.default_rng(seed)
    n = w * h
    acc = np.zeros((n, 4), np.float32)
    acc[:, 3] = rng.integers(0, 9, n)
    acc[:, :3] = rng.exponential(0.4, (n, 3)).astype(np.float32) * acc[:, 3:4]
    acc[::7, :3] = rng.uniform(0, 0.004, (len(acc[::7]), 3)) * acc[::7, 3:4]   # the linear segment
    acc[::11, :3] = 0
    return acc


@pytest.mark.parametrize("gamma", [True, False])
@pytest.mark.parametrize("w,h", [(1, 1), (37, 23), (256, 256), (300, 2)])
def test_tonemap_matches_oracle(native, ctx, oracle, gamma, w, h):
    acc = _accum(w, h, w * 1000 + h)
    if not gamma:   # linear output of values above 1 spills into the next channel, as in the reference
        acc[:, :3] = np.minimum(acc[:, :3], acc[:, 3:4] * 1.5)
    dev = torch.from_numpy(acc).cuda()
    out = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    native.tonemap(dev, w, h, out, gamma=gamma)
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint32)
    want = oracle.create_pixels(acc, w, h, gamma)
    bad = np.flatnonzero(got != want)
    assert bad.size == 0, f"{bad.size} pixels differ, e.g. {bad[:4]}: {got[bad[:4]]} vs {want[bad[:4]]}"


def test_framebuffer_render_read_tonemap(native, ctx, oracle):
    spec = scenes.box_room(sphere_level=2)
    cam = scenes.camera(40, 30)
    scene = native.Scene.from_spec(ctx, spec)
    fb = native.Framebuffer(ctx, 40, 30)
    acc_dev, casts_dev = fb.device_buffers()
    scene.render(cam, acc_dev, casts_dev, spp=3, max_depth=6)
    scene.render(cam, acc_dev, casts_dev, spp=2, sample_offset=3, max_depth=6)
    acc, casts, total = fb.read()

    ref = torch.zeros((1200, 4), dtype=torch.float32, device="cuda")
    rc = torch.zeros(1200, dtype=torch.int32, device="cuda")
    scene.render(cam, ref, rc, spp=5, max_depth=6)
    torch.cuda.synchronize()
    assert np.array_equal(acc.view(np.uint32), ref.cpu().numpy().view(np.uint32))
    assert np.array_equal(casts, rc.cpu().numpy().astype(np.uint32))
    assert total == int(casts.astype(np.uint64).sum()) > 0

    px = fb.tonemap(gamma=True)
    assert np.array_equal(px, oracle.create_pixels(acc, 40, 30, True))
    assert np.array_equal(fb.tonemap(gamma=False), oracle.create_pixels(acc, 40, 30, False))

    fb.clear()
    acc2, casts2, total2 = fb.read()
    assert not acc2.any() and not casts2.any() and total2 == 0
    assert np.all(fb.tonemap() == np.uint32(0xFF000000))
    fb.close()


def test_framebuffer_invalid_arguments(native, ctx):
    with pytest.raises(native.DrError):
        native.Framebuffer(ctx, 0, 10)
    with pytest.raises(native.DrError):
        native.Framebuffer(ctx, 10, 70000)


@pytest.mark.parametrize("mode", [0, 1])
def test_alias_build_host_equals_oracle(native, ctx, oracle, mode):
    w = oracle.lognormal_input(5000, seed=7)
    table = np.zeros(len(w), native.ALIAS_DTYPE)
    native.check(native.load().dr_alias_build_host(ctx.handle, native._ptr(w), len(w), native._ptr(table), mode))
    want = oracle.alias_build_ref(w) if mode == 0 else oracle.alias_build_sweep(w)
    assert table.tobytes() == want.tobytes()


def _read_pfm(path):
    data = path.read_bytes()
    parts = data.split(b"\n", 3)
    assert parts[0] == b"PF"
    w, h = (int(x) for x in parts[1].split())
    assert float(parts[2]) < 0  # little-endian
    return np.frombuffer(parts[3], dtype="<f4").reshape(h, w, 3), w, h


def test_resolve_and_pfm_output(native, ctx, tmp_path):
    """Headless output: dr_resolve gives sum / samples on the device (0 where
    a pixel has no samples), bit for bit the FP32 quotient, and the
    framebuffer's PFM file holds the same values, bottom row first."""
    w, h = 37, 23
    acc = _accum(w, h, 5)
    dev = torch.from_numpy(acc).cuda()
    rgb = torch.full((w * h, 3), -1.0, dtype=torch.float32, device="cuda")
    native.resolve(dev, w, h, rgb)
    torch.cuda.synchronize()
    got = rgb.cpu().numpy()
    want = np.where(acc[:, 3:4] != 0, acc[:, :3] / np.where(acc[:, 3:4] != 0, acc[:, 3:4], 1), 0).astype(np.float32)
    assert np.array_equal(got, want)

    spec = scenes.box_room(sphere_level=2)
    scene = native.Scene.from_spec(ctx, spec)
    fb = native.Framebuffer(ctx, 40, 30)
    acc_dev, casts_dev = fb.device_buffers()
    scene.render(scenes.camera(40, 30), acc_dev, casts_dev, spp=3, max_depth=6)
    path = tmp_path / "image.pfm"
    fb.write_pfm(path)
    img, pw, ph = _read_pfm(path)
    assert (pw, ph) == (40, 30)
    a, _, _ = fb.read()
    lin = (a[:, :3] / a[:, 3:4]).reshape(30, 40, 3)
    assert np.array_equal(img, lin)
    fb.close()
