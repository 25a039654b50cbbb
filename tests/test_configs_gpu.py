"""Parity at the benchmark configurations' own sizes.

The reduced cases of test_trace_gpu.py and test_render_gpu.py cover layouts,
triangle tests and edge cases. These tests run the workloads the benchmark
reports, at their stated sizes or on a stated pixel subset of them, against
the oracle:

* incoherent traversal: 2^20 triangles and 16,777,216 rays (the benchmark's
  scene and rays), closest hit with t and triangle index bit for bit, and any
  hit;
* box room: 256x256, 16 spp, depth 8, level-3 glass icosphere; the image and
  the path-ray counts bit for bit;
* many-light: 2^20 triangles and 65,536 emitters at 1920x1080, depth 16; the
  GPU renders the whole image, and the oracle renders three 32x32 windows plus
  1,024 scattered pixels, which must match bit for bit; the light tables of
  both builds (sweep and reference pairing) equal the oracle's;
* batched uneven scenes: the 64-scene batch (1k-2M triangles, 128^2-1024^2,
  32 spp, depth 12) as one graph-captured schedule; four of its images (the
  three scenes with the fewest triangles and the median one) match the
  oracle on pixel subsets.
"""
from __future__ import annotations

import numpy as np
import pytest

from devilray_gb300 import scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_incoherent_traversal_full_size(native, ctx, oracle):
    soup, _, _ = scenes.incoherent_soup(1 << 20, seed=0)
    rays = scenes.incoherent_rays(1 << 24, seed=0)
    n = len(rays)
    scene = native.Scene(ctx, soup)
    assert scene.info().layout == 8
    d_rays = torch.from_numpy(rays).cuda()
    hits = torch.empty((n, 2), dtype=torch.int32, device="cuda")
    scene.trace_closest(d_rays, n, hits, native.DR_TRI_REFERENCE)
    torch.cuda.synchronize()
    h = hits.cpu().numpy()
    t, prim = h[:, 0].copy().view(np.float32), h[:, 1].copy()
    b = oracle.BBH(soup)
    tc, pc = b.trace_canonical(rays, slack=scene.info().slack)
    mism = np.flatnonzero((_bits(t) != _bits(tc)) | (prim != pc))
    assert mism.size == 0, f"{mism.size} of {n} rays differ, first {mism[:5]}"
    assert 0.1 < (prim >= 0).mean() < 0.5
    # any hit: the same rays with tmax uniform in [0, 60]
    rng = np.random.default_rng(7)
    rays[:, 3] = rng.uniform(0.0, 60.0, n).astype(np.float32)
    d_rays.copy_(torch.from_numpy(rays))
    occ = torch.empty(n, dtype=torch.uint8, device="cuda")
    scene.trace_any(d_rays, n, occ, native.DR_TRI_REFERENCE)
    torch.cuda.synchronize()
    occ_o = b.trace_any(rays, slack=scene.info().slack)
    assert np.array_equal(occ.cpu().numpy(), occ_o)
    assert 0.05 < occ_o.mean() < 0.95


def test_box_room_full_config_bit_exact(native, ctx, oracle):
    spec = scenes.box_room(sphere_level=3)
    assert spec.positions.shape[0] == 1292
    cam = scenes.camera(256, 256)
    n = 256 * 256
    scene = native.Scene.from_spec(ctx, spec)
    acc = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    casts = torch.zeros(n, dtype=torch.int32, device="cuda")
    scene.render(cam, acc, casts, spp=16, max_depth=8, seed=0)
    torch.cuda.synchronize()
    oacc, ocasts, _ = oracle.RenderScene(spec).render(cam, 16, max_depth=8, seed=0)
    got = acc.cpu().numpy()
    mism = np.flatnonzero((got.view(np.uint32) != oacc.view(np.uint32)).any(1))
    assert mism.size == 0, f"{mism.size} pixels differ, e.g. {mism[:3]}"
    assert np.array_equal(casts.cpu().numpy().astype(np.uint32), ocasts)
    assert (got[:, 3] == 16).all() and got[:, :3].sum() > 0


def _windows(width, height, size, corners, extra, seed):
    """Pixel indices of size x size windows at the given top-left corners plus
    `extra` scattered pixels."""
    pix = []
    for (x0, y0) in corners:
        ys, xs = np.mgrid[y0:y0 + size, x0:x0 + size]
        pix.append((ys * width + xs).reshape(-1))
    rng = np.random.default_rng(seed)
    pix.append(rng.choice(width * height, extra, replace=False))
    return np.unique(np.concatenate(pix)).astype(np.int64)


def test_many_light_1080p_windows_bit_exact(native, ctx, oracle):
    spec = scenes.many_light()
    cam = scenes.outside_camera(1920, 1080)
    n = 1920 * 1080
    osc = oracle.RenderScene(spec)
    scene = native.Scene.from_spec(ctx, spec)
    # the object light table of 66,356 objects (65,536 emitters), both builds
    assert len(spec.objects) > 65536
    assert scene.light_table().tobytes() == osc.light_table().tobytes()
    ref_scene = native.Scene.from_spec(ctx, spec, light_tables=native.DR_LIGHT_TABLES_REFERENCE)
    assert ref_scene.light_table().tobytes() == oracle.RenderScene(spec, light_tables=1).light_table().tobytes()
    del ref_scene
    acc = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    casts = torch.zeros(n, dtype=torch.int32, device="cuda")
    scene.render(cam, acc, casts, spp=2, max_depth=16, seed=3)
    torch.cuda.synchronize()
    pix = _windows(1920, 1080, 32, [(944, 524), (300, 700), (1500, 100)], 1024, seed=11)
    oacc, ocasts, _ = osc.render(cam, 2, max_depth=16, seed=3, pixels=pix)
    got = acc.cpu().numpy()[pix]
    mism = np.flatnonzero((got.view(np.uint32) != oacc[pix].view(np.uint32)).any(1))
    assert mism.size == 0, f"{mism.size} of {pix.size} pixels differ, e.g. {pix[mism[:3]]}"
    assert np.array_equal(casts.cpu().numpy().astype(np.uint32)[pix], ocasts[pix])
    assert (got[:, :3] > 0).mean() > 0.05


def test_uneven_batch_images_match_oracle(native, ctx, oracle):
    specs = scenes.uneven_batch(64)
    spp, depth = 32, 12
    scs = [native.Scene.from_spec(ctx, spec) for spec, _ in specs]
    jobs, outs = [], []
    for i, ((spec, cam), sc) in enumerate(zip(specs, scs)):
        npx = cam["width"] * cam["height"]
        acc = torch.zeros((npx, 4), dtype=torch.float32, device="cuda")
        casts = torch.zeros(npx, dtype=torch.int32, device="cuda")
        jobs.append(native.make_job(sc, cam, acc, casts, spp=spp, max_depth=depth, seed=i))
        outs.append((acc, casts))
    b = native.Batch(ctx, jobs, use_graph=True)
    b.render()
    torch.cuda.synchronize()
    assert b.info().graph_nodes > 0
    sizes = np.array([s.positions.shape[0] for s, _ in specs])
    order = np.argsort(sizes, kind="stable")
    chosen = list(order[:3]) + [order[len(order) // 2]]
    for i in chosen:
        spec, cam = specs[i]
        w, h = cam["width"], cam["height"]
        pix = _windows(w, h, 16, [(w // 2 - 8, h // 2 - 8)], min(1024, w * h - 256), seed=int(i))
        oacc, ocasts, _ = oracle.RenderScene(spec).render(cam, spp, max_depth=depth, seed=int(i), pixels=pix)
        acc, casts = outs[i]
        got = acc.cpu().numpy()[pix]
        mism = np.flatnonzero((got.view(np.uint32) != oacc[pix].view(np.uint32)).any(1))
        assert mism.size == 0, f"image {i} ({sizes[i]} triangles, {w}x{h}): {mism.size} of {pix.size} pixels differ"
        assert np.array_equal(casts.cpu().numpy().astype(np.uint32)[pix], ocasts[pix])
        assert (got[:, 3] == spp).all()
    b.close()
