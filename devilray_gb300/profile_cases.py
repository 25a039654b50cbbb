"""Small, fixed workloads for profiling single kernels (ncu, CUDA events).

    python -m devilray_gb300.profile_cases guide_infer [kernel]   # 0: tcgen05, 1: mma.sync
    python -m devilray_gb300.profile_cases guide_train [rows]     # Adam steps on random samples
    python -m devilray_gb300.profile_cases render_box_room         # 256x256, 16 spp, depth 8
    python -m devilray_gb300.profile_cases batch_small             # 8 uneven scenes, graph, 2 renders
    python -m devilray_gb300.profile_cases guided [spp]            # occluded-light scene, plain vs guided

Each case prints one line with its timing; run it once plainly before running
it under a profiler.
"""
from __future__ import annotations

import sys
import time

import numpy as np


def _ctx():
    from devilray_gb300 import native
    native.load()
    return native, native.Context(0)


def guide_infer(kernel: int = 0, rows: int = 1 << 20) -> None:
    import torch
    native, ctx = _ctx()
    g = native.Guide(ctx, seed=1, half_extent=10.0, infer_kernel=kernel)
    rng = np.random.default_rng(0)
    pos = torch.from_numpy(rng.uniform(-10, 10, (rows, 3)).astype(np.float32)).cuda()
    d = rng.normal(size=(rows, 3))
    nrm = torch.from_numpy((d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)).cuda()
    y = torch.zeros((rows, 40), dtype=torch.float32, device="cuda")
    for _ in range(3):
        g.infer(pos, nrm, rows, y)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(20):
        g.infer(pos, nrm, rows, y)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 20
    flop = 2 * (80 * 64 + 3 * 64 * 64 + 64 * 48) * rows
    print(f"guide_infer kernel {kernel}: {ms:.3f} ms for {rows} rows, {flop / ms / 1e9:.1f} TFLOP/s, "
          f"{rows / ms / 1e3:.1f} Mrows/s")
    ctx.check()


def guide_train(rows: int = 16384, steps: int = 100) -> None:
    import torch
    native, ctx = _ctx()
    g = native.Guide(ctx, seed=1, half_extent=10.0)
    rng = np.random.default_rng(0)

    def unit(k):
        d = rng.normal(size=(k, 3))
        return torch.from_numpy((d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)).cuda()

    pos = torch.from_numpy(rng.uniform(-10, 10, (rows, 3)).astype(np.float32)).cuda()
    nrm, sdir = unit(rows), unit(rows)
    w = torch.from_numpy(rng.exponential(1.0, rows).astype(np.float32)).cuda()
    for _ in range(3):
        g.train_step(pos, nrm, sdir, w, rows)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        g.train_step(pos, nrm, sdir, w, rows)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    print(f"guide_train: {ms:.4f} ms per Adam step of {rows} rows, loss {g.last_loss():.4f}")
    ctx.check()


def render_box_room() -> None:
    import torch
    from devilray_gb300 import scenes
    native, ctx = _ctx()
    scene = native.Scene.from_spec(ctx, scenes.box_room(3))
    cam = scenes.camera(256, 256)
    acc = torch.zeros((256 * 256, 4), dtype=torch.float32, device="cuda")
    casts = torch.zeros(256 * 256, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    t = time.perf_counter()
    scene.render(cam, acc, casts, spp=16, max_depth=8)
    torch.cuda.synchronize()
    print(f"render_box_room: {time.perf_counter() - t:.4f} s (first call), samples {float(acc[:, 3].sum()):.0f}")
    ctx.check()


def render_many_light(spp: int = 16) -> None:
    """Many-light 1080p: scenes.many_light() (2^20 triangles, 65,536 emitters)
    through the outside camera, depth 16, default schedule."""
    import torch
    from devilray_gb300 import scenes
    native, ctx = _ctx()
    scene = native.Scene.from_spec(ctx, scenes.many_light())
    cam = scenes.outside_camera(1920, 1080)
    n = 1920 * 1080
    acc = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    scene.render(cam, acc, spp=1, max_depth=16)
    torch.cuda.synchronize()
    t = time.perf_counter()
    scene.render(cam, acc, spp=spp, max_depth=16)
    torch.cuda.synchronize()
    print(f"render_many_light: {time.perf_counter() - t:.4f} s for {spp} spp")
    ctx.check()


def batch_small() -> None:
    import torch
    from devilray_gb300 import scenes  # noqa: F401
    native, ctx = _ctx()
    sys.path.insert(0, str(__import__("pathlib").Path(__file__).resolve().parents[1]))
    import bench
    specs = bench.batch_specs(8, seed=7)
    scs = [native.Scene.from_spec(ctx, s) for s, _ in specs]
    jobs, outs = [], []
    for i, ((s, cam), sc) in enumerate(zip(specs, scs)):
        n = cam["width"] * cam["height"]
        acc = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        jobs.append(native.make_job(sc, cam, acc, spp=4, max_depth=12, seed=i))
        outs.append(acc)
    b = native.Batch(ctx, jobs, use_graph=True)
    b.render()
    b.render()
    torch.cuda.synchronize()
    i = b.info()
    print(f"batch_small: {i.num_waves} waves, {i.graph_nodes} graph nodes, {i.paths_per_render} paths per render")
    ctx.check()


def guided(spp: int = 32) -> None:
    """Plain and guided renders of the single-gap occluded-light scene at
    480x270 with the benchmark's guided schedule: alpha 0.75, the first 3
    bounces guided, 16 Adam steps of 65,536 samples after every 16-spp wave
    (at most 512 steps), a fresh network."""
    import torch
    from devilray_gb300 import scenes
    native, ctx = _ctx()
    spec = scenes.occluded_light(slab_gap=0.15)
    scene = native.Scene.from_spec(ctx, spec)
    cam = scenes.lower_camera(480, 270)
    n = 480 * 270
    acc = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    pos = spec.positions.reshape(-1, 3)
    lo, hi = pos.min(0), pos.max(0)
    g = native.Guide(ctx, seed=1, center=tuple(float(x) for x in (lo + hi) / 2),
                     half_extent=float((hi - lo).max() / 2))

    def timed(fn):
        acc.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t

    tp = timed(lambda: scene.render(cam, acc, spp=spp, max_depth=16, seed=1, wave_paths=16 * n))
    tg = timed(lambda: scene.render_guided(g, cam, acc, spp=spp, max_depth=16, seed=2, alpha=0.75, train=True,
                                           train_batch=65536, train_steps=16, train_budget=512, bounces=3,
                                           wave_paths=16 * n))
    print(f"guided: plain {tp:.3f} s, guided with training {tg:.3f} s for {spp} spp at 480x270")
    ctx.check()


if __name__ == "__main__":
    case = sys.argv[1] if len(sys.argv) > 1 else "guide_infer"
    args = [int(a) for a in sys.argv[2:]]
    {"guide_infer": guide_infer, "guide_train": guide_train, "render_box_room": render_box_room,
     "render_many_light": render_many_light,
     "batch_small": batch_small, "guided": guided}[case](*args)
