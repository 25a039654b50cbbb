"""Benchmark: incoherent closest-hit traversal, Mrays/s.

Workload (one step): closest hit of 16,777,216 incoherent rays against a
2^20-triangle soup of level-3 icospheres (centres uniform in [-50,50]^3, radii
log-uniform in [0.5,3]; rays with origins uniform in the cube and directions
uniform on the sphere), FP32, reference triangle test (bit-exact t and hit
index against the reference). Synthetic, seeded inputs.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``value``  : rays/s with rays resident in device memory (CUDA events on the
             launching stream, max over ranks), in Mrays/s.
``e2e``    : the same through dr_trace_closest_host with pinned host buffers:
             the ray upload and the hit download are inside the timed region.
``--impl reference`` times the reference's CPU traversal (the oracle's port of
getIntersectionImpl over the reference's median-split BBH) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NUM_TRIS = 1 << 20
NUM_RAYS = 1 << 24
# DRAM bytes of one full 16.8 M-ray launch of the dominant kernel, from one
# `ncu --set full` capture of this workload (the profiles named beside them).
NCU_TRAFFIC = {8: 930_092_288 + 130_737_664, 2: 1_652_000_000 + 152_000_000}
NCU_PROFILE = {8: "trace_closest_p8_incoherent_1M_tris_16M_rays.md",
               2: "trace_closest_bvh2_incoherent_1M_tris_16M_rays.md"}
# Warp instructions per ray of the dominant kernel (smsp__inst_executed.sum of
# the same capture / 16,777,216 rays): with the launch time and the sampled SM
# clock it gives the issue-slot fraction (4 schedulers per SM, one instruction
# per scheduler and cycle).
NCU_WARP_INST_PER_RAY = {8: 3_200_962_454 / NUM_RAYS}
METRIC = "Mrays/s closest-hit"
# Seconds the reference arm's timed steps may take in all (it sizes its
# per-step sample of the workload to fit).
REF_TIMED_BUDGET_S = 150
WORKLOAD = "incoherent closest-hit: 2^20-triangle icosphere soup, 16,777,216 rays"
L2_BYTES = 129 * 1024 * 1024


def _env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().strip().splitlines() if r.strip()]
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, name in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.file.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_workload(rank: int):
    from devilray_gb300 import scenes
    soup, _, _ = scenes.incoherent_soup(NUM_TRIS, seed=0)
    rays = scenes.incoherent_rays(NUM_RAYS, seed=rank)
    return soup, rays


def cpu_baseline(soup, rays, sample: int, threads: int):
    """The reference's traversal (oracle port) on a bounded sample; Mrays/s."""
    from oracle import pyoracle as po
    po.build(ref=False)
    t0 = time.perf_counter()
    bbh = po.BBH(soup)
    build_s = time.perf_counter() - t0
    from devilray_gb300.scenes import rays6
    r6 = rays6(rays[:sample])
    t0 = time.perf_counter()
    t, prim, nb, nt = bbh.trace_reference(r6, threads=threads)
    dt = time.perf_counter() - t0
    return {"value": sample / dt / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"{sample} of the {NUM_RAYS} rays, reference median-split BBH (built in {build_s:.1f} s, untimed), "
                      f"reference triangle test, std::thread over ray chunks",
            "seconds": dt, "box_tests_per_ray": float(nb.mean()), "tri_tests_per_ray": float(nt.mean())}, (t, prim)


def run_reference(args):
    rank, local, world = _env_rank()
    if rank != 0:
        return 0
    soup, rays = build_workload(0)
    threads = os.cpu_count() or 1
    from oracle import pyoracle as po
    po.build(ref=False)
    bbh = po.BBH(soup)
    from devilray_gb300.scenes import rays6
    # Rays per timed step: the whole workload when the timed steps fit about
    # REF_TIMED_BUDGET_S at the rate the warm-up measures, else the largest
    # multiple of 2^16 rays that does (--ref-sample fixes it instead).
    warm = rays6(rays[: 1 << 18])
    rate = 0.0
    for _ in range(args.warmup):
        t0 = time.perf_counter()
        bbh.trace_reference(warm, threads=threads)
        rate = max(rate, len(warm) / (time.perf_counter() - t0))
    if args.ref_sample:
        sample = min(NUM_RAYS, args.ref_sample)
    else:
        fit = int(rate * REF_TIMED_BUDGET_S / max(1, args.steps))
        sample = NUM_RAYS if fit >= NUM_RAYS else max(1 << 16, fit >> 16 << 16)
    r6 = rays6(rays[:sample])
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        bbh.trace_reference(r6, threads=threads)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = sample * args.steps / total / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "num_triangles": NUM_TRIS, "num_rays": NUM_RAYS,
                   "step_sample_rays": sample, "tri_mode": "reference"},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": (f"all {NUM_RAYS} rays of the workload every step" if sample == NUM_RAYS else
                                    f"{sample} rays per step of the {NUM_RAYS}-ray workload (the timed steps "
                                    f"kept to about {REF_TIMED_BUDGET_S} s)") +
                                   "; the reference's median-split BBH and getIntersectionImpl restated in C++ "
                                   "(oracle), std::thread over ray chunks on all host cores"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def max_over_ranks(values, dist, device):
    """Each timing's maximum over the ranks (the slowest replica sets the
    job's time)."""
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def job_rate(world: int, units_per_rank: int, steps: int, seconds: float) -> float:
    """Whole-job millions of units per second: every replica processes its own
    units each step (weak scaling), the job takes the slowest rank's time."""
    return world * units_per_rank * steps / seconds / 1e6


def run_ours(args):
    import torch
    rank, local, world = _env_rank()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from devilray_gb300 import native
    soup, rays = build_workload(rank)
    ctx = native.Context(local)
    scene = native.Scene(ctx, soup, layout=args.layout)
    info = scene.info()
    stream = torch.cuda.Stream()
    d_rays = torch.from_numpy(rays).to(f"cuda:{local}")
    d_hits = torch.empty((NUM_RAYS, 2), dtype=torch.int32, device=f"cuda:{local}")
    torch.cuda.synchronize()

    # Counting pass (untimed): node and triangle visits per ray for the
    # algorithmic-byte count of the roofline.
    with torch.cuda.stream(stream):
        cnt = scene.trace_closest(d_rays, NUM_RAYS, d_hits, native.DR_TRI_REFERENCE, counters=True, stream=stream)
    stream.synchronize()
    nodes_per_ray = cnt.node_visits / NUM_RAYS
    tris_per_ray = cnt.tri_tests / NUM_RAYS
    hit_frac = cnt.hits / NUM_RAYS

    for _ in range(args.warmup):
        scene.trace_closest(d_rays, NUM_RAYS, d_hits, native.DR_TRI_REFERENCE, stream=stream)
    stream.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for k in range(args.steps):
            starts[k].record(stream)
            scene.trace_closest(d_rays, NUM_RAYS, d_hits, native.DR_TRI_REFERENCE, stream=stream)
            ends[k].record(stream)
        stream.synchronize()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = sum(step_ms)
    ctx.check()

    # End to end through the host-buffer entry point, pinned host memory.
    h_rays = torch.from_numpy(rays).pin_memory()
    h_hits = torch.empty((NUM_RAYS, 2), dtype=torch.int32).pin_memory()
    e2e_steps = max(1, min(args.steps, 10))
    for _ in range(1):
        native.check(native.load().dr_trace_closest_host(scene.handle, h_rays.data_ptr(), NUM_RAYS,
                                                         h_hits.data_ptr(), 0, stream.cuda_stream))
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        native.check(native.load().dr_trace_closest_host(scene.handle, h_rays.data_ptr(), NUM_RAYS,
                                                         h_hits.data_ptr(), 0, stream.cuda_stream))
    e2e_s = time.perf_counter() - t0
    # the host copy of the hits equals the device-resident result
    same = torch.equal(h_hits, d_hits.cpu())

    if dist:
        total_ms, e2e_s = max_over_ranks([total_ms, e2e_s], dist, f"cuda:{local}")
    value = job_rate(world, NUM_RAYS, args.steps, total_ms / 1e3)
    e2e_value = job_rate(world, NUM_RAYS, e2e_steps, e2e_s)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    hbm_peak, peak_kind = _peaks()
    node_bytes, tri_bytes = (80 if info.layout == 8 else 64), 48
    bytes_per_ray = 32 + 8 + nodes_per_ray * node_bytes + tris_per_ray * tri_bytes
    per_launch_ms = total_ms / args.steps
    achieved = bytes_per_ray * NUM_RAYS / (per_launch_ms / 1e3) / 1e9
    # reference mode reads the nodes, the reference triangle records and the
    # triangle index map: 64 or 80 B per node + 52 B per triangle
    working_set = info.num_nodes * node_bytes + NUM_TRIS * 52
    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "num_triangles": NUM_TRIS, "num_rays": NUM_RAYS, "tri_mode": "reference",
                   "layout": ("compressed 8-wide BVH (80-byte nodes), binned SAH" if info.layout == 8
                              else "binary two-box BVH, binned SAH"), "bvh_nodes": info.num_nodes, "bvh_depth": info.depth,
                   "scene_device_bytes": working_set, "bvh_build_s": round(info.build_seconds, 3),
                   "l2": "rays 512 MiB per step > L2; scene arrays stay L2-resident across steps",
                   "parallelism": f"replicas{world}" if world > 1 else "single"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": NCU_TRAFFIC.get(info.layout),
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one full launch "
                                       "(profiles/" + NCU_PROFILE.get(info.layout, "") + ")",
                     "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                     "kernel": ("k_trace_closest_p8<0,false>" if info.layout == 8 else "k_trace_closest<0,false,2>"),
                     "bytes_per_ray": bytes_per_ray, "node_visits_per_ray": nodes_per_ray,
                     "tri_tests_per_ray": tris_per_ray, "hit_fraction": hit_frac,
                     "per_launch_ms": per_launch_ms, "working_set_bytes": working_set,
                     "working_set_fits_l2": working_set < L2_BYTES},
        "clocks": clocks.summary(),
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": NUM_RAYS * 32,
                "d2h_bytes_per_step": NUM_RAYS * 8, "steps": e2e_steps, "api": "dr_trace_closest_host",
                "matches_device_result": bool(same)},
        "gpu_launches": args.steps,
    }
    l2, hbm_read = _read_probes(ctx, local)
    rf = line["roofline"]
    rf["l2_read_gbs_measured"] = l2
    rf["hbm_read_gbs_measured"] = hbm_read
    rf["frac_of_l2"] = achieved / l2
    # The scene's arrays fit L2 and stay resident across launches, so the
    # memory level of this roofline is L2 (its denominator: our streaming read
    # probe over a buffer smaller than L2); the HBM copy peak is kept beside it.
    if working_set < L2_BYTES:
        rf["hbm"] = {"peak": hbm_peak, "frac": achieved / hbm_peak, "peak_kind": rf["peak_kind"]}
        rf.update({"bound": "l2", "peak": l2, "frac": achieved / l2,
                   "peak_kind": "measured: dr_probe_read_bandwidth, L2-cached 16-byte loads over a 48 MiB buffer"})
    # issue slots: warp instructions of the launch over the SMs' schedulers at the sampled clock
    sm_mhz = line["clocks"].get("sm_mhz")
    wpr = NCU_WARP_INST_PER_RAY.get(info.layout)
    if sm_mhz and wpr:
        slots = torch.cuda.get_device_properties(local).multi_processor_count * 4 * sm_mhz * 1e6 * per_launch_ms / 1e3
        rf["issue"] = {"warp_instructions_per_ray": wpr, "frac": wpr * NUM_RAYS / slots,
                       "source": "smsp__inst_executed.sum of profiles/" + NCU_PROFILE[info.layout]}
        rf["binding"] = "instruction issue (see issue.frac)"
    if world == 1 and not args.no_cpu_baseline:
        cb, _ = cpu_baseline(soup, rays, args.cpu_sample, os.cpu_count() or 1)
        line["cpu_baseline"] = cb
    if not args.no_render:
        del d_rays, d_hits, h_rays, h_hits
        torch.cuda.empty_cache()
        line["render"] = render_section(ctx, native, local, stream, cpu=(world == 1 and not args.no_cpu_baseline),
                                        threads=os.cpu_count() or 1, layout=args.render_layout)
    if not args.no_batch:
        torch.cuda.empty_cache()
        line["batch"] = batch_section(ctx, native, local, stream, scenes_n=args.batch_scenes)
    if not args.no_guided:
        torch.cuda.empty_cache()
        line["guided"] = guided_section(ctx, native, local, stream, ref_spp=args.guided_ref_spp,
                                        scene=args.guided_scene, width=args.guided_size[0],
                                        height=args.guided_size[1], spp=args.guided_spp,
                                        hd=args.guided_size[0] < 1920)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def render_section(ctx, native, device: int, stream, cpu: bool, threads: int, layout: int = 0):
    """1080p samples/s on the many-light configuration (1920x1080, 64 spp,
    depth 16, 65,536 emitters) and the box room (256x256, 16 spp, depth 8),
    rendered with the schedule dr_autotune picks (the default schedule's time
    is reported beside it); each with the reference's CPU integrator (oracle
    port: per-object cast, reference random-number order) timed on a pixel
    subset."""
    import torch
    from devilray_gb300 import scenes
    out = {}
    cases = [
        ("box_room", scenes.box_room(3), scenes.camera(256, 256), 16, 8, 3),
        ("many_light_1080p", scenes.many_light(), scenes.outside_camera(1920, 1080), 64, 16, 1),
    ]
    for name, spec, cam, spp, depth, reps in cases:
        t0 = time.perf_counter()
        scene = native.Scene.from_spec(ctx, spec, layout=layout)
        build_s = time.perf_counter() - t0
        npix = cam["width"] * cam["height"]
        accum = torch.zeros((npix, 4), dtype=torch.float32, device=f"cuda:{device}")
        casts = torch.zeros(npix, dtype=torch.int32, device=f"cuda:{device}")
        # the autotuner's schedule (dr_autotune: probe renders, untimed); the
        # images do not depend on it
        t0 = time.perf_counter()
        # probes of the full sample count where that is cheap (a probe with
        # fewer samples runs smaller waves and can favour another layout)
        probe = spp if npix * spp <= (1 << 22) else min(spp, 4)
        tune = native.autotune(ctx, spec, cam, spp=spp, max_depth=depth, probe_spp=probe, reps=2,
                               try_layouts=layout == 0)
        tune_s = time.perf_counter() - t0
        tuned = scene
        if layout == 0 and tune.layout != scene.info().layout:
            tuned = native.Scene.from_spec(ctx, spec, layout=tune.layout)
        sched = dict(wave_paths=tune.wave_paths, streams=tune.streams, chunk=tune.chunk, stack=tune.stack)

        def timed(sc, kw):
            sc.render(cam, accum, casts, spp=1, max_depth=depth, stream=stream, **kw)  # warm-up
            stream.synchronize()
            times = []
            for r in range(reps):
                accum.zero_()
                casts.zero_()
                torch.cuda.synchronize()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                sc.render(cam, accum, casts, spp=spp, max_depth=depth, stream=stream, **kw)
                b.record(stream)
                stream.synchronize()
                times.append(a.elapsed_time(b) / 1e3)
            return min(times)

        t_default = timed(scene, {})
        t = timed(tuned, sched)
        path_rays = int(casts.sum().item())
        stats = tuned.render_stats()
        entry = {"width": cam["width"], "height": cam["height"], "spp": spp, "max_depth": depth,
                 "layout": tuned.info().layout, "schedule": sched, "autotune_s": round(tune_s, 3),
                 "default_schedule_seconds": t_default,
                 "triangles": int(spec.positions.shape[0]), "objects": len(spec.objects),
                 "scene_build_s": round(build_s, 3), "seconds": t,
                 "samples_per_s": npix * spp / t, "path_mrays_per_s": path_rays / t / 1e6,
                 "path_and_shadow_mrays_per_s": (stats.path_rays + stats.shadow_rays) / t / 1e6,
                 "path_rays_per_sample": path_rays / (npix * spp),
                 "shadow_rays_per_sample": stats.shadow_rays / (npix * spp)}
        if cpu:
            entry["cpu_baseline"] = render_cpu_baseline(spec, cam, depth, threads,
                                                        pixels=65536 if name == "box_room" else 1024)
        out[name] = entry
        del scene, tuned, accum, casts
    torch.cuda.empty_cache()
    return out


def batch_section(ctx, native, device: int, stream, scenes_n: int = 64, spp: int = 32, depth: int = 12):
    """Batched uneven scenes: `scenes_n` scenes and cameras traced as one
    schedule (dr_batch) captured in a CUDA graph, wave size / streams / fetch
    size and hierarchy width picked by the autotuner; samples/s over the whole
    batch, beside the same images rendered one dr_render call at a time."""
    import torch
    t0 = time.perf_counter()
    from devilray_gb300 import scenes
    specs = scenes.uneven_batch(scenes_n)
    gen_s = time.perf_counter() - t0
    sizes = [s.positions.shape[0] for s, _ in specs]
    median = int(np.argsort(sizes)[len(sizes) // 2])
    t0 = time.perf_counter()
    tune_scene = native.autotune(ctx, specs[median][0], specs[median][1], spp=2, max_depth=depth, reps=2)
    tune_scene_s = time.perf_counter() - t0
    layout = tune_scene.layout
    t0 = time.perf_counter()
    scs = [native.Scene.from_spec(ctx, spec, layout=layout) for spec, _ in specs]
    build_s = time.perf_counter() - t0
    jobs, outs = [], []
    for i, ((spec, cam), sc) in enumerate(zip(specs, scs)):
        n = cam["width"] * cam["height"]
        acc = torch.zeros((n, 4), dtype=torch.float32, device=f"cuda:{device}")
        casts = torch.zeros(n, dtype=torch.int32, device=f"cuda:{device}")
        jobs.append(native.make_job(sc, cam, acc, casts, spp=spp, max_depth=depth, seed=i))
        outs.append((acc, casts))
    t0 = time.perf_counter()
    tune = native.autotune_batch(ctx, jobs, probe_spp=1, reps=2)
    tune_batch_s = time.perf_counter() - t0
    b = native.Batch(ctx, jobs, wave_paths=tune.wave_paths, streams=tune.streams, chunk=tune.chunk, use_graph=True,
                     stack=tune.stack)
    b.render(stream=stream)  # captures the graph
    stream.synchronize()
    times = []
    for _ in range(2):
        for acc, casts in outs:
            acc.zero_()
            casts.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.render(sample_offsets=[0] * len(jobs), stream=stream)
        e1.record(stream)
        stream.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    t = min(times)
    info = b.info()
    path_rays = sum(int(c.sum().item()) for _, c in outs)
    samples = int(info.paths_per_render)
    # the same scenes built on the device (linear BVH collapsed into the same
    # hierarchy width): build time and the batch's samples/s with them
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dscs = [native.Scene.from_spec(ctx, spec, builder=1, layout=layout) for spec, _ in specs]
    torch.cuda.synchronize()
    dev_build_s = time.perf_counter() - t0
    djobs = [native.make_job(sc, cam, acc, casts, spp=spp, max_depth=depth, seed=i)
             for i, ((spec, cam), sc, (acc, casts)) in enumerate(zip(specs, dscs, outs))]
    db = native.Batch(ctx, djobs, wave_paths=tune.wave_paths, streams=tune.streams, chunk=tune.chunk, use_graph=True,
                      stack=tune.stack)
    db.render(stream=stream)
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    db.render(sample_offsets=[0] * len(djobs), stream=stream)
    e1.record(stream)
    stream.synchronize()
    t_dev = e0.elapsed_time(e1) / 1e3
    db.close()
    del dscs, djobs
    # the same images one dr_render call at a time (default schedule)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for (spec, cam), sc, (acc, casts) in zip(specs, scs, outs):
        sc.render(cam, acc, casts, spp=spp, max_depth=depth, stream=stream)
    e1.record(stream)
    stream.synchronize()
    t_seq = e0.elapsed_time(e1) / 1e3
    out = {"scenes": scenes_n, "triangles_total": int(sum(sizes)), "triangles_min": int(min(sizes)),
           "triangles_max": int(max(sizes)), "pixels_total": int(sum(c["width"] * c["height"] for _, c in specs)),
           "spp": spp, "max_depth": depth, "layout": layout, "seconds": t, "samples_per_s": samples / t,
           "path_mrays_per_s": path_rays / t / 1e6, "num_waves": info.num_waves,
           "wave_paths": info.max_wave_paths, "graph_nodes": int(info.graph_nodes),
           "sequential_dr_render_seconds": t_seq, "sequential_samples_per_s": samples / t_seq,
           "autotune_scene": tune_scene.as_dict(), "autotune_batch": tune.as_dict(),
           "autotune_seconds": round(tune_scene_s + tune_batch_s, 3), "scene_build_s": round(build_s, 3),
           "device_lbvh": {"scene_build_s": round(dev_build_s, 3), "samples_per_s": samples / t_dev,
                           "layout": layout,
                           "note": f"the same {scenes_n} scenes built on the device (linear BVH, collapsed into "
                                   f"{'8-wide' if layout == 8 else 'binary'} nodes), light tables included"},
           "scene_generation_s": round(gen_s, 3)}
    b.close()
    del jobs, outs, scs
    torch.cuda.empty_cache()
    return out


def guided_section(ctx, native, device: int, stream, width: int = 480, height: int = 270, spp: int = 1024,
                   depth: int = 16, ref_spp: int = 65536, hd_spp: int = 16, seeds: int = 5, scene: str = "gap",
                   hd: bool = True):
    """Learned path guiding on the occluded-light scene (the many-light
    geometry, emitters only above an occluding slab): RMSE of the guided and of
    the plain MIS tracer against a converged render (the plain tracer,
    `ref_spp` samples accumulated in FP64), at equal samples and at equal time
    (training included), plus guided samples/s at 1920x1080. Each RMSE is the
    root of the mean squared error over `seeds` independent renders (the
    guided ones each train a fresh network), because single renders of this
    scene differ by tens of percent in squared error."""
    import torch
    from devilray_gb300 import scenes
    scene_kw = {"gap": dict(slab_gap=0.15), "centered": {}}[scene]
    spec = scenes.occluded_light(**scene_kw)
    sc = native.Scene.from_spec(ctx, spec)
    cam = scenes.lower_camera(width, height)
    npix = width * height
    dev = f"cuda:{device}"
    acc = torch.zeros((npix, 4), dtype=torch.float32, device=dev)

    # converged reference: two halves of ref_spp samples, each summed in FP64
    # from chunks of 1024; the squared difference of the halves estimates the
    # reference's own variance, which every MSE below has subtracted
    t0 = time.perf_counter()
    halves = []
    for h in range(2):
        ref = torch.zeros((npix, 4), dtype=torch.float64, device=dev)
        for off in range(0, ref_spp // 2, 1024):
            acc.zero_()
            sc.render(cam, acc, spp=min(1024, ref_spp // 2 - off), max_depth=depth,
                      sample_offset=h * (ref_spp // 2) + off, seed=12345, stream=stream)
            stream.synchronize()
            ref += acc.double()
        halves.append(ref[:, :3] / ref[:, 3:4])
    ref_img = 0.5 * (halves[0] + halves[1])
    var_ref = float(torch.mean((halves[0] - halves[1]) ** 2).item()) / 4.0
    del halves
    ref_s = time.perf_counter() - t0
    # the share of indirect light: 1 - (image mean at depth 1) / (converged mean)
    acc.zero_()
    sc.render(cam, acc, spp=64, max_depth=1, seed=7, stream=stream)
    stream.synchronize()
    indirect = 1.0 - float((acc[:, :3].double() / acc[:, 3:4].double()).mean()) / float(ref_img.mean())

    def mse():
        img = acc[:, :3].double() / acc[:, 3:4].double()
        return float(torch.mean((img - ref_img) ** 2).item()) - var_ref

    def timed(fn):
        acc.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1) / 1e3

    wave = npix * 16  # 16 samples per pixel per wave: a training round after every 16 spp
    alpha, steps, batch, budget, bounces = 0.75, 16, 65536, 512, 3

    def runs(fn):
        ts, ms = [], []
        for sd in range(seeds):
            ts.append(timed(lambda: fn(sd)))
            ms.append(mse())
        return float(np.mean(ts)), float(np.mean(ms)), ms

    t_plain, m_plain, m_plain_s = runs(lambda sd: sc.render(cam, acc, spp=spp, max_depth=depth, seed=100 + sd,
                                                             wave_paths=wave, stream=stream))
    pos = spec.positions.reshape(-1, 3)
    lo, hi = pos.min(0), pos.max(0)
    center = tuple(float(x) for x in (lo + hi) / 2)
    half = float((hi - lo).max() / 2)
    guides = []

    def guided(sd):
        g = native.Guide(ctx, seed=1 + sd, center=center, half_extent=half)
        guides.append(g)
        sc.render_guided(g, cam, acc, spp=spp, max_depth=depth, seed=200 + sd, alpha=alpha, train=True,
                         train_batch=batch, train_steps=steps, train_budget=budget, bounces=bounces,
                         wave_paths=wave, stream=stream)

    t_guided, m_guided, m_guided_s = runs(guided)
    loss = guides[-1].last_loss()
    # equal time: the plain tracer with the samples it renders in the guided time
    spp_eq = max(1, int(round(spp * t_guided / t_plain)))
    t_eq, m_eq, m_eq_s = runs(lambda sd: sc.render(cam, acc, spp=spp_eq, max_depth=depth, seed=300 + sd,
                                                    wave_paths=wave, stream=stream))
    # the trained networks on their own (no further training), equal samples
    t_trained, m_trained, _ = runs(lambda sd: sc.render_guided(guides[sd], cam, acc, spp=spp, max_depth=depth,
                                                                seed=400 + sd, alpha=alpha, train=False,
                                                                bounces=bounces, wave_paths=wave, stream=stream))
    # 1080p throughput of the guided tracer (training on), unless the section itself runs at 1080p
    hd_out = None
    if hd:
        hd_cam = scenes.lower_camera(1920, 1080)
        hd_acc = torch.zeros((1920 * 1080, 4), dtype=torch.float32, device=dev)
        g = native.Guide(ctx, seed=9, center=center, half_extent=half)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sc.render_guided(g, hd_cam, hd_acc, spp=hd_spp, max_depth=depth, seed=5, alpha=alpha, train=True,
                         train_batch=batch, train_steps=steps, bounces=bounces, stream=stream)
        e1.record(stream)
        stream.synchronize()
        t_hd = e0.elapsed_time(e1) / 1e3
        e0.record(stream)
        sc.render(hd_cam, hd_acc, spp=hd_spp, max_depth=depth, seed=6, stream=stream)
        e1.record(stream)
        stream.synchronize()
        t_hd_plain = e0.elapsed_time(e1) / 1e3
        g.close()
        del hd_acc
        hd_out = {"spp": hd_spp, "guided_samples_per_s": 1920 * 1080 * hd_spp / t_hd,
                  "plain_samples_per_s": 1920 * 1080 * hd_spp / t_hd_plain}
    desc = {"gap": "slab over the whole room but a gap of 0.15 half-widths along one wall",
            "centered": "centred slab over 0.7 of the width"}[scene]
    out = {"scene": f"occluded_light (2^20 triangles, 65,536 emitters above the slab, {desc}; floor and walls of "
                    f"albedo 0.4; half the spheres glass)",
           "indirect_fraction": indirect, "width": width, "height": height, "max_depth": depth,
           "reference_spp": ref_spp, "reference_accumulation": "fp64", "reference_seconds": round(ref_s, 2),
           "reference_variance": var_ref,
           "mse": "mean over pixels and channels of the squared error against the reference, minus the "
                  "reference's variance (a quarter of the mean squared difference of its two halves)",
           "spp": spp, "seeds": seeds, "alpha": alpha,
           "plain": {"rmse": m_plain ** 0.5, "seconds": t_plain, "mse_per_seed": m_plain_s},
           "guided": {"rmse": m_guided ** 0.5, "seconds": t_guided, "mse_per_seed": m_guided_s, "final_loss": loss,
                      "training": f"{steps} Adam steps x {batch} samples after every 16 spp, at most {budget} steps",
                      "guided_bounces": bounces},
           "plain_equal_time": {"rmse": m_eq ** 0.5, "spp": spp_eq, "seconds": t_eq, "mse_per_seed": m_eq_s},
           "guided_trained_equal_spp": {"rmse": m_trained ** 0.5, "seconds": t_trained},
           "rmse_ratio_equal_spp": (m_plain / m_guided) ** 0.5, "rmse_ratio_equal_time": (m_eq / m_guided) ** 0.5,
           "rmse_ratio_trained_equal_spp": (m_plain / m_trained) ** 0.5,
           "hd_1080p": hd_out}
    for g in guides:
        g.close()
    del sc, acc, ref_img
    torch.cuda.empty_cache()
    return out


def render_cpu_baseline(spec, cam, depth: int, threads: int, pixels: int):
    """The reference's integrator on the CPU (oracle port of sampleColor with the
    reference's per-object cast), `pixels` pixels x 1 sample; samples/s."""
    from oracle import pyoracle as po
    po.build(ref=False)
    sub = dict(cam)
    # a centred window of the image with the same camera geometry
    wsub = int(np.sqrt(pixels))
    sub["width"] = sub["height"] = wsub
    sub["cx"] = np.float32(cam["cx"] - np.float32((cam["width"] - wsub) // 2) * cam["psx"])
    sub["cy"] = np.float32(cam["cy"] - np.float32((cam["height"] - wsub) // 2) * cam["psy"])
    sc = po.RenderScene(spec)
    t0 = time.perf_counter()
    sc.render(sub, 1, max_depth=depth, cast_mode=1, tri_table_order=1, threads=threads)
    dt = time.perf_counter() - t0
    return {"value": wsub * wsub / dt, "unit": "samples/s", "cores": threads, "kind": "port",
            "sample": f"{wsub}x{wsub} pixels x 1 sample, reference integrator and per-object cast (oracle)",
            "seconds": dt}


def _read_probes(ctx, device: int):
    """Streaming-read bandwidth (dr_probe_read_bandwidth, our own kernel) of a
    48 MiB buffer (L2-resident) and of a 2 GiB buffer (HBM), GB/s."""
    import torch
    small = torch.ones(12 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{device}")
    big = torch.ones(512 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{device}")
    l2 = max(ctx.read_bandwidth(small, small.numel() * 4, reps=50) for _ in range(3))
    hbm = max(ctx.read_bandwidth(big, big.numel() * 4, reps=3) for _ in range(2))
    del small, big
    torch.cuda.empty_cache()
    return l2, hbm


# ---- profiling cases ---------------------------------------------------------------
# Small, fixed workloads for profiling single kernels (ncu, CUDA events):
#   python bench.py --case guide_infer [kernel]   # 0: tcgen05, 1: mma.sync
#   python bench.py --case guide_train [rows]     # Adam steps on random samples
#   python bench.py --case render_box_room        # 256x256, 16 spp, depth 8
#   python bench.py --case render_many_light [spp]
#   python bench.py --case batch_small            # 8 uneven scenes, graph, 2 renders
#   python bench.py --case guided [spp]           # occluded-light scene, plain vs guided
#   python bench.py --case guided_phases          # training, plain and frozen guided renders (NVTX ranges)
# Each case prints one line with its timing; run it once plainly before running
# it under a profiler.

def _case_ctx():
    from devilray_gb300 import native
    native.load()
    return native, native.Context(0)


def case_guide_infer(kernel: int = 0, rows: int = 1 << 20) -> None:
    import torch
    native, ctx = _case_ctx()
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


def case_guide_train(rows: int = 16384, steps: int = 100) -> None:
    import torch
    native, ctx = _case_ctx()
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


def case_render_box_room() -> None:
    import torch
    from devilray_gb300 import scenes
    native, ctx = _case_ctx()
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


def case_render_many_light(spp: int = 16) -> None:
    """Many-light 1080p: scenes.many_light() (2^20 triangles, 65,536 emitters)
    through the outside camera, depth 16, default schedule."""
    import torch
    from devilray_gb300 import scenes
    native, ctx = _case_ctx()
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


def case_batch_small() -> None:
    import torch
    from devilray_gb300 import scenes
    native, ctx = _case_ctx()
    specs = scenes.uneven_batch(8, seed=7)
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


def case_guided(spp: int = 32) -> None:
    """Plain and guided renders of the single-gap occluded-light scene at
    480x270 with the benchmark's guided schedule: alpha 0.75, the first 3
    bounces guided, 16 Adam steps of 65,536 samples after every 16-spp wave
    (at most 512 steps), a fresh network."""
    import torch
    from devilray_gb300 import scenes
    native, ctx = _case_ctx()
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



def case_guided_phases(width: int = 480, height: int = 270, later_spp: int = 448) -> None:
    """The guided render's phases for a launch list, at width x height
    (480x270 by default), depth 16, waves of 16 spp: a fresh network trains
    over 64 spp inside the NVTX range "train" (alpha 0.75, 3 guided bounces,
    16 Adam steps of 65,536 samples after every wave) and over `later_spp`
    more outside any range (448: 512 steps in all); then, inside the range
    "measure", the plain tracer renders 64 spp and the guided one 64 spp with
    the network frozen. Torch fills mark the phases."""
    import torch
    from devilray_gb300 import scenes
    native, ctx = _case_ctx()
    spec = scenes.occluded_light(slab_gap=0.15)
    sc = native.Scene.from_spec(ctx, spec)
    cam = scenes.lower_camera(width, height)
    n = width * height
    acc = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    pos = spec.positions.reshape(-1, 3)
    lo, hi = pos.min(0), pos.max(0)
    g = native.Guide(ctx, seed=1, center=tuple(float(x) for x in (lo + hi) / 2),
                     half_extent=float((hi - lo).max() / 2))
    kw = dict(max_depth=16, alpha=0.75, train_batch=65536, train_steps=16, train_budget=512, bounces=3,
              wave_paths=16 * n)
    marker = torch.zeros(7777, device="cuda")
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("train")
    marker.fill_(0.5)
    sc.render_guided(g, cam, acc, spp=64, seed=11, train=True, **kw)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    if later_spp:
        sc.render_guided(g, cam, acc, spp=later_spp, seed=1, train=True, **kw)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("measure")
    marker.fill_(1.0)
    sc.render(cam, acc, spp=64, max_depth=16, seed=2, wave_paths=16 * n)
    torch.cuda.synchronize()
    marker.fill_(2.0)
    sc.render_guided(g, cam, acc, spp=64, seed=3, train=False, **{k: kw[k] for k in ("max_depth", "alpha", "bounces",
                                                                                       "wave_paths")})
    torch.cuda.synchronize()
    marker.fill_(3.0)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    print(f"guided_phases: loss {g.last_loss():.4f}")
    g.close()
    ctx.check()


CASES = {"guide_infer": case_guide_infer, "guide_train": case_guide_train, "render_box_room": case_render_box_room,
         "render_many_light": case_render_many_light, "batch_small": case_batch_small, "guided": case_guided,
         "guided_phases": case_guided_phases}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-sample", type=int, default=1 << 20)
    ap.add_argument("--ref-sample", type=int, default=0,
                    help="rays per timed step of --impl reference (0: the whole workload if the steps fit)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-render", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-guided", action="store_true")
    ap.add_argument("--guided-ref-spp", type=int, default=65536)
    ap.add_argument("--guided-scene", choices=["gap", "centered"], default="gap")
    ap.add_argument("--guided-size", type=int, nargs=2, default=[480, 270], metavar=("W", "H"))
    ap.add_argument("--guided-spp", type=int, default=1024)
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--layout", type=int, default=0, help="BVH layout of the trace workload: 0 default, 2, 8")
    ap.add_argument("--render-layout", type=int, default=0, help="BVH layout of the render workloads")
    ap.add_argument("--case", nargs="+", metavar=("NAME", "ARG"),
                    help=f"run one profiling case instead of the benchmark: {', '.join(CASES)}")
    args = ap.parse_args()
    if args.case:
        CASES[args.case[0]](*[int(a) for a in args.case[1:]])
        return 0
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
