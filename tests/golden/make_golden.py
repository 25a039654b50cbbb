"""Writes the golden fixtures of tests/golden/ from DevilRay's OWN code.

Run where the DevilRay sources exist (it builds oracle/_ref/libref_harness.so
from them): ``python tests/golden/make_golden.py``. Every expected value in the
fixtures comes from calling the reference function through the harness; the
inputs are either the known-answer cases of the reference's tests (file:line
beside each) or seeded random cases. The fixtures are committed; the tests read
them and never need the reference tree.
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import pyoracle as po  # noqa: E402
from devilray_gb300 import scenes  # noqa: E402

OUT = Path(__file__).resolve().parent
NAN = np.float32(np.nan)


def tri_fixture():
    unit = [0, 0, 0, 1, 0, 0, 0, 1, 0]
    # Known-answer cases of test/src/test_intersection.cpp:33-200.
    kat = [
        ([0.2, 0.2, 5, 0, 0, -1], unit),               # HitsCenterOfTriangle :38-54
        ([0, 0, 10, 0, 0, -1], unit),                  # HitsExactlyOnVertex :56-64
        ([-0.01, 0.5, 1, 0, 0, -1], unit),             # MissesJustOutsideEdge :67-72
        ([0.2, 0.2, 1, 0, 0, 1], unit),                # MissesBehindRayOrigin :74-79
        ([-1, 0.2, 1, 1, 0, 0], unit),                 # ParallelRayDoesNotIntersect :82-87
        ([0, 0, 1, 0, 0, -1], [0] * 9),                # DegenerateTriangleFails :89-95
        ([0.2, 0.2, -1, 0, 0, 1], unit),               # NoBackfaceCulling :97-106
        ([0.2, 0.2, 10000, 0, 0, -1], unit),           # VeryDistantIntersection :108-115
        ([0.5, 0, 1, 0, 0, -1], [0, 0, 0, 1, 0, 0, 2, 0, 0]),       # DegenerateTriangleCollinear :119-126
        ([0.2, 0.2, 1, 0, 0, 0], unit),                # DegenerateRayZeroDirection :128-134
        ([0, 0, 0, NAN, NAN, NAN], unit),              # DegenerateRayNaNInDirection :136-142
        ([50, 1e-9, 1, 0, 0, -1], [0, 0, 0, 100, 0, 0, 100, 2e-8, 0]),  # ExtremelyThinTriangle :144-153
    ]
    # MultipleAngleSanityCheck :155-200: rays from four origins towards an
    # inside point (0.2, 0.2, 0) and an outside point (5, 5, 0).
    for o in ([0.2, 0.2, 10], [10, 0.2, 10], [-5, -5, 2], [0, 0, 1]):
        o32 = np.array(o, np.float32)
        for target in ([0.2, 0.2, 0], [5, 5, 0]):
            d = np.array(target, np.float32) - o32
            kat.append(([*o32.tolist(), *d.tolist()], unit))
    kat_rays = np.array([k[0] for k in kat], np.float32)
    kat_tris = np.array([k[1] for k in kat], np.float32)

    rng = np.random.default_rng(20240531)
    n = 8192
    tris = rng.normal(size=(n, 9)).astype(np.float32)
    # axis-aligned and shared-edge cases
    tris[: n // 8, 2::3] = 0.0
    tris[n // 8: n // 4, 3:6] = tris[n // 8: n // 4, 0:3]
    o = rng.normal(size=(n, 3)) * 3.0
    target = tris.reshape(n, 3, 3).mean(1) + rng.normal(size=(n, 3)) * 0.6
    d = target - o
    d[::2] /= np.linalg.norm(d[::2], axis=1, keepdims=True)
    rays = np.concatenate([o, d], 1).astype(np.float32)
    rays[7::97, 3] = 0.0  # zero direction components
    all_rays = np.concatenate([kat_rays, rays])
    all_tris = np.concatenate([kat_tris, tris])
    hit = np.zeros(len(all_rays), np.int8)
    out = np.zeros((len(all_rays), 4), np.float32)
    for i in range(len(all_rays)):
        h, o4 = po.ref_tri_test(all_rays[i], all_tris[i])
        hit[i] = h
        out[i] = o4 if h else 0.0
    np.savez_compressed(OUT / "tri_test.npz", rays=all_rays, tris=all_tris, hit=hit, out=out,
                        num_kat=np.int32(len(kat)))


def box_fixture():
    unit = [-1, -1, -1, 1, 1, 1]
    # test/src/test_tracing.cpp:91-131
    cases = [([0, 0, -5, 0, 0, 1], unit), ([0, 0, 0, 0, 0, 1], unit), ([0, 0, 5, 0, 0, 1], unit),
             ([0.5, -0.5, -5, 0, 0, 1], unit), ([5, 0, -5, 0, 0, 1], unit), ([-5, -5, 0, 1, 1, 0], unit)]
    rng = np.random.default_rng(7)
    for _ in range(4000):
        lo = rng.normal(size=3) * 4
        hi = lo + np.abs(rng.normal(size=3)) * 2
        o = rng.normal(size=3) * 6
        d = rng.normal(size=3)
        d[rng.random(3) < 0.1] = 0.0
        cases.append(([*o, *d], [*lo, *hi]))
    rays = np.array([c[0] for c in cases], np.float32)
    boxes = np.array([c[1] for c in cases], np.float32)
    hit = np.zeros(len(cases), np.int8)
    t = np.zeros(len(cases), np.float32)
    for i in range(len(cases)):
        h, tt = po.ref_box_test(boxes[i], rays[i])
        hit[i] = h
        t[i] = tt if h else 0.0
    np.savez_compressed(OUT / "box_test.npz", rays=rays, boxes=boxes, hit=hit, t=t)


def bbh_fixture():
    # Two spheres of the incoherent soup family plus scattered slivers, and
    # rays from inside the cube in all directions (closest hit through the
    # reference's generateSimpleBBH + getIntersectionBenchmark).
    rng = np.random.default_rng(99)
    unit = scenes.icosphere_soup(2)  # 320 triangles
    parts = []
    for c, r in (([0, 0, 0], 2.0), ([3, 1, -2], 1.0), ([-4, 2, 1], 1.5)):
        parts.append((np.array(c)[None, :] + r * unit.reshape(-1, 3, 3)).reshape(-1, 9))
    cent = rng.uniform(-6, 6, (1000, 3))
    scatter = (cent[:, None, :] + rng.normal(size=(1000, 3, 3)) * 0.4).reshape(-1, 9)
    # axis-aligned quads (coplanar pairs sharing a diagonal)
    quads = []
    for z in (-5.0, 5.0):
        quads += [[-6, -6, z, 6, -6, z, 6, 6, z], [-6, -6, z, 6, 6, z, -6, 6, z]]
    soup = np.concatenate(parts + [scatter, np.array(quads)]).astype(np.float32)
    m = 6000
    o = rng.uniform(-6, 6, (m, 3))
    u = rng.random((m, 2))
    d = scenes.sphere_directions(u[:, 0], u[:, 1])
    rays6 = np.concatenate([o, d], 1).astype(np.float32)
    res = po.ref_bbh_trace(soup, rays6)
    np.savez_compressed(OUT / "bbh_trace.npz", soup=soup, rays6=rays6, **{k: v for k, v in res.items()})


def alias_fixture():
    # test/src/test_alias.cpp:64-189 inputs, then seeded random tables.
    cases = [[], [42.0], [10, 10, 10], [1, 3], [0.1, 1000], [0, 0, 0, 0], [-5, 10],
             [float(i + 1) for i in range(100)], [1.00001, 0.99999, 1.0], [0.1, 10, 0.1, 10, 0.1, 10]]
    rng = np.random.default_rng(3)
    for n in (7, 64, 333, 1000, 4096):
        cases.append(rng.lognormal(0, 1.5, n).tolist())
        w = rng.random(n)
        w[rng.random(n) < 0.3] = 0.0
        cases.append(w.tolist())
    w_all, off, tables = [], [0], []
    for c in cases:
        c32 = np.array(c, np.float32)
        w_all.append(c32)
        off.append(off[-1] + len(c32))
        tables.append(po.ref_alias_build(c32))
    w_all = np.concatenate(w_all).astype(np.float32)
    tab = np.concatenate(tables)
    # StressTest :193-229: 200,000 lognormal(0,1) weights from std::mt19937(42).
    stress_w = po.ref_lognormal(200000, 42)
    stress = po.ref_alias_build(stress_w)
    # A 65,536-entry emitter-power table (many-light configuration).
    em = np.exp(np.random.default_rng(11).normal(0, 1.5, 65536)).astype(np.float32)
    em_tab = po.ref_alias_build(em)
    # sample() on the 100-item table with seeded uniforms (incl. 0 and the
    # values just below 1).
    t100 = tables[7]
    u = np.random.default_rng(5).random((4000, 2)).astype(np.float32)
    u[:4] = [[0.0, 0.0], [np.nextafter(np.float32(1), np.float32(0)), 0.5], [0.5, 1.0], [0.999, 0.0]]
    idx = np.zeros(len(u), np.int32)
    pdf = np.zeros(len(u), np.float32)
    po.ref().refh_alias_sample(t100["p_A"].copy(), t100["pdf_A"].copy(), t100["pdf_B"].copy(), t100["A"].copy(),
                               t100["B"].copy(), len(t100), u.reshape(-1).copy(), len(u), idx, pdf)
    np.savez_compressed(
        OUT / "alias.npz", sample_uniforms=u, sample_index=idx, sample_pdf=pdf, weights=w_all, offsets=np.array(off, np.int64),
        p_A=tab["p_A"], pdf_A=tab["pdf_A"], pdf_B=tab["pdf_B"], A=tab["A"], B=tab["B"],
        stress_input_sha=np.frombuffer(hashlib.sha256(stress_w.tobytes()).digest(), np.uint8),
        stress_table_sha=np.frombuffer(hashlib.sha256(stress.tobytes()).digest(), np.uint8),
        stress_head=stress[:256].view(np.uint8).copy(),
        emitter_weights=em, emitter_table_sha=np.frombuffer(hashlib.sha256(em_tab.tobytes()).digest(), np.uint8))


def render_fixture():
    # sampleColor (include/tracing/PathGeneration.hpp:363-515) of the
    # reference on the box room with a level-1 glass icosphere, every pixel
    # sample fed a replayed stream of uniforms.
    spec = scenes.box_room(sphere_level=1)
    w, h, spp, stride = 12, 9, 6, 96
    cam = scenes.camera(w, h)
    replay = np.random.default_rng(7).random((w * h, spp, stride)).astype(np.float32)
    out = {}
    for sampling in (0, 1):
        rgb, casts, _ = po.ref_render_samples(spec, cam, spp, replay, sampling)
        out[f"rgb_{sampling}"] = rgb
        out[f"casts_{sampling}"] = casts
    np.savez_compressed(OUT / "render_pin.npz", positions=spec.positions, objects=spec.objects_array(),
                        materials=spec.materials_array(), replay=replay, width=np.int32(w), height=np.int32(h),
                        spp=np.int32(spp), **out)


def debug_fixture():
    # The first-hit debug views of sampleColor / sampleColorDebug
    # (include/tracing/PathGeneration.hpp:274-299, 393-429) on the box room,
    # materials given distinct debug colours; camera jitter replayed.
    spec = scenes.box_room(sphere_level=1)
    for i, m in enumerate(spec.materials):
        m["debug"] = (0.9 - 0.1 * i, 0.2 + 0.15 * i, 0.5, 0.0)
    w, h, spp, stride = 16, 12, 3, 4
    cam = scenes.camera(w, h)
    replay = np.random.default_rng(11).random((w * h, spp, stride)).astype(np.float32)
    out = {}
    for view in (1, 2, 3):
        rgb, casts, sw = po.ref_render_samples(spec, cam, spp, replay, 1, debug=view)
        out[f"rgb_{view}"] = rgb
        out[f"casts_{view}"] = casts
        out[f"w_{view}"] = sw
    np.savez_compressed(OUT / "render_debug_pin.npz", positions=spec.positions, materials=spec.materials_array(),
                        replay=replay, width=np.int32(w), height=np.int32(h), spp=np.int32(spp), **out)


# OBJ texts of the loader's grammar and error cases (ours); the reference's
# model files are read from its tree.
MESH_TEXTS = {
    "grammar": "# corners in every form\nmtllib scene.mtl\no tetra_1\nv 0 0 0\nv 1.5 0 -0.25\r\n"
               "v 0 1 0.5 \t\nv 0.25 0.125 2\nvt 0.5 0.5\nvn 0 0 1\nvn 0.6 0.8 0\ns off\n"
               "f 1 2 3\nf 1//2 2//2 4//1\nf 1/1/1 3/1/2 4/1/1\nf 2/1 3/1 4/1\nf 4 3\n\n",
    "no_normals": "v -1 -1 0\nv 1 -1 0\nv 0 1 0\nv 0 0 1\nf 1 2 3\nf 1 2 4\n",
    "quad": "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1 2 3 4\n",
    "unknown_tag": "v 0 0 0\nusemtl red\n",
    "index_range": "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 4\n",
    "normal_range": "v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//2 3//1\n",
    "negative_index": "v 0 0 0\nv 1 0 0\nv 0 1 0\nf -1 -2 -3\n",
    "bad_number": "v 0 x 0\n",
    "four_indices": "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1/1/1/1 2 3\n",
}


def mesh_fixture():
    """loadMesh, then normalizeMeshSize and generateCoarseNormals, of the
    reference (src/models/Mesh.cpp:117-243) on its three model files and on
    the OBJ texts above; a case that throws keeps only its text and the flag."""
    import os
    import tempfile
    ref_root = Path(os.environ.get("DEVILRAY_REF_ROOT", "/root/reference"))
    cases = {name: (ref_root / "models" / f"{name}.obj").read_bytes() for name in ("ico", "cube", "suzanne")}
    cases.update({k: v.encode() for k, v in MESH_TEXTS.items()})
    out = {"names": np.array(list(cases.keys()))}
    with tempfile.TemporaryDirectory() as d:
        for name, text in cases.items():
            path = Path(d) / f"{name}.obj"
            path.write_bytes(text)
            out[f"{name}_obj"] = np.frombuffer(text, np.uint8)
            m = po.ref_mesh_load(str(path))
            out[f"{name}_ok"] = np.int32(m is not None)
            if m is None:
                continue
            for k, v in m.items():
                out[f"{name}_{k}"] = v
            if len(m["points"]):
                for k, v in po.ref_mesh_load(str(path), normalize=True).items():
                    out[f"{name}_norm_{k}"] = v
    np.savez_compressed(OUT / "mesh.npz", **out)


FIXTURES = {"render": lambda: (render_fixture(), debug_fixture()), "tri": tri_fixture, "box": box_fixture,
            "bbh": bbh_fixture, "alias": alias_fixture, "mesh": mesh_fixture}


def main():
    """Writes every fixture, or those named on the command line."""
    po.build(ref=True)
    for name in (sys.argv[1:] or list(FIXTURES)):
        FIXTURES[name]()
    for p in sorted(OUT.glob("*.npz")):
        print(f"{p.name}: {p.stat().st_size} bytes")


if __name__ == "__main__":
    main()
