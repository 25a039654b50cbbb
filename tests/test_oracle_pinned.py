"""The CPU oracle against golden vectors produced by DevilRay's own code.

The fixtures in tests/golden/ were written by tests/golden/make_golden.py,
which calls the reference's testTriangleIntersection, testBoxIntersection,
generateSimpleBBH + getIntersectionBenchmark and generateAliasTable. Here the
oracle's restatement of each must reproduce them bit for bit.
"""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

pytestmark = []


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_triangle_test_matches_reference(oracle, golden):
    g = golden("tri_test.npz")
    rays, tris, hit, out = g["rays"], g["tris"], g["hit"], g["out"]
    for i in range(len(rays)):
        h, o = oracle.tri_test(rays[i], tris[i])
        assert h == bool(hit[i]), f"case {i}"
        if h:
            assert np.array_equal(_bits(o), _bits(out[i])), f"case {i}: {o} vs {out[i]}"


def test_known_answers_of_reference_tests(oracle, golden):
    """test/src/test_intersection.cpp expectations, evaluated on the oracle."""
    g = golden("tri_test.npz")
    rays, tris = g["rays"], g["tris"]
    expect_hit = [True, True, False, False, False, False, True, True, False, False, False, True]
    for i, e in enumerate(expect_hit):
        h, o = oracle.tri_test(rays[i], tris[i])
        assert h == e, f"known-answer case {i}"
    assert abs(oracle.tri_test(rays[0], tris[0])[1][0] - 5.0) < 1e-5
    assert abs(oracle.tri_test(rays[1], tris[1])[1][0] - 10.0) < 1e-5
    assert abs(oracle.tri_test(rays[7], tris[7])[1][0] - 10000.0) < 1e-2
    # MultipleAngleSanityCheck: hits at t ~ 1 with barycentrics (0.6, 0.2, 0.2)
    for k in range(4):
        h, o = oracle.tri_test(rays[12 + 2 * k], tris[12 + 2 * k])
        assert h and abs(o[0] - 1.0) < 1e-4
        assert np.allclose(o[1:], [0.6, 0.2, 0.2], atol=1e-4)
        assert not oracle.tri_test(rays[13 + 2 * k], tris[13 + 2 * k])[0]


def test_box_test_matches_reference(oracle, golden):
    g = golden("box_test.npz")
    for i in range(len(g["rays"])):
        h, t = oracle.box_test(g["boxes"][i], g["rays"][i])
        assert h == bool(g["hit"][i]), f"case {i}"
        if h:
            assert np.float32(t).view(np.uint32) == g["t"][i].view(np.uint32), f"case {i}"
    # test/src/test_tracing.cpp:91-131
    assert g["hit"][:6].tolist() == [1, 1, 0, 1, 0, 1]
    assert g["t"][[0, 1, 3, 5]].tolist() == [4.0, 0.0, 4.0, 4.0]


def test_bbh_structure_matches_reference(oracle, golden):
    g = golden("bbh_trace.npz")
    b = oracle.BBH(g["soup"])
    boxes, links, order = b.export()
    assert np.array_equal(_bits(boxes), _bits(g["boxes"]))
    assert np.array_equal(links, g["links"])
    assert np.array_equal(order, g["order"])
    assert b.depth == int(g["depth"])


def test_bbh_traversal_matches_reference(oracle, golden):
    g = golden("bbh_trace.npz")
    b = oracle.BBH(g["soup"])
    t, prim, nb, nt = b.trace_reference(g["rays6"])
    assert np.array_equal(_bits(t), _bits(g["t"]))
    ok = g["prim"] != -2  # -2: the harness found a bit-identical tie
    assert np.array_equal(prim[ok], g["prim"][ok])
    assert np.array_equal(nb, g["box_tests"])
    assert np.array_equal(nt, g["tri_tests"])


def test_canonical_closest_hit_equals_brute_force(oracle, golden):
    """The canonical semantics (min t, ties to the smaller index) shared with
    the GPU: conservative BBH traversal == brute-force scan; and it agrees with
    the reference's own traversal on every ray of the fixture."""
    g = golden("bbh_trace.npz")
    soup = g["soup"]
    r6 = g["rays6"]
    r8 = np.zeros((len(r6), 8), np.float32)
    r8[:, 0:3], r8[:, 3], r8[:, 4:7] = r6[:, 0:3], np.inf, r6[:, 3:6]
    b = oracle.BBH(soup)
    tc, pc = b.trace_canonical(r8, slack=1e-3)
    tb, pb = oracle.trace_brute(soup, r8)
    assert np.array_equal(_bits(tc), _bits(tb))
    assert np.array_equal(pc, pb)
    ok = g["prim"] != -2
    assert np.array_equal(_bits(tc), _bits(g["t"]))
    assert np.array_equal(pc[ok], g["prim"][ok])


def test_alias_tables_match_reference(oracle, golden):
    g = golden("alias.npz")
    off = g["offsets"]
    for c in range(len(off) - 1):
        w = g["weights"][off[c]:off[c + 1]]
        tab = oracle.alias_build_ref(w)
        sl = slice(off[c], off[c + 1])
        assert np.array_equal(_bits(tab["p_A"]), _bits(g["p_A"][sl])), f"case {c}"
        assert np.array_equal(_bits(tab["pdf_A"]), _bits(g["pdf_A"][sl])), f"case {c}"
        assert np.array_equal(_bits(tab["pdf_B"]), _bits(g["pdf_B"][sl])), f"case {c}"
        assert np.array_equal(tab["A"], g["A"][sl]), f"case {c}"
        assert np.array_equal(tab["B"], g["B"][sl]), f"case {c}"


def test_alias_stress_input_and_table_match_reference(oracle, golden):
    g = golden("alias.npz")
    w = oracle.lognormal_input(200000, 42)
    assert hashlib.sha256(w.tobytes()).digest() == g["stress_input_sha"].tobytes()
    tab = oracle.alias_build_ref(w)
    assert tab[:256].view(np.uint8).tobytes() == g["stress_head"].tobytes()
    assert hashlib.sha256(tab.tobytes()).digest() == g["stress_table_sha"].tobytes()
    em = oracle.alias_build_ref(g["emitter_weights"])
    assert hashlib.sha256(em.tobytes()).digest() == g["emitter_table_sha"].tobytes()


def _fidelity(w, tab):
    """VerifyTableFidelity (test/src/test_alias.cpp:17-57) in double precision."""
    w = np.maximum(np.asarray(w, np.float64), 0.0)
    n = len(w)
    total = w.sum()
    expected = w / total if total > 0 else np.zeros(n)
    actual = np.zeros(n)
    np.add.at(actual, tab["A"], tab["p_A"].astype(np.float64) / n)
    m = (tab["p_A"] < 1.0) & (tab["B"] >= 0)
    np.add.at(actual, tab["B"][m], (1.0 - tab["p_A"][m].astype(np.float64)) / n)
    return np.abs(actual - expected).max()


@pytest.mark.parametrize("n", [1, 2, 3, 100, 4096, 200000])
def test_sweep_alias_fidelity(oracle, n):
    """The device build's CPU restatement is a valid alias table (same fidelity
    bound as the reference's VerifyTableFidelity)."""
    w = oracle.lognormal_input(n, 42) if n > 3 else np.arange(1, n + 1, dtype=np.float32)
    tab = oracle.alias_build_sweep(w)
    assert _fidelity(w, tab) < 1e-6
    assert (tab["p_A"] >= 0.5).all() and (tab["p_A"] <= 1.0).all()
    assert ((tab["p_A"] == 1.0) | (tab["B"] >= 0)).all()


def test_sweep_alias_edge_cases(oracle):
    assert oracle.alias_build_sweep(np.zeros(0, np.float32)).size == 0
    z = oracle.alias_build_sweep(np.zeros(4, np.float32))
    assert (z["p_A"] == 1).all() and (z["A"] == np.arange(4)).all()
    neg = oracle.alias_build_sweep(np.array([-5, 10], np.float32))
    assert _fidelity([0, 10], neg) < 1e-7


def test_philox_known_answers(oracle):
    """Random123 known-answer vectors for philox4x32_10."""
    assert oracle.philox([0, 0, 0, 0], [0, 0]).tolist() == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert oracle.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2).tolist() == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert oracle.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]).tolist() == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_alias_sample_matches_reference(oracle, golden):
    g = golden("alias.npz")
    off = g["offsets"]
    sl = slice(off[7], off[8])
    tab = np.zeros(off[8] - off[7], oracle.ALIAS_DTYPE)
    for k in ("p_A", "pdf_A", "pdf_B", "A", "B"):
        tab[k] = g[k][sl]
    for (u0, u1), i, p in zip(g["sample_uniforms"], g["sample_index"], g["sample_pdf"]):
        idx, pdf = oracle.alias_sample(tab, float(u0), float(u1))
        assert idx == i and np.float32(pdf) == p


def test_integrator_matches_reference_sample_color(oracle, golden):
    """The oracle's integrator with the reference's random-number order, the
    reference's cast (per-object BBH) and std sin/cos/acos reproduces the
    reference's own sampleColor on every pixel sample (colour bits and path-ray
    counts), for both pixel-sampling modes."""
    from devilray_gb300 import scenes
    g = golden("render_pin.npz")
    spec = scenes.box_room(sphere_level=1)
    assert np.array_equal(spec.positions, g["positions"])
    w, h, spp = int(g["width"]), int(g["height"]), int(g["spp"])
    cam = scenes.camera(w, h)
    sc = oracle.RenderScene(spec, light_tables=1)
    for sampling in (0, 1):
        acc, casts, rgb = sc.render(cam, spp, max_depth=10, rng_mode=1, trig_mode=1, cast_mode=1, tri_table_order=1,
                                    replay=g["replay"], per_sample=True, pixel_sampling=sampling)
        assert np.array_equal(rgb.view(np.uint32), g[f"rgb_{sampling}"].view(np.uint32))
        assert np.array_equal(casts, g[f"casts_{sampling}"])
        assert (rgb != 0).any()


def test_create_pixels_known_values(oracle):
    # 2 x 2 image; row 0 is the bottom row of the output
    acc = np.array([[0, 0, 0, 0],            # never sampled: black
                    [2, 4, 6, 2],            # averages above 1 clamp to 255
                    [0.2, 0.2, 0.2, 1],      # linear 0.2 -> 51; sRGB 0.2 -> 124
                    [0.001, 0, 1, 1]],       # 0.001 is on the linear segment: 0.01292 * 255 -> 3
                   np.float32)
    g = oracle.create_pixels(acc, 2, 2, True)
    lin = oracle.create_pixels(acc, 2, 2, False)
    # flipped: input row 0 lands in output row 1
    assert g[2] == 0xFF000000 and g[3] == 0xFFFFFFFF
    assert g[0] == 0xFF000000 | (124 << 16) | (124 << 8) | 124
    assert g[1] == 0xFF000000 | (255 << 16) | 3
    assert lin[0] == 0xFF000000 | (51 << 16) | (51 << 8) | 51


@pytest.mark.parametrize("view", [1, 2, 3])
def test_debug_views_match_reference(oracle, golden, view):
    """First-hit debug views (UV checker, barycentrics, winding order) of the
    oracle against the reference's own sampleColor with that DebugOptions."""
    from devilray_gb300 import scenes
    g = golden("render_debug_pin.npz")
    spec = scenes.box_room(sphere_level=1)
    for i, m in enumerate(spec.materials):
        m["debug"] = (0.9 - 0.1 * i, 0.2 + 0.15 * i, 0.5, 0.0)
    assert np.array_equal(spec.materials_array(), g["materials"])
    w, h, spp = int(g["width"]), int(g["height"]), int(g["spp"])
    cam = scenes.camera(w, h)
    sc = oracle.RenderScene(spec, light_tables=1)
    acc, casts, rgb = sc.render(cam, spp, rng_mode=1, trig_mode=1, cast_mode=1, tri_table_order=1,
                                replay=g["replay"], per_sample=True, pixel_sampling=1, debug=view)
    assert np.array_equal(rgb.view(np.uint32), g[f"rgb_{view}"].view(np.uint32))
    assert np.array_equal(casts, g[f"casts_{view}"])
    assert np.array_equal(acc[:, 3], g[f"w_{view}"].sum(0))
    assert (rgb != 0).any()
    if view == 1:
        assert (g["w_1"] == 0).any() and (g["w_1"] == 1).any()   # misses add no sample
