"""GPU traversal parity through the C ABI.

Closest hit: the GPU's (t, prim) must equal the oracle's canonical closest hit
bit for bit (smallest t of the reference triangle test over the soup, ties to
the smaller triangle index), and the reference's own traversal on the golden
fixture. Any hit: the occlusion flag must equal the oracle's.
"""
from __future__ import annotations

import numpy as np
import pytest

from devilray_gb300 import scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def gpu_closest(native, scene, rays8, mode=0, counters=False):
    r = torch.from_numpy(np.ascontiguousarray(rays8, np.float32)).cuda()
    hits = torch.empty((len(rays8), 2), dtype=torch.int32, device="cuda")
    cnt = scene.trace_closest(r, len(rays8), hits, mode, counters=counters)
    torch.cuda.synchronize()
    h = hits.cpu().numpy()
    return h[:, 0].copy().view(np.float32), h[:, 1].copy(), cnt


def gpu_any(native, scene, rays8, mode=0):
    r = torch.from_numpy(np.ascontiguousarray(rays8, np.float32)).cuda()
    occ = torch.empty(len(rays8), dtype=torch.uint8, device="cuda")
    scene.trace_any(r, len(rays8), occ, mode)
    torch.cuda.synchronize()
    return occ.cpu().numpy()


def rays8_from6(r6, tmax=np.inf):
    r8 = np.zeros((len(r6), 8), np.float32)
    r8[:, 0:3], r8[:, 3], r8[:, 4:7] = r6[:, 0:3], tmax, r6[:, 3:6]
    return r8


def test_closest_hit_matches_reference_fixture(native, ctx, oracle, golden):
    g = golden("bbh_trace.npz")
    scene = native.Scene(ctx, g["soup"])
    r8 = rays8_from6(g["rays6"])
    t, prim, _ = gpu_closest(native, scene, r8)
    assert np.array_equal(_bits(t), _bits(g["t"])), "t differs from the reference's getIntersection"
    ok = g["prim"] != -2
    assert np.array_equal(prim[ok], g["prim"][ok])
    b = oracle.BBH(g["soup"])
    tc, pc = b.trace_canonical(r8, slack=scene.info().slack)
    assert np.array_equal(_bits(t), _bits(tc)) and np.array_equal(prim, pc)


@pytest.mark.parametrize("layout", [2, 8])
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("ntri,nray,leaf", [(1, 4096, 0), (37, 20000, 1), (5000, 100000, 0), (65536, 262144, 0),
                                            (65536, 262144, 8)])
def test_closest_hit_bit_exact_vs_oracle(native, ctx, oracle, mode, ntri, nray, leaf, layout):
    half = max(1.0, scenes.density_half(ntri))
    soup, _, _ = scenes.incoherent_soup(ntri, seed=ntri, half=half)
    rays = scenes.incoherent_rays(nray, seed=nray, half=half)
    scene = native.Scene(ctx, soup, max_leaf_size=leaf, layout=layout)
    assert scene.info().layout == layout
    t, prim, _ = gpu_closest(native, scene, rays, mode)
    b = oracle.BBH(soup)
    tc, pc = b.trace_canonical(rays, slack=scene.info().slack, tri_mode=mode)
    assert (pc >= 0).sum() > 0 or ntri == 1
    mism = np.flatnonzero((_bits(t) != _bits(tc)) | (prim != pc))
    assert mism.size == 0, f"{mism.size} mismatches, first {mism[:5]}: gpu {t[mism[:5]]},{prim[mism[:5]]} oracle {tc[mism[:5]]},{pc[mism[:5]]}"


def test_closest_hit_brute_force_small(native, ctx, oracle):
    half = scenes.density_half(2000)
    soup, _, _ = scenes.incoherent_soup(2000, seed=5, half=half)
    rays = scenes.incoherent_rays(20000, seed=6, half=half)
    scene = native.Scene(ctx, soup)
    t, prim, _ = gpu_closest(native, scene, rays)
    tb, pb = oracle.trace_brute(soup, rays)
    assert np.array_equal(_bits(t), _bits(tb)) and np.array_equal(prim, pb)


@pytest.mark.parametrize("layout", [2, 8])
@pytest.mark.parametrize("mode", [0, 1])
def test_any_hit_matches_oracle(native, ctx, oracle, mode, layout):
    half = scenes.density_half(30000)
    soup, _, _ = scenes.incoherent_soup(30000, seed=9, half=half)
    rays = scenes.incoherent_rays(200000, seed=10, half=half)
    rng = np.random.default_rng(1)
    rays[:, 3] = rng.uniform(0, 40, len(rays)).astype(np.float32)
    scene = native.Scene(ctx, soup, layout=layout)
    occ = gpu_any(native, scene, rays, mode)
    b = oracle.BBH(soup)
    occ_o = b.trace_any(rays, slack=scene.info().slack, tri_mode=mode)
    assert np.array_equal(occ, occ_o)
    t, prim, _ = gpu_closest(native, scene, rays, mode)
    assert np.array_equal(occ.astype(bool), prim >= 0)  # closest hit honours tmax too
    assert 0.05 < occ.mean() < 0.95


def grazing_rays(soup, n, seed):
    """Rays aimed exactly at triangle vertices and edge midpoints (so they graze
    the boxes of the hierarchy), from origins 1 to 10^4 scene units away, a
    quarter of them along a coordinate axis (two direction components 0)."""
    rng = np.random.default_rng(seed)
    tri = soup.reshape(-1, 3, 3).astype(np.float64)
    k = rng.integers(0, len(tri), n)
    a, b = rng.integers(0, 3, n), rng.integers(0, 3, n)
    mid = rng.random(n) < 0.3
    target = np.where(mid[:, None], 0.5 * (tri[k, a] + tri[k, b]), tri[k, a])
    d = rng.normal(size=(n, 3))
    axis = rng.random(n) < 0.25
    ax = np.zeros((n, 3))
    ax[np.arange(n), rng.integers(0, 3, n)] = rng.choice([-1.0, 1.0], n)
    d = np.where(axis[:, None], ax, d / np.linalg.norm(d, axis=1, keepdims=True))
    dist = 10.0 ** rng.uniform(0, 4, n)
    r8 = np.zeros((n, 8), np.float32)
    r8[:, 0:3] = (target - d * dist[:, None]).astype(np.float32)
    r8[:, 3] = np.inf
    r8[:, 4:7] = d.astype(np.float32)
    return r8


@pytest.mark.parametrize("layout", [2, 8])
@pytest.mark.parametrize("mode", [0, 1])
def test_grazing_rays_match_brute_force(native, ctx, oracle, layout, mode):
    """The box tests are conservative: rays that pass exactly through vertices
    and edges (the faces of the quantised child boxes) from near and far find
    the brute-force closest hit."""
    half = scenes.density_half(6000)
    soup, _, _ = scenes.incoherent_soup(6000, seed=21, half=half)
    rays = grazing_rays(soup, 40000, seed=22)
    scene = native.Scene(ctx, soup, layout=layout)
    t, prim, _ = gpu_closest(native, scene, rays, mode)
    tb, pb = oracle.trace_brute(soup, rays, tri_mode=mode)
    assert (pb >= 0).mean() > 0.5
    mism = np.flatnonzero((_bits(t) != _bits(tb)) | (prim != pb))
    assert mism.size == 0, f"{mism.size} mismatches, first {mism[:5]}: gpu {prim[mism[:5]]} brute {pb[mism[:5]]}"
    occ = gpu_any(native, scene, rays, mode)
    assert np.array_equal(occ.astype(bool), pb >= 0)


@pytest.mark.parametrize("layout", [2, 8])
def test_edge_cases(native, ctx, oracle, layout):
    unit = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32)
    degenerate = np.array([[0, 0, 0, 0, 0, 0, 0, 0, 0], [0, 0, 0, 1, 0, 0, 2, 0, 0]], np.float32)
    dup = np.concatenate([unit, unit, unit + np.float32([0, 0, -1] * 3)])
    quad = np.array([[-1, -1, 0, 1, -1, 0, 1, 1, 0], [-1, -1, 0, 1, 1, 0, -1, 1, 0]], np.float32)
    soup = np.concatenate([degenerate, dup, quad + np.float32([5, 0, 0] * 3)])
    r6 = np.array([
        [0.2, 0.2, 5, 0, 0, -1],       # hits the duplicated unit triangle -> smaller index wins
        [0.2, 0.2, -5, 0, 0, 1],       # from below: the lower copy first
        [0, 0, 10, 0, 0, -1],          # on a vertex
        [5.0, 0.0, 3, 0, 0, -1],       # on the shared diagonal of the quad
        [5.5, -0.5, 3, 0, 0, -1],
        [0.2, 0.2, 5, 0, 0, 0],        # zero direction
        [0, 0, 0, np.nan, np.nan, np.nan],
        [np.inf, 0, 0, 0, 0, -1],
        [-1, 0.2, 1, 1, 0, 0],         # parallel
        [0.2, 0.2, 0, 0, 0, -1],       # starts on the surface (t = 0)
    ], np.float32)
    r8 = rays8_from6(r6)
    scene = native.Scene(ctx, soup, layout=layout)
    t, prim, _ = gpu_closest(native, scene, r8)
    tb, pb = oracle.trace_brute(soup, r8)
    assert np.array_equal(_bits(t), _bits(tb)) and np.array_equal(prim, pb)
    assert prim[0] == 2 and prim[1] == 4 and prim[5] == -1 and prim[6] == -1 and prim[7] == -1
    assert np.isinf(t[5]) and prim[8] == -1
    assert np.array_equal(gpu_any(native, scene, r8).astype(bool), pb >= 0)
    # tmax: a hit at exactly t == tmax counts; below it does not
    r8b = r8[:1].copy()
    r8b[0, 3] = np.float32(5.0)
    assert gpu_closest(native, scene, r8b)[1][0] == 2
    r8b[0, 3] = np.nextafter(np.float32(5.0), np.float32(0))
    assert gpu_closest(native, scene, r8b)[1][0] == -1


@pytest.mark.parametrize("layout", [2, 8])
def test_coincident_and_zero_area_triangles_match_brute_force(native, ctx, oracle, layout):
    """Thousands of copies of one triangle (zero-extent splits, equal costs in
    the wide collapse), zero-area triangles and a few ordinary ones: the
    smallest index among the coincident copies must win."""
    rng = np.random.default_rng(11)
    tri = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32)
    copies = np.repeat(tri, 3000, axis=0)
    points = np.repeat(np.float32([[0.25, 0.25, 0.5] * 3]), 500, axis=0)
    centres = rng.uniform(-3, 3, size=(200, 1, 3))
    centres[:, 0, 2] = rng.uniform(-3, -0.5, 200)  # below the copies
    others = (centres + rng.uniform(-0.3, 0.3, size=(200, 3, 3))).reshape(200, 9).astype(np.float32)
    soup = np.concatenate([others[:100], copies, points, others[100:]])
    o = np.column_stack([rng.uniform(0, 0.5, 4000), rng.uniform(0, 0.5, 4000), np.full(4000, 2.0)])
    dvec = np.column_stack([rng.normal(0, 0.05, 4000), rng.normal(0, 0.05, 4000), -np.ones(4000)])
    r6 = np.concatenate([np.column_stack([o, dvec]), rng.uniform(-3, 3, size=(4000, 6))]).astype(np.float32)
    r8 = rays8_from6(r6)
    scene = native.Scene(ctx, soup, layout=layout)
    t, prim, _ = gpu_closest(native, scene, r8)
    tb, pb = oracle.trace_brute(soup, r8)
    assert np.array_equal(_bits(t), _bits(tb)) and np.array_equal(prim, pb)
    assert (prim[:4000] == 100).sum() > 3000  # the first copy
    assert np.array_equal(gpu_any(native, scene, r8).astype(bool), pb >= 0)


@pytest.mark.parametrize("layout", [2, 8])
def test_empty_and_single_triangle_scenes(native, ctx, layout):
    rays = scenes.incoherent_rays(1000, seed=3)
    empty = native.Scene(ctx, np.zeros((0, 9), np.float32), layout=layout)
    t, prim, _ = gpu_closest(native, empty, rays)
    assert (prim == -1).all() and np.isinf(t).all()
    assert gpu_any(native, empty, rays).sum() == 0
    one = native.Scene(ctx, np.array([[-60, -60, 0, 60, -60, 0, 0, 60, 0]], np.float32), layout=layout)
    t, prim, _ = gpu_closest(native, one, rays)
    assert set(np.unique(prim)) <= {-1, 0} and (prim == 0).sum() > 50


@pytest.mark.parametrize("layout", [2, 8])
def test_counters_and_host_path(native, ctx, oracle, layout):
    half = scenes.density_half(20000)
    soup, _, _ = scenes.incoherent_soup(20000, seed=2, half=half)
    rays = scenes.incoherent_rays(50000, seed=4, half=half)
    scene = native.Scene(ctx, soup, layout=layout)
    t, prim, cnt = gpu_closest(native, scene, rays, counters=True)
    assert cnt.rays == len(rays) and cnt.hits == (prim >= 0).sum()
    assert cnt.node_visits >= len(rays) and cnt.tri_tests > 0
    if layout == 2:
        assert cnt.box_tests == 2 * cnt.node_visits
    else:
        assert cnt.node_visits <= cnt.box_tests <= 8 * cnt.node_visits
    hits = scene.trace_closest_host(rays)
    assert np.array_equal(hits["prim"], prim) and np.array_equal(_bits(hits["t"]), _bits(t))
    info = scene.info()
    assert info.depth < 64 and info.num_nodes > 0 and info.slack > 0


def test_concurrent_launches_on_two_streams(native, ctx, oracle):
    """Persistent launches on different streams run at the same time; each
    takes its own work counter, so both results stay exact (including the
    host-buffer path, which alternates two compute streams itself)."""
    half = scenes.density_half(30000)
    soup, _, _ = scenes.incoherent_soup(30000, seed=12, half=half)
    rays_a = scenes.incoherent_rays(300000, seed=13, half=half)
    rays_b = scenes.incoherent_rays(300000, seed=14, half=half)
    scene = native.Scene(ctx, soup, layout=8)
    ta, pa, _ = gpu_closest(native, scene, rays_a)
    tb, pb, _ = gpu_closest(native, scene, rays_b)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    da, db = torch.from_numpy(rays_a).cuda(), torch.from_numpy(rays_b).cuda()
    torch.cuda.synchronize()
    for _ in range(3):
        ha = torch.empty((len(rays_a), 2), dtype=torch.int32, device="cuda")
        hb = torch.empty((len(rays_b), 2), dtype=torch.int32, device="cuda")
        occ = torch.empty(len(rays_b), dtype=torch.uint8, device="cuda")
        scene.trace_closest(da, len(rays_a), ha, stream=s1)
        scene.trace_closest(db, len(rays_b), hb, stream=s2)
        scene.trace_any(db, len(rays_b), occ, stream=s1)
        torch.cuda.synchronize()
        a, b = ha.cpu().numpy(), hb.cpu().numpy()
        assert np.array_equal(a[:, 1], pa) and np.array_equal(a[:, 0].view(np.float32).view(np.uint32), _bits(ta))
        assert np.array_equal(b[:, 1], pb) and np.array_equal(b[:, 0].view(np.float32).view(np.uint32), _bits(tb))
        assert np.array_equal(occ.cpu().numpy().astype(bool), pb >= 0)
    hits = scene.trace_closest_host(np.concatenate([rays_a, rays_b]))
    assert np.array_equal(hits["prim"], np.concatenate([pa, pb]))


def test_invalid_arguments_return_status(native, ctx):
    scene = native.Scene(ctx, np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32))
    with pytest.raises(native.DrError) as e:
        scene.trace_closest(0, 10, 0)
    assert e.value.status == 1
    bad = np.array([[0, 0, np.nan, 1, 0, 0, 0, 1, 0]], np.float32)
    with pytest.raises(native.DrError):
        native.Scene(ctx, bad)


def test_read_bandwidth_probe(native, ctx):
    buf = torch.ones(8 * 1024 * 1024, dtype=torch.float32, device="cuda")
    gbs = ctx.read_bandwidth(buf, buf.numel() * 4, reps=5)
    assert 100.0 < gbs < 1e6


@pytest.mark.parametrize("n,dup", [(1, 0), (2, 0), (3, 0), (100, 0), (4096, 0), (1 << 18, 0), (5000, 3)])
def test_device_lbvh_build_matches_host_build(native, ctx, oracle, n, dup):
    """The device linear BVH (DR_BUILD_DEVICE_LBVH) gives the same hits, bit for
    bit, as the host binned-SAH build and the oracle; `dup` repeats every
    triangle (equal Morton codes)."""
    soup, _, _ = scenes.incoherent_soup(n, seed=n + 3)
    if dup:
        soup = np.repeat(soup, dup, axis=0)
    rays = scenes.incoherent_rays(20000, seed=5)
    dev = native.Scene(ctx, soup, builder=1)
    host = native.Scene(ctx, soup, layout=2)
    assert dev.info().layout == 2 and dev.info().num_nodes == max(1, len(soup) - 1)
    d_rays = torch.from_numpy(rays).cuda()
    out = []
    for sc in (dev, host):
        h = torch.empty((len(rays), 2), dtype=torch.int32, device="cuda")
        sc.trace_closest(d_rays, len(rays), h)
        occ = torch.empty(len(rays), dtype=torch.uint8, device="cuda")
        sc.trace_any(d_rays, len(rays), occ)
        torch.cuda.synchronize()
        out.append((h.cpu().numpy(), occ.cpu().numpy()))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    if len(soup) <= 4096:
        t, prim = oracle.BBH(soup).trace_canonical(rays, slack=host.info().slack)
        assert np.array_equal(out[0][0][:, 1], prim)
    ctx.check()


def test_device_lbvh_render_matches_host(native, ctx):
    spec = scenes.box_room(sphere_level=2)
    cam = scenes.camera(32, 24)
    outs = []
    for kw in ({"builder": 1}, {"layout": 2}):
        sc = native.Scene.from_spec(ctx, spec, **kw)
        acc = torch.zeros((32 * 24, 4), dtype=torch.float32, device="cuda")
        sc.render(cam, acc, spp=4, max_depth=8)
        torch.cuda.synchronize()
        outs.append(acc.cpu().numpy())
    assert np.array_equal(outs[0].view(np.uint32), outs[1].view(np.uint32))


@pytest.mark.parametrize("n,dup", [(1, 0), (2, 0), (3, 0), (9, 0), (100, 0), (4096, 0), (1 << 18, 0), (5000, 3)])
def test_device_wide_build_matches_host_build(native, ctx, oracle, n, dup):
    """The device build collapsed into compressed 8-wide nodes
    (DR_BUILD_DEVICE_LBVH, layout 8) gives the same closest and any hits, bit
    for bit, as the host-built 8-wide scene and the oracle; `dup` repeats every
    triangle (equal Morton codes)."""
    soup, _, _ = scenes.incoherent_soup(n, seed=n + 7)
    if dup:
        soup = np.repeat(soup, dup, axis=0)
    rays = scenes.incoherent_rays(20000, seed=8)
    rng = np.random.default_rng(n)
    rays[:, 3] = np.where(rng.random(len(rays)) < 0.5, np.inf, rng.uniform(0, 60, len(rays))).astype(np.float32)
    dev = native.Scene(ctx, soup, builder=1, layout=8)
    host = native.Scene(ctx, soup, layout=8)
    assert dev.info().layout == 8 and 1 <= dev.info().num_nodes <= max(1, len(soup) - 1)
    assert dev.info().depth >= 1
    d_rays = torch.from_numpy(rays).cuda()
    out = []
    for sc in (dev, host):
        h = torch.empty((len(rays), 2), dtype=torch.int32, device="cuda")
        sc.trace_closest(d_rays, len(rays), h)
        occ = torch.empty(len(rays), dtype=torch.uint8, device="cuda")
        sc.trace_any(d_rays, len(rays), occ)
        torch.cuda.synchronize()
        out.append((h.cpu().numpy(), occ.cpu().numpy()))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    if len(soup) <= 4096:
        t, prim = oracle.BBH(soup).trace_canonical(rays, slack=host.info().slack)
        assert np.array_equal(out[0][0][:, 1], prim)
        assert np.array_equal(out[0][0][:, 0].view(np.float32).view(np.uint32), t.view(np.uint32))
    ctx.check()


def test_device_wide_build_renders_like_host_build(native, ctx):
    spec = scenes.many_light(6 * 1280, 40, seed=3, half=6.0)
    cam = scenes.outside_camera(40, 30, distance=20.0, half=6.0)
    outs = []
    for kw in ({"builder": 1, "layout": 8}, {"layout": 8}):
        sc = native.Scene.from_spec(ctx, spec, **kw)
        acc = torch.zeros((40 * 30, 4), dtype=torch.float32, device="cuda")
        sc.render(cam, acc, spp=4, max_depth=12)
        torch.cuda.synchronize()
        outs.append(acc.cpu().numpy())
    assert np.array_equal(outs[0].view(np.uint32), outs[1].view(np.uint32))
    assert outs[0][:, :3].sum() > 0
