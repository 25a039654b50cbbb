"""Seeded synthetic workloads (triangle soups and ray sets).

The reference's benchmark casts rays at a loaded mesh (bunny.obj, absent from
the reference tree); these generators stand in for it with procedural geometry
of the stated shapes and sizes:

* ``incoherent_soup``: icospheres of subdivision level 3 (1,280 triangles
  each) with centres uniform in [-50, 50]^3 and radii log-uniform in
  [0.5, 3], truncated to exactly ``num_triangles`` (2^20 = 819 spheres plus
  256 triangles of an 820th).
* ``incoherent_rays``: origins uniform in the same cube, directions uniform on
  the sphere in the form of uniformSphereSample (DevilRay
  include/tracing/DistributionSamplers.hpp:8-20).
"""
from __future__ import annotations

import numpy as np

CUBE_HALF = 50.0


def icosphere(level: int = 3) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: (vertices [V,3] float64, faces [F,3] int32), F = 20 * 4^level."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
             (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
             (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
             (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
             (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = [np.array(p, np.float64) / np.linalg.norm(p) for p in verts]
    f = list(faces)
    for _ in range(level):
        cache: dict[tuple[int, int], int] = {}

        def mid(a: int, b: int) -> int:
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = (v[a] + v[b]) / 2.0
                v.append(m / np.linalg.norm(m))
                cache[key] = len(v) - 1
            return cache[key]

        nf = []
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    return np.array(v), np.array(f, np.int32)


def icosphere_soup(level: int = 3) -> np.ndarray:
    """Unit icosphere as a soup [F, 9] (float64)."""
    v, f = icosphere(level)
    return v[f].reshape(-1, 9)


def density_half(num_triangles: int) -> float:
    """Cube half-size that keeps the 2^20-triangle sphere density for a
    smaller soup (used by the tests' reduced workloads)."""
    return CUBE_HALF * (num_triangles / float(1 << 20)) ** (1.0 / 3.0)


def incoherent_soup(num_triangles: int = 1 << 20, seed: int = 0, level: int = 3, half: float = CUBE_HALF):
    """Soup [num_triangles, 9] float32 plus (centres, radii) of the spheres."""
    unit = icosphere_soup(level)
    per = unit.shape[0]
    nsph = (num_triangles + per - 1) // per
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-half, half, size=(nsph, 3))
    radii = np.exp(rng.uniform(np.log(0.5), np.log(3.0), size=nsph))
    soup = (centres[:, None, :] + radii[:, None, None] * unit.reshape(1, per * 3, 3)).reshape(nsph * per, 9)
    return soup[:num_triangles].astype(np.float32), centres, radii


def sphere_directions(u0: np.ndarray, u1: np.ndarray) -> np.ndarray:
    """uniformSphereSample's mapping of two uniforms (float64 math)."""
    theta0 = 2.0 * np.pi * u0
    theta1 = np.arccos(1.0 - 2.0 * u1)
    return np.stack([np.sin(theta1) * np.sin(theta0), np.sin(theta1) * np.cos(theta0), np.cos(theta1)], axis=-1)


def incoherent_rays(n: int, seed: int = 0, tmax: float = np.inf, chunk: int = 1 << 22,
                    half: float = CUBE_HALF) -> np.ndarray:
    """Rays [n, 8] float32 (dr_ray layout): origins uniform in the cube,
    directions uniform on the sphere."""
    rng = np.random.default_rng(seed + 0x5EED)
    out = np.empty((n, 8), np.float32)
    for b in range(0, n, chunk):
        m = min(chunk, n - b)
        o = rng.uniform(-half, half, size=(m, 3))
        u = rng.random((m, 2))
        d = sphere_directions(u[:, 0], u[:, 1])
        out[b:b + m, 0:3] = o
        out[b:b + m, 3] = tmax
        out[b:b + m, 4:7] = d
        out[b:b + m, 7] = 0.0
    return out


def rays6(rays8: np.ndarray) -> np.ndarray:
    """dr_ray [n, 8] -> reference Ray {p, v} [n, 6]."""
    return np.ascontiguousarray(np.concatenate([rays8[:, 0:3], rays8[:, 4:7]], axis=1), np.float32)


# ---- scenes with materials (flattened: objects are contiguous triangle ranges) ----

def _f32(x):
    return np.asarray(x, np.float32)


def _cross32(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
                     a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], axis=-1).astype(np.float32)


def tri_area_f32(soup: np.ndarray) -> np.ndarray:
    """triangleArea (include/Utils.hpp:218-224) in FP32, one rounding per op."""
    s = _f32(soup).reshape(-1, 3, 3)
    A, B, C = s[:, 0], s[:, 1], s[:, 2]
    c = _cross32((A - B).astype(np.float32), (A - C).astype(np.float32))
    l2 = ((c[:, 0] * c[:, 0]).astype(np.float32) + (c[:, 1] * c[:, 1]).astype(np.float32)).astype(np.float32)
    l2 = (l2 + (c[:, 2] * c[:, 2]).astype(np.float32)).astype(np.float32)
    return (np.sqrt(l2).astype(np.float32) / np.float32(2)).astype(np.float32)


def surface_area(soup: np.ndarray) -> float:
    """totalSurfaceArea (src/GpuTris.cpp:40-58): FP32 triangle areas summed in
    order in double, then rounded to FP32."""
    a = tri_area_f32(soup).astype(np.float64)
    return float(np.float32(np.cumsum(a)[-1] if a.size else 0.0))


def quad(center, normal, right, size) -> np.ndarray:
    """createQuadMesh (src/GpuTris.cpp:87-107) in FP32: two triangles (0,2,1), (0,3,2)."""
    c, n, r = _f32(center), _f32(normal), _f32(right)
    up = _cross32(r, n)
    h = np.float32(size) / np.float32(2)
    pts = [((c + r * -h).astype(np.float32) + up * -h).astype(np.float32),
           ((c + r * h).astype(np.float32) + up * -h).astype(np.float32),
           ((c + r * h).astype(np.float32) + up * h).astype(np.float32),
           ((c + r * -h).astype(np.float32) + up * h).astype(np.float32)]
    return np.array([np.concatenate([pts[0], pts[2], pts[1]]), np.concatenate([pts[0], pts[3], pts[2]])], np.float32)


def rect_y(x0: float, x1: float, z0: float, z1: float, y: float) -> np.ndarray:
    """Two triangles covering [x0, x1] x [z0, z1] at height y."""
    a, b, c, d = (x0, y, z0), (x1, y, z0), (x1, y, z1), (x0, y, z1)
    return np.array([a + c + b, a + d + c], np.float32)


def material(kind=0, emission=(0, 0, 0), albedo=(0, 0, 0), ior=1.0, debug=(0.5, 0.5, 0.5)):
    return {"kind": int(kind), "ior": float(ior), "emission": tuple(emission) + (0.0,) * (4 - len(emission)),
            "albedo": tuple(albedo) + (0.0,) * (4 - len(albedo)), "debug": tuple(debug) + (0.0,) * (4 - len(debug))}


class SceneSpec:
    """A flattened scene: soup [N, 9] float32, objects (tri_begin, tri_count,
    material, surface_area) and materials."""

    def __init__(self):
        self.parts: list[np.ndarray] = []
        self.objects: list[tuple[int, int, int, float]] = []
        self.materials: list[dict] = []
        self.count = 0
        self._soup: np.ndarray | None = None  # the joined parts, read-only, until the next add_object

    def add_material(self, m: dict) -> int:
        self.materials.append(m)
        return len(self.materials) - 1

    def add_object(self, soup: np.ndarray, mat: int, area: float | None = None) -> int:
        soup = _f32(soup).reshape(-1, 9)
        self.parts.append(soup)
        self._soup = None
        self.objects.append((self.count, soup.shape[0], mat, surface_area(soup) if area is None else area))
        self.count += soup.shape[0]
        return len(self.objects) - 1

    @property
    def positions(self) -> np.ndarray:
        """The soup [N, 9] float32, joined once and shared by later reads (read-only)."""
        if self._soup is None:
            soup = np.concatenate(self.parts) if self.parts else np.zeros((0, 9), np.float32)
            soup = soup.astype(np.float32, copy=False)
            soup.flags.writeable = False
            self._soup = soup
        return self._soup

    def materials_array(self) -> np.ndarray:
        """dr_material layout: [kind, ior, 0, 0, emission4, albedo4, debug4] as float32
        (kind stored as its int32 bit pattern)."""
        ms = self.materials
        out = np.zeros((len(ms), 16), np.float32)
        if ms:
            out[:, 0] = np.array([m["kind"] for m in ms], np.int32).view(np.float32)
            out[:, 1] = [m["ior"] for m in ms]
            out[:, 4:8] = [m["emission"] for m in ms]
            out[:, 8:12] = [m["albedo"] for m in ms]
            out[:, 12:16] = [m["debug"] for m in ms]
        return out

    def objects_array(self) -> np.ndarray:
        dt = np.dtype([("tri_begin", "<u4"), ("tri_count", "<u4"), ("material", "<i4"), ("surface_area", "<f4")])
        return np.array(self.objects, dt)


def camera(width: int, height: int, focal: float = 1.0, fov_half_width: float = 0.375, transform=None) -> dict:
    """Pinhole camera (include/tracing/Camera.hpp) with the principal point at
    the image centre; `fov_half_width` = half the sensor width / focal length."""
    ps = np.float32(2.0 * fov_half_width * focal / width)
    m = np.eye(4, dtype=np.float32) if transform is None else _f32(transform)
    return {"m": m.reshape(16), "focal": np.float32(focal), "cx": np.float32(width / 2.0) * ps,
            "cy": np.float32(height / 2.0) * ps, "width": int(width), "height": int(height), "psx": ps, "psy": ps}


def box_room(sphere_level: int = 3, glass_sphere: bool = True) -> SceneSpec:
    """The box room of the plain-method configuration: five axis-aligned
    quads (albedo 0.75, red/green side walls 0.6), a ceiling light quad
    (radiance 15) and a dielectric icosphere (IOR 1.5) in the middle; laid out
    like the reference's interactive scene (renderer/src/SceneSetup.cpp:120-131).
    With glass_sphere=False the sphere is diffuse (albedo 0.75)."""
    s = SceneSpec()
    white = s.add_material(material(0, albedo=(0.75, 0.75, 0.75)))
    red = s.add_material(material(0, albedo=(0.6, 0.1, 0.1)))
    green = s.add_material(material(0, albedo=(0.1, 0.6, 0.1)))
    light = s.add_material(material(0, emission=(15.0, 15.0, 15.0)))
    glass = s.add_material(material(1, ior=1.5)) if glass_sphere else white
    s.add_object(quad((0, 0, 2.5), (0, 0, -1), (1, 0, 0), 1.0), white)
    s.add_object(quad((0.5, 0, 2), (-1, 0, 0), (0, 1, 0), 1.0), red)
    s.add_object(quad((-0.5, 0, 2), (1, 0, 0), (0, 1, 0), 1.0), green)
    s.add_object(quad((0, 0.5, 2), (0, -1, 0), (0, 0, 1), 1.0), white)
    s.add_object(quad((0, -0.5, 2), (0, 1, 0), (0, 0, 1), 1.0), white)
    s.add_object(quad((0, 0.4999, 2), (0, -1, 0), (0, 0, 1), 0.4), light)
    sph = (np.array([0.0, -0.2, 2.0]) + 0.25 * icosphere_soup(sphere_level).reshape(-1, 3, 3)).reshape(-1, 9)
    s.add_object(sph.astype(np.float32), glass)
    return s


def many_light(num_triangles: int = 1 << 20, num_emitters: int = 65536, seed: int = 0,
               half: float = CUBE_HALF) -> SceneSpec:
    """The many-light configuration: the incoherent soup's spheres; a seeded
    choice of `num_emitters` triangles emit grey radiance exp(N(0, 1.5^2)); of
    the remaining spheres half are diffuse (albedo uniform in [0.2, 0.8]) and
    half dielectric (IOR uniform in [1.3, 1.7]). Materials are per object as in
    the reference's data model: each sphere's non-emitting triangles form one
    object, each emitting triangle is an object of its own."""
    soup, centres, radii = incoherent_soup(num_triangles, seed=seed, half=half)
    per = 1280
    rng = np.random.default_rng(seed + 17)
    n = soup.shape[0]
    num_emitters = min(num_emitters, n)
    emit_idx = rng.permutation(n)[:num_emitters]
    emissive = np.zeros(n, bool)
    emissive[emit_idx] = True
    radiance = np.exp(rng.normal(0.0, 1.5, n)).astype(np.float32)
    nsph = (n + per - 1) // per
    kind = rng.random(nsph) < 0.5
    albedo = rng.uniform(0.2, 0.8, nsph)
    ior = rng.uniform(1.3, 1.7, nsph)
    s = SceneSpec()
    for k in range(nsph):
        tris = np.arange(k * per, min(n, (k + 1) * per))
        body = tris[~emissive[tris]]
        if body.size:
            m = s.add_material(material(0, albedo=(albedo[k],) * 3) if kind[k] else material(1, ior=ior[k]))
            s.add_object(soup[body], m)
        for t in tris[emissive[tris]]:
            L = float(radiance[t])
            m = s.add_material(material(0, emission=(L, L, L)))
            s.add_object(soup[t:t + 1], m)
    return s


def occluded_light(num_triangles: int = 1 << 20, num_emitters: int = 65536, seed: int = 0,
                   half: float = CUBE_HALF, light_y: float = 0.4, slab_y: float = 0.3,
                   slab_extent: float = 0.7, enclose="box", room_albedo: float = 0.4,
                   dielectric_fraction: float = 0.5, slab_gap: float | None = None) -> SceneSpec:
    """The guided configuration: the many-light scene with its emitters only on
    spheres whose centre lies above `light_y` * half, and a diffuse occluding
    slab (albedo 0.8, two triangles) at height `slab_y` * half covering
    `slab_extent` of the cube's width in x and z, so light reaches the
    spheres below mostly through the gaps at the slab's edges, off a floor
    and walls (`enclose`, albedo `room_albedo`): indirect light dominates the
    camera's view of the lower region."""
    soup, centres, radii = incoherent_soup(num_triangles, seed=seed, half=half)
    per = 1280
    rng = np.random.default_rng(seed + 17)
    n = soup.shape[0]
    nsph = (n + per - 1) // per
    upper = np.flatnonzero(centres[:nsph, 1] > light_y * half)
    candidates = np.concatenate([np.arange(k * per, min(n, (k + 1) * per)) for k in upper]) if upper.size else \
        np.arange(0)
    num_emitters = min(num_emitters, candidates.size)
    emissive = np.zeros(n, bool)
    emissive[rng.permutation(candidates)[:num_emitters]] = True
    radiance = np.exp(rng.normal(0.0, 1.5, n)).astype(np.float32)
    kind = rng.random(nsph) < 1.0 - dielectric_fraction
    albedo = rng.uniform(0.2, 0.8, nsph)
    ior = rng.uniform(1.3, 1.7, nsph)
    s = SceneSpec()
    for k in range(nsph):
        tris = np.arange(k * per, min(n, (k + 1) * per))
        body = tris[~emissive[tris]]
        if body.size:
            m = s.add_material(material(0, albedo=(albedo[k],) * 3) if kind[k] else material(1, ior=ior[k]))
            s.add_object(soup[body], m)
        for t in tris[emissive[tris]]:
            L = float(radiance[t])
            m = s.add_material(material(0, emission=(L, L, L)))
            s.add_object(soup[t:t + 1], m)
    w = 1.15 * half
    if slab_gap is None:
        e = slab_extent * half
        slab = quad((0.0, slab_y * half, 0.0), (0.0, -1.0, 0.0), (1.0, 0.0, 0.0), 2 * e)
    else:
        # the whole width of the room but a gap of slab_gap * half along the -x wall
        slab = rect_y(-w + slab_gap * half, w, -w, w, slab_y * half)
    grey = s.add_material(material(0, albedo=(room_albedo,) * 3))
    s.add_object(slab, grey)
    if enclose:
        # a floor, a back wall and side walls (open towards the camera) catch the
        # light that passes the slab's edges and scatter it under the slab
        s.add_object(quad((0.0, -w, 0.0), (0.0, 1.0, 0.0), (1.0, 0.0, 0.0), 2 * w), grey)
        s.add_object(quad((0.0, 0.0, w), (0.0, 0.0, -1.0), (1.0, 0.0, 0.0), 2 * w), grey)
        if enclose == "box":
            s.add_object(quad((-w, 0.0, 0.0), (1.0, 0.0, 0.0), (0.0, 0.0, 1.0), 2 * w), grey)
            s.add_object(quad((w, 0.0, 0.0), (-1.0, 0.0, 0.0), (0.0, 0.0, 1.0), 2 * w), grey)
            s.add_object(quad((0.0, w, 0.0), (0.0, -1.0, 0.0), (1.0, 0.0, 0.0), 2 * w), grey)
    return s


def lower_camera(width: int, height: int, distance: float = 150.0, half: float = CUBE_HALF,
                 look_y: float = -0.3) -> dict:
    """Camera on the -z axis outside the cube, aimed at height look_y * half so
    the region below the slab of occluded_light fills the view."""
    m = np.eye(4, dtype=np.float32)
    m[1, 3] = look_y * half
    m[2, 3] = -distance
    return camera(width, height, focal=1.0, fov_half_width=0.62 * half / distance * 1.6, transform=m)


def outside_camera(width: int, height: int, distance: float = 150.0, half: float = CUBE_HALF) -> dict:
    """Camera on the -z axis outside the cube, looking at its centre."""
    m = np.eye(4, dtype=np.float32)
    m[2, 3] = -distance
    return camera(width, height, focal=1.0, fov_half_width=0.62 * half / distance * 1.6, transform=m)


def uneven_batch(n: int = 64, seed: int = 2024) -> list:
    """The batched configuration: `n` procedural scenes with triangle counts
    log-uniform in [1k, 2M] and square resolutions from {128, 256, 512, 1024};
    the many-light material mix (1/64 of the triangles emissive, at least 16;
    the rest half diffuse, half dielectric); each seen by a camera outside its
    cube. Returns [(SceneSpec, camera)]."""
    rng = np.random.default_rng(seed)
    tris = np.exp(rng.uniform(np.log(1e3), np.log(2e6), n)).astype(np.int64)
    res = rng.choice([128, 256, 512, 1024], n)
    out = []
    for i in range(n):
        spec = many_light(int(tris[i]), max(16, int(tris[i]) // 64), seed=seed + i)
        out.append((spec, outside_camera(int(res[i]), int(res[i]))))
    return out
