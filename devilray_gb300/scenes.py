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
