"""OBJ loading of the C++ interface against the reference's own loader.

tests/golden/mesh.npz holds, for the reference's three model files (ico,
cube, suzanne) and for OBJ texts of the grammar's and the errors' cases, what
the reference's loadMesh returns (src/models/Mesh.cpp:117-243) and the mesh
after its normalizeMeshSize and generateCoarseNormals, written by
tests/golden/make_golden.py through the reference harness. The C++ driver's
dump-mesh mode runs devilray_gb300/cxx/Mesh.cpp on the same texts; points,
normals, triangle indices and names must be equal bit for bit, and the same
texts must throw.
"""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

from tests.test_cxx_interface import driver  # noqa: F401  (fixture)


def _read_stage(buf, off):
    np_, nn, nt = np.frombuffer(buf, np.int32, 3, off)
    off += 12
    pts = np.frombuffer(buf, np.float32, 3 * np_, off).reshape(-1, 3)
    off += 12 * np_
    nrm = np.frombuffer(buf, np.float32, 3 * nn, off).reshape(-1, 3)
    off += 12 * nn
    tri = np.frombuffer(buf, np.uint32, 6 * nt, off).reshape(-1, 6)
    off += 24 * nt
    ln = int(np.frombuffer(buf, np.int32, 1, off)[0])
    off += 4
    name = bytes(buf[off:off + ln]).decode()
    return {"points": pts, "normals": nrm, "triangles": tri, "name": name}, off + ln


def _dump(exe, tmp_path, name, text):
    obj = tmp_path / f"{name}.obj"
    obj.write_bytes(text)
    out = tmp_path / f"{name}.bin"
    r = subprocess.run([str(exe), "dump-mesh", str(obj), str(out)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    buf = out.read_bytes()
    ok = int(np.frombuffer(buf, np.int32, 1, 0)[0])
    if not ok:
        return None, None
    loaded, off = _read_stage(buf, 4)
    norm = _read_stage(buf, off)[0] if off < len(buf) else None
    return loaded, norm


def _same(got, g, prefix):
    for k in ("points", "normals"):
        assert np.array_equal(got[k].view(np.uint32), g[f"{prefix}{k}"].view(np.uint32)), f"{prefix}{k}"
    assert np.array_equal(got["triangles"], g[f"{prefix}triangles"]), f"{prefix}triangles"
    assert got["name"] == str(g[f"{prefix}name"]), f"{prefix}name"


def test_obj_loader_matches_reference_loader(driver, golden, tmp_path):  # noqa: F811
    g = golden("mesh.npz")
    names = [str(n) for n in g["names"]]
    assert {"ico", "cube", "suzanne"} <= set(names)
    for name in names:
        loaded, norm = _dump(driver, tmp_path, name, g[f"{name}_obj"].tobytes())
        if not int(g[f"{name}_ok"]):
            assert loaded is None, f"{name}: the reference's loadMesh throws, ours did not"
            continue
        assert loaded is not None, f"{name}: ours throws, the reference's loadMesh does not"
        _same(loaded, g, f"{name}_")
        if f"{name}_norm_points" in g:
            _same(norm, g, f"{name}_norm_")
    assert g["suzanne_triangles"].shape == (967, 6)
