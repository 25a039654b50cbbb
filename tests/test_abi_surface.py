"""The C-ABI library loads and exports every symbol the public headers declare
(no compute calls: these run without a GPU)."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    syms = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(dr_\w+)\s*\(", text, flags=re.M):
            syms.add(m.group(1))
    return syms


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("dr_context_create", "dr_scene_create", "dr_trace_closest", "dr_trace_any",
              "dr_trace_closest_host", "dr_last_error_string"):
        assert s in syms


def test_library_exports_every_declared_symbol(native):
    lib = ctypes.CDLL(str(native.LIB_PATH))
    missing = [s for s in sorted(declared_symbols()) if not hasattr(lib, s)]
    assert not missing, f"declared but not exported: {missing}"


def test_binding_covers_every_declared_symbol(native):
    assert declared_symbols() <= set(native.SIGNATURES)


def test_abi_version_and_no_device_error(native):
    lib = native.load()
    header = (ROOT / "include" / "devilray_gb300.h").read_text()
    version = int(re.search(r"#define DR_ABI_VERSION (\d+)", header).group(1))
    assert lib.dr_abi_version() == version
    # Without a GPU the context call fails with a status, never exits.
    import torch
    if not torch.cuda.is_available():
        h = ctypes.c_void_p()
        st = lib.dr_context_create(None, ctypes.byref(h))
        assert st == 4  # DR_ERR_NO_DEVICE
        assert b"no CUDA device" in lib.dr_last_error_string()


def test_scene_records_match_the_struct_layouts(native):
    """The numpy object and material records handed to dr_scene_create hold
    the same bytes as dr_object / dr_material structs filled field by field,
    so the vectorised descriptors change nothing the library reads."""
    import numpy as np
    from devilray_gb300 import scenes
    spec = scenes.box_room()
    spec.add_object(scenes.quad((0, 1, 0), (0, -1, 0), (1, 0, 0), 0.5),
                    spec.add_material(scenes.material(kind=0, emission=(3.5, 2.25, 1.0), albedo=(0.1, 0.2, 0.3))),
                    area=0.1234567)
    objs = [native.Object(int(b), int(c), int(m), float(a)) for (b, c, m, a) in spec.objects]
    mats = []
    for m in spec.materials:
        mm = native.Material()
        mm.kind, mm.ior = m["kind"], m["ior"]
        for i in range(4):
            mm.emission[i], mm.albedo[i], mm.debug_color[i] = m["emission"][i], m["albedo"][i], m["debug"][i]
        mats.append(mm)
    d1, keep1 = native.scene_desc(spec.positions, objs, mats)
    d2, keep2 = native.scene_desc(spec.positions, *native.spec_parts(spec))
    assert d1.num_objects == d2.num_objects == len(spec.objects)
    assert d1.num_materials == d2.num_materials == len(spec.materials)
    for ptr, n, size in (("objects_host", d1.num_objects, 16), ("materials_host", d1.num_materials, 64)):
        a = ctypes.string_at(getattr(d1, ptr), n * size)
        b = ctypes.string_at(getattr(d2, ptr), n * size)
        assert a == b, ptr
    with np.testing.assert_raises(ValueError):
        native.scene_desc(spec.positions, np.zeros((2, 3), np.float32))
    assert not spec.positions.flags.writeable and spec.positions is spec.positions
