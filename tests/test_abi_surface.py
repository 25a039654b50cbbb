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
