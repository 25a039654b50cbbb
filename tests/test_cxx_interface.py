"""The C++ interface (include/devilray: Renderer, Scene, GpuTris,
DistributionSamplers, Mesh, Image) through its own test driver,
tests/cpp/test_devilray_cxx.cpp, built here with g++ against the in-tree
libraries. CPU cases (OBJ loading, mesh utilities, PNG output) run anywhere;
the renderer and alias-table cases need the GPU."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "test_devilray_cxx.cpp"
BIN = ROOT / "tests" / "cpp" / "bin"
EXE = BIN / "test_devilray_cxx"


@pytest.fixture(scope="module")
def driver(native):
    from devilray_gb300 import build
    build.build_cxx()
    BIN.mkdir(parents=True, exist_ok=True)
    newest = max(p.stat().st_mtime for p in [SRC, build.CXX_LIB, *build.CXX_INCLUDE.rglob("*.hpp")])
    if not EXE.exists() or EXE.stat().st_mtime < newest:
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, "-std=c++20", "-O1", "-I", str(ROOT / "include"), "-I", str(build.CXX_INCLUDE), str(SRC),
               "-o", str(EXE), "-L", str(build.LIB_DIR), "-ldevilray_cxx", "-ldevilray_gb300",
               f"-Wl,-rpath,{build.LIB_DIR}"]
        out = subprocess.run(cmd, capture_output=True, text=True)
        assert out.returncode == 0, out.stderr
    return EXE


def _run(exe, group):
    out = subprocess.run([str(exe), group, str(BIN / "scratch")], capture_output=True, text=True, timeout=600)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
    return out.stdout


def test_cxx_interface_cpu_cases(driver):
    text = _run(driver, "cpu")
    assert "0 failed" in text


@pytest.mark.gpu
def test_cxx_interface_gpu_cases(driver):
    text = _run(driver, "gpu")
    assert "ok   renderer_progressive_equals_one_call" in text and "0 failed" in text
