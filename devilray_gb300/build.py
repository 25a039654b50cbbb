"""Builds the in-tree CUDA library ``devilray_gb300/lib/libdevilray_gb300.so``.

Every translation unit is compiled for sm_103a only (``-gencode
arch=compute_103a,code=sm_103a``). The units whose results are bit-exact
against the oracle (traversal, shading, tonemap, alias tables, BVH builds) are
compiled with ``-fmad=false``: the FP32 triangle tests and the shading restate
the reference's expression order, so no multiply/add pair may be contracted
into an FMA unless the source writes ``fmaf``. The guiding network's kernels
are checked against their FP64 oracle within a tolerance, not bit for bit, so
they keep the compiler's FMA contraction. Host C++ is compiled with
``-ffp-contract=off`` (the triangle records are precomputed on the host).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB_DIR = PKG / "lib"
LIB = LIB_DIR / "libdevilray_gb300.so"
INCLUDE = ROOT / "include"
CXX_SRC = PKG / "cxx"
CXX_LIB = LIB_DIR / "libdevilray_cxx.so"
CXX_INCLUDE = INCLUDE / "devilray"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Translation units compared with their oracle within a tolerance: FMA contraction allowed.
FMAD_UNITS = {"guiding.cu"}


def _nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = Path(cuda) / "bin" / "nvcc"
    if exe.exists():
        return str(exe)
    found = shutil.which("nvcc")
    if not found:
        raise RuntimeError("nvcc not found (set CUDA_HOME)")
    return found


def _sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers():
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))


def _compile_cmd(src: Path, obj: Path) -> list[str]:
    common = ["-O3", "-std=c++17", "-I", str(INCLUDE), "-I", str(CSRC)]
    host = ["-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fno-fast-math"]
    if src.suffix == ".cu":
        fmad = "-fmad=true" if src.name in FMAD_UNITS else "-fmad=false"
        return [_nvcc(), *ARCH, "-lineinfo", fmad, "--expt-relaxed-constexpr",
                "-Xptxas", "-v" if os.environ.get("DR_PTXAS_VERBOSE") else "-O3",
                *common, *host, "-c", str(src), "-o", str(obj)]
    return [_nvcc(), "-x", "c++", *common, *host, "-c", str(src), "-o", str(obj)]


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    srcs = _sources()
    newest_header = max((h.stat().st_mtime for h in _headers()), default=0.0)
    jobs = []
    objs = []
    for src in srcs:
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        stale = (force or not obj.exists() or obj.stat().st_mtime < src.stat().st_mtime
                 or obj.stat().st_mtime < newest_header or obj.stat().st_mtime < Path(__file__).stat().st_mtime)
        if stale:
            jobs.append((src, obj))

    def run(job):
        src, obj = job
        cmd = _compile_cmd(src, obj)
        out = subprocess.run(cmd, capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError(f"compile failed: {src.name}\n{' '.join(cmd)}\n{out.stdout}\n{out.stderr}")
        if verbose and (out.stdout or out.stderr):
            sys.stderr.write(out.stdout + out.stderr)
        return src.name

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for name in ex.map(run, jobs):
                if verbose:
                    print(f"  compiled {name}", file=sys.stderr)
    if jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-Xcompiler", "-pthread"]
        out = subprocess.run(cmd, capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{out.stdout}\n{out.stderr}")
        os.replace(tmp, LIB)
    build_cxx(force=force or bool(jobs))
    return LIB


def _cxx() -> str:
    return os.environ.get("CXX") or shutil.which("g++") or "g++"


def build_cxx(force: bool = False) -> Path:
    """The C++ interface (Renderer, Scene, GpuTris, DistributionSamplers over
    the C ABI) as ``lib/libdevilray_cxx.so``, linked to the CUDA library."""
    srcs = sorted(CXX_SRC.glob("*.cpp"))
    headers = list(CXX_INCLUDE.rglob("*.hpp")) + list(INCLUDE.glob("*.h"))
    newest = max([p.stat().st_mtime for p in srcs + headers] + [Path(__file__).stat().st_mtime])
    if not force and CXX_LIB.exists() and CXX_LIB.stat().st_mtime >= newest:
        return CXX_LIB
    BUILD.mkdir(exist_ok=True)
    flags = ["-std=c++20", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-I", str(INCLUDE),
             "-I", str(CXX_INCLUDE)]

    def run(src):
        obj = BUILD / ("cxx_" + src.name + ".o")
        cmd = [_cxx(), *flags, "-c", str(src), "-o", str(obj)]
        out = subprocess.run(cmd, capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError(f"compile failed: {src.name}\n{' '.join(cmd)}\n{out.stdout}\n{out.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(run, srcs))
    tmp = CXX_LIB.with_suffix(".so.tmp")
    cmd = [_cxx(), "-shared", "-o", str(tmp), *map(str, objs), "-L", str(LIB_DIR), "-ldevilray_gb300",
           "-Wl,-rpath,$ORIGIN", "-pthread"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{out.stdout}\n{out.stderr}")
    os.replace(tmp, CXX_LIB)
    return CXX_LIB


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build(verbose=True, force=force))
