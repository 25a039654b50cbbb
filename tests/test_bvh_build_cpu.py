"""Host checks of the hierarchy builders (no GPU).

`tests/cpp/bvh_check.cpp` links the library's builder source
(`devilray_gb300/csrc/bvh_build.cpp`) and checks the 8-wide and binary
hierarchies of a soup: the leaf order is a permutation, every node is reached
once, the leaves cover the order once, and every triangle lies inside the
(dequantised) box of every slot or child on its path. The builds are
parallel (binning, subtree construction, the wide collapse and its emission),
so each soup is built with one host thread and with four, and the two
hierarchies must be the same bytes.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from devilray_gb300 import scenes

ROOT = Path(__file__).resolve().parents[1]
CUDA_INCLUDE = Path("/usr/local/cuda/include")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None or not (CUDA_INCLUDE / "cuda_runtime.h").exists():
        pytest.skip("needs g++ and the CUDA headers")
    exe = tmp_path_factory.mktemp("bvh") / "bvh_check"
    subprocess.run([cxx, "-O2", "-std=c++20", "-ffp-contract=off", "-fno-fast-math", "-I", str(ROOT / "include"),
                    "-I", str(ROOT / "devilray_gb300" / "csrc"), "-I", str(CUDA_INCLUDE),
                    str(ROOT / "tests" / "cpp" / "bvh_check.cpp"),
                    str(ROOT / "devilray_gb300" / "csrc" / "bvh_build.cpp"), "-o", str(exe), "-pthread"],
                   check=True, capture_output=True, text=True)
    return exe


def _soups():
    rng = np.random.default_rng(7)
    one = rng.normal(size=(1, 9)).astype(np.float32)
    flat = rng.normal(size=(4000, 9)).astype(np.float32)
    flat[:, 2::3] = 0.0
    signed_zeros = rng.normal(size=(6000, 9)).astype(np.float32)
    signed_zeros[rng.random(signed_zeros.shape) < 0.3] = -0.0
    signed_zeros[rng.random(signed_zeros.shape) < 0.3] = 0.0
    return {
        "one": one,
        "three": rng.normal(size=(3, 9)).astype(np.float32),
        "coincident": np.repeat(one, 3000, axis=0),
        "flat": flat,
        "signed_zeros": signed_zeros,
        "box_room": scenes.box_room().positions,
        # above the sizes that bin on several threads and pass bounds down
        "spheres": scenes.incoherent_soup(300_000, seed=3)[0],
        "far_from_origin": (rng.normal(size=(20000, 9)) * 5.0 + 1.0e4).astype(np.float32),
    }


@pytest.mark.parametrize("name", list(_soups()))
def test_hierarchies_are_valid_and_thread_independent(checker, tmp_path, name):
    soup = np.ascontiguousarray(_soups()[name], np.float32)
    path = tmp_path / f"{name}.f32"
    soup.tofile(path)
    outs = []
    for threads in (1, 4):
        r = subprocess.run([str(checker), str(path), str(threads)], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        outs.append(r.stdout.strip())
    assert outs[0] == outs[1], outs
    assert f"triangles {soup.shape[0]} " in outs[0]
