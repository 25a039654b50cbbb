"""The code examples of INTEGRATION.md compile against the public headers.

Each fenced example (C++ interface, C binding, guided render in C) is wrapped
in a function whose parameters declare the example's free variables, and
compiled with -fsyntax-only, so a renamed entry point, field or argument in
the headers fails here rather than in a reader's build. Elided parts of an
example (`{...}`) become empty initialisers.
"""
from __future__ import annotations

import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CUDA_INCLUDE = Path("/usr/local/cuda/include")

# first line of the example -> (language, declarations of its free variables)
PARAMS = {
    '#include "Renderer.hpp"': (
        "c++",
        "Camera camera, Vec3 center, Vec3 normal, Vec3 right, float size, std::vector<float> weights, DemoRng &rng",
    ),
    '#include "devilray_gb300.h"': (
        "c++",
        "const float *soup, uint32_t num_tris, const dr_object *objects, uint32_t num_objects, "
        "const dr_material *materials, uint32_t num_materials, const dr_ray *d_rays, uint64_t n, dr_hit *d_hits, "
        "const dr_ray *d_shadow_rays, uint8_t *d_occluded, dr_camera camera, dr_render_config cfg, float *d_accum, "
        "uint32_t *d_casts, void *stream",
    ),
    "dr_guide_config gc =": (
        "c",
        "dr_context *ctx, dr_scene *scene, dr_camera camera, uint32_t width, uint32_t height, float *d_accum, "
        "void *stream, float cx, float cy, float cz, float h, dr_guide *guide2",
    ),
}

PRELUDE = {
    "c++": "#include <cstdint>\n#include <span>\n#include <stdexcept>\n#include <vector>\n"
           "struct DemoRng { float rnd() { return 0.5f; } };\n",
    "c": "#include <stdint.h>\n#include <stdlib.h>\n#include \"devilray_gb300.h\"\n",
}


def _examples():
    text = (ROOT / "INTEGRATION.md").read_text()
    return re.findall(r"```(?:c|cpp)\n(.*?)```", text, flags=re.S)


def test_every_example_has_declarations():
    firsts = [ex.strip().splitlines()[0].strip() for ex in _examples()]
    assert len(firsts) == 3
    for f in firsts:
        assert any(f.startswith(k) for k in PARAMS), f


@pytest.mark.parametrize("index", range(3))
def test_example_compiles(index, tmp_path):
    ex = _examples()[index]
    first = ex.strip().splitlines()[0].strip()
    lang, params = next(v for k, v in PARAMS.items() if first.startswith(k))
    compiler = shutil.which("g++" if lang == "c++" else "gcc")
    if compiler is None or not (CUDA_INCLUDE / "cuda_runtime.h").exists():
        pytest.skip("needs gcc/g++")
    lines = ex.replace("{...}", "{}").splitlines()
    includes = [ln for ln in lines if ln.startswith("#include")]
    body = [ln for ln in lines if not ln.startswith("#include")]
    src = PRELUDE[lang] + "\n".join(includes) + f"\nvoid example({params})\n{{\n" + "\n".join(body) + "\n}\n"
    path = tmp_path / ("example.cpp" if lang == "c++" else "example.c")
    path.write_text(src)
    std = ["-std=c++20"] if lang == "c++" else ["-std=c11"]
    r = subprocess.run([compiler, *std, "-fsyntax-only", "-Wno-unused-variable", "-I", str(ROOT / "include"),
                        "-I", str(ROOT / "include" / "devilray"), "-I", str(CUDA_INCLUDE), str(path)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + "\n" + src
