"""ctypes bindings of the CPU oracle and of the reference harness.

TEST INFRASTRUCTURE. Only the tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module; the product package never
does. ``liboracle.so`` is the CPU restatement of DevilRay's tracing path;
``libref_harness.so`` (built only where the DevilRay sources exist) calls the
reference's own host code and pins the restatement.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "lib" / "liboracle.so"
REF_SO = HERE / "_ref" / "libref_harness.so"
# The DevilRay source tree: DEVILRAY_REF_ROOT when set, else the location
# oracle/Makefile names (the recipe that reads the sources there).
REF_ROOT_ENV = os.environ.get("DEVILRAY_REF_ROOT")

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")

ALIAS_DTYPE = np.dtype([("p_A", "<f4"), ("pdf_A", "<f4"), ("pdf_B", "<f4"), ("A", "<i4"), ("B", "<i4")])


def build(ref: bool | None = None, quiet: bool = True) -> None:
    """Compiles liboracle.so (and the reference harness when the sources exist)."""
    targets = ["all"]
    root = [f"REF_ROOT={REF_ROOT_ENV}"] if REF_ROOT_ENV else []
    if ref is None:
        probe = subprocess.run(["make", "-s", "-C", str(HERE), *root, "ref-present"], capture_output=True, text=True)
        ref = probe.returncode == 0 and probe.stdout.strip() == "yes"
    if ref:
        targets.append("ref")
    out = subprocess.run(["make", "-C", str(HERE), *root, "-j4", *targets], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{out.stdout}\n{out.stderr}")


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not ORACLE_SO.exists():
            build(ref=False)
        L = C.CDLL(str(ORACLE_SO))
        L.or_tri_test_ref.argtypes = [_f32p, _f32p, _f32p]
        L.or_tri_test_watertight.argtypes = [_f32p, _f32p, _f32p]
        L.or_box_test_ref.argtypes = [_f32p, _f32p, _f32p]
        L.or_bbh_create.argtypes = [_f32p, C.c_int32]
        L.or_bbh_create.restype = C.c_void_p
        L.or_bbh_destroy.argtypes = [C.c_void_p]
        L.or_bbh_num_nodes.argtypes = [C.c_void_p]
        L.or_bbh_depth.argtypes = [C.c_void_p]
        L.or_bbh_export.argtypes = [C.c_void_p, _f32p, _i32p, _i32p]
        L.or_bbh_trace_reference.argtypes = [C.c_void_p, _f32p, C.c_int64, _f32p, _i32p, _i64p, _i64p,
                                             C.c_int32, C.c_int32]
        L.or_bbh_trace_canonical.argtypes = [C.c_void_p, _f32p, C.c_int64, C.c_float, _f32p, _i32p,
                                             C.c_int32, C.c_int32]
        L.or_bbh_trace_any.argtypes = [C.c_void_p, _f32p, C.c_int64, C.c_float, _u8p, C.c_int32, C.c_int32]
        L.or_trace_brute.argtypes = [_f32p, C.c_int32, _f32p, C.c_int64, _f32p, _i32p, C.c_int32, C.c_int32]
        L.or_alias_build_ref.argtypes = [_f32p, C.c_int32, C.c_void_p]
        L.or_alias_build_sweep.argtypes = [_f32p, C.c_int32, C.c_void_p]
        L.or_alias_sample.argtypes = [C.c_void_p, C.c_int32, C.c_float, C.c_float,
                                      C.POINTER(C.c_int32), C.POINTER(C.c_float)]
        L.or_lognormal_input.argtypes = [C.c_int32, C.c_uint32, _f32p]
        L.or_philox4x32_10.argtypes = [_u32p, _u32p, _u32p]
        L.or_create_pixels.argtypes = [_f32p, C.c_int32, C.c_int32, C.c_int32, _u32p]
        _lib = L
    return _lib


def create_pixels(accum, width: int, height: int, gamma: bool = True) -> np.ndarray:
    """Renderer::createPixels restated: RGBA8 pixels, rows top first."""
    a = _f32(accum).reshape(-1)
    assert a.size == 4 * width * height
    out = np.zeros(width * height, np.uint32)
    lib().or_create_pixels(a, width, height, 1 if gamma else 0, out)
    return out


def ref_available() -> bool:
    return REF_SO.exists()


def ref():
    """The harness over the reference's own code (only where it was built)."""
    global _ref
    if _ref is None:
        if not REF_SO.exists():
            raise FileNotFoundError("reference harness not built (needs the DevilRay sources)")
        L = C.CDLL(str(REF_SO))
        L.refh_tri_test.argtypes = [_f32p, _f32p, _f32p]
        L.refh_box_test.argtypes = [_f32p, _f32p, _f32p]
        L.refh_bbh_create.argtypes = [_f32p, C.c_int]
        L.refh_bbh_create.restype = C.c_void_p
        L.refh_bbh_destroy.argtypes = [C.c_void_p]
        L.refh_bbh_num_nodes.argtypes = [C.c_void_p]
        L.refh_bbh_depth.argtypes = [C.c_void_p]
        L.refh_bbh_export.argtypes = [C.c_void_p, _f32p, _i32p, _i32p]
        L.refh_bbh_trace.argtypes = [C.c_void_p, _f32p, C.c_int, _f32p, _i32p, C.c_void_p, C.c_void_p,
                                     _i64p, _i64p]
        L.refh_alias_build.argtypes = [_f32p, C.c_int, _f32p, _f32p, _f32p, _i32p, _i32p]
        L.refh_alias_sample.argtypes = [_f32p, _f32p, _f32p, _i32p, _i32p, C.c_int, _f32p, C.c_int, _i32p, _f32p]
        L.refh_lognormal.argtypes = [C.c_int, C.c_uint, _f32p]
        L.refh_sphere_sample.argtypes = [_f32p, C.c_int, _f32p]
        L.refh_cosine_sample.argtypes = [_f32p, _f32p, C.c_int, _f32p]
        L.refh_camera_ray.argtypes = [_f32p, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                      C.c_float, C.c_float, C.c_int, _f32p, _f32p]
        _ref = L
    return _ref


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


# ---- oracle wrappers ---------------------------------------------------------

def tri_test(ray6, tri9, mode: int = 0):
    out = np.zeros(4, np.float32)
    fn = lib().or_tri_test_watertight if mode == 1 else lib().or_tri_test_ref
    hit = fn(_f32(ray6), _f32(tri9), out)
    return (bool(hit), out)


def box_test(box6, ray6):
    out = np.zeros(1, np.float32)
    hit = lib().or_box_test_ref(_f32(box6), _f32(ray6), out)
    return bool(hit), float(out[0])


class BBH:
    """The reference's median-split BBH (src/models/BBH.cpp) over a soup."""

    def __init__(self, positions: np.ndarray):
        self.positions = _f32(positions).reshape(-1, 9)
        self.ntri = self.positions.shape[0]
        self.h = lib().or_bbh_create(self.positions.reshape(-1), self.ntri)

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_bbh_destroy(self.h)
            self.h = None

    @property
    def num_nodes(self) -> int:
        return lib().or_bbh_num_nodes(self.h)

    @property
    def depth(self) -> int:
        return lib().or_bbh_depth(self.h)

    def export(self):
        n = self.num_nodes
        boxes = np.zeros((n, 6), np.float32)
        links = np.zeros((n, 5), np.int32)
        order = np.zeros(self.ntri, np.int32)
        lib().or_bbh_export(self.h, boxes.reshape(-1), links.reshape(-1), order)
        return boxes, links, order

    def trace_reference(self, rays6: np.ndarray, tri_mode: int = 0, threads: int = 0):
        rays6 = _f32(rays6).reshape(-1, 6)
        n = rays6.shape[0]
        t = np.zeros(n, np.float32)
        prim = np.zeros(n, np.int32)
        nb = np.zeros(n, np.int64)
        nt = np.zeros(n, np.int64)
        lib().or_bbh_trace_reference(self.h, rays6.reshape(-1), n, t, prim, nb, nt, tri_mode, threads)
        return t, prim, nb, nt

    def trace_canonical(self, rays8: np.ndarray, slack: float, tri_mode: int = 0, threads: int = 0):
        rays8 = _f32(rays8).reshape(-1, 8)
        n = rays8.shape[0]
        t = np.zeros(n, np.float32)
        prim = np.zeros(n, np.int32)
        lib().or_bbh_trace_canonical(self.h, rays8.reshape(-1), n, slack, t, prim, tri_mode, threads)
        return t, prim

    def trace_any(self, rays8: np.ndarray, slack: float, tri_mode: int = 0, threads: int = 0):
        rays8 = _f32(rays8).reshape(-1, 8)
        n = rays8.shape[0]
        occ = np.zeros(n, np.uint8)
        lib().or_bbh_trace_any(self.h, rays8.reshape(-1), n, slack, occ, tri_mode, threads)
        return occ


def trace_brute(positions, rays8, tri_mode: int = 0, threads: int = 0):
    positions = _f32(positions).reshape(-1)
    rays8 = _f32(rays8).reshape(-1, 8)
    n = rays8.shape[0]
    t = np.zeros(n, np.float32)
    prim = np.zeros(n, np.int32)
    lib().or_trace_brute(positions, positions.size // 9, rays8.reshape(-1), n, t, prim, tri_mode, threads)
    return t, prim


def alias_build_ref(weights) -> np.ndarray:
    w = _f32(weights)
    out = np.zeros(w.size, ALIAS_DTYPE)
    lib().or_alias_build_ref(w, w.size, out.ctypes.data)
    return out


def alias_build_sweep(weights) -> np.ndarray:
    w = _f32(weights)
    out = np.zeros(w.size, ALIAS_DTYPE)
    lib().or_alias_build_sweep(w, w.size, out.ctypes.data)
    return out


def alias_sample(table: np.ndarray, u0: float, u1: float):
    idx = C.c_int32()
    pdf = C.c_float()
    lib().or_alias_sample(table.ctypes.data, table.size, u0, u1, C.byref(idx), C.byref(pdf))
    return idx.value, pdf.value


def lognormal_input(n: int, seed: int = 42) -> np.ndarray:
    out = np.zeros(n, np.float32)
    lib().or_lognormal_input(n, seed, out)
    return out


def philox(ctr, key) -> np.ndarray:
    out = np.zeros(4, np.uint32)
    lib().or_philox4x32_10(np.ascontiguousarray(ctr, np.uint32), np.ascontiguousarray(key, np.uint32), out)
    return out


# ---- reference harness wrappers ------------------------------------------------

def ref_tri_test(ray6, tri9):
    out = np.zeros(4, np.float32)
    hit = ref().refh_tri_test(_f32(ray6), _f32(tri9), out)
    return bool(hit), out


def ref_box_test(box6, ray6):
    out = np.zeros(1, np.float32)
    hit = ref().refh_box_test(_f32(box6), _f32(ray6), out)
    return bool(hit), float(out[0])


def ref_bbh_trace(positions, rays6):
    positions = _f32(positions).reshape(-1)
    ntri = positions.size // 9
    h = ref().refh_bbh_create(positions, ntri)
    try:
        rays6 = _f32(rays6).reshape(-1, 6)
        n = rays6.shape[0]
        t = np.zeros(n, np.float32)
        prim = np.zeros(n, np.int32)
        nrm = np.zeros((n, 3), np.float32)
        area = np.zeros(n, np.float32)
        nb = np.zeros(n, np.int64)
        nt = np.zeros(n, np.int64)
        ref().refh_bbh_trace(h, rays6.reshape(-1), n, t, prim, nrm.ctypes.data, area.ctypes.data, nb, nt)
        nn = ref().refh_bbh_num_nodes(h)
        boxes = np.zeros((nn, 6), np.float32)
        links = np.zeros((nn, 5), np.int32)
        order = np.zeros(ntri, np.int32)
        ref().refh_bbh_export(h, boxes.reshape(-1), links.reshape(-1), order)
        depth = ref().refh_bbh_depth(h)
    finally:
        ref().refh_bbh_destroy(h)
    return dict(t=t, prim=prim, normal=nrm, area=area, box_tests=nb, tri_tests=nt,
                boxes=boxes, links=links, order=order, depth=depth)


def ref_alias_build(weights) -> np.ndarray:
    w = _f32(weights)
    n = w.size
    pA, pdfA, pdfB = (np.zeros(n, np.float32) for _ in range(3))
    A, B = np.zeros(n, np.int32), np.zeros(n, np.int32)
    ref().refh_alias_build(w, n, pA, pdfA, pdfB, A, B)
    out = np.zeros(n, ALIAS_DTYPE)
    out["p_A"], out["pdf_A"], out["pdf_B"], out["A"], out["B"] = pA, pdfA, pdfB, A, B
    return out


def ref_mesh_load(path: str, normalize: bool = False):
    """The reference's loadMesh (then normalizeMeshSize and
    generateCoarseNormals when `normalize`): dict of points [n, 3], normals
    [m, 3], triangles [k, 6] (a.pi, a.ni, b.pi, b.ni, c.pi, c.ni) and name, or
    None when it throws."""
    L = ref()
    if not getattr(L, "_mesh_bound", False):
        L.refh_mesh_load.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
        L.refh_mesh_load.restype = C.c_void_p
        L.refh_mesh_free.argtypes = [C.c_void_p]
        L.refh_mesh_sizes.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.refh_mesh_export.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_int]
        L.refh_mesh_normalize_and_coarse_normals.argtypes = [C.c_void_p]
        L._mesh_bound = True
    err = C.create_string_buffer(512)
    h = L.refh_mesh_load(path.encode(), err, 512)
    if not h:
        return None
    try:
        if normalize:
            L.refh_mesh_normalize_and_coarse_normals(h)
        np_, nn, nt = C.c_int(), C.c_int(), C.c_int()
        L.refh_mesh_sizes(h, C.byref(np_), C.byref(nn), C.byref(nt))
        pts = np.zeros((np_.value, 3), np.float32)
        nrm = np.zeros((nn.value, 3), np.float32)
        tri = np.zeros((nt.value, 6), np.uint32)
        name = C.create_string_buffer(256)
        L.refh_mesh_export(h, pts.ctypes.data, nrm.ctypes.data, tri.ctypes.data, name, 256)
    finally:
        L.refh_mesh_free(h)
    return {"points": pts, "normals": nrm, "triangles": tri, "name": np.array(name.value.decode())}


def ref_lognormal(n: int, seed: int = 42) -> np.ndarray:
    out = np.zeros(n, np.float32)
    ref().refh_lognormal(n, seed, out)
    return out


# ---- integrator ------------------------------------------------------------------

class RenderCfg(C.Structure):
    _fields_ = [("max_depth", C.c_int32), ("spp", C.c_int32), ("sample_offset", C.c_int32),
                ("pixel_sampling", C.c_int32), ("seed", C.c_uint64), ("rng_mode", C.c_int32),
                ("trig_mode", C.c_int32), ("cast_mode", C.c_int32), ("tri_table_order", C.c_int32),
                ("threads", C.c_int32), ("replay_stride", C.c_int32), ("replay", C.c_void_p),
                ("debug", C.c_int32), ("pixels", C.c_void_p), ("num_pixels", C.c_int64)]


class Camera(C.Structure):
    _fields_ = [("m", C.c_float * 16), ("focal", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
                ("width", C.c_int32), ("height", C.c_int32), ("psx", C.c_float), ("psy", C.c_float)]


def make_camera(cam: dict) -> Camera:
    c = Camera()
    for i in range(16):
        c.m[i] = float(cam["m"][i])
    c.focal, c.cx, c.cy = float(cam["focal"]), float(cam["cx"]), float(cam["cy"])
    c.width, c.height = int(cam["width"]), int(cam["height"])
    c.psx, c.psy = float(cam["psx"]), float(cam["psy"])
    return c


def _render_lib():
    L = lib()
    if not getattr(L, "_render_bound", False):
        L.or_scene_create.argtypes = [_f32p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p,
                                      C.c_int32]
        L.or_scene_create.restype = C.c_void_p
        L.or_scene_destroy.argtypes = [C.c_void_p]
        L.or_scene_total_power.argtypes = [C.c_void_p]
        L.or_scene_total_power.restype = C.c_float
        L.or_scene_light_table.argtypes = [C.c_void_p, C.c_void_p]
        L.or_render.argtypes = [C.c_void_p, C.POINTER(Camera), C.POINTER(RenderCfg), C.c_void_p, C.c_void_p,
                                C.c_void_p]
        L.or_render_f64.argtypes = [C.c_void_p, C.POINTER(Camera), C.POINTER(RenderCfg), C.c_void_p]
        L._render_bound = True
    return L


class RenderScene:
    """Oracle scene for the integrator restatement. light_tables: 0 = sweep
    tables (the GPU scene's default), 1 = the reference's pairing."""

    def __init__(self, spec, light_tables: int = 0):
        L = _render_lib()
        self.pos = _f32(spec.positions).reshape(-1)
        self.objs = spec.objects_array()
        self.mats = spec.materials_array()
        self.h = L.or_scene_create(self.pos, self.pos.size // 9, self.objs.ctypes.data, len(self.objs),
                                   self.mats.ctypes.data, len(self.mats), None, int(light_tables))

    def __del__(self):
        if getattr(self, "h", None):
            _render_lib().or_scene_destroy(self.h)
            self.h = None

    @property
    def total_power(self) -> float:
        return _render_lib().or_scene_total_power(self.h)

    def light_table(self) -> np.ndarray:
        out = np.zeros(len(self.objs), ALIAS_DTYPE)
        _render_lib().or_scene_light_table(self.h, out.ctypes.data)
        return out

    def render(self, cam: dict, spp: int, max_depth: int = 10, seed: int = 0, sample_offset: int = 0,
               pixel_sampling: int = 1, rng_mode: int = 0, trig_mode: int = 0, cast_mode: int = 0,
               tri_table_order: int = 0, replay: np.ndarray | None = None, threads: int = 0,
               per_sample: bool = False, debug: int = 0, pixels: np.ndarray | None = None):
        """accum [h*w, 4], casts [h*w], per-sample rgb or None. With `pixels`
        (pixel indices y * width + x) only those pixels are rendered; the
        others stay zero."""
        cfg = RenderCfg(max_depth, spp, sample_offset, pixel_sampling, seed, rng_mode, trig_mode, cast_mode,
                        tri_table_order, threads, 0, None, debug, None, 0)
        if pixels is not None:
            pixels = np.ascontiguousarray(pixels, np.int64)
            cfg.pixels = pixels.ctypes.data
            cfg.num_pixels = pixels.size
        if replay is not None:
            replay = _f32(replay)
            cfg.replay_stride = replay.shape[-1]
            cfg.replay = replay.ctypes.data
        w, h = cam["width"], cam["height"]
        accum = np.zeros((h * w, 4), np.float32)
        casts = np.zeros(h * w, np.uint32)
        rgb = np.zeros((spp, h * w, 3), np.float32) if per_sample else None
        c = make_camera(cam)
        _render_lib().or_render(self.h, C.byref(c), C.byref(cfg), rgb.ctypes.data if rgb is not None else None,
                                accum.ctypes.data, casts.ctypes.data)
        return accum, casts, rgb


    def render_f64(self, cam: dict, spp: int, max_depth: int = 10, seed: int = 0, sample_offset: int = 0,
                   pixel_sampling: int = 1, threads: int = 0, pixels: np.ndarray | None = None) -> np.ndarray:
        """FP64 restatement of the integrator: mean radiance [h*w, 3] (float64)
        over `spp` samples per pixel (pixels outside `pixels` stay zero)."""
        cfg = RenderCfg(max_depth, spp, sample_offset, pixel_sampling, seed, 0, 0, 0, 0, threads, 0, None, 0,
                        None, 0)
        if pixels is not None:
            pixels = np.ascontiguousarray(pixels, np.int64)
            cfg.pixels = pixels.ctypes.data
            cfg.num_pixels = pixels.size
        w, h = cam["width"], cam["height"]
        out = np.zeros((h * w, 3), np.float64)
        c = make_camera(cam)
        _render_lib().or_render_f64(self.h, C.byref(c), C.byref(cfg), out.ctypes.data)
        return out / float(spp)


def ref_render_samples(spec, cam: dict, spp: int, replay: np.ndarray, sampling: int = 1, debug: int = 0):
    """The reference's own sampleColor (depth 10) on every pixel sample:
    per-sample colours, per-pixel path-ray counts and per-sample counts (w)."""
    L = ref()
    if not getattr(L, "_render_bound", False):
        L.refh_render_samples.argtypes = [_f32p, _i32p, _i32p, _i32p, _f32p, C.c_int, _f32p, C.c_int, _f32p,
                                          C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, C.c_float, C.c_float,
                                          C.c_int, C.c_int, _f32p, C.c_int, _f32p, _u32p, C.c_int, _f32p]
        L._render_bound = True
    objs = spec.objects_array()
    w, h = cam["width"], cam["height"]
    rgb = np.zeros((spp, h * w, 3), np.float32)
    sw = np.zeros((spp, h * w), np.float32)
    casts = np.zeros(h * w, np.uint32)
    replay = _f32(replay)
    L.refh_render_samples(_f32(spec.positions).reshape(-1), objs["tri_begin"].astype(np.int32),
                          objs["tri_count"].astype(np.int32), objs["material"].astype(np.int32),
                          objs["surface_area"].astype(np.float32), len(objs), spec.materials_array().reshape(-1),
                          len(spec.materials), _f32(cam["m"]), float(cam["focal"]), float(cam["cx"]),
                          float(cam["cy"]), w, h, float(cam["psx"]), float(cam["psy"]), sampling, spp,
                          replay.reshape(-1), replay.shape[-1], rgb.reshape(-1), casts, debug, sw.reshape(-1))
    return rgb, casts, sw


# ---- path-guiding network (FP64 restatement) --------------------------------

def _guide_lib():
    L = lib()
    if not getattr(L, "_guide_bound", False):
        L.or_mlp_num_params.restype = C.c_int32
        L.or_guide_encode.argtypes = [_f32p, _f32p, _f32p, C.c_float, _f32p]
        L.or_mlp_forward.argtypes = [_f32p, _f32p, C.c_int32, _f32p]
        L.or_vmf_mixture_log_pdf.argtypes = [_f32p, _f32p]
        L.or_vmf_mixture_log_pdf.restype = C.c_double
        L.or_mlp_loss_grad.argtypes = [_f32p, _f32p, _f32p, _f32p, C.c_int32, C.POINTER(C.c_double),
                                       np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")]
        L.or_adam_step.argtypes = [_f32p, _f32p, _f32p, _f32p, C.c_int32, C.c_int32, C.c_float, C.c_float,
                                   C.c_float, C.c_float]
        L._guide_bound = True
    return L


def mlp_num_params() -> int:
    return int(_guide_lib().or_mlp_num_params())


def guide_encode(pos, dirs, center, half) -> np.ndarray:
    pos, dirs = _f32(pos).reshape(-1, 3), _f32(dirs).reshape(-1, 3)
    out = np.zeros((pos.shape[0], 80), np.float32)
    c = _f32(center)
    for i in range(pos.shape[0]):
        row = np.zeros(80, np.float32)
        _guide_lib().or_guide_encode(np.ascontiguousarray(pos[i]), np.ascontiguousarray(dirs[i]), c, float(half), row)
        out[i] = row
    return out


def mlp_forward(params, inputs) -> np.ndarray:
    inputs = _f32(inputs).reshape(-1, 80)
    out = np.zeros((inputs.shape[0], 48), np.float32)
    _guide_lib().or_mlp_forward(_f32(params), inputs, inputs.shape[0], out)
    return out


def vmf_mixture_log_pdf(y, w) -> float:
    return float(_guide_lib().or_vmf_mixture_log_pdf(_f32(y).reshape(-1)[:40].copy(), _f32(w)))


def mlp_loss_grad(params, inputs, dirs, weights):
    inputs = _f32(inputs).reshape(-1, 80)
    grad = np.zeros(mlp_num_params(), np.float64)
    loss = C.c_double()
    _guide_lib().or_mlp_loss_grad(_f32(params), inputs, _f32(dirs).reshape(-1), _f32(weights), inputs.shape[0],
                                  C.byref(loss), grad)
    return loss.value, grad


def adam_step(params, m, v, grad, t, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    p, m, v = _f32(params).copy(), _f32(m).copy(), _f32(v).copy()
    _guide_lib().or_adam_step(p, m, v, _f32(grad), p.size, int(t), lr, b1, b2, eps)
    return p, m, v
