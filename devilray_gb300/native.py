"""ctypes binding of ``libdevilray_gb300.so`` (the C ABI of include/devilray_gb300.h).

The library is built in-tree by :mod:`devilray_gb300.build`. Loading fails
loudly when it is missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB

DR_OK = 0
STATUS_NAMES = {
    0: "DR_OK", 1: "DR_ERR_INVALID_ARGUMENT", 2: "DR_ERR_CUDA", 3: "DR_ERR_OUT_OF_MEMORY",
    4: "DR_ERR_NO_DEVICE", 5: "DR_ERR_TIMEOUT", 6: "DR_ERR_STACK_OVERFLOW", 7: "DR_ERR_UNSUPPORTED",
    8: "DR_ERR_TOO_LARGE",
}

DR_ALIAS_REFERENCE = 0
DR_ALIAS_SWEEP = 1
DR_LIGHT_TABLES_SWEEP = 0
DR_LIGHT_TABLES_REFERENCE = 1
ALIAS_DTYPE = np.dtype([("p_A", "<f4"), ("pdf_A", "<f4"), ("pdf_B", "<f4"), ("A", "<i4"), ("B", "<i4")])

DR_TRI_REFERENCE = 0
DR_TRI_WATERTIGHT = 1
DR_MAT_DIFFUSE = 0
DR_MAT_DIELECTRIC = 1

RAY_DTYPE = np.dtype([("ox", "<f4"), ("oy", "<f4"), ("oz", "<f4"), ("tmax", "<f4"),
                      ("dx", "<f4"), ("dy", "<f4"), ("dz", "<f4"), ("pad", "<f4")])
HIT_DTYPE = np.dtype([("t", "<f4"), ("prim", "<i4")])


class DrError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class ContextConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("flags", C.c_uint32)]


class Material(C.Structure):
    _fields_ = [("kind", C.c_int32), ("ior", C.c_float), ("pad0", C.c_float), ("pad1", C.c_float),
                ("emission", C.c_float * 4), ("albedo", C.c_float * 4), ("debug_color", C.c_float * 4)]


class Object(C.Structure):
    _fields_ = [("tri_begin", C.c_uint32), ("tri_count", C.c_uint32), ("material", C.c_int32),
                ("surface_area", C.c_float)]


class SceneDesc(C.Structure):
    _fields_ = [("positions_host", C.c_void_p), ("num_triangles", C.c_uint32),
                ("objects_host", C.c_void_p), ("num_objects", C.c_uint32),
                ("materials_host", C.c_void_p), ("num_materials", C.c_uint32),
                ("tri_material_host", C.c_void_p), ("tri_weight_host", C.c_void_p),
                ("light_tables", C.c_uint32)]


class BuildConfig(C.Structure):
    _fields_ = [("max_leaf_size", C.c_uint32), ("sah_bins", C.c_uint32), ("threads", C.c_uint32),
                ("layout", C.c_uint32), ("builder", C.c_uint32)]


class SceneInfo(C.Structure):
    _fields_ = [("num_triangles", C.c_uint32), ("num_nodes", C.c_uint32), ("depth", C.c_uint32),
                ("layout", C.c_uint32), ("slack", C.c_float), ("total_radiant_power", C.c_float),
                ("device_bytes", C.c_uint64), ("build_seconds", C.c_double)]


class Camera(C.Structure):
    _fields_ = [("transform", C.c_float * 16), ("focal_length", C.c_float), ("center", C.c_float * 2),
                ("width", C.c_int32), ("height", C.c_int32), ("pixel_size", C.c_float * 2)]


class RenderConfig(C.Structure):
    _fields_ = [("max_depth", C.c_uint32), ("spp", C.c_uint32), ("sample_offset", C.c_uint32),
                ("pixel_sampling", C.c_int32), ("seed", C.c_uint64), ("tri_mode", C.c_int32),
                ("wave_paths", C.c_uint32), ("flags", C.c_uint32), ("debug", C.c_int32),
                ("streams", C.c_uint32), ("chunk", C.c_uint32), ("stack", C.c_uint32)]


class RenderStats(C.Structure):
    _fields_ = [("path_rays", C.c_uint64), ("shadow_rays", C.c_uint64)]


class Job(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", Camera), ("config", RenderConfig), ("accum_dev", C.c_void_p),
                ("casts_dev", C.c_void_p)]


class BatchConfig(C.Structure):
    _fields_ = [("wave_paths", C.c_uint32), ("streams", C.c_uint32), ("chunk", C.c_uint32),
                ("use_graph", C.c_uint32), ("stack", C.c_uint32)]


class AutotuneConfig(C.Structure):
    _fields_ = [("probe_spp", C.c_uint32), ("reps", C.c_uint32), ("try_layouts", C.c_uint32),
                ("max_leaf_size", C.c_uint32)]


class AutotuneCandidate(C.Structure):
    _fields_ = [("layout", C.c_uint32), ("wave_paths", C.c_uint32), ("streams", C.c_uint32),
                ("chunk", C.c_uint32), ("stack", C.c_uint32), ("ms", C.c_float)]


class AutotuneResult(C.Structure):
    _fields_ = [("layout", C.c_uint32), ("wave_paths", C.c_uint32), ("streams", C.c_uint32),
                ("chunk", C.c_uint32), ("stack", C.c_uint32), ("best_ms", C.c_float),
                ("num_candidates", C.c_uint32), ("candidates", AutotuneCandidate * 64)]

    def as_dict(self) -> dict:
        return {"layout": self.layout, "wave_paths": self.wave_paths, "streams": self.streams, "chunk": self.chunk,
                "stack": self.stack, "best_ms": self.best_ms,
                "candidates": [{"layout": c.layout, "wave_paths": c.wave_paths, "streams": c.streams,
                                "chunk": c.chunk, "stack": c.stack, "ms": c.ms}
                               for c in self.candidates[:self.num_candidates]]}


class BatchInfo(C.Structure):
    _fields_ = [("num_jobs", C.c_uint32), ("num_waves", C.c_uint32), ("max_wave_paths", C.c_uint32),
                ("layout", C.c_uint32), ("graph_nodes", C.c_uint64), ("paths_per_render", C.c_uint64),
                ("device_bytes", C.c_uint64), ("streams", C.c_uint32), ("chunk", C.c_uint32)]


def make_camera(cam: dict) -> Camera:
    """dr_camera from the dict of devilray_gb300.scenes.camera()."""
    c = Camera()
    for i in range(16):
        c.transform[i] = float(cam["m"][i])
    c.focal_length = float(cam["focal"])
    c.center[0], c.center[1] = float(cam["cx"]), float(cam["cy"])
    c.width, c.height = int(cam["width"]), int(cam["height"])
    c.pixel_size[0], c.pixel_size[1] = float(cam["psx"]), float(cam["psy"])
    return c


class TraceCounters(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("node_visits", C.c_uint64), ("box_tests", C.c_uint64),
                ("tri_tests", C.c_uint64), ("hits", C.c_uint64)]


# Every symbol the public header declares, with its ctypes signature.
SIGNATURES = {
    "dr_abi_version": (C.c_uint32, []),
    "dr_last_error_string": (C.c_char_p, []),
    "dr_context_create": (C.c_int, [C.POINTER(ContextConfig), C.POINTER(C.c_void_p)]),
    "dr_context_destroy": (C.c_int, [C.c_void_p]),
    "dr_context_check": (C.c_int, [C.c_void_p]),
    "dr_scene_create": (C.c_int, [C.c_void_p, C.POINTER(SceneDesc), C.POINTER(BuildConfig), C.POINTER(C.c_void_p)]),
    "dr_scene_destroy": (C.c_int, [C.c_void_p]),
    "dr_scene_get_info": (C.c_int, [C.c_void_p, C.POINTER(SceneInfo)]),
    "dr_trace_closest": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_int32,
                                   C.POINTER(TraceCounters), C.c_void_p]),
    "dr_trace_any": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_int32, C.c_void_p]),
    "dr_trace_closest_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_int32, C.c_void_p]),
    "dr_render": (C.c_int, [C.c_void_p, C.POINTER(Camera), C.POINTER(RenderConfig), C.c_void_p, C.c_void_p,
                            C.c_void_p]),
    "dr_synchronize": (C.c_int, [C.c_void_p, C.c_void_p]),
    "dr_device_allocate": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    "dr_device_free": (C.c_int, [C.c_void_p, C.c_void_p]),
    "dr_device_copy_from_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64]),
    "dr_device_copy_to_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64]),
    "dr_device_zero": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "dr_scene_get_light_table": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32)]),
    "dr_scene_get_render_stats": (C.c_int, [C.c_void_p, C.c_void_p]),
    "dr_framebuffer_create": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "dr_framebuffer_destroy": (C.c_int, [C.c_void_p]),
    "dr_framebuffer_clear": (C.c_int, [C.c_void_p, C.c_void_p]),
    "dr_framebuffer_device_buffers": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "dr_framebuffer_read": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64)]),
    "dr_framebuffer_tonemap": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "dr_tonemap": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "dr_resolve": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "dr_framebuffer_write_pfm": (C.c_int, [C.c_void_p, C.c_char_p]),
    "dr_batch_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(C.c_void_p)]),
    "dr_batch_render": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "dr_batch_get_info": (C.c_int, [C.c_void_p, C.c_void_p]),
    "dr_batch_destroy": (C.c_int, [C.c_void_p]),
    "dr_render_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    "dr_autotune": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "dr_autotune_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    "dr_guide_num_params": (C.c_uint32, []),
    "dr_guide_create": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "dr_guide_destroy": (C.c_int, [C.c_void_p]),
    "dr_guide_set_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "dr_guide_get_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "dr_guide_state_bytes": (C.c_uint64, []),
    "dr_guide_get_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "dr_guide_set_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "dr_guide_encode": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "dr_guide_infer": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    "dr_guide_gradients": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                     C.c_void_p, C.c_void_p]),
    "dr_guide_train_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                      C.c_void_p]),
    "dr_guide_last_loss": (C.c_int, [C.c_void_p, C.c_void_p]),
    "dr_guide_mixture_sample": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "dr_guide_mixture_pdf": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    "dr_render_guided": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p]),
    "dr_alias_build_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_int32]),
    "dr_alias_build": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_int32, C.c_void_p]),
    "dr_alias_build_noalloc": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    "dr_alias_sample": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p,
                                  C.c_void_p]),
    "dr_probe_read_bandwidth": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32, C.POINTER(C.c_double),
                                          C.c_void_p]),
    "dr_debug_expire_wait": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "dr_debug_stack_limit": (C.c_int, [C.c_void_p, C.c_uint32]),
    "dr_debug_fail_allocation": (C.c_int, [C.c_uint32]),
}

_lib = None


def load(path: Path | str | None = None):
    """Loads the library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        _build.build()
    if not p.exists():
        raise FileNotFoundError(f"{p} is missing: build the CUDA library first")
    L = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(status: int) -> None:
    if status != DR_OK:
        msg = load().dr_last_error_string()
        raise DrError(status, msg.decode() if msg else "")


def _ptr(a) -> int:
    """Device or host address of a torch tensor / numpy array / int."""
    if a is None:
        return 0
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


def _stream_ptr(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class Context:
    def __init__(self, device: int = 0):
        L = load()
        self.handle = C.c_void_p()
        cfg = ContextConfig(device, 0)
        check(L.dr_context_create(C.byref(cfg), C.byref(self.handle)))
        self.device = device

    def close(self):
        if self.handle:
            load().dr_context_destroy(self.handle)
            self.handle = C.c_void_p()

    def check(self):
        check(load().dr_context_check(self.handle))

    def read_bandwidth(self, buf_dev, nbytes: int, reps: int = 20, stream=None) -> float:
        """GB/s of streaming reads over a device buffer (dr_probe_read_bandwidth)."""
        out = C.c_double()
        check(load().dr_probe_read_bandwidth(self.handle, _ptr(buf_dev), nbytes, reps, C.byref(out),
                                             _stream_ptr(stream)))
        return out.value

    def alias_build(self, weights_dev, n: int, table_dev, mode: int = DR_ALIAS_SWEEP, stream=None):
        check(load().dr_alias_build(self.handle, _ptr(weights_dev), n, _ptr(table_dev), mode, _stream_ptr(stream)))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def alias_sample(table_dev, n: int, uniforms_dev, ndraws: int, index_dev, pdf_dev, stream=None):
    check(load().dr_alias_sample(_ptr(table_dev), n, _ptr(uniforms_dev), ndraws, _ptr(index_dev), _ptr(pdf_dev),
                                 _stream_ptr(stream)))


def scene_desc(positions: np.ndarray, objects=None, materials=None, tri_material=None, tri_weight=None,
               light_tables: int = 0):
    """dr_scene_desc over numpy/ctypes arrays; returns (desc, arrays to keep alive).
    light_tables: DR_LIGHT_TABLES_SWEEP (0) or DR_LIGHT_TABLES_REFERENCE (1)."""
    positions = np.ascontiguousarray(positions, np.float32).reshape(-1, 9)
    desc = SceneDesc()
    desc.light_tables = light_tables
    desc.positions_host = positions.ctypes.data
    desc.num_triangles = positions.shape[0]
    keep = [positions]
    if objects is not None:
        objs = _records(objects, Object)
        keep.append(objs)
        desc.objects_host = objs.ctypes.data
        desc.num_objects = len(objs)
    if materials is not None:
        mats = _records(materials, Material)
        keep.append(mats)
        desc.materials_host = mats.ctypes.data
        desc.num_materials = len(mats)
    if tri_material is not None:
        tm = np.ascontiguousarray(tri_material, np.int32)
        keep.append(tm)
        desc.tri_material_host = tm.ctypes.data
    if tri_weight is not None:
        tw = np.ascontiguousarray(tri_weight, np.float32)
        keep.append(tw)
        desc.tri_weight_host = tw.ctypes.data
    return desc, keep


def _records(items, struct) -> np.ndarray:
    """Contiguous bytes of `struct` records: a sequence of ctypes `struct`
    instances, or a numpy array whose rows have the struct's size (the
    structured arrays of SceneSpec.objects_array / materials_array)."""
    size = C.sizeof(struct)
    if isinstance(items, np.ndarray):
        a = np.ascontiguousarray(items)
        if a.dtype.itemsize * (a.shape[1] if a.ndim == 2 else 1) != size:
            raise ValueError(f"{struct.__name__} records are {size} bytes")
        return a.view(np.uint8).reshape(-1, size)
    out = np.empty((len(items), size), np.uint8)
    for i, it in enumerate(items):
        out[i] = np.frombuffer(bytes(it), np.uint8)
    return out


def spec_parts(spec):
    """(objects, materials) records of a devilray_gb300.scenes.SceneSpec, as
    numpy arrays laid out like dr_object and dr_material."""
    return spec.objects_array(), spec.materials_array()


def autotune(ctx: "Context", spec, cam: dict, spp: int = 1, max_depth: int = 10, pixel_sampling: int = 1,
             seed: int = 0, probe_spp: int = 0, reps: int = 2, try_layouts: bool = True) -> "AutotuneResult":
    """dr_autotune for a SceneSpec rendered through `cam`."""
    objs, mats = spec_parts(spec)
    desc, keep = scene_desc(spec.positions, objs, mats)
    c = make_camera(cam)
    cfg = RenderConfig(max_depth, spp, 0, pixel_sampling, seed, DR_TRI_REFERENCE, 0, 0, 0, 0, 0, 0)
    tc = AutotuneConfig(probe_spp, reps, 1 if try_layouts else 0, 0)
    out = AutotuneResult()
    check(load().dr_autotune(ctx.handle, C.byref(desc), C.byref(c), C.byref(cfg), C.byref(tc), C.byref(out)))
    del keep
    return out


class Scene:
    """A triangle soup uploaded with its BVH (dr_scene_create)."""

    @classmethod
    def from_spec(cls, ctx: "Context", spec, **kw) -> "Scene":
        """Scene from a devilray_gb300.scenes.SceneSpec (objects + materials)."""
        objs, mats = spec_parts(spec)
        return cls(ctx, spec.positions, objects=objs, materials=mats, **kw)

    def __init__(self, ctx: Context, positions: np.ndarray, objects=None, materials=None,
                 tri_material=None, tri_weight=None, max_leaf_size: int = 0, sah_bins: int = 0,
                 threads: int = 0, layout: int = 0, builder: int = 0, light_tables: int = 0):
        self.ctx = ctx
        self.positions = np.ascontiguousarray(positions, np.float32).reshape(-1, 9)
        desc, keep = scene_desc(self.positions, objects, materials, tri_material, tri_weight, light_tables)
        cfg = BuildConfig(max_leaf_size, sah_bins, threads, layout, builder)
        self.handle = C.c_void_p()
        check(load().dr_scene_create(ctx.handle, C.byref(desc), C.byref(cfg), C.byref(self.handle)))
        self._keep = keep

    def render_stats(self) -> RenderStats:
        """Path and shadow rays of the last render (synchronous)."""
        st = RenderStats()
        check(load().dr_scene_get_render_stats(self.handle, C.byref(st)))
        return st

    def info(self) -> SceneInfo:
        info = SceneInfo()
        check(load().dr_scene_get_info(self.handle, C.byref(info)))
        return info

    def light_table(self) -> np.ndarray:
        """The object light table (dr_scene_get_light_table), ALIAS_DTYPE entries."""
        count = C.c_uint32()
        check(load().dr_scene_get_light_table(self.handle, None, 0, C.byref(count)))
        out = np.zeros(count.value, ALIAS_DTYPE)
        if count.value:
            check(load().dr_scene_get_light_table(self.handle, out.ctypes.data, count.value, C.byref(count)))
        return out

    def close(self):
        if self.handle:
            load().dr_scene_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- traversal on device buffers (torch tensors or raw addresses) --
    def trace_closest(self, rays_dev, n: int, hits_dev, tri_mode: int = DR_TRI_REFERENCE,
                      counters: bool = False, stream=None):
        cnt = TraceCounters() if counters else None
        check(load().dr_trace_closest(self.handle, _ptr(rays_dev), n, _ptr(hits_dev), tri_mode,
                                      C.byref(cnt) if cnt is not None else None, _stream_ptr(stream)))
        return cnt

    def trace_any(self, rays_dev, n: int, occluded_dev, tri_mode: int = DR_TRI_REFERENCE, stream=None):
        check(load().dr_trace_any(self.handle, _ptr(rays_dev), n, _ptr(occluded_dev), tri_mode,
                                  _stream_ptr(stream)))

    # -- rendering --
    def render(self, cam: dict, accum_dev, casts_dev=None, spp: int = 1, max_depth: int = 10,
               sample_offset: int = 0, pixel_sampling: int = 1, seed: int = 0, tri_mode: int = DR_TRI_REFERENCE,
               wave_paths: int = 0, debug: int = 0, streams: int = 0, chunk: int = 0, stack: int = 0, stream=None):
        c = make_camera(cam)
        cfg = RenderConfig(max_depth, spp, sample_offset, pixel_sampling, seed, tri_mode, wave_paths, 0, debug,
                           streams, chunk, stack)
        check(load().dr_render(self.handle, C.byref(c), C.byref(cfg), _ptr(accum_dev), _ptr(casts_dev),
                               _stream_ptr(stream)))

    def render_guided(self, guide: "Guide", cam: dict, accum_dev, casts_dev=None, spp: int = 1,
                      max_depth: int = 10, sample_offset: int = 0, pixel_sampling: int = 1, seed: int = 0,
                      alpha: float = 0.5, train: bool = True, train_batch: int = 0, train_steps: int = 0,
                      train_budget: int = 0, target: int = 0, bounces: int = 0, wave_paths: int = 0, streams: int = 0,
                      alpha_ramp: int = 0, stream=None):
        c = make_camera(cam)
        cfg = RenderConfig(max_depth, spp, sample_offset, pixel_sampling, seed, DR_TRI_REFERENCE, wave_paths, 0, 0,
                           streams, 0, 0)
        g = GuidedConfig(alpha, 1 if train else 0, train_batch, train_steps, train_budget, target, bounces, alpha_ramp)
        check(load().dr_render_guided(self.handle, C.byref(c), C.byref(cfg), guide.handle, C.byref(g), _ptr(accum_dev),
                                      _ptr(casts_dev), _stream_ptr(stream)))

    # -- traversal on host buffers --
    def trace_closest_host(self, rays: np.ndarray, hits: np.ndarray | None = None,
                           tri_mode: int = DR_TRI_REFERENCE, stream=None) -> np.ndarray:
        rays = np.ascontiguousarray(rays)
        assert rays.dtype == RAY_DTYPE or (rays.dtype == np.float32 and rays.shape[-1] == 8)
        n = rays.shape[0]
        if hits is None:
            hits = np.empty(n, HIT_DTYPE)
        check(load().dr_trace_closest_host(self.handle, _ptr(rays), n, _ptr(hits), tri_mode,
                                           _stream_ptr(stream)))
        return hits


class Framebuffer:
    """Accumulation buffers of a progressive render (Buffers of the reference)."""

    def __init__(self, ctx: "Context", width: int, height: int):
        self.ctx = ctx
        self.width, self.height = int(width), int(height)
        h = C.c_void_p()
        check(load().dr_framebuffer_create(ctx.handle, self.width, self.height, C.byref(h)))
        self.handle = h.value

    def close(self) -> None:
        if getattr(self, "handle", None):
            load().dr_framebuffer_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def clear(self, stream=None) -> None:
        check(load().dr_framebuffer_clear(self.handle, _stream_ptr(stream)))

    def device_buffers(self) -> tuple[int, int]:
        a, c = C.c_void_p(), C.c_void_p()
        check(load().dr_framebuffer_device_buffers(self.handle, C.byref(a), C.byref(c)))
        return a.value, c.value

    def read(self):
        n = self.width * self.height
        acc = np.zeros((n, 4), np.float32)
        casts = np.zeros(n, np.uint32)
        total = C.c_uint64()
        check(load().dr_framebuffer_read(self.handle, _ptr(acc), _ptr(casts), C.byref(total)))
        return acc, casts, total.value

    def tonemap(self, gamma: bool = True) -> np.ndarray:
        out = np.zeros(self.width * self.height, np.uint32)
        check(load().dr_framebuffer_tonemap(self.handle, 1 if gamma else 0, _ptr(out)))
        return out

    def write_pfm(self, path) -> None:
        """The linear image as a PFM file (rows from the bottom)."""
        check(load().dr_framebuffer_write_pfm(self.handle, str(path).encode()))


def resolve(accum_dev, width: int, height: int, rgb_dev, stream=None) -> None:
    """dr_resolve: the linear image (sum / samples) of a device accumulation buffer."""
    check(load().dr_resolve(_ptr(accum_dev), width, height, _ptr(rgb_dev), _stream_ptr(stream)))


def make_job(scene: "Scene", cam: dict, accum_dev, casts_dev=None, spp: int = 1, max_depth: int = 10,
             sample_offset: int = 0, pixel_sampling: int = 1, seed: int = 0,
             tri_mode: int = DR_TRI_REFERENCE) -> Job:
    j = Job()
    j.scene = scene.handle.value if isinstance(scene.handle, C.c_void_p) else scene.handle
    j.camera = make_camera(cam)
    j.config = RenderConfig(max_depth, spp, sample_offset, pixel_sampling, seed, tri_mode, 0, 0, 0, 0, 0, 0)
    j.accum_dev = _ptr(accum_dev)
    j.casts_dev = _ptr(casts_dev) if casts_dev is not None else None
    return j


class Batch:
    """Many images of many scenes rendered as one schedule (dr_batch)."""

    def __init__(self, ctx: "Context", jobs: list, wave_paths: int = 0, streams: int = 0, chunk: int = 0,
                 use_graph: bool = True, stack: int = 0):
        self.ctx = ctx
        self._jobs = (Job * len(jobs))(*jobs)
        cfg = BatchConfig(wave_paths, streams, chunk, 1 if use_graph else 0, stack)
        h = C.c_void_p()
        check(load().dr_batch_create(ctx.handle, self._jobs, len(jobs), C.byref(cfg), C.byref(h)))
        self.handle = h.value

    def render(self, sample_offsets=None, stream=None) -> None:
        offs = None
        if sample_offsets is not None:
            offs = (C.c_uint32 * len(sample_offsets))(*[int(x) for x in sample_offsets])
        check(load().dr_batch_render(self.handle, offs, _stream_ptr(stream)))

    def info(self) -> BatchInfo:
        i = BatchInfo()
        check(load().dr_batch_get_info(self.handle, C.byref(i)))
        return i

    def close(self) -> None:
        if getattr(self, "handle", None):
            load().dr_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune_batch(ctx: "Context", jobs: list, probe_spp: int = 1, reps: int = 2) -> AutotuneResult:
    arr = (Job * len(jobs))(*jobs)
    tc = AutotuneConfig(probe_spp, reps, 0, 0)
    out = AutotuneResult()
    check(load().dr_autotune_batch(ctx.handle, arr, len(jobs), C.byref(tc), C.byref(out)))
    return out


def render_batch(ctx: "Context", jobs: list, wave_paths: int = 0, streams: int = 0, chunk: int = 0,
                 stack: int = 0, stream=None) -> None:
    arr = (Job * len(jobs))(*jobs)
    cfg = BatchConfig(wave_paths, streams, chunk, 0, stack)
    check(load().dr_render_batch(ctx.handle, arr, len(jobs), C.byref(cfg), _stream_ptr(stream)))


class GuidedConfig(C.Structure):
    _fields_ = [("alpha", C.c_float), ("train", C.c_uint32), ("train_batch", C.c_uint32), ("train_steps", C.c_uint32),
                ("train_budget", C.c_uint32), ("target", C.c_uint32), ("bounces", C.c_uint32),
                ("alpha_ramp", C.c_uint32)]


class GuideConfig(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("learning_rate", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float),
                ("epsilon", C.c_float), ("center", C.c_float * 3), ("half_extent", C.c_float),
                ("infer_kernel", C.c_uint32), ("warmup_steps", C.c_uint32)]


class Guide:
    """The path-guiding network (dr_guide)."""

    def __init__(self, ctx: "Context", seed: int = 0, learning_rate: float = 1e-3, center=(0.0, 0.0, 0.0),
                 half_extent: float = 1.0, infer_kernel: int = 0, warmup_steps: int = 0):
        self.ctx = ctx
        cfg = GuideConfig(seed, learning_rate, 0.9, 0.999, 1e-8, (C.c_float * 3)(*center), half_extent, infer_kernel,
                          warmup_steps)
        h = C.c_void_p()
        check(load().dr_guide_create(ctx.handle, C.byref(cfg), C.byref(h)))
        self.handle = h.value
        self.num_params = int(load().dr_guide_num_params())

    def params(self) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        check(load().dr_guide_get_params(self.handle, _ptr(out), self.num_params))
        return out

    def get_state(self) -> np.ndarray:
        """The network's whole training state (configuration, Adam step,
        parameters, Adam moments) as bytes, for a checkpoint."""
        out = np.zeros(int(load().dr_guide_state_bytes()), np.uint8)
        check(load().dr_guide_get_state(self.handle, _ptr(out), out.size))
        return out

    def set_state(self, state: np.ndarray) -> None:
        """Restores a state from get_state (of any network of this library)."""
        state = np.ascontiguousarray(state, np.uint8)
        check(load().dr_guide_set_state(self.handle, _ptr(state), state.size))

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        check(load().dr_guide_set_params(self.handle, _ptr(p), self.num_params))

    def encode(self, pos_dev, dir_dev, n: int, out_dev) -> None:
        check(load().dr_guide_encode(self.handle, _ptr(pos_dev), _ptr(dir_dev), n, _ptr(out_dev)))

    def infer(self, pos_dev, dir_dev, n: int, y_dev, stream=None) -> None:
        check(load().dr_guide_infer(self.handle, _ptr(pos_dev), _ptr(dir_dev), n, _ptr(y_dev), _stream_ptr(stream)))

    def gradients(self, pos_dev, dir_dev, sdir_dev, w_dev, n: int):
        loss = C.c_float()
        grad = np.zeros(self.num_params, np.float32)
        check(load().dr_guide_gradients(self.handle, _ptr(pos_dev), _ptr(dir_dev), _ptr(sdir_dev), _ptr(w_dev), n,
                                        C.byref(loss), _ptr(grad)))
        return float(loss.value), grad

    def train_step(self, pos_dev, dir_dev, sdir_dev, w_dev, n: int, stream=None) -> None:
        check(load().dr_guide_train_step(self.handle, _ptr(pos_dev), _ptr(dir_dev), _ptr(sdir_dev), _ptr(w_dev), n,
                                         _stream_ptr(stream)))

    def last_loss(self) -> float:
        v = C.c_float()
        check(load().dr_guide_last_loss(self.handle, C.byref(v)))
        return float(v.value)

    def close(self) -> None:
        if getattr(self, "handle", None):
            load().dr_guide_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tonemap(accum_dev, width: int, height: int, rgba_dev, gamma: bool = True, stream=None) -> None:
    check(load().dr_tonemap(_ptr(accum_dev), width, height, 1 if gamma else 0, _ptr(rgba_dev),
                            _stream_ptr(stream)))


def make_rays(origins: np.ndarray, dirs: np.ndarray, tmax=np.inf) -> np.ndarray:
    """Packs origins/directions into the 32-byte dr_ray layout (float32 [n, 8])."""
    n = origins.shape[0]
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = origins
    r[:, 3] = tmax
    r[:, 4:7] = dirs
    return r
