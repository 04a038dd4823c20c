"""ctypes binding of the C ABI in include/fnd_rt.h.

This is the Python face of the path-tracer pass: a ``Context`` (one CUDA
stream on one device, the counterpart of ``Renderer::Renderer(device,
allocator)`` in src/Renderer/Renderer.hpp:41) owns ``Scene`` objects (BVH +
triangles in device memory) and traces ray batches. Errors come back as
``FndError`` carrying the library status code and message; there is no CPU
fallback: if the native library is missing, importing this module's entry
points raises.

Buffers: numpy arrays are host memory (the library copies in and out and
synchronises); objects exposing ``data_ptr()`` and ``is_cuda`` (torch CUDA
tensors) are passed as device pointers and the call only enqueues work on
the context stream.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref

import numpy as np

from . import _build

LIB_PATH = _build.LIB_PATH

FND_OK = 0
STATUS_NAMES = {
    -1: "FND_ERR_INVALID_ARG", -2: "FND_ERR_OUT_OF_MEMORY", -3: "FND_ERR_CUDA", -4: "FND_ERR_NO_DEVICE",
    -5: "FND_ERR_INVALID_SCENE", -6: "FND_ERR_STACK_OVERFLOW", -7: "FND_ERR_TIMEOUT", -8: "FND_ERR_UNSUPPORTED",
    -9: "FND_ERR_IO",
}
FND_MEM_HOST, FND_MEM_DEVICE = 0, 1
ABI_VERSION = 2
INVALID_ID = 0xFFFFFFFF

HIT_DTYPE = np.dtype([("prim", np.uint32), ("t", np.float32)])
MATERIAL_DTYPE = np.dtype([("type", "<u4"), ("albedo", "<f4", 3), ("roughness", "<f4"), ("emission", "<f4", 3),
                           ("light", "<i4"), ("reserved", "<f4", 3)])
LIGHT_DTYPE = np.dtype([("corner", "<f4", 3), ("edge_u", "<f4", 3), ("edge_v", "<f4", 3), ("radiance", "<f4", 3)])
MAT_LAMBERT, MAT_GGX, MAT_EMISSIVE = 0, 1, 2
RENDER_ACCUMULATE = 1
BVH_SPATIAL_SPLITS = 1
BVH_GPU_BUILD = 2
BVH_SAH_COLLAPSE = 4
BVH_GPU_CLUSTER = 8
RENDER_CACHE = 2
RENDER_WAVEFRONT = 4
RENDER_TRAIN_ONLY = 8
TONEMAP_CLAMP, TONEMAP_REINHARD, TONEMAP_ACES = 0, 1, 2
CACHE_NUM_PARAMS = 22720
CACHE_NUM_FEATURES = 96


def BVH_CLUSTER_RADIUS(r: int) -> int:
    """FND_BVH_CLUSTER_RADIUS: the clustering search radius in bits 8..15 of the BVH flags."""
    return (int(r) & 255) << 8


def BVH_NODE_WIDTH(w: int) -> int:
    """FND_BVH_NODE_WIDTH: children per wide node (2..8) in bits 16..19 of the BVH flags."""
    return (int(w) & 15) << 16


class FndError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class _Desc(C.Structure):
    _fields_ = [("abi_version", C.c_uint32), ("device", C.c_int32), ("stream", C.c_void_p), ("flags", C.c_uint32)]


class _BvhDesc(C.Structure):
    _fields_ = [("sah_bins", C.c_uint32), ("max_leaf_tris", C.c_uint32), ("build_threads", C.c_uint32),
                ("flags", C.c_uint32), ("traversal_cost", C.c_float), ("split_budget", C.c_float),
                ("margin_scale", C.c_float), ("collapse_tri_cost", C.c_float)]


class SceneInfo(C.Structure):
    _fields_ = [("num_tris", C.c_uint32), ("num_binary_nodes", C.c_uint32), ("num_wide_nodes", C.c_uint32),
                ("binary_depth", C.c_uint32), ("wide_depth", C.c_uint32), ("num_leaves", C.c_uint32),
                ("node_bytes", C.c_uint64), ("tri_bytes", C.c_uint64), ("sah_cost", C.c_double),
                ("build_ms", C.c_double), ("collapse_ms", C.c_double), ("upload_ms", C.c_double),
                ("bounds_lo", C.c_float * 3), ("bounds_hi", C.c_float * 3), ("box_margin", C.c_float),
                ("num_refs", C.c_uint32)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["bounds_lo"] = list(self.bounds_lo)
        d["bounds_hi"] = list(self.bounds_hi)
        return d


class _Camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("target", C.c_float * 3), ("up", C.c_float * 3), ("vfov_deg", C.c_float)]


class _RenderDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_uint32), ("max_depth", C.c_uint32),
                ("rr_start", C.c_uint32), ("flags", C.c_uint32), ("seed", C.c_uint64), ("camera", _Camera),
                ("sky", C.c_float * 3), ("sun_dir", C.c_float * 3), ("sun_irradiance", C.c_float * 3),
                ("wave_paths", C.c_uint32), ("tail_paths", C.c_uint32)]


class RenderStats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("waves", C.c_uint32), ("samples_accumulated", C.c_uint32)]


class TraceConfig(C.Structure):
    _fields_ = [("block", C.c_uint32), ("short_stack", C.c_uint32), ("refill_min", C.c_uint32),
                ("postpone_min", C.c_uint32), ("sort_bits", C.c_uint32)]

    def as_dict(self):
        return dict(block=self.block, short_stack=self.short_stack, refill_min=self.refill_min,
                    postpone_min=self.postpone_min, sort_bits=self.sort_bits)


RASTER_VERTEX_DTYPE = np.dtype([("pos", "<f4", 2), ("color", "<f4", 3), ("uv", "<f4", 2)])
# the reference renderer's quad (src/Renderer/Renderer.cpp:153-157, 175)
REFERENCE_QUAD = np.array([((-0.5, -0.5), (1.0, 0.0, 0.0), (1.0, 0.0)), ((0.5, -0.5), (0.0, 1.0, 0.0), (0.0, 0.0)),
                           ((0.5, 0.5), (0.0, 0.0, 1.0), (0.0, 1.0)), ((-0.5, 0.5), (1.0, 1.0, 1.0), (1.0, 1.0))],
                          RASTER_VERTEX_DTYPE)
REFERENCE_QUAD_INDICES = np.array([0, 1, 2, 2, 3, 0], np.uint16)


class RasterDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("model", C.c_float * 16), ("view", C.c_float * 16),
                ("proj", C.c_float * 16), ("clear", C.c_float * 4), ("cull_back", C.c_uint32)]


def raster_uniforms(time_s: float, aspect: float = 1920.0 / 1080.0):
    """The reference renderer's model, view and proj matrices at time t
    (column-major float32 arrays of 16)."""
    m, v, p = (np.zeros(16, np.float32) for _ in range(3))
    rc = load().fnd_rt_raster_uniforms(C.c_float(time_s), C.c_float(aspect), _ptr(m), _ptr(v), _ptr(p))
    if rc != 0:
        raise FndError(rc, "fnd_rt_raster_uniforms: invalid arguments")
    return m, v, p


class TuneEntry(C.Structure):
    _fields_ = [("config", TraceConfig), ("ms", C.c_float)]


class BatchJobDesc(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("rays", C.c_void_p), ("out", C.c_void_p), ("n", C.c_uint32),
                ("kind", C.c_uint32)]


QUERY_CLOSEST, QUERY_ANY = 0, 1
BATCH_NO_GRAPH = 1


class CacheDesc(C.Structure):
    _fields_ = [("train_paths", C.c_uint32), ("train_steps", C.c_uint32), ("batch", C.c_uint32),
                ("learning_rate", C.c_float), ("specular_alpha", C.c_float), ("flags", C.c_uint32),
                ("seed", C.c_uint64), ("weight_average", C.c_float)]


class CacheStats(C.Structure):
    _fields_ = [("steps", C.c_uint64), ("samples_last", C.c_uint64), ("queries_last", C.c_uint64),
                ("loss_last", C.c_double)]


class TraceStats(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("node_fetches", C.c_uint64), ("tri_tests", C.c_uint64),
                ("warp_node_steps", C.c_uint64), ("warp_tri_steps", C.c_uint64)]


# every symbol include/fnd_rt.h declares, with (restype, argtypes)
_P, _U32, _I32, _SZ = C.c_void_p, C.c_uint32, C.c_int, C.c_size_t
SIGNATURES = {
    "fnd_rt_create": (_I32, [_P, _P]),
    "fnd_rt_destroy": (_I32, [_P]),
    "fnd_rt_last_error": (C.c_char_p, [_P]),
    "fnd_rt_sync": (_I32, [_P]),
    "fnd_rt_stream": (_P, [_P]),
    "fnd_rt_host_alloc": (_I32, [_SZ, _P]),
    "fnd_rt_host_free": (_I32, [_P]),
    "fnd_rt_scene_upload": (_I32, [_P, _P, _U32, _P, _U32, _P, _P]),
    "fnd_rt_scene_info_get": (_I32, [_P, _P]),
    "fnd_rt_scene_destroy": (_I32, [_P]),
    "fnd_rt_trace_closest": (_I32, [_P, _P, _P, _U32, _P, _I32]),
    "fnd_rt_trace_any": (_I32, [_P, _P, _P, _U32, _P, _I32]),
    "fnd_rt_trace_closest_stats": (_I32, [_P, _P, _P, _U32, _P, _I32, _P]),
    "fnd_rt_trace_closest_noalloc": (_I32, [_P, _P, _U32, _P, _P]),
    "fnd_rt_scene_set_materials": (_I32, [_P, _P, _U32, _P, _U32]),
    "fnd_rt_scene_set_lights": (_I32, [_P, _P, _U32]),
    "fnd_rt_render": (_I32, [_P, _P, _P, _P, _I32]),
    "fnd_rt_render_stats_get": (_I32, [_P, _P]),
    "fnd_rt_tonemap": (_I32, [_P, _P, _U32, _U32, _I32, C.c_float, _U32, _P, _I32]),
    "fnd_rt_raster_uniforms": (_I32, [C.c_float, C.c_float, _P, _P, _P]),
    "fnd_rt_instances_upload": (_I32, [_P, _P, _U32, _P]),
    "fnd_rt_raster_draw": (_I32, [_P, _P, _P, _U32, _P, _U32, _P, _U32, _U32, _P, _I32]),
    "fnd_rt_set_trace_config": (_I32, [_P, _P]),
    "fnd_rt_get_trace_config": (_I32, [_P, _P]),
    "fnd_rt_tune": (_I32, [_P, _P, _P, _U32, _U32, _U32, _P, _U32, _P, _P]),
    "fnd_rt_batch_create": (_I32, [_P, _P, _U32, _U32, _P]),
    "fnd_rt_batch_launch": (_I32, [_P]),
    "fnd_rt_batch_tune": (_I32, [_P, _U32, _P, _U32, _P, _P]),
    "fnd_rt_batch_destroy": (_I32, [_P]),
    "fnd_rt_cache_create": (_I32, [_P, _P, _P]),
    "fnd_rt_cache_destroy": (_I32, [_P]),
    "fnd_rt_cache_stats_get": (_I32, [_P, _P]),
    "fnd_rt_cache_get_weights": (_I32, [_P, _P, _U32]),
    "fnd_rt_cache_set_weights": (_I32, [_P, _P, _U32]),
    "fnd_rt_cache_save": (_I32, [_P, C.c_char_p]),
    "fnd_rt_cache_load": (_I32, [_P, C.c_char_p]),
    "fnd_rt_cache_eval": (_I32, [_P, _P, _U32, _P]),
    "fnd_rt_cache_gradient": (_I32, [_P, _P, _P, _U32, _P, _P]),
    "fnd_rt_cache_adam_step": (_I32, [_P, _P, C.c_float]),
    "fnd_rt_cache_encode": (_I32, [_P, _P, _U32, _P]),
}

_lib = None


def load(path: str | None = None):
    """Loads libfnd_rt.so (built by foundation_gb300._build.build())."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FndError(-8, f"native library not built: {p} (run __graft_entry__.build())")
    L = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = L
    return L


def _check(rc: int, ctx=None):
    if rc != FND_OK:
        msg = load().fnd_rt_last_error(ctx)
        raise FndError(rc, msg.decode() if msg else "")


def _is_device(a) -> bool:
    return hasattr(a, "data_ptr") and getattr(a, "is_cuda", False)


def _ptr(a):
    if _is_device(a):
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)


class Context:
    """One device + one CUDA stream (``stream``: an int cudaStream_t handle, or
    None for a private non-blocking stream)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self._h = None
        d = _Desc(ABI_VERSION, device, C.c_void_p(stream) if stream else None, 0)
        h = C.c_void_p()
        _check(load().fnd_rt_create(C.byref(d), C.byref(h)))
        self._h = h
        self.device = device
        self._scenes = weakref.WeakSet()

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return int(load().fnd_rt_stream(self._h) or 0)

    def sync(self):
        _check(load().fnd_rt_sync(self._h), self._h)

    def close(self):
        """Destroys the scenes still open on this context, then the context."""
        if self._h is not None:
            # two-level scenes first: they hold their bottom levels
            for sc in sorted(self._scenes, key=lambda x: not getattr(x, "two_level", False)):
                sc.close()
            rc = load().fnd_rt_destroy(self._h)
            if rc == -1:  # refused (scenes still alive): the context is intact
                _check(rc, self._h)
            self._h = None  # freed; a failure message is in the global slot
            _check(rc, None)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def instances(self, instances) -> "InstanceScene":
        """Two-level scene: instances = [(scene, transform (3, 4) object->world, prim_offset)]."""
        return InstanceScene(self, instances)

    def upload(self, verts, idx, bins: int = 32, max_leaf: int = 4, threads: int = 0,
               spatial_splits: bool = False, traversal_cost: float = 0.0, gpu_build: bool = False,
               split_budget: float = 0.0, margin_scale: float = 0.0, sah_collapse: bool = False,
               collapse_tri_cost: float = 0.0, cluster: bool = False, cluster_radius: int = 0,
               node_width: int = 0) -> "Scene":
        """cluster (with gpu_build): the binary tree by locally-ordered clustering
        with search radius cluster_radius (1..64; 0: 2) instead of the Karras
        hierarchy. node_width: children per wide node (2..8; 0: 8)."""
        return Scene(self, verts, idx, bins, max_leaf, threads, spatial_splits, traversal_cost, gpu_build,
                     split_budget, margin_scale, sah_collapse, collapse_tri_cost, cluster, cluster_radius,
                     node_width)

    def render(self, scene: "Scene", width: int, height: int, spp: int, camera: dict, *, max_depth: int = 8,
               rr_start: int = 3, seed: int = 1, sky=(0.0, 0.0, 0.0), sun_dir=(0.0, 0.0, 0.0),
               sun_irradiance=(0.0, 0.0, 0.0), accumulate: bool = False, wave_paths: int = 0, out=None,
               cache: bool = False, tail_paths: int = 0, wavefront: bool = False, train_only: bool = False):
        """Path-traces spp samples per pixel. Host: returns (height, width, 3)
        float32 mean radiance. Device: out is a CUDA tensor of
        width*height*3 floats, filled asynchronously. tail_paths: threshold
        of the tail megakernel (0: automatic); wavefront: never use it;
        train_only (with cache): only train the cache, render nothing."""
        cam = _Camera((C.c_float * 3)(*camera["eye"]), (C.c_float * 3)(*camera["target"]),
                      (C.c_float * 3)(*camera.get("up", (0.0, 1.0, 0.0))), camera.get("vfov_deg", 45.0))
        flags = (RENDER_ACCUMULATE if accumulate else 0) | (RENDER_CACHE if cache else 0) | \
            (RENDER_WAVEFRONT if wavefront else 0) | (RENDER_TRAIN_ONLY if train_only else 0)
        d = _RenderDesc(width, height, spp, max_depth, rr_start, flags, seed, cam,
                        (C.c_float * 3)(*sky), (C.c_float * 3)(*sun_dir), (C.c_float * 3)(*sun_irradiance),
                        wave_paths, tail_paths)
        if train_only:
            _check(load().fnd_rt_render(self._h, scene.handle, C.byref(d), None, FND_MEM_DEVICE), self._h)
            return None
        if out is not None and _is_device(out):
            _check(load().fnd_rt_render(self._h, scene.handle, C.byref(d), _ptr(out), FND_MEM_DEVICE), self._h)
            return out
        img = np.empty((height, width, 3), np.float32) if out is None else out
        _check(load().fnd_rt_render(self._h, scene.handle, C.byref(d), _ptr(img), FND_MEM_HOST), self._h)
        return img

    def tonemap(self, rgb, width: int, height: int, exposure: float = 1.0, mode: int = 2, out=None):
        """Linear RGB (host array or CUDA tensor of width*height*3 floats) to
        R8G8B8A8_UNORM pixels: (height, width, 4) uint8 on the host, or into
        `out` (a CUDA uint8 tensor of width*height*4), asynchronously."""
        mem_in = FND_MEM_DEVICE if _is_device(rgb) else FND_MEM_HOST
        if mem_in == FND_MEM_HOST:
            rgb = np.ascontiguousarray(rgb, np.float32)
        if out is not None and _is_device(out):
            _check(load().fnd_rt_tonemap(self._h, _ptr(rgb), width, height, mem_in, exposure, mode, _ptr(out),
                                         FND_MEM_DEVICE), self._h)
            return out
        img = np.empty((height, width, 4), np.uint8)
        _check(load().fnd_rt_tonemap(self._h, _ptr(rgb), width, height, mem_in, exposure, mode, _ptr(img),
                                     FND_MEM_HOST), self._h)
        return img

    def raster_draw(self, width: int, height: int, model, view, proj, texture, verts=None, indices=None,
                    clear=(0.0, 0.0, 0.0, 1.0), cull_back: bool = True, out=None):
        """The raster pass (the reference renderer's DrawIndexed): texture is a
        (h, w, 4) uint8 array; verts / indices default to the reference quad.
        Returns (height, width, 4) uint8, or fills the CUDA tensor `out`."""
        verts = REFERENCE_QUAD if verts is None else np.ascontiguousarray(verts, RASTER_VERTEX_DTYPE)
        indices = REFERENCE_QUAD_INDICES if indices is None else np.ascontiguousarray(indices, np.uint16)
        tex = np.ascontiguousarray(texture, np.uint8)
        d = RasterDesc(width, height, (C.c_float * 16)(*model), (C.c_float * 16)(*view), (C.c_float * 16)(*proj),
                       (C.c_float * 4)(*clear), 1 if cull_back else 0)
        args = (self._h, C.byref(d), _ptr(verts), len(verts), _ptr(indices), len(indices), _ptr(tex), tex.shape[1],
                tex.shape[0])
        if out is not None and _is_device(out):
            _check(load().fnd_rt_raster_draw(*args, _ptr(out), FND_MEM_DEVICE), self._h)
            return out
        img = np.empty((height, width, 4), np.uint8)
        _check(load().fnd_rt_raster_draw(*args, _ptr(img), FND_MEM_HOST), self._h)
        return img

    # ---- launch shape -------------------------------------------------
    def set_trace_config(self, block: int = 128, short_stack: int = 8, refill_min: int = 8, postpone_min: int = 0,
                         sort_bits: int = 0):
        c = TraceConfig(block, short_stack, refill_min, postpone_min, sort_bits)
        _check(load().fnd_rt_set_trace_config(self._h, C.byref(c)), self._h)

    def trace_config(self) -> dict:
        c = TraceConfig()
        _check(load().fnd_rt_get_trace_config(self._h, C.byref(c)), self._h)
        return c.as_dict()

    def tune(self, scene: "Scene", rays, kind: int = QUERY_CLOSEST, reps: int = 3):
        """Times every launch shape on device rays; returns (best, table)."""
        n = rays.numel() * rays.element_size() // 32
        table = (TuneEntry * 128)()
        tn = C.c_uint32()
        best = TraceConfig()
        _check(load().fnd_rt_tune(self._h, scene.handle, _ptr(rays), n, kind, reps, table, 128, C.byref(tn),
                                  C.byref(best)), self._h)
        return best.as_dict(), [dict(table[i].config.as_dict(), ms=table[i].ms) for i in range(tn.value)]

    # ---- radiance cache -------------------------------------------------
    def cache_create(self, scene: "Scene", train_paths: int = 65536, train_steps: int = 4, batch: int = 16384,
                     learning_rate: float = 1e-2, specular_alpha: float = 0.1, seed: int = 1,
                     weight_average: float = 0.0):
        d = CacheDesc(train_paths, train_steps, batch, learning_rate, specular_alpha, 0, seed, weight_average)
        _check(load().fnd_rt_cache_create(self._h, scene.handle, C.byref(d)), self._h)

    def cache_destroy(self):
        _check(load().fnd_rt_cache_destroy(self._h), self._h)

    def cache_stats(self) -> dict:
        st = CacheStats()
        _check(load().fnd_rt_cache_stats_get(self._h, C.byref(st)), self._h)
        return {k: getattr(st, k) for k, _ in st._fields_}

    def cache_weights(self) -> np.ndarray:
        w = np.empty(CACHE_NUM_PARAMS, np.float32)
        _check(load().fnd_rt_cache_get_weights(self._h, _ptr(w), len(w)), self._h)
        return w

    def cache_set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        _check(load().fnd_rt_cache_set_weights(self._h, _ptr(w), len(w)), self._h)

    def cache_save(self, path: str):
        _check(load().fnd_rt_cache_save(self._h, str(path).encode()), self._h)

    def cache_load(self, path: str):
        _check(load().fnd_rt_cache_load(self._h, str(path).encode()), self._h)

    def cache_eval(self, features) -> np.ndarray:
        f = np.ascontiguousarray(features, np.float32).reshape(-1, CACHE_NUM_FEATURES)
        out = np.empty((len(f), 3), np.float32)
        _check(load().fnd_rt_cache_eval(self._h, _ptr(f), len(f), _ptr(out)), self._h)
        return out

    def cache_gradient(self, features, targets):
        f = np.ascontiguousarray(features, np.float32).reshape(-1, CACHE_NUM_FEATURES)
        t = np.ascontiguousarray(targets, np.float32).reshape(-1, 3)
        g = np.empty(CACHE_NUM_PARAMS, np.float32)
        loss = C.c_double()
        _check(load().fnd_rt_cache_gradient(self._h, _ptr(f), _ptr(t), len(f), _ptr(g), C.byref(loss)), self._h)
        return g, loss.value

    def cache_encode(self, points) -> np.ndarray:
        """points: (n, 13) position, outgoing direction, normal, roughness,
        albedo -> (n, 96) network input features."""
        p = np.ascontiguousarray(points, np.float32).reshape(-1, 13)
        out = np.empty((len(p), CACHE_NUM_FEATURES), np.float32)
        _check(load().fnd_rt_cache_encode(self._h, _ptr(p), len(p), _ptr(out)), self._h)
        return out

    def cache_adam_step(self, grad, learning_rate: float = 1e-2):
        g = np.ascontiguousarray(grad, np.float32)
        _check(load().fnd_rt_cache_adam_step(self._h, _ptr(g), learning_rate), self._h)

    def render_stats(self) -> dict:
        st = RenderStats()
        _check(load().fnd_rt_render_stats_get(self._h, C.byref(st)), self._h)
        return {k: getattr(st, k) for k, _ in st._fields_}


class Scene:
    def __init__(self, ctx: Context, verts, idx, bins=32, max_leaf=4, threads=0, spatial_splits=False,
                 traversal_cost=0.0, gpu_build=False, split_budget=0.0, margin_scale=0.0, sah_collapse=False,
                 collapse_tri_cost=0.0, cluster=False, cluster_radius=0, node_width=0):
        self._h = None
        self.ctx = ctx
        v = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 3)
        f = np.ascontiguousarray(idx, dtype=np.uint32).reshape(-1, 3)
        flags = ((BVH_SPATIAL_SPLITS if spatial_splits else 0) | (BVH_GPU_BUILD if gpu_build else 0) |
                 (BVH_SAH_COLLAPSE if sah_collapse else 0) | (BVH_GPU_CLUSTER if cluster else 0) |
                 BVH_CLUSTER_RADIUS(cluster_radius) | BVH_NODE_WIDTH(node_width))
        bd = _BvhDesc(bins, max_leaf, threads, flags, traversal_cost, split_budget, margin_scale, collapse_tri_cost)
        h = C.c_void_p()
        _check(load().fnd_rt_scene_upload(ctx.handle, _ptr(v), len(v), _ptr(f), len(f), C.byref(bd), C.byref(h)),
               ctx.handle)
        self._h = h
        ctx._scenes.add(self)

    @property
    def handle(self):
        return self._h

    def set_materials(self, tri_material, materials):
        tm = np.ascontiguousarray(tri_material, dtype=np.uint32)
        mats = np.ascontiguousarray(materials, dtype=MATERIAL_DTYPE)
        _check(load().fnd_rt_scene_set_materials(self._h, _ptr(tm), len(tm), _ptr(mats), len(mats)), self.ctx.handle)

    def set_lights(self, lights):
        ls = np.ascontiguousarray(lights, dtype=LIGHT_DTYPE)
        _check(load().fnd_rt_scene_set_lights(self._h, _ptr(ls) if len(ls) else None, len(ls)), self.ctx.handle)

    def info(self) -> dict:
        out = SceneInfo()
        _check(load().fnd_rt_scene_info_get(self._h, C.byref(out)))
        return out.as_dict()

    def close(self):
        if self._h is not None:
            _check(load().fnd_rt_scene_destroy(self._h), self.ctx.handle)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _trace(self, rays, out, any_hit: bool, stats: bool = False):
        dev = _is_device(rays)
        if dev != _is_device(out):
            raise FndError(-1, "rays and output must both be host or both be device buffers")
        n = (rays.numel() * rays.element_size() if dev else rays.nbytes) // 32
        mem = FND_MEM_DEVICE if dev else FND_MEM_HOST
        L = load()
        if stats:
            st = TraceStats()
            _check(L.fnd_rt_trace_closest_stats(self.ctx.handle, self._h, _ptr(rays), n, _ptr(out), mem,
                                                C.byref(st)), self.ctx.handle)
            return dict(rays=st.rays, node_fetches=st.node_fetches, tri_tests=st.tri_tests,
                        warp_node_steps=st.warp_node_steps, warp_tri_steps=st.warp_tri_steps)
        fn = L.fnd_rt_trace_any if any_hit else L.fnd_rt_trace_closest
        _check(fn(self.ctx.handle, self._h, _ptr(rays), n, _ptr(out), mem), self.ctx.handle)
        return None

    def closest(self, rays, out=None, stats: bool = False):
        """Closest hit. Host: rays (n, 8) float32 -> structured (prim, t)
        array. Device: rays / out are CUDA tensors (out: n*2 int32/float32
        words); asynchronous on the context stream."""
        if _is_device(rays):
            if out is None:
                raise FndError(-1, "device call needs an output tensor")
            st = self._trace(rays, out, False, stats)
            return st if stats else out
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        out = np.empty(len(rays), HIT_DTYPE) if out is None else out
        st = self._trace(rays, out, False, stats)
        return (out, st) if stats else out

    def any(self, rays, out=None):
        if _is_device(rays):
            if out is None:
                raise FndError(-1, "device call needs an output tensor")
            self._trace(rays, out, True)
            return out
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        out = np.empty(len(rays), np.uint8) if out is None else out
        self._trace(rays, out, True)
        return out


class PinnedBuffer:
    """Page-locked host memory from fnd_rt_host_alloc, viewed as numpy."""

    def __init__(self, nbytes: int):
        p = C.c_void_p()
        _check(load().fnd_rt_host_alloc(nbytes, C.byref(p)))
        self._p = p
        self.nbytes = nbytes

    def view(self, dtype, shape):
        buf = (C.c_char * self.nbytes).from_address(self._p.value)
        return np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def __del__(self):
        if getattr(self, "_p", None):
            load().fnd_rt_host_free(self._p)
            self._p = None


class _Instance(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("transform", C.c_float * 12), ("prim_offset", C.c_uint32)]


class InstanceScene(Scene):
    """Instances of uploaded scenes under a top-level tree (fnd_rt_instances_upload).
    Traced with closest() / any(); hit ids are prim_offset + bottom-level ids."""

    two_level = True

    def __init__(self, ctx: Context, instances):
        self.ctx = ctx
        self._h = None
        arr = (_Instance * max(1, len(instances)))()
        self._blas = []
        for i, (scene, m, off) in enumerate(instances):
            m = np.asarray(m, np.float32).reshape(3, 4)
            arr[i] = _Instance(scene.handle.value, (C.c_float * 12)(*m.ravel()), int(off))
            self._blas.append(scene)
        h = C.c_void_p()
        _check(load().fnd_rt_instances_upload(ctx.handle, arr, len(instances), C.byref(h)), ctx.handle)
        self._h = h
        ctx._scenes.add(self)


class Batch:
    """Batched traversal: jobs = [(scene, rays, out, kind)] with CUDA tensors
    (rays: n x 8 float32; out: 2n int32 words for closest, n uint8 for any).
    One persistent launch over all jobs, captured in a CUDA graph."""

    def __init__(self, ctx: Context, jobs, graph: bool = True):
        self.ctx = ctx
        self._keep = jobs  # keeps the tensors alive
        arr = (BatchJobDesc * len(jobs))()
        for i, (scene, rays, out, kind) in enumerate(jobs):
            n = rays.numel() * rays.element_size() // 32
            arr[i] = BatchJobDesc(scene.handle.value, rays.data_ptr(), out.data_ptr(), n, kind)
        h = C.c_void_p()
        _check(load().fnd_rt_batch_create(ctx.handle, arr, len(jobs), 0 if graph else BATCH_NO_GRAPH, C.byref(h)),
               ctx.handle)
        self._h = h
        self.total_rays = sum(r.numel() * r.element_size() // 32 for _, r, _, _ in jobs)

    def launch(self):
        _check(load().fnd_rt_batch_launch(self._h), self.ctx.handle)

    def tune(self, reps: int = 2):
        table = (TuneEntry * 128)()
        tn = C.c_uint32()
        best = TraceConfig()
        _check(load().fnd_rt_batch_tune(self._h, reps, table, 128, C.byref(tn), C.byref(best)), self.ctx.handle)
        return best.as_dict(), [dict(table[i].config.as_dict(), ms=table[i].ms) for i in range(tn.value)]

    def close(self):
        if getattr(self, "_h", None) is not None:
            _check(load().fnd_rt_batch_destroy(self._h), self.ctx.handle)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
