"""TEST INFRASTRUCTURE ONLY: ctypes front end of the scalar CPU oracle.

Imported by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg,
always as the checker or the timed CPU baseline, never as a product path.
Parity against the reference is unpinned: mos9527/Foundation contains no
ray-tracing code (its only pass is a raster draw, src/Renderer/Renderer.cpp
:312-366). The oracle restates published methods (binned SAH, Wald 2007;
watertight intersection, Woop/Benthin/Wald 2013; PCG32, O'Neill 2014) and is
pinned by hand-derived known-answer tests and brute-force cross-checks.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "librt_oracle.so")
SOURCES = ["rt_oracle.cpp", "pt_oracle.cpp", "mlp_oracle.cpp", "raster_oracle.cpp"]
HEADERS = ["rt_oracle.h", "oracle_common.hpp", "rt_oracle_internal.hpp"]
CXXFLAGS = ["-O3", "-std=c++20", "-ffp-contract=off", "-fPIC", "-shared", "-pthread"]

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (portable flags, no FMA contraction)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, h) for h in HEADERS]
    if not force and os.path.exists(LIB_PATH):
        t = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", *CXXFLAGS, "-o", tmp, *srcs])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P, U32, U64, F = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float
        L.orc_bvh_build.restype = P
        L.orc_bvh_build.argtypes = [P, U32, P, U32, U32, U32]
        L.orc_bvh_free.argtypes = [P]
        L.orc_bvh_stats.argtypes = [P, P, P]
        L.orc_bvh_validate.argtypes = [P]
        L.orc_bvh_validate.restype = C.c_int
        L.orc_bvh_margin.argtypes = [P]
        L.orc_bvh_margin.restype = F
        L.orc_trace_closest.argtypes = [P, P, U64, P, U32, P]
        L.orc_trace_any.argtypes = [P, P, U64, P, U32, P]
        L.orc_brute_closest.argtypes = [P, U32, P, U32, P, U64, P, U32]
        L.orc_brute_any.argtypes = [P, U32, P, U32, P, U64, P, U32]
        L.orc_intersect1.argtypes = [P, P, P]
        L.orc_intersect1.restype = C.c_int
        L.orc_pcg32_fill.argtypes = [U64, U64, P, U64]
        L.orc_time_build_ms.argtypes = [P, U32, P, U32, U32, U32]
        L.orc_time_build_ms.restype = C.c_double
        L.orc_pt_render.argtypes = [P, P, P, U32, P, U32, P, U32, U32, U32, U32, U32, U64, P, U32, U32, U32, U32,
                                    U32, P]
        L.orc_mlp_num_params.restype = U64
        L.orc_mlp_forward_backward.argtypes = [P, P, P, U64, C.c_int, P, P, P, P]
        L.orc_adam_step.argtypes = [P, P, P, P, U64, U64, C.c_double]
        L.orc_nrc_encode.argtypes = [P, P, P, P]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


HIT_DTYPE = np.dtype([("prim", np.uint32), ("t", np.float32)])


class OracleBVH:
    """Binary binned-SAH BVH of the oracle (32 bins, <= 4 triangles/leaf)."""

    def __init__(self, verts, idx, bins: int = 32, max_leaf: int = 4):
        self.verts = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 3)
        self.idx = np.ascontiguousarray(idx, dtype=np.uint32).reshape(-1, 3)
        self._h = lib().orc_bvh_build(_ptr(self.verts), len(self.verts), _ptr(self.idx), len(self.idx), bins,
                                      max_leaf)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_bvh_free(self._h)
            self._h = None

    def stats(self) -> dict:
        out = np.zeros(4, np.uint64)
        sah = C.c_double()
        lib().orc_bvh_stats(self._h, _ptr(out), C.byref(sah))
        return dict(nodes=int(out[0]), leaves=int(out[1]), depth=int(out[2]), max_leaf=int(out[3]),
                    sah=sah.value, margin=float(lib().orc_bvh_margin(self._h)))

    def validate(self) -> int:
        return int(lib().orc_bvh_validate(self._h))

    def closest(self, rays, threads: int = 0, with_stats: bool = False):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        hits = np.empty(len(rays), HIT_DTYPE)
        st = np.zeros(2, np.uint64)
        lib().orc_trace_closest(self._h, _ptr(rays), len(rays), _ptr(hits), threads, _ptr(st))
        return (hits, dict(node_fetches=int(st[0]), tri_tests=int(st[1]))) if with_stats else hits

    def any(self, rays, threads: int = 0, with_stats: bool = False):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        out = np.empty(len(rays), np.uint8)
        st = np.zeros(2, np.uint64)
        lib().orc_trace_any(self._h, _ptr(rays), len(rays), _ptr(out), threads, _ptr(st))
        return (out, dict(node_fetches=int(st[0]), tri_tests=int(st[1]))) if with_stats else out


def brute_closest(verts, idx, rays, threads: int = 0):
    verts = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 3)
    idx = np.ascontiguousarray(idx, dtype=np.uint32).reshape(-1, 3)
    rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
    hits = np.empty(len(rays), HIT_DTYPE)
    lib().orc_brute_closest(_ptr(verts), len(verts), _ptr(idx), len(idx), _ptr(rays), len(rays), _ptr(hits),
                            threads)
    return hits


def brute_any(verts, idx, rays, threads: int = 0):
    verts = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 3)
    idx = np.ascontiguousarray(idx, dtype=np.uint32).reshape(-1, 3)
    rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
    out = np.empty(len(rays), np.uint8)
    lib().orc_brute_any(_ptr(verts), len(verts), _ptr(idx), len(idx), _ptr(rays), len(rays), _ptr(out), threads)
    return out


def intersect1(ray, tri):
    """One ray (8 floats) vs one triangle (9 floats) -> (hit, t, U, V, W, det)."""
    r = np.ascontiguousarray(ray, dtype=np.float32).reshape(8)
    v = np.ascontiguousarray(tri, dtype=np.float32).reshape(9)
    out = np.zeros(5, np.float32)
    h = lib().orc_intersect1(_ptr(r), _ptr(v), _ptr(out))
    return bool(h), float(out[0]), out[1:].copy()


def pcg32(seed: int, seq: int, n: int) -> np.ndarray:
    out = np.empty(n, np.uint32)
    lib().orc_pcg32_fill(seed, seq, _ptr(out), n)
    return out


def time_build_ms(verts, idx, bins: int = 32, max_leaf: int = 4) -> float:
    verts = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 3)
    idx = np.ascontiguousarray(idx, dtype=np.uint32).reshape(-1, 3)
    return float(lib().orc_time_build_ms(_ptr(verts), len(verts), _ptr(idx), len(idx), bins, max_leaf))


def pt_render(bvh: OracleBVH, tri_material, materials, lights, camera: dict, width: int, height: int, spp: int, *,
              max_depth: int = 8, rr_start: int = 3, seed: int = 1, sky=(0, 0, 0), sun_dir=(0, 0, 0),
              sun_irradiance=(0, 0, 0), crop=None, threads: int = 0) -> np.ndarray:
    """FP64 path-traced crop (x0, y0, w, h) of a width x height image:
    (h, w, 3) float64 mean radiance. materials / lights: fnd_material /
    fnd_quad_light records (numpy structured arrays)."""
    x0, y0, cw, ch = crop if crop else (0, 0, width, height)
    tm = np.ascontiguousarray(tri_material, dtype=np.uint32) if tri_material is not None else None
    mats = np.ascontiguousarray(materials)
    ls = np.ascontiguousarray(lights)
    cam = np.array([*camera["eye"], *camera["target"], *camera.get("up", (0, 1, 0)), camera.get("vfov_deg", 45.0)],
                   np.float64)
    env = np.array([*sky, *sun_dir, *sun_irradiance], np.float64)
    out = np.zeros((ch, cw, 3), np.float64)
    lib().orc_pt_render(bvh._h, _ptr(tm) if tm is not None else None, _ptr(mats), len(mats),
                        _ptr(ls) if len(ls) else None, len(ls), _ptr(cam), width, height, spp, max_depth, rr_start,
                        seed, _ptr(env), x0, y0, cw, ch, threads, _ptr(out))
    return out


MLP_DIMS = (96, 64, 64, 64, 64, 64, 3)


def mlp_num_params() -> int:
    return int(lib().orc_mlp_num_params())


def mlp_forward_backward(w, x, t=None, emulate_bf16: bool = True, grad: bool = True, fixed_den=None):
    """FP64 radiance-cache network: returns (y (B x 3), loss, dW) — loss / dW
    None without targets. fixed_den (B x 3) replaces the loss denominators
    y^2 + 0.01 by constants."""
    w = np.ascontiguousarray(w, np.float32)
    x = np.ascontiguousarray(x, np.float32).reshape(-1, 96)
    B = len(x)
    y = np.zeros((B, 3), np.float64)
    loss = C.c_double()
    dw = np.zeros(len(w), np.float64) if (t is not None and grad) else None
    tt = np.ascontiguousarray(t, np.float32).reshape(-1, 3) if t is not None else None
    fd = np.ascontiguousarray(fixed_den, np.float64).reshape(-1, 3) if fixed_den is not None else None
    lib().orc_mlp_forward_backward(_ptr(w), _ptr(x), _ptr(tt) if tt is not None else None, B, int(emulate_bf16),
                                   _ptr(y), C.byref(loss) if t is not None else None,
                                   _ptr(dw) if dw is not None else None,
                                   _ptr(fd) if fd is not None else None)
    return y, (loss.value if t is not None else None), dw


def adam_step(w, m, v, g, step: int, lr: float):
    """In-place FP64 Adam on float64 arrays."""
    lib().orc_adam_step(_ptr(w), _ptr(m), _ptr(v), _ptr(np.ascontiguousarray(g, np.float64)), len(w), step, lr)


def nrc_encode(p, wo, n, rough, albedo, lo, hi) -> np.ndarray:
    rec = np.array([*p, *wo, *n, rough, *albedo], np.float32)
    out = np.zeros(96, np.float32)
    lo = np.asarray(lo, np.float32)
    hi = np.asarray(hi, np.float32)
    lib().orc_nrc_encode(_ptr(rec), _ptr(lo), _ptr(hi), _ptr(out))
    return out


# ---- display encoding (foundation_gb300/csrc/pt/tonemap.cu) -----------------
def tonemap_rgba8(rgb, exposure: float = 1.0, mode: int = 2) -> np.ndarray:
    """Linear RGB (h, w, 3) -> R8G8B8A8 (h, w, 4): exposure, tone curve (0
    clamp, 1 Reinhard x/(1+x), 2 the ACES fit of Narkowicz 2015:
    x(2.51x+0.03)/(x(2.43x+0.59)+0.14)), clamp to [0,1], sRGB transfer
    function (IEC 61966-2-1), round to 8 bits; alpha 255. Float32 operations
    in the device's order except the power, evaluated in float64 (so codes
    agree to within one step)."""
    f = np.float32
    x = np.asarray(rgb, np.float32) * f(exposure)
    pos = x > 0
    x = np.where(pos, x, f(0))
    with np.errstate(invalid="ignore", over="ignore"):
        if mode == 1:
            x = x / (f(1) + x)
        elif mode == 2:
            x = (x * (f(2.51) * x + f(0.03))) / (x * (f(2.43) * x + f(0.59)) + f(0.14))
    with np.errstate(invalid="ignore"):
        x = np.fmin(x, f(1)).astype(np.float32)  # drops NaN (inf / inf of the curves) like fminf
    lin = f(12.92) * x
    gam = (f(1.055) * np.power(x.astype(np.float64), 1.0 / 2.4).astype(np.float32) - f(0.055)).astype(np.float32)
    s = np.where(x <= f(0.0031308), lin, gam).astype(np.float32)
    q = np.clip(np.floor(s * f(255) + f(0.5)), 0, 255).astype(np.uint8)
    q = np.where(pos, q, 0).astype(np.uint8)
    a = np.full(q.shape[:-1] + (1,), 255, np.uint8)
    return np.concatenate([q, a], -1)


# ---- raster pass (raster_oracle.cpp) -----------------------------------------
def raster_draw(width: int, height: int, model, view, proj, texture, verts, indices, clear=(0.0, 0.0, 0.0, 1.0),
                cull_back: bool = True) -> np.ndarray:
    """The scalar raster pass: verts (n, 7) float32 (pos xy, colour rgb, uv),
    indices uint16, texture (h, w, 4) uint8 -> (height, width, 4) uint8."""
    L = lib()
    f = L.orc_raster_draw
    f.restype = None
    P = C.c_void_p
    f.argtypes = [C.c_uint32, C.c_uint32, P, P, P, P, C.c_int, P, C.c_uint32, P, C.c_uint32, P, C.c_uint32,
                  C.c_uint32, P]
    m, v, p = (np.ascontiguousarray(x, np.float32) for x in (model, view, proj))
    cl = np.ascontiguousarray(clear, np.float32)
    vt = np.ascontiguousarray(verts, np.float32).reshape(-1, 7)
    ix = np.ascontiguousarray(indices, np.uint16)
    tex = np.ascontiguousarray(texture, np.uint8)
    out = np.zeros((height, width, 4), np.uint8)
    ptr = lambda a: a.ctypes.data_as(P)  # noqa: E731
    f(width, height, ptr(m), ptr(v), ptr(p), ptr(cl), 1 if cull_back else 0, ptr(vt), len(vt), ptr(ix), len(ix),
      ptr(tex), tex.shape[1], tex.shape[0], ptr(out))
    return out


# ---- two-level scenes (rt_oracle.cpp orc_instances_trace) ---------------------
def instances_trace(levels, instances, rays, any_hit: bool = False, threads: int = 0):
    """levels: [(verts (nv, 3) float32, idx (nt, 3) uint32)]; instances:
    [(level index, transform (3, 4) object->world, prim_offset)]. Returns the
    closest-hit records (prim, t) or the occlusion flags, brute force."""
    L = lib()
    f = L.orc_instances_trace
    f.restype = None
    P = C.c_void_p
    f.argtypes = [P, P, P, P, P, P, P, C.c_uint32, P, C.c_uint64, P, P, C.c_int, C.c_uint32]
    verts, idx, base, count, vb = [], [], [], [], 0
    tb = 0
    for v, ix in levels:
        v = np.asarray(v, np.float32).reshape(-1, 3)
        ix = np.asarray(ix, np.uint32).reshape(-1, 3)
        verts.append(v)
        idx.append(ix + np.uint32(vb))
        base.append(tb)
        count.append(len(ix))
        vb += len(v)
        tb += len(ix)
    verts = np.ascontiguousarray(np.concatenate(verts), np.float32)
    idx = np.ascontiguousarray(np.concatenate(idx), np.uint32)
    base = np.asarray(base, np.uint32)
    count = np.asarray(count, np.uint32)
    lev = np.asarray([i[0] for i in instances], np.uint32)
    tr = np.ascontiguousarray(np.stack([np.asarray(i[1], np.float32).reshape(12) for i in instances]), np.float32)
    off = np.asarray([i[2] for i in instances], np.uint32)
    rays = np.ascontiguousarray(rays, np.float32)
    n = len(rays)
    hits = np.zeros(n, HIT_DTYPE) if not any_hit else None
    occ = np.zeros(n, np.uint8) if any_hit else None
    ptr = lambda a: a.ctypes.data_as(P) if a is not None else None  # noqa: E731
    f(ptr(verts), ptr(idx), ptr(base), ptr(count), ptr(lev), ptr(tr), ptr(off), len(instances), ptr(rays), n,
      ptr(hits), ptr(occ), 1 if any_hit else 0, threads)
    return occ if any_hit else hits
