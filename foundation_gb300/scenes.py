"""Seeded synthetic scenes and ray batches for the path-tracer workloads.

Every generator is deterministic: random numbers come from PCG32 streams
(O'Neill 2014, PCG-XSH-RR 64/32), one stream per object / ray, evaluated
vectorised in numpy with wrapping uint64 arithmetic. Only IEEE-exact
operations (+, -, *, /, sqrt) touch the generated floats, so the same seed
gives the same bits on x86-64 and aarch64 hosts.

The reference renderer has no scene or mesh loader (its only geometry is the
hard-coded 4-vertex quad of src/Renderer/Renderer.cpp:153-157); the scene
shapes follow the workloads the path-tracer pass is measured on:

* ``icosphere_scene`` unit icosphere subdivided 6 times (81,920 tris) plus
                      1,024 random triangles in [-2,2]^3 (seed 0)
* ``camera_rays``     pinhole camera, glm lookAt convention (right-handed,
                      looking down -Z, as src/Renderer/Renderer.cpp:374-380)
* ``cornell_scene``   Cornell box (5 wall quads + 0.25 m^2 light) holding 200
                      icospheres of level 3 (256,012 tris; seed 1)
* ``incoherent_rays`` origins uniform in a box, directions uniform on S^2
* ``soup_scene``      triangle soup in the unit cube, edge lengths
                      log-uniform in [1e-3, 0.1] (seed 2)
* ``terrain_scene``   value-noise heightfield (2237^2 vertices, 9,999,392
                      tris) plus 4,096 level-4 icospheres (20,971,520 tris),
                      sun + sky (seed 3)
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

_MULT = np.uint64(6364136223846793005)
_U64 = np.uint64


class Pcg32Streams:
    """N independent PCG32 generators (one per element of ``seq``)."""

    def __init__(self, seed: int, seq):
        seq = np.asarray(seq, dtype=np.uint64)
        self.inc = (seq << _U64(1)) | _U64(1)
        self.state = np.zeros_like(seq)
        self.next_u32()
        self.state = self.state + _U64(seed & 0xFFFFFFFFFFFFFFFF)
        self.next_u32()

    def next_u32(self, mask=None) -> np.ndarray:
        old = self.state if mask is None else self.state[mask]
        inc = self.inc if mask is None else self.inc[mask]
        new = old * _MULT + inc
        if mask is None:
            self.state = new
        else:
            self.state[mask] = new
        xorshifted = (((old >> _U64(18)) ^ old) >> _U64(27)) & _U64(0xFFFFFFFF)
        rot = (old >> _U64(59)).astype(np.uint64)
        res = (xorshifted >> rot) | (xorshifted << ((_U64(32) - rot) & _U64(31)))
        return (res & _U64(0xFFFFFFFF)).astype(np.uint32)

    def next_f32(self, mask=None) -> np.ndarray:
        """Uniform float32 in [0, 1) from the top 24 bits."""
        return (self.next_u32(mask) >> np.uint32(8)).astype(np.float32) * np.float32(1.0 / 16777216.0)

    def next_f64(self, mask=None) -> np.ndarray:
        return (self.next_u32(mask) >> np.uint32(8)).astype(np.float64) * (1.0 / 16777216.0)


def _exp2_det(y: np.ndarray) -> np.ndarray:
    """2**y in float64 from IEEE-exact ufuncs only (range split + Taylor
    series of exp(f ln2) on f in [0,1)), so the bits do not depend on the
    host's libm or SIMD math library."""
    y = np.asarray(y, dtype=np.float64)
    n = np.floor(y)
    f = (y - n) * 0.6931471805599453
    acc = np.ones_like(f)
    term = np.ones_like(f)
    for k in range(1, 22):
        term = term * f / float(k)
        acc = acc + term
    return np.ldexp(acc, n.astype(np.int64))


# ---------------------------------------------------------------------------
# meshes
# ---------------------------------------------------------------------------

def icosphere(level: int):
    """Unit icosphere: 10*4^L+2 vertices, 20*4^L triangles (float64 verts)."""
    phi = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, phi, 0], [1, phi, 0], [-1, -phi, 0], [1, -phi, 0],
                  [0, -1, phi], [0, 1, phi], [0, -1, -phi], [0, 1, -phi],
                  [phi, 0, -1], [phi, 0, 1], [-phi, 0, -1], [-phi, 0, 1]], dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    v = v / np.sqrt((v * v).sum(1, keepdims=True))
    for _ in range(level):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], 0)
        key = np.minimum(e[:, 0], e[:, 1]) * (len(v) + 1) + np.maximum(e[:, 0], e[:, 1])
        uniq, inv = np.unique(key, return_inverse=True)
        a = uniq // (len(v) + 1)
        b = uniq % (len(v) + 1)
        mid = (v[a] + v[b]) * 0.5
        mid = mid / np.sqrt((mid * mid).sum(1, keepdims=True))
        mid_idx = inv + len(v)
        nf = len(f)
        m01, m12, m20 = mid_idx[:nf], mid_idx[nf:2 * nf], mid_idx[2 * nf:]
        v = np.concatenate([v, mid], 0)
        f = np.concatenate([
            np.stack([f[:, 0], m01, m20], 1),
            np.stack([f[:, 1], m12, m01], 1),
            np.stack([f[:, 2], m20, m12], 1),
            np.stack([m01, m12, m20], 1)], 0)
    return v, f.astype(np.uint32)


@dataclass
class Scene:
    verts: np.ndarray            # (nv, 3) float32
    idx: np.ndarray              # (nt, 3) uint32
    tri_material: np.ndarray | None = None   # (nt,) uint32
    materials: np.ndarray | None = None      # (nm, 8) float32: type, albedo rgb, roughness, emission rgb
    lights: list = field(default_factory=list)
    bounds: tuple | None = None  # ((lo), (hi)) of the region rays start in
    name: str = ""

    @property
    def num_tris(self) -> int:
        return int(self.idx.shape[0])


def _merge(parts):
    verts, idx, off = [], [], 0
    for v, f in parts:
        verts.append(np.asarray(v, dtype=np.float32))
        idx.append(np.asarray(f, dtype=np.uint64) + off)
        off += len(v)
    return np.concatenate(verts, 0), np.concatenate(idx, 0).astype(np.uint32)


def random_triangles(n: int, seed: int, lo: float, hi: float, stream_base: int = 0):
    """n triangles with all 9 coordinates uniform in [lo, hi]^3 (one PCG32
    stream per triangle)."""
    g = Pcg32Streams(seed, np.arange(stream_base, stream_base + n, dtype=np.uint64))
    c = np.stack([g.next_f32() for _ in range(9)], 1).astype(np.float32)
    c = np.float32(lo) + c * np.float32(hi - lo)
    v = c.reshape(n * 3, 3)
    f = np.arange(n * 3, dtype=np.uint32).reshape(n, 3)
    return v, f


def icosphere_scene() -> Scene:
    """Unit icosphere subdivided 6 times (81,920 tris) + 1,024 random
    triangles with vertices uniform in [-2,2]^3, seed 0: 82,944 triangles."""
    sv, sf = icosphere(6)
    rv, rf = random_triangles(1024, seed=0, lo=-2.0, hi=2.0)
    v, f = _merge([(sv.astype(np.float32), sf), (rv, rf)])
    return Scene(v, f, bounds=((-2.0, -2.0, -2.0), (2.0, 2.0, 2.0)), name="icosphere6+1024")


def camera_basis(eye, target, up):
    eye = np.asarray(eye, np.float64)
    fwd = np.asarray(target, np.float64) - eye
    fwd /= math.sqrt(float((fwd * fwd).sum()))
    right = np.cross(fwd, np.asarray(up, np.float64))
    right /= math.sqrt(float((right * right).sum()))
    upv = np.cross(right, fwd)
    return eye, fwd, right, upv


def camera_rays(width: int, height: int, eye=(0.0, 0.0, 5.0), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0),
                vfov_deg: float = 45.0, tmin: float = 0.0, tmax: float = math.inf) -> np.ndarray:
    """One ray through each pixel centre; returns (H*W, 8) float32 rows in the
    fnd_ray layout (org xyz, tmin, dir xyz, tmax), row-major from the top."""
    eye, fwd, right, upv = camera_basis(eye, target, up)
    th = (math.sqrt(2.0) - 1.0) if vfov_deg == 45.0 else math.tan(math.radians(vfov_deg) * 0.5)
    aspect = width / height
    px = (np.arange(width, dtype=np.float64) + 0.5) / width * 2.0 - 1.0
    py = 1.0 - (np.arange(height, dtype=np.float64) + 0.5) / height * 2.0
    X, Y = np.meshgrid(px * th * aspect, py * th)
    d = fwd[None, None, :] + X[..., None] * right[None, None, :] + Y[..., None] * upv[None, None, :]
    d /= np.sqrt((d * d).sum(-1, keepdims=True))
    rays = np.empty((height * width, 8), np.float32)
    rays[:, 0:3] = eye.astype(np.float32)
    rays[:, 3] = tmin
    rays[:, 4:7] = d.reshape(-1, 3).astype(np.float32)
    rays[:, 7] = tmax
    return rays


def unit_vectors(g: Pcg32Streams) -> np.ndarray:
    """Directions uniform on S^2 by rejection from the cube [-1,1]^3 (one
    stream per vector, each stream draws until it accepts)."""
    n = g.state.shape[0]
    out = np.zeros((n, 3), np.float64)
    pending = np.ones(n, bool)
    while pending.any():
        m = pending
        x = g.next_f64(m) * 2.0 - 1.0
        y = g.next_f64(m) * 2.0 - 1.0
        z = g.next_f64(m) * 2.0 - 1.0
        r2 = x * x + y * y + z * z
        ok = (r2 > 1e-6) & (r2 <= 1.0)
        idx = np.nonzero(m)[0]
        acc = idx[ok]
        s = np.sqrt(r2[ok])
        out[acc, 0] = x[ok] / s
        out[acc, 1] = y[ok] / s
        out[acc, 2] = z[ok] / s
        pending[acc] = False
    return out


def incoherent_rays(n: int, lo, hi, seed: int, stream_base: int = 1 << 40, tmin: float = 0.0,
                    tmax: float = math.inf) -> np.ndarray:
    """n rays, origins uniform in the box [lo, hi], directions uniform on the
    sphere; (n, 8) float32 fnd_ray rows."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    g = Pcg32Streams(seed, np.arange(stream_base, stream_base + n, dtype=np.uint64))
    o = np.stack([lo[i] + g.next_f64() * (hi[i] - lo[i]) for i in range(3)], 1)
    d = unit_vectors(g)
    rays = np.empty((n, 8), np.float32)
    rays[:, 0:3] = o.astype(np.float32)
    rays[:, 3] = tmin
    rays[:, 4:7] = d.astype(np.float32)
    rays[:, 7] = tmax
    return rays


# Material table rows: [type, r, g, b, roughness, er, eg, eb]
MAT_LAMBERT = 0.0
MAT_GGX = 1.0
MAT_LIGHT = 2.0


def cornell_scene(num_spheres: int = 200, level: int = 3, seed: int = 1) -> Scene:
    """Cornell box [-1,1] x [0,2] x [-1,1] open towards +z: floor, ceiling, back
    wall, red left wall, green right wall (2 tris each), a 0.5 m x 0.5 m area
    light (0.25 m^2, radiance 15) just below the ceiling, and ``num_spheres``
    icospheres of ``level`` with centres uniform in the box and radii uniform
    in [0.02, 0.15]; half Lambertian (albedo U[0.1,0.9]^3), half GGX
    (roughness U[0.05,0.8], specular colour U[0.1,0.9]^3). 256,012 triangles
    for the defaults."""
    def quad(p, u, v):
        p, u, v = (np.asarray(a, np.float64) for a in (p, u, v))
        verts = np.stack([p, p + u, p + u + v, p + v])
        return verts, np.array([[0, 1, 2], [0, 2, 3]], np.uint32)

    parts, tri_mat = [], []
    mats = [
        [MAT_LAMBERT, 0.73, 0.73, 0.73, 1.0, 0, 0, 0],   # 0 white
        [MAT_LAMBERT, 0.65, 0.05, 0.05, 1.0, 0, 0, 0],   # 1 red
        [MAT_LAMBERT, 0.12, 0.45, 0.15, 1.0, 0, 0, 0],   # 2 green
        [MAT_LIGHT, 0.0, 0.0, 0.0, 1.0, 15.0, 15.0, 15.0],  # 3 light
    ]
    walls = [
        (quad((-1, 0, -1), (0, 0, 2), (2, 0, 0)), 0),    # floor  (normal +y)
        (quad((-1, 2, -1), (2, 0, 0), (0, 0, 2)), 0),    # ceiling (normal -y)
        (quad((-1, 0, -1), (2, 0, 0), (0, 2, 0)), 0),    # back   (normal +z)
        (quad((-1, 0, -1), (0, 2, 0), (0, 0, 2)), 1),    # left   (normal +x)
        (quad((1, 0, -1), (0, 0, 2), (0, 2, 0)), 2),     # right  (normal -x)
    ]
    for (v, f), m in walls:
        parts.append((v, f))
        tri_mat += [m, m]
    ly = 2.0 - 1e-3
    light = quad((-0.25, ly, -0.25), (0.5, 0, 0), (0, 0, 0.5))
    parts.append(light)
    tri_mat += [3, 3]
    sv, sf = icosphere(level)
    g = Pcg32Streams(seed, np.arange(num_spheres, dtype=np.uint64))
    cx = g.next_f64() * 2.0 - 1.0
    cy = g.next_f64() * 2.0
    cz = g.next_f64() * 2.0 - 1.0
    rad = 0.02 + g.next_f64() * 0.13
    kind = g.next_u32() & np.uint32(1)
    col = np.stack([0.1 + g.next_f64() * 0.8 for _ in range(3)], 1)
    rough = 0.05 + g.next_f64() * 0.75
    for i in range(num_spheres):
        c = np.array([cx[i], cy[i], cz[i]])
        parts.append((sv * rad[i] + c, sf))
        mats.append([MAT_GGX if kind[i] else MAT_LAMBERT, col[i, 0], col[i, 1], col[i, 2],
                     rough[i] if kind[i] else 1.0, 0, 0, 0])
        tri_mat += [len(mats) - 1] * len(sf)
    v, f = _merge(parts)
    lv = light[0]
    lights = [dict(kind="quad", corner=lv[0].tolist(), edge_u=(lv[1] - lv[0]).tolist(),
                   edge_v=(lv[3] - lv[0]).tolist(), radiance=[15.0, 15.0, 15.0])]
    return Scene(v, f, tri_material=np.asarray(tri_mat, np.uint32), materials=np.asarray(mats, np.float32),
                 lights=lights, bounds=((-1.0, 0.0, -1.0), (1.0, 2.0, 1.0)), name="cornell200")


CORNELL_CAMERA = dict(eye=(0.0, 1.0, 3.4), target=(0.0, 1.0, 0.0), up=(0.0, 1.0, 0.0), vfov_deg=45.0)


def soup_scene(n: int, seed: int = 2, stream_base: int = 0) -> Scene:
    """n triangles in the unit cube: first vertex uniform in [0,1]^3, the two
    edges from it with directions uniform on S^2 and lengths log-uniform in
    [1e-3, 0.1]."""
    g = Pcg32Streams(seed, np.arange(stream_base, stream_base + n, dtype=np.uint64))
    p = np.stack([g.next_f64() for _ in range(3)], 1)
    l1 = _exp2_det(math.log2(1e-3) + g.next_f64() * (math.log2(0.1) - math.log2(1e-3)))
    l2 = _exp2_det(math.log2(1e-3) + g.next_f64() * (math.log2(0.1) - math.log2(1e-3)))
    d1 = unit_vectors(g)
    d2 = unit_vectors(g)
    v = np.stack([p, p + d1 * l1[:, None], p + d2 * l2[:, None]], 1).astype(np.float32)
    f = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    return Scene(v.reshape(-1, 3), f, bounds=((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), name=f"soup{n}")


def value_noise(x: np.ndarray, z: np.ndarray, seed: int, octaves: int = 8, amplitude: float = 0.2) -> np.ndarray:
    """Value noise on [0,1]^2: octave o has a (2^(o+2)+1)^2 lattice of values
    uniform in [-1, 1) (one PCG32 stream per lattice point, seed ``seed``),
    blended with smoothstep weights t^2 (3 - 2t); octaves are summed with
    weights 2^-o and scaled so the sum lies in [-amplitude, amplitude)."""
    x = np.asarray(x, np.float64)
    z = np.asarray(z, np.float64)
    h = np.zeros(np.broadcast(x, z).shape, np.float64)
    wsum = 0.0
    base = 0
    for o in range(octaves):
        f = 1 << (o + 2)
        g = Pcg32Streams(seed, np.arange(base, base + (f + 1) * (f + 1), dtype=np.uint64))
        lat = (g.next_f64() * 2.0 - 1.0).reshape(f + 1, f + 1)
        base += (f + 1) * (f + 1)
        fx, fz = x * f, z * f
        ix = np.minimum(np.floor(fx).astype(np.int64), f - 1)
        iz = np.minimum(np.floor(fz).astype(np.int64), f - 1)
        tx, tz = fx - ix, fz - iz
        sx, sz = tx * tx * (3.0 - 2.0 * tx), tz * tz * (3.0 - 2.0 * tz)
        a = lat[ix, iz] * (1.0 - sx) + lat[ix + 1, iz] * sx
        b = lat[ix, iz + 1] * (1.0 - sx) + lat[ix + 1, iz + 1] * sx
        w = 1.0 / (1 << o)
        h += w * (a * (1.0 - sz) + b * sz)
        wsum += w
    return h * (amplitude / wsum)


def terrain_scene(grid: int = 2237, instances: int = 4096, level: int = 4, seed: int = 3) -> Scene:
    """Large scene: a heightfield over [0,1]^2 on a ``grid`` x ``grid`` vertex
    lattice ((grid-1)^2 x 2 triangles; 9,999,392 for 2237), heights from
    8-octave value noise (seed ``seed``, amplitude 0.2), and ``instances``
    icospheres of ``level`` (5,120 tris each at level 4) at positions uniform
    on the terrain, radii uniform in [0.001, 0.01], resting half sunk into
    the ground; half Lambertian (albedo U[0.1,0.9]^3), half GGX (roughness
    U[0.05,0.8]). The instances are stored flattened (one triangle list).
    Lit by a directional sun and a constant sky (``TERRAIN_LIGHTING``)."""
    n = grid
    t = np.arange(n, dtype=np.float64) / float(n - 1)
    X, Z = np.meshgrid(t, t, indexing="ij")
    H = value_noise(X, Z, seed)
    tv = np.stack([X, H, Z], -1).reshape(-1, 3)
    i = np.arange(n - 1, dtype=np.uint32)
    I, J = np.meshgrid(i, i, indexing="ij")
    v00 = (I * n + J).ravel()
    v01, v10, v11 = v00 + 1, v00 + n, v00 + n + 1
    # winding with +y normals: (v00, v01, v10) and (v10, v01, v11)
    tf = np.concatenate([np.stack([v00, v01, v10], 1), np.stack([v10, v01, v11], 1)], 0).astype(np.uint32)
    parts = [(tv, tf)]
    mats = [[MAT_LAMBERT, 0.42, 0.38, 0.33, 1.0, 0, 0, 0]]
    tri_mat = [np.zeros(len(tf), np.uint32)]
    sv, sf = icosphere(level)
    g = Pcg32Streams(seed, np.arange(1 << 32, (1 << 32) + instances, dtype=np.uint64))
    cx, cz = g.next_f64(), g.next_f64()
    rad = 0.001 + g.next_f64() * 0.009
    kind = g.next_u32() & np.uint32(1)
    col = np.stack([0.1 + g.next_f64() * 0.8 for _ in range(3)], 1)
    rough = 0.05 + g.next_f64() * 0.75
    cy = value_noise(cx, cz, seed) + 0.5 * rad
    iv = (sv[None, :, :] * rad[:, None, None] + np.stack([cx, cy, cz], 1)[:, None, :]).reshape(-1, 3)
    off = (np.arange(instances, dtype=np.uint64) * np.uint64(len(sv)))[:, None, None]
    if_ = (sf[None, :, :].astype(np.uint64) + off).reshape(-1, 3)
    parts.append((iv, if_))
    for k in range(instances):
        mats.append([MAT_GGX if kind[k] else MAT_LAMBERT, col[k, 0], col[k, 1], col[k, 2],
                     rough[k] if kind[k] else 1.0, 0, 0, 0])
    tri_mat.append(np.repeat(np.arange(1, instances + 1, dtype=np.uint32), len(sf)))
    v, f = _merge(parts)
    return Scene(v, f, tri_material=np.concatenate(tri_mat), materials=np.asarray(mats, np.float32), lights=[],
                 bounds=((0.0, -0.2, 0.0), (1.0, 0.25, 1.0)), name=f"terrain{n}x{instances}")


TERRAIN_CAMERA = dict(eye=(0.5, 0.42, 1.32), target=(0.5, 0.0, 0.42), up=(0.0, 1.0, 0.0), vfov_deg=40.0)
TERRAIN_LIGHTING = dict(sky=(0.30, 0.40, 0.55), sun_dir=(0.35, 0.6, 0.25), sun_irradiance=(3.0, 2.8, 2.5))


def material_records(scene: Scene) -> np.ndarray:
    """fnd_material records of a scene's material table; the k-th emissive
    material is tied to the k-th quad light."""
    from .rt import MATERIAL_DTYPE
    rows = scene.materials if scene.materials is not None else np.array([[0, 0.8, 0.8, 0.8, 1, 0, 0, 0]], np.float32)
    out = np.zeros(len(rows), MATERIAL_DTYPE)
    k = 0
    for i, r in enumerate(rows):
        out[i]["type"] = int(r[0])
        out[i]["albedo"] = r[1:4]
        out[i]["roughness"] = r[4]
        out[i]["emission"] = r[5:8]
        out[i]["light"] = -1
        if int(r[0]) == int(MAT_LIGHT):
            out[i]["light"] = k
            k += 1
    return out


def light_records(scene: Scene) -> np.ndarray:
    from .rt import LIGHT_DTYPE
    out = np.zeros(len(scene.lights), LIGHT_DTYPE)
    for i, L in enumerate(scene.lights):
        out[i]["corner"] = L["corner"]
        out[i]["edge_u"] = L["edge_u"]
        out[i]["edge_v"] = L["edge_v"]
        out[i]["radiance"] = L["radiance"]
    return out


def sphere_scene(level: int = 4, radius: float = 1.0, material=(0, 0.5, 0.5, 0.5, 1.0, 0, 0, 0)) -> Scene:
    """One icosphere at the origin with one material (furnace tests)."""
    v, f = icosphere(level)
    return Scene((v * radius).astype(np.float32), f, tri_material=np.zeros(len(f), np.uint32),
                 materials=np.asarray([material], np.float32), bounds=((-radius,) * 3, (radius,) * 3),
                 name=f"sphere{level}")


def write_obj(scene: Scene, path: str) -> None:
    """Writes the scene as OBJ + MTL (+ "#fnd quad_light" lines), the format
    the C++ pass's ObjLoader reads."""
    import os
    mtl = os.path.splitext(path)[0] + ".mtl"
    rows = scene.materials if scene.materials is not None else np.array([[0, 0.8, 0.8, 0.8, 1, 0, 0, 0]])
    with open(mtl, "w") as f:
        for i, r in enumerate(rows):
            f.write(f"newmtl m{i}\n")
            t = int(r[0])
            if t == int(MAT_GGX):
                f.write(f"Pm 1\nKs {r[1]:.9g} {r[2]:.9g} {r[3]:.9g}\nPr {r[4]:.9g}\n")
            elif t == int(MAT_LIGHT):
                f.write(f"Kd 0 0 0\nKe {r[5]:.9g} {r[6]:.9g} {r[7]:.9g}\n")
            else:
                f.write(f"Kd {r[1]:.9g} {r[2]:.9g} {r[3]:.9g}\n")
    tm = scene.tri_material if scene.tri_material is not None else np.zeros(scene.num_tris, np.uint32)
    with open(path, "w") as f:
        f.write(f"mtllib {os.path.basename(mtl)}\n")
        for L in scene.lights:
            vals = [*L["corner"], *L["edge_u"], *L["edge_v"], *L["radiance"]]
            f.write("#fnd quad_light " + " ".join(f"{float(x):.9g}" for x in vals) + "\n")
        f.write("".join(f"v {x:.9g} {y:.9g} {z:.9g}\n" for x, y, z in scene.verts.astype(np.float64)))
        cur = None
        for t in range(scene.num_tris):
            if tm[t] != cur:
                cur = tm[t]
                f.write(f"usemtl m{cur}\n")
            a, b, c = scene.idx[t] + 1
            f.write(f"f {a} {b} {c}\n")


def log_uniform_ints(n: int, lo: int, hi: int, seed: int, stream_base: int) -> np.ndarray:
    g = Pcg32Streams(seed, np.arange(stream_base, stream_base + n, dtype=np.uint64))
    u = g.next_f64()
    return np.round(_exp2_det(math.log2(lo) + u * (math.log2(hi) - math.log2(lo)))).astype(np.int64)


def cube_camera_rays(n: int) -> np.ndarray:
    """n coherent primary rays looking at the unit cube from (0.5, 0.5, 2.5)."""
    w = max(1, int(math.ceil(math.sqrt(n))))
    h = max(1, int(math.ceil(n / w)))
    return camera_rays(w, h, eye=(0.5, 0.5, 2.5), target=(0.5, 0.5, 0.5), vfov_deg=40.0)[:n]


def shadow_segments(n: int, seed: int, stream_base: int) -> np.ndarray:
    """n any-hit queries: segments between two uniform points of the unit
    cube (unnormalised direction p1 - p0, t in [0, 1])."""
    g = Pcg32Streams(seed, np.arange(stream_base, stream_base + n, dtype=np.uint64))
    p0 = np.stack([g.next_f64() for _ in range(3)], 1)
    p1 = np.stack([g.next_f64() for _ in range(3)], 1)
    rays = np.empty((n, 8), np.float32)
    rays[:, 0:3] = p0
    rays[:, 3] = 0.0
    rays[:, 4:7] = p1 - p0
    rays[:, 7] = 1.0
    return rays


def batch_plan(num_scenes: int = 256, seed: int = 2, tris=(1000, 500000), rays=(4096, 1 << 20)) -> dict:
    """Sizes and PCG stream bases of the batched-traversal workload: scene i
    has nt[i] triangles (streams tri_base[i]...) and nr[i] rays per query
    kind (closest: camera + random from ray_base[i], any: shadow segments
    from ray_base[i] + nr[i])."""
    nt = log_uniform_ints(num_scenes, tris[0], tris[1], seed, 1 << 50)
    nr = log_uniform_ints(num_scenes, rays[0], rays[1], seed, (1 << 50) + 4096)
    tri_base = np.concatenate([[0], np.cumsum(nt[:-1].astype(np.int64))]).astype(np.int64)
    ray_base = (1 << 44) + np.concatenate([[0], np.cumsum(2 * nr[:-1].astype(np.int64))]).astype(np.int64)
    return dict(seed=seed, nt=nt, nr=nr, tri_base=tri_base, ray_base=ray_base)


def batch_item(plan: dict, i: int) -> dict:
    """Scene i of a batch plan: a triangle soup in the unit cube and its ray
    batches (half coherent camera rays, half uniform-random rays for closest
    hit; as many shadow segments for any hit)."""
    seed = plan["seed"]
    sc = soup_scene(int(plan["nt"][i]), seed=seed, stream_base=int(plan["tri_base"][i]))
    n = int(plan["nr"][i])
    base = int(plan["ray_base"][i])
    cam = cube_camera_rays(n // 2)
    rnd = incoherent_rays(n - n // 2, (0, 0, 0), (1, 1, 1), seed=seed, stream_base=base)
    sh = shadow_segments(n, seed, base + n)
    return dict(scene=sc, closest=np.concatenate([cam, rnd], 0), any=sh)


def batch_workload(num_scenes: int = 256, seed: int = 2, tris=(1000, 500000), rays=(4096, 1 << 20)):
    """The batched-traversal workload: `num_scenes` triangle soups in the unit
    cube (log-uniform triangle counts, edge lengths log-uniform in [1e-3,
    0.1]), each with a ray batch of log-uniform size: half coherent camera
    rays, half uniform-random rays (closest hit), plus as many any-hit
    shadow segments. Returns a list of dicts (scene, closest_rays, any_rays)."""
    plan = batch_plan(num_scenes, seed, tris, rays)
    return [batch_item(plan, i) for i in range(num_scenes)]
