"""Generates the committed golden fixtures of the traversal tests.

The reference (mos9527/Foundation) has no ray-tracing code and therefore no
golden vectors for this path; these fixtures are outputs of the CPU oracle
(oracle/, itself pinned by hand-derived known-answer tests) on seeded inputs,
committed so that any later change of the oracle, of the scene generators or
of the device kernels shows up as a diff. Run from the repository root:

    python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from foundation_gb300 import scenes  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def main():
    # 1) a small seeded soup scene with uniform random rays through it
    soup = scenes.soup_scene(1024, seed=7)
    rays = scenes.incoherent_rays(2048, (-0.1, -0.1, -0.1), (1.1, 1.1, 1.1), seed=7)
    b = oracle.OracleBVH(soup.verts, soup.idx)
    h = b.closest(rays)
    a = b.any(rays)
    np.savez_compressed(os.path.join(OUT, "soup1k.npz"), verts=soup.verts, idx=soup.idx, rays=rays,
                        prim=h["prim"], t=h["t"], occluded=a)
    # 2) first 4096 primary rays of the 1024x1024 icosphere workload; the
    #    scene itself is pinned by a digest of the generator output
    ico = scenes.icosphere_scene()
    r1 = scenes.camera_rays(1024, 1024)
    b1 = oracle.OracleBVH(ico.verts, ico.idx)
    sel = np.concatenate([np.arange(4096), np.arange(512 * 1024, 512 * 1024 + 4096)])
    h1 = b1.closest(r1[sel])
    np.savez_compressed(os.path.join(OUT, "icosphere_rows.npz"), sel=sel, rays=r1[sel], prim=h1["prim"], t=h1["t"],
                        scene_sha256=np.array(digest(ico.verts, ico.idx)),
                        rays_sha256=np.array(digest(r1)))
    # 3) the Cornell-box scene digest and 2048 incoherent rays
    cs = scenes.cornell_scene()
    ir = scenes.incoherent_rays(2048, *cs.bounds, seed=1)
    bc = oracle.OracleBVH(cs.verts, cs.idx)
    hc = bc.closest(ir)
    np.savez_compressed(os.path.join(OUT, "cornell_rows.npz"), rays=ir, prim=hc["prim"], t=hc["t"],
                        scene_sha256=np.array(digest(cs.verts, cs.idx, cs.tri_material, cs.materials)))
    # 4) FP64 oracle render of the Cornell box at 96x54, 4096 spp
    cam = scenes.CORNELL_CAMERA
    img = oracle.pt_render(bc, cs.tri_material, scenes.material_records(cs), scenes.light_records(cs), cam, 96, 54,
                           4096, max_depth=8, rr_start=3, seed=7)
    np.savez_compressed(os.path.join(OUT, "cornell_fp64_96x54.npz"), image=img.astype(np.float32), spp=4096,
                        max_depth=8, rr_start=3)
    print("written to", OUT)


if __name__ == "__main__":
    main()
