// ObjLoader.hpp — Wavefront OBJ / MTL reader for the path-tracer pass.
//
// The reference renderer has no mesh loader (its only geometry is the
// hard-coded quad of src/Renderer/Renderer.cpp:153-157); scenes reach the
// pass through this reader. Supported subset:
//   OBJ: v x y z | f i j k ... (polygons fan-triangulated; v, v/t, v/t/n,
//        v//n and negative indices) | usemtl name | mtllib file
//   MTL: newmtl name | Kd r g b (Lambert albedo) | Ks r g b (GGX specular
//        colour) | Pm m (m > 0 selects GGX) | Pr alpha (GGX roughness) |
//        Ke r g b (emitter radiance, makes the material emissive)
//   light directive (an OBJ comment): "#fnd quad_light cx cy cz ux uy uz
//        vx vy vz r g b" — the k-th emissive material is tied to the k-th
//        quad light for multiple-importance weighting.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <fnd_rt.h>

namespace Foundation {
namespace Renderer {

struct ObjScene {
    std::vector<float> verts;
    std::vector<uint32_t> indices;
    std::vector<uint32_t> tri_material;
    std::vector<fnd_material> materials;
    std::vector<fnd_quad_light> lights;
};

// Throws std::runtime_error on an unreadable or malformed file.
ObjScene LoadObj(const std::string& path);

}  // namespace Renderer
}  // namespace Foundation
