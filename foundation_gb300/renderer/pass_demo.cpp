// pass_demo.cpp — drives the path-tracer pass the way the reference's Editor
// drives its renderer (src/Editor/Editor.cpp:14-28: create, then Draw() per
// frame), headless: loads an OBJ scene, renders, writes the frame to a file:
// out.pfm keeps the linear radiance, out.png the display pixels
// (R8G8B8A8_UNORM through fnd_rt_tonemap, ACES curve, exposure 1).
//
// usage: fnd_pass_demo scene.obj out.{pfm,png} width height spp_per_draw draws
//                      eye_x eye_y eye_z target_x target_y target_z vfov_deg [sky]
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "ImageIO.hpp"
#include "ObjLoader.hpp"
#include "PathTracerPass.hpp"

using namespace Foundation;

static bool EndsWith(const std::string& s, const char* suffix) {
    const std::string x(suffix);
    return s.size() >= x.size() && s.compare(s.size() - x.size(), x.size(), x) == 0;
}

int main(int argc, char** argv) {
    if (argc == 3 && std::string(argv[1]) == "--write-test-png") {
        // no GPU: a 37 x 23 gradient (r = 7x, g = 11y, b = x ^ y, a = 255 - x - y)
        // through the PNG writer, for the CPU test of the encoder
        const uint32_t w = 37, h = 23;
        std::vector<uint8_t> rgba(4 * (size_t)w * h);
        for (uint32_t y = 0; y < h; ++y)
            for (uint32_t x = 0; x < w; ++x) {
                uint8_t* p = &rgba[4 * ((size_t)y * w + x)];
                p[0] = (uint8_t)(7 * x);
                p[1] = (uint8_t)(11 * y);
                p[2] = (uint8_t)(x ^ y);
                p[3] = (uint8_t)(255 - x - y);
            }
        try {
            Renderer::WritePng(argv[2], rgba, w, h);
        } catch (const Core::FndError& e) {
            std::fprintf(stderr, "error %d: %s\n", e.code(), e.what());
            return 1;
        }
        return 0;
    }
    if (argc == 3 && std::string(argv[1]) == "--parse") {
        // load only (no GPU): prints the counts the pass would upload
        try {
            const Renderer::ObjScene obj = Renderer::LoadObj(argv[2]);
            std::printf("verts %zu tris %zu materials %zu lights %zu\n", obj.verts.size() / 3, obj.indices.size() / 3,
                        obj.materials.size(), obj.lights.size());
            for (const auto& m : obj.materials)
                std::printf("material type %u albedo %g %g %g roughness %g emission %g %g %g light %d\n", m.type,
                            m.albedo[0], m.albedo[1], m.albedo[2], m.roughness, m.emission[0], m.emission[1],
                            m.emission[2], m.light);
            return 0;
        } catch (const Core::FndError& e) {
            std::fprintf(stderr, "error %d: %s\n", e.code(), e.what());
            return 1;
        }
    }
    if (argc < 14) {
        std::fprintf(stderr, "usage: %s scene.obj out.pfm w h spp draws ex ey ez tx ty tz vfov [sky]\n", argv[0]);
        return 2;
    }
    try {
        Core::HeapAllocator allocator;
        Renderer::PathTracerDesc desc;
        desc.width = (uint32_t)std::atoi(argv[3]);
        desc.height = (uint32_t)std::atoi(argv[4]);
        desc.spp_per_draw = (uint32_t)std::atoi(argv[5]);
        const int draws = std::atoi(argv[6]);
        {
            Renderer::PathTracerPass pass(desc, &allocator);
            const Renderer::ObjScene obj = Renderer::LoadObj(argv[1]);
            Renderer::SceneDesc sd;
            sd.verts = obj.verts;
            sd.indices = obj.indices;
            sd.tri_material = obj.tri_material;
            sd.materials = obj.materials;
            sd.lights = obj.lights;
            pass.SetScene(sd);
            fnd_camera cam{{(float)std::atof(argv[7]), (float)std::atof(argv[8]), (float)std::atof(argv[9])},
                           {(float)std::atof(argv[10]), (float)std::atof(argv[11]), (float)std::atof(argv[12])},
                           {0.0f, 1.0f, 0.0f},
                           (float)std::atof(argv[13])};
            pass.SetCamera(cam);
            const float sky_v = argc > 14 ? (float)std::atof(argv[14]) : 0.0f;
            const float sky[3] = {sky_v, sky_v, sky_v}, zero[3] = {0, 0, 0};
            pass.SetEnvironment(sky, zero, zero);
            for (int i = 0; i < draws; ++i) pass.Draw();
            std::vector<float> rgb(3 * (size_t)desc.width * desc.height);
            pass.Readback(rgb);
            if (EndsWith(argv[2], ".png")) {
                std::vector<uint8_t> rgba(4 * (size_t)desc.width * desc.height);
                pass.ReadbackRGBA8(rgba);
                Renderer::WritePng(argv[2], rgba, desc.width, desc.height);
            } else {
                Renderer::WritePfm(argv[2], rgb, desc.width, desc.height);
            }
            std::printf("rendered %u x %u, %u spp, %u triangles, %zu materials, %zu lights\n", desc.width, desc.height,
                        pass.SamplesAccumulated(), pass.SceneInfo().num_tris, obj.materials.size(), obj.lights.size());
        }
        std::printf("host memory still allocated: %zu bytes\n", allocator.GetUsedMemory());
        return allocator.GetUsedMemory() == 0 ? 0 : 3;
    } catch (const Core::FndError& e) {
        std::fprintf(stderr, "error %d: %s\n", e.code(), e.what());
        return 1;
    }
}
