// pass_demo.cpp — drives the path-tracer pass the way the reference's Editor
// drives its renderer (src/Editor/Editor.cpp:14-28: create, then Draw() per
// frame; FrameLoop.hpp), headless: loads an OBJ scene, renders, writes the
// frame to a file:
// out.pfm keeps the linear radiance, out.png the display pixels
// (R8G8B8A8_UNORM through fnd_rt_tonemap, ACES curve, exposure 1).
//
// usage: fnd_pass_demo scene.obj out.{pfm,png} width height spp_per_draw draws
//                      eye_x eye_y eye_z target_x target_y target_z vfov_deg [sky]
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "FrameLoop.hpp"
#include "ImageIO.hpp"
#include "ObjLoader.hpp"

using namespace Foundation;

namespace {

// The host allocator the demo hands the pass, in place of the application's
// heap allocator: operator new with the requested alignment, and a count of
// the bytes still allocated (checked to be 0 at exit). Blocks carry a 64-byte
// header with their size and alignment so the size-less Deallocate and
// Reallocate work.
class CountingAllocator final : public Core::Allocator {
public:
    pointer Allocate(size_type size) override { return Allocate(size, alignof(std::max_align_t)); }
    pointer Allocate(size_type size, size_t alignment) override {
        const size_t align = alignment < kHeader ? kHeader : alignment;
        auto* base = static_cast<unsigned char*>(::operator new(align + size, std::align_val_t(align)));
        auto* h = reinterpret_cast<size_t*>(base + align - kHeader);
        h[0] = size;
        h[1] = align;
        m_used += size;
        return base + align;
    }
    void Deallocate(pointer ptr, size_type) override { Deallocate(ptr); }
    void Deallocate(pointer ptr) override {
        if (!ptr) return;
        auto* p = static_cast<unsigned char*>(ptr);
        const size_t* h = reinterpret_cast<const size_t*>(p - kHeader);
        const size_t size = h[0], align = h[1];
        m_used -= size;
        ::operator delete(p - align, std::align_val_t(align));
    }
    pointer Reallocate(pointer ptr, size_type new_size, size_t alignment) override {
        pointer q = Allocate(new_size, alignment);
        if (ptr) {
            const size_t old = reinterpret_cast<const size_t*>(static_cast<unsigned char*>(ptr) - kHeader)[0];
            std::memcpy(q, ptr, old < new_size ? old : new_size);
            Deallocate(ptr);
        }
        return q;
    }
    size_type GetUsedMemory() const noexcept override { return m_used.load(); }

private:
    static constexpr size_t kHeader = 64;
    std::atomic<size_t> m_used{0};
};

}  // namespace

namespace Foundation::Platform {
void ExceptionHandler(const std::exception& e, std::vector<std::string>) { std::fprintf(stderr, "%s\n", e.what()); }
}  // namespace Foundation::Platform

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
        } catch (const std::exception& e) {
            std::fprintf(stderr, "error: %s\n", e.what());
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
        } catch (const std::exception& e) {
            std::fprintf(stderr, "error: %s\n", e.what());
            return 1;
        }
    }
    if (argc < 14) {
        std::fprintf(stderr, "usage: %s scene.obj out.pfm w h spp draws ex ey ez tx ty tz vfov [sky]\n", argv[0]);
        return 2;
    }
    try {
        CountingAllocator allocator;
        Renderer::FrameLoopDesc desc;
        desc.pass.width = (uint32_t)std::atoi(argv[3]);
        desc.pass.height = (uint32_t)std::atoi(argv[4]);
        desc.pass.spp_per_draw = (uint32_t)std::atoi(argv[5]);
        desc.draws = (uint32_t)std::atoi(argv[6]);
        desc.camera = fnd_camera{{(float)std::atof(argv[7]), (float)std::atof(argv[8]), (float)std::atof(argv[9])},
                                 {(float)std::atof(argv[10]), (float)std::atof(argv[11]), (float)std::atof(argv[12])},
                                 {0.0f, 1.0f, 0.0f},
                                 (float)std::atof(argv[13])};
        const float sky_v = argc > 14 ? (float)std::atof(argv[14]) : 0.0f;
        desc.sky[0] = desc.sky[1] = desc.sky[2] = sky_v;
        {
            const Renderer::ObjScene obj = Renderer::LoadObj(argv[1]);
            Renderer::SceneDesc sd;
            sd.verts = obj.verts;
            sd.indices = obj.indices;
            sd.tri_material = obj.tri_material;
            sd.materials = obj.materials;
            sd.lights = obj.lights;
            const size_t px = (size_t)desc.pass.width * desc.pass.height;
            std::vector<float> rgb(3 * px);
            std::vector<uint8_t> rgba(EndsWith(argv[2], ".png") ? 4 * px : 0);
            const uint32_t spp = Renderer::RenderFrames(&allocator, desc, sd, rgb, rgba);
            if (!rgba.empty())
                Renderer::WritePng(argv[2], rgba, desc.pass.width, desc.pass.height);
            else
                Renderer::WritePfm(argv[2], rgb, desc.pass.width, desc.pass.height);
            std::printf("rendered %u x %u, %u spp, %zu triangles, %zu materials, %zu lights\n", desc.pass.width,
                        desc.pass.height, spp, obj.indices.size() / 3, obj.materials.size(), obj.lights.size());
        }
        std::printf("host memory still allocated: %zu bytes\n", allocator.GetUsedMemory());
        return allocator.GetUsedMemory() == 0 ? 0 : 3;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
