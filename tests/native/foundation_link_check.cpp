// foundation_link_check.cpp — TEST HARNESS: a minimal Foundation
// application around the path-tracer pass. Built two ways by
// tests/test_pass_foundation.py:
//  * with FND_IN_FOUNDATION against Foundation's own src/Core headers (the
//    pass then takes Foundation's Core::Allocator and fails through its
//    BugCheck), linked with the pass sources and libfnd_rt.so: proves the
//    pass compiles and links into a Foundation build; run without a GPU it
//    must reach BugCheck with the library's message;
//  * against the standalone declarations (renderer/FoundationCore.hpp): on a
//    GPU it draws a frame of a one-triangle scene and checks the pixels and
//    that every host byte went back to the allocator.
// The stubs below stand in for the application's: BugCheck reports and
// exits with status 3 instead of terminating (Foundation's terminates,
// src/Core/Core.cpp:7-10), and the allocator counts bytes.
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../foundation_gb300/renderer/FrameLoop.hpp"

namespace Foundation {
namespace Platform {
void ExceptionHandler(const std::exception& e, std::vector<std::string>) {
    std::printf("ExceptionHandler: %s\n", e.what());
}
}  // namespace Platform
#if defined(FND_IN_FOUNDATION)
namespace Core {
void BugCheck(const std::exception& e, const std::source_location loc) {
    Platform::ExceptionHandler(e, {});
    std::printf("BugCheck at %s:%u\n", loc.file_name(), (unsigned)loc.line());
    std::fflush(stdout);
    std::exit(3);
}
}  // namespace Core
#endif
}  // namespace Foundation

namespace {

class TestAllocator final : public Foundation::Core::Allocator {
public:
    pointer Allocate(size_type size) override { return Allocate(size, alignof(std::max_align_t)); }
    pointer Allocate(size_type size, size_t alignment) override {
        void* p = ::operator new(size ? size : 1, std::align_val_t(kAlign));
        (void)alignment;
        used += size;
        return p;
    }
    void Deallocate(pointer ptr, size_type size) override {
        if (!ptr) return;
        used -= size;
        ::operator delete(ptr, std::align_val_t(kAlign));
    }
    void Deallocate(pointer) override { std::abort(); }  // the pass always passes the size
    pointer Reallocate(pointer, size_type, size_t) override { std::abort(); }
    size_type GetUsedMemory() const noexcept override { return used.load(); }
    static constexpr size_t kAlign = 64;
    std::atomic<size_t> used{0};
};

}  // namespace

int main() {
    using namespace Foundation::Renderer;
    // one Lambertian triangle facing the camera, filling the frame's centre
    const std::vector<float> verts = {-1, -1, 0, 1, -1, 0, 0, 1, 0};
    const std::vector<uint32_t> idx = {0, 1, 2};
    fnd_material white{};
    white.type = FND_MAT_LAMBERT;
    white.albedo[0] = white.albedo[1] = white.albedo[2] = 0.5f;
    white.roughness = 1.0f;
    white.light = -1;
    const std::vector<fnd_material> mats = {white};
    SceneDesc scene;
    scene.verts = verts;
    scene.indices = idx;
    scene.materials = mats;
    FrameLoopDesc desc;
    desc.pass.width = 16;
    desc.pass.height = 16;
    desc.pass.spp_per_draw = 4;
    desc.draws = 2;
    desc.sky[0] = desc.sky[1] = desc.sky[2] = 1.0f;  // a white sky lights the triangle
    TestAllocator allocator;
    std::vector<float> rgb(3 * 16 * 16);
    const uint32_t spp = RenderFrames(&allocator, desc, scene, rgb);
    // centre pixel: the triangle under a white sky (albedo 0.5, one bounce to
    // the sky: 0.5 exactly for a Lambertian surface); corner: the sky itself
    const float* c = &rgb[3 * (8 * 16 + 8)];
    const float* k = &rgb[0];
    std::printf("spp %u centre %.4f %.4f %.4f corner %.4f %.4f %.4f used %zu\n", spp, c[0], c[1], c[2], k[0], k[1],
                k[2], (size_t)allocator.GetUsedMemory());
    const bool ok = spp == 8 && std::abs(c[0] - 0.5f) < 1e-5f && std::abs(k[0] - 1.0f) < 1e-5f &&
                    allocator.GetUsedMemory() == 0;
    return ok ? 0 : 1;
}
