// FoundationCore.hpp — the host conventions the path-tracer pass is written
// against: Foundation's polymorphic allocator and its CHECK -> BugCheck
// failure path.
//
// Inside a Foundation build (FND_IN_FOUNDATION defined, the application's
// src/ directory on the include path) this is the application's own
// headers, src/Core/Core.hpp and src/Core/Allocator/Allocator.hpp, so the
// pass takes the very Foundation::Core::Allocator the Renderer is given
// (src/Renderer/Renderer.hpp:41) and fails through the application's
// BugCheck, which reports and terminates (src/Core/Core.cpp:7-10).
//
// Built on its own (this repository's demo and tests), the same three
// declarations are made here. The allocator interface keeps the reference's
// members and virtual-function order (Allocate(size), Allocate(size,
// alignment), Deallocate(ptr, size), Deallocate(ptr), Reallocate,
// GetUsedMemory; no virtual destructor), so an object of either build has the
// same virtual table layout. The standalone BugCheck is defined in
// FoundationCoreStandalone.cpp.
#pragma once

#if defined(FND_IN_FOUNDATION)

#include <Core/Core.hpp>
#include <Core/Allocator/Allocator.hpp>

#else

#include <cstddef>
#include <exception>
#include <source_location>
#include <stdexcept>
#include <string>
#include <vector>

namespace Foundation {
namespace Platform {
// Reports an unrecoverable error with the log lines that led to it.
extern void ExceptionHandler(const std::exception& e, std::vector<std::string> backtrace);
}  // namespace Platform
namespace Core {

// Called on a failed CHECK; does not return to the failed statement.
extern void BugCheck(const std::exception& e, const std::source_location loc = std::source_location::current());

class Allocator {
public:
    using size_type = std::size_t;
    using pointer = void*;
    struct Arena {
        pointer memory;
        size_type size;
    };

    virtual pointer Allocate(size_type size) = 0;
    virtual pointer Allocate(size_type size, size_t alignment) = 0;
    virtual void Deallocate(pointer ptr, size_type size) = 0;
    virtual void Deallocate(pointer ptr) = 0;
    virtual pointer Reallocate(pointer ptr, size_type new_size, size_t alignment) = 0;

    Arena AllocateArena(size_type size, size_t alignment) { return {Allocate(size, alignment), size}; }
    Arena AllocateArena(size_type size) { return {Allocate(size), size}; }
    void DeallocateArena(Arena arena) {
        if (arena.memory) Deallocate(arena.memory, arena.size);
    }
    virtual size_type GetUsedMemory() const noexcept = 0;

    Allocator* Ptr() { return this; }
};

}  // namespace Core
}  // namespace Foundation

#define CHECK(expr) \
    if (!(expr)) Foundation::Core::BugCheck(std::runtime_error("Check Failed: " #expr));

#endif
