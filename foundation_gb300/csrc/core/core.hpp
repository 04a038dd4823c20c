// core.hpp — host-side conventions of the Foundation codebase, restated
// without its third-party dependencies (spdlog, fmt and mimalloc are not
// available here):
//  * CHECK(expr): the reference routes a failed check to BugCheck and
//    terminates (src/Core/Core.hpp:17, src/Core/Core.cpp:7-10). Inside this
//    library a failed check throws FndError instead, and the C ABI layer turns
//    it into a negative status code, because nothing may terminate a host
//    process from behind a C ABI.
//  * LOG_RUNTIME(TAG, level, fmt, ...): tagged logging in the shape of
//    src/Core/Logging.hpp:34-35, printf-style, to stderr, filtered by the
//    FND_LOG_LEVEL environment variable (0 = off, 1 = err, 2 = warn, 3 = info).
//  * Allocator: the polymorphic host allocator interface of
//    src/Core/Allocator/Allocator.hpp:17-41 (Allocate / Deallocate /
//    GetUsedMemory), with a counting heap implementation.
#pragma once

#include <atomic>
#include <cstdarg>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <new>
#include <stdexcept>
#include <string>

#include "../../../include/fnd_rt.h"

namespace Foundation {
namespace Core {

class FndError : public std::runtime_error {
public:
    FndError(int code, const std::string& msg) : std::runtime_error(msg), m_code(code) {}
    int code() const noexcept { return m_code; }

private:
    int m_code;
};

[[noreturn]] inline void Fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    throw FndError(code, buf);
}

int LogLevel();
void LogWrite(const char* tag, int level, const char* fmt, ...);

class Allocator {
public:
    using size_type = std::size_t;
    using pointer = void*;
    virtual ~Allocator() = default;
    virtual pointer Allocate(size_type size, size_t alignment) = 0;
    virtual void Deallocate(pointer ptr, size_type size) = 0;
    virtual size_type GetUsedMemory() const noexcept = 0;
};

// Heap allocator that counts live bytes (thread-safe counter). Every block is
// 64-byte aligned; larger alignments are rejected.
class HeapAllocator final : public Allocator {
public:
    static constexpr size_t kAlign = 64;
    pointer Allocate(size_type size, size_t alignment) override {
        CHECK_ALIGN(alignment);
        void* p = ::operator new(size ? size : 1, std::align_val_t(kAlign), std::nothrow);
        if (!p) Fail(FND_ERR_OUT_OF_MEMORY, "host allocation of %zu bytes failed", size);
        m_used.fetch_add(size, std::memory_order_relaxed);
        return p;
    }
    void Deallocate(pointer ptr, size_type size) override {
        if (!ptr) return;
        ::operator delete(ptr, std::align_val_t(kAlign));
        m_used.fetch_sub(size, std::memory_order_relaxed);
    }
    size_type GetUsedMemory() const noexcept override { return m_used.load(std::memory_order_relaxed); }

private:
    static void CHECK_ALIGN(size_t alignment) {
        if (alignment > kAlign) Fail(FND_ERR_INVALID_ARG, "alignment %zu above %zu", alignment, kAlign);
    }
    std::atomic<size_type> m_used{0};
};

}  // namespace Core
}  // namespace Foundation

#define FND_STR2(x) #x
#define FND_STR(x) FND_STR2(x)
#define CHECK(expr)                                                                                         \
    do {                                                                                                    \
        if (!(expr))                                                                                        \
            ::Foundation::Core::Fail(FND_ERR_INVALID_ARG, "Check Failed: " #expr " (" __FILE__ ":" FND_STR( \
                                                              __LINE__) ")");                               \
    } while (0)
#define CHECK_CODE(expr, code, ...)                                    \
    do {                                                               \
        if (!(expr)) ::Foundation::Core::Fail((code), __VA_ARGS__);    \
    } while (0)

#define FND_LOG_ERR 1
#define FND_LOG_WARN 2
#define FND_LOG_INFO 3
#define LOG_RUNTIME(TAG, LEVEL, ...)                                                                  \
    do {                                                                                              \
        if (::Foundation::Core::LogLevel() >= FND_LOG_##LEVEL)                                        \
            ::Foundation::Core::LogWrite(#TAG, FND_LOG_##LEVEL, __VA_ARGS__);                         \
    } while (0)
