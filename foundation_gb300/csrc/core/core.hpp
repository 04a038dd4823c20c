// core.hpp — host-side conventions inside libfnd_rt.so, in the shape of the
// Foundation codebase but in a namespace of their own (Foundation::RtCore),
// so the library's symbols never meet the host application's
// Foundation::Core (its Allocator, BugCheck, logging) in one process:
//  * CHECK(expr): the reference routes a failed check to BugCheck and
//    terminates (src/Core/Core.hpp:17, src/Core/Core.cpp:7-10). Inside this
//    library a failed check throws FndError instead, and the C ABI layer turns
//    it into a negative status code, because nothing may terminate a host
//    process from behind a C ABI.
//  * LOG_RUNTIME(TAG, level, fmt, ...): tagged logging in the shape of
//    src/Core/Logging.hpp:34-35, printf-style, to stderr, filtered by the
//    FND_LOG_LEVEL environment variable (0 = off, 1 = err, 2 = warn, 3 = info).
// The C++ pass that a Foundation build compiles (renderer/) takes the
// application's Foundation::Core::Allocator instead (renderer/FoundationCore.hpp).
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
namespace RtCore {

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

}  // namespace RtCore
}  // namespace Foundation

#define FND_STR2(x) #x
#define FND_STR(x) FND_STR2(x)
#define CHECK(expr)                                                                                         \
    do {                                                                                                    \
        if (!(expr))                                                                                        \
            ::Foundation::RtCore::Fail(FND_ERR_INVALID_ARG, "Check Failed: " #expr " (" __FILE__ ":" FND_STR( \
                                                              __LINE__) ")");                               \
    } while (0)
#define CHECK_CODE(expr, code, ...)                                    \
    do {                                                               \
        if (!(expr)) ::Foundation::RtCore::Fail((code), __VA_ARGS__);    \
    } while (0)

#define FND_LOG_ERR 1
#define FND_LOG_WARN 2
#define FND_LOG_INFO 3
#define LOG_RUNTIME(TAG, LEVEL, ...)                                                                  \
    do {                                                                                              \
        if (::Foundation::RtCore::LogLevel() >= FND_LOG_##LEVEL)                                        \
            ::Foundation::RtCore::LogWrite(#TAG, FND_LOG_##LEVEL, __VA_ARGS__);                         \
    } while (0)
