// core.cpp — tagged logging (see core.hpp).
#include "core.hpp"

#include <mutex>

namespace Foundation {
namespace RtCore {

int LogLevel() {
    static const int level = [] {
        const char* s = std::getenv("FND_LOG_LEVEL");
        return s ? std::atoi(s) : FND_LOG_WARN;
    }();
    return level;
}

void LogWrite(const char* tag, int level, const char* fmt, ...) {
    static std::mutex mu;
    static const char* names[] = {"", "error", "warning", "info"};
    char buf[2048];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    std::lock_guard<std::mutex> lock(mu);
    std::fprintf(stderr, "[%s] [%s] %s\n", tag, names[level < 0 ? 0 : (level > 3 ? 3 : level)], buf);
}

}  // namespace RtCore
}  // namespace Foundation
