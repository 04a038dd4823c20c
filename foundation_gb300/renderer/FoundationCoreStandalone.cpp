// FoundationCoreStandalone.cpp — BugCheck for builds of the pass outside a
// Foundation application (this repository's demo and tests). Foundation's
// own BugCheck hands the error to Platform::ExceptionHandler and terminates
// (src/Core/Core.cpp:7-10); here the error is rethrown as a
// std::runtime_error naming the failed check's source location, so a
// command-line driver can report it and exit with a status.
#ifndef FND_IN_FOUNDATION

#include "FoundationCore.hpp"

#include <string>

namespace Foundation {
namespace Core {

void BugCheck(const std::exception& e, const std::source_location loc) {
    throw std::runtime_error(std::string(e.what()) + " (" + loc.file_name() + ":" + std::to_string(loc.line()) + ")");
}

}  // namespace Core
}  // namespace Foundation

#endif
