// Error state and version of the C ABI.
#include <string>

#include "fdfd_internal.h"

namespace fdfd {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

}  // namespace fdfd

extern "C" const char *fdfd_last_error(void) { return fdfd::g_last_error.c_str(); }

extern "C" int fdfd_version(void) { return 1; }
