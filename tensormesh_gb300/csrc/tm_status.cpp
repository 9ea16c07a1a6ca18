// Error reporting of the C ABI: a status code plus a thread-local message.
#include "tm_status.h"

#include <cstdio>
#include <cstring>

namespace {
thread_local char g_message[512] = "";
}

int tm_set_error(int status, const char* message) {
    std::snprintf(g_message, sizeof(g_message), "%s", message ? message : "");
    return status;
}

extern "C" const char* tm_last_error_message(void) { return g_message; }

extern "C" const char* tm_error_string(int status) {
    switch (status) {
        case TM_OK: return "ok";
        case TM_ERR_INVALID_ARG: return "invalid argument";
        case TM_ERR_UNSUPPORTED: return "unsupported element type or form";
        case TM_ERR_CUDA: return "CUDA error";
        case TM_ERR_PLAN: return "plan construction failed";
        case TM_ERR_TOO_LARGE: return "size above a supported limit";
        case TM_ERR_DEVICE_WAIT: return "a device-side wait ran out";
        default: return "unknown status";
    }
}

extern "C" int tm_version(void) { return 2; }
