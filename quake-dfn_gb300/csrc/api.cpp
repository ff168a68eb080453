// Library-level entry points: version, status strings, thread-local errors.
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "qdfn_internal.h"

namespace qdfn {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
    g_last_error = std::string(qdfn_status_string(code)) + ": " + msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string("CUDA error ") + cudaGetErrorName(e) + " (" +
                   cudaGetErrorString(e) + ") in " + what;
    return QDFN_ERR_CUDA;
}

int num_sms() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    return n;
}

}  // namespace qdfn

extern "C" const char* qdfn_version(void) { return "qdfn-gb300 0.1.0 (sm_103a)"; }

extern "C" const char* qdfn_status_string(int status) {
    switch (status) {
        case QDFN_OK: return "ok";
        case QDFN_ERR_INVALID: return "invalid argument";
        case QDFN_ERR_CUDA: return "CUDA error";
        case QDFN_ERR_NOMEM: return "out of device memory";
        case QDFN_ERR_STATE: return "call out of order";
        case QDFN_ERR_DOMAIN: return "domain error (log or sqrt of a negative number)";
        case QDFN_ERR_EMPTY: return "time-step control reduced over an empty set";
        case QDFN_ERR_RETRIES: return "step retry cap exceeded";
        case QDFN_ERR_NO_CONVERGE: return "per-patch iteration cap exceeded";
        case QDFN_ERR_TIMEOUT: return "device deadline passed";
        case QDFN_ERR_HALF_SPACE: return "point above the free surface";
        default: return "unknown status";
    }
}

extern "C" int qdfn_last_error(char* buf, size_t n) {
    if (!buf || n == 0) return QDFN_ERR_INVALID;
    const std::string& s = qdfn::g_last_error;
    size_t k = s.size() < n - 1 ? s.size() : n - 1;
    std::memcpy(buf, s.data(), k);
    buf[k] = '\0';
    return QDFN_OK;
}
