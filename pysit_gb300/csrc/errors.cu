// Error state of the C ABI: one message per calling thread.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <exception>
#include <new>

#include "common.cuh"

namespace pgb {

namespace {
thread_local char g_msg[1024] = {0};
}

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t e, const char* what) {
    set_error("CUDA error %d (%s: %s) in %s", (int)e, cudaGetErrorName(e), cudaGetErrorString(e),
              what);
    return PYSIT_ECUDA;
}

int host_exception(const char* where) noexcept {
    try {
        throw;
    } catch (const std::bad_alloc&) {
        set_error("%s: host memory allocation failed", where);
    } catch (const std::exception& e) {
        set_error("%s: %s", where, e.what());
    } catch (...) {
        set_error("%s: unexpected C++ exception", where);
    }
    return PYSIT_EHOST;
}

}  // namespace pgb

extern "C" const char* pysit_cuda_last_error(void) { return pgb::g_msg; }

extern "C" int pysit_cuda_version(void) { return PYSIT_ABI_VERSION; }
