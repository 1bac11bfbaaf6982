// Shared device/host helpers for the pysit_gb300 CUDA library (sm_103a only).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/pysit_gb300.h"

namespace pgb {

// ---------------------------------------------------------------------------
// Central finite-difference weights of order 2R (R = 1..4).  First derivative:
// sum_m a_m (v[i+m] - v[i-m]); second derivative: b_0 v[i] + sum_m b_m (v[i+m] + v[i-m]).
// These are the standard central weights that the reference hard-codes as the
// "bulk" (shift 0) rows of pysit/solvers/fd_tools/fd_manual.hpp:8-69.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr double d1w(int R, int m) {
    return R == 1 ? (m == 1 ? 0.5 : 0.0)
         : R == 2 ? (m == 1 ? 2.0 / 3.0 : m == 2 ? -1.0 / 12.0 : 0.0)
         : R == 3 ? (m == 1 ? 3.0 / 4.0 : m == 2 ? -3.0 / 20.0 : m == 3 ? 1.0 / 60.0 : 0.0)
         : R == 4 ? (m == 1 ? 4.0 / 5.0 : m == 2 ? -1.0 / 5.0 : m == 3 ? 4.0 / 105.0
                     : m == 4 ? -1.0 / 280.0 : 0.0)
         : 0.0;
}
__host__ __device__ constexpr double d2w(int R, int m) {
    return R == 1 ? (m == 0 ? -2.0 : m == 1 ? 1.0 : 0.0)
         : R == 2 ? (m == 0 ? -5.0 / 2.0 : m == 1 ? 4.0 / 3.0 : m == 2 ? -1.0 / 12.0 : 0.0)
         : R == 3 ? (m == 0 ? -49.0 / 18.0 : m == 1 ? 3.0 / 2.0 : m == 2 ? -3.0 / 20.0
                     : m == 3 ? 1.0 / 90.0 : 0.0)
         : R == 4 ? (m == 0 ? -205.0 / 72.0 : m == 1 ? 8.0 / 5.0 : m == 2 ? -1.0 / 5.0
                     : m == 3 ? 8.0 / 315.0 : m == 4 ? -1.0 / 560.0 : 0.0)
         : 0.0;
}

// signed first-derivative tap weight for offset m in [-R, R]
__host__ __device__ constexpr double d1tap(int R, int m) {
    return m > 0 ? d1w(R, m) : m < 0 ? -d1w(R, -m) : 0.0;
}
__host__ __device__ constexpr double d2tap(int R, int m) { return d2w(R, m < 0 ? -m : m); }

// ---------------------------------------------------------------------------
// Error reporting across the C ABI: a thread-local message plus an int code.
// ---------------------------------------------------------------------------
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* what);
// Called from a catch (...) handler: records the exception in flight and returns PYSIT_EHOST,
// so that no C++ exception leaves an extern "C" entry point.
int host_exception(const char* where) noexcept;

// Closes every extern "C" entry point written as a function-try-block.
#define PGB_API_CATCH(name) \
    catch (...) { return ::pgb::host_exception(name); }

#define PGB_CHECK_CUDA(call)                                         \
    do {                                                             \
        cudaError_t _e = (call);                                     \
        if (_e != cudaSuccess) return ::pgb::cuda_status(_e, #call); \
    } while (0)

#define PGB_REQUIRE(cond, ...)                                       \
    do {                                                             \
        if (!(cond)) {                                               \
            ::pgb::set_error(__VA_ARGS__);                           \
            return PYSIT_EINVAL;                                     \
        }                                                            \
    } while (0)

inline bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace pgb
