// Per-shot residual and misfit with no device allocation.
//
// Callers that cannot allocate device memory: a host application that reserves
// all of its device memory up front in its own pool (common in seismic
// processing frameworks that run many jobs per GPU) and must not call
// cudaMalloc afterwards, and C or Fortran codes that pass device pointers they
// own but link no allocator at all.  pysit_plan_misfit needs a plan workspace
// bound by the caller; this entry point needs nothing but its inputs and
// outputs: its only scratch is a fixed array in device memory that the library
// holds on every GPU that loads it, until the process exits.
//
// Scratch: kMaxShots * kBlocksPerShot doubles (256 * 64 * 8 B = 128 KiB).  A
// __device__ array has one address per CUDA context, so the address is looked up
// (cudaGetSymbolAddress) on the first call made in each context and kept with
// that context's unique ID: a host that switches between contexts of its own, or
// a context rebuilt after cudaDeviceReset, gets the address that belongs to it.
// Make the first call of each context before any stream capture.  Every call
// overwrites every partial sum it reads, so nothing has to start at zero; but all
// calls share the one array, so calls that overlap on the GPU (different streams,
// or host threads) race and give wrong results.
#include <cuda.h>

#include <mutex>

#include "common.cuh"

namespace pgb {
namespace {

constexpr int kMaxShots = 256;
constexpr int kBlocksPerShot = 64;
constexpr int kThreadsNA = 256;

static __device__ __align__(256) double g_noalloc_partials[kMaxShots * kBlocksPerShot];

// stage 1: block b of shot s sums (dobs - dsim)^2 over its slice in FP64 and
// writes one partial; optional residual written back.  resid may be dobs or dsim
// (an in-place call): each element is read before it is written, by one thread.
template <typename T>
__global__ void __launch_bounds__(kThreadsNA) na_partials(const T* dobs, const T* dsim, long long per_shot, T* resid,
                                                          double* __restrict__ partials) {
    const int s = blockIdx.y, b = blockIdx.x;
    const T* o = dobs + (long long)s * per_shot;
    const T* d = dsim + (long long)s * per_shot;
    T* r = resid ? resid + (long long)s * per_shot : nullptr;
    double acc = 0.0;
    for (long long i = (long long)b * kThreadsNA + threadIdx.x; i < per_shot; i += (long long)kBlocksPerShot * kThreadsNA) {
        const T v = o[i] - d[i];
        if (r) r[i] = v;
        acc += (double)v * (double)v;
    }
    __shared__ double sm[kThreadsNA];
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kThreadsNA / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[s * kBlocksPerShot + b] = sm[0];
}

// stage 2: one warp per shot adds its kBlocksPerShot partials in a fixed order
__global__ void na_finish(const double* __restrict__ partials, int nshots, double* __restrict__ out) {
    const int s = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (s >= nshots) return;
    double a = 0.0;
    for (int b = lane; b < kBlocksPerShot; b += 32) a += partials[s * kBlocksPerShot + b];
    for (int off = 16; off > 0; off >>= 1) a += __shfl_down_sync(0xffffffffu, a, off);
    if (lane == 0) out[s] = a;
}

// ---- the scratch address of the current context -------------------------------------
// Two driver entry points, fetched through the runtime (no link against the driver
// library): the calling thread's current context and its process-unique ID.
using GetCurrentFn = CUresult (*)(CUcontext*);
using GetIdFn = CUresult (*)(CUcontext, unsigned long long*);

struct CtxAddr {
    unsigned long long id;
    double* ptr;
};
constexpr int kCtxSlots = 64;  // contexts remembered at once (the oldest entry is replaced)

std::mutex g_mu;
GetCurrentFn g_get_current = nullptr;
GetIdFn g_get_id = nullptr;
bool g_fns_tried = false;
CtxAddr g_cache[kCtxSlots];
int g_cached = 0, g_next = 0;

int driver_fns() {  // under g_mu
    if (!g_fns_tried) {
        g_fns_tried = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_get_current = reinterpret_cast<GetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_get_id = reinterpret_cast<GetIdFn>(f);
        cudaGetLastError();  // a failed query leaves no sticky runtime error behind
    }
    PGB_REQUIRE(g_get_current && g_get_id, "the CUDA driver offers no cuCtxGetCurrent / cuCtxGetId (CUDA >= 12 needed)");
    return PYSIT_OK;
}

// ID of the calling thread's current context; the runtime makes the device's primary
// context current first if no context is current yet
int current_context(unsigned long long* id) {  // under g_mu
    CUcontext ctx = nullptr;
    PGB_REQUIRE(g_get_current(&ctx) == CUDA_SUCCESS, "cuCtxGetCurrent failed");
    if (!ctx) {
        int dev = 0;
        PGB_CHECK_CUDA(cudaGetDevice(&dev));
        PGB_CHECK_CUDA(cudaSetDevice(dev));  // initialises and binds the primary context
        PGB_REQUIRE(g_get_current(&ctx) == CUDA_SUCCESS && ctx, "no CUDA context is current");
    }
    PGB_REQUIRE(g_get_id(ctx, id) == CUDA_SUCCESS, "cuCtxGetId failed");
    return PYSIT_OK;
}

int scratch_address(double** out) {
    std::lock_guard<std::mutex> lock(g_mu);
    int rc = driver_fns();
    if (rc) return rc;
    unsigned long long id = 0;
    if ((rc = current_context(&id))) return rc;
    for (int i = 0; i < g_cached; ++i)
        if (g_cache[i].id == id) {
            *out = g_cache[i].ptr;
            return PYSIT_OK;
        }
    // first call in this context: look the symbol up (not inside a stream capture)
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_noalloc_partials)");
    const int slot = g_cached < kCtxSlots ? g_cached++ : g_next;
    if (g_cached == kCtxSlots && slot == g_next) g_next = (g_next + 1) % kCtxSlots;
    g_cache[slot] = CtxAddr{id, static_cast<double*>(p)};
    *out = static_cast<double*>(p);
    return PYSIT_OK;
}

}  // namespace
}  // namespace pgb

using namespace pgb;

extern "C" int pysit_misfit_per_shot_noalloc(int dtype, const void* dobs, const void* dsim, int nshots,
                                             int64_t per_shot, void* resid, double* rnorm2, void* stream) try {
    PGB_REQUIRE(dtype == PYSIT_F32 || dtype == PYSIT_F64, "dtype must be PYSIT_F32 or PYSIT_F64 (got %d)", dtype);
    PGB_REQUIRE(nshots >= 1 && nshots <= kMaxShots,
                "nshots must be in [1, %d]: the fixed scratch holds %d shots (got %d)", kMaxShots, kMaxShots,
                nshots);
    PGB_REQUIRE(per_shot >= 1, "per_shot must be >= 1 (got %lld)", (long long)per_shot);
    PGB_REQUIRE(dobs && dsim && rnorm2, "NULL array argument");
    double* partials = nullptr;
    int rc = scratch_address(&partials);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    dim3 grid(kBlocksPerShot, nshots);
    if (dtype == PYSIT_F64)
        na_partials<double><<<grid, kThreadsNA, 0, s>>>((const double*)dobs, (const double*)dsim, per_shot,
                                                        (double*)resid, partials);
    else
        na_partials<float><<<grid, kThreadsNA, 0, s>>>((const float*)dobs, (const float*)dsim, per_shot,
                                                       (float*)resid, partials);
    PGB_CHECK_CUDA(cudaGetLastError());
    na_finish<<<(nshots + 7) / 8, 256, 0, s>>>(partials, nshots, rnorm2);
    PGB_CHECK_CUDA(cudaGetLastError());
    return PYSIT_OK;
} PGB_API_CATCH("pysit_misfit_per_shot_noalloc")
