// Batched 2D leapfrog step: persistent warps fed by per-warp shared-memory row
// rings (forward, recompute, adjoint).
//
// Same maths as the reference step cda_time_scalar_2D (pysit/solvers/
// constant_density_acoustic/time/scalar/constant_density_acoustic_time_scalar_2D.h:88-179)
// with the fusions of the batched pipeline:
//   kFwd    trace recording of u_k (recorder blocks at the front of the grid,
//           receivers.py:462-510);
//   kRecomp the imaging operand dWaveOp_k (constant_density_acoustic_base.py:24-40)
//           from the stencil's own bracket F: C^2 F where the step and mesh
//           sigmas agree, plus the sigma differences elsewhere (the right PML,
//           whose step profile is read one node further out, _2D.h:143-157);
//   kAdj    the time-reversed adjoint step with ic += q_k * dWaveOp_k fused
//           (temporal_modeling.py:312-365).
//
// Work decomposition: a table of warp tasks (x0, x1, zs, ze, kind) covers the
// padded grid of one shot once.  The warps of the launch are persistent: each
// takes the next (shot, task) from a global counter until the launch's tasks
// are used up, so no wave of blocks runs half empty at the end.  A task owns the
// cells z in [zs, ze) of the rows x0..x1-1; lane L holds the V consecutive cells
// from zs + L*V.  Per row x, lane 0 has already asked (A rows ahead) for
//   * row x+R of u_k, with an R-cell z-halo each side, into the warp's x-ring
//     of 2R+A rows (the x-derivatives read rows x-R..x+R from it);
//   * the centre rows of u_{k-1}, C^2 (and dWaveOp, ic for the adjoint; Phi_z
//     with its halo, row x+R of Phi_x for the PML) into one of A stages,
// with 1-D bulk copies (cp.async.bulk) completing on the stage's mbarrier.  Every
// operand then comes from shared memory with aligned vector loads; the loop body
// is one row (no unrolling), which keeps the kernel small enough for the
// instruction cache.  Warps never wait for each other.
// Task kinds (warp-uniform branch):
//   kind 0  interior: at least R cells away from the padding, 16-byte lane
//           vectors, no PML state;
//   kind 1  PML shell: the padding and its R-wide rim, 8-byte lane vectors (more
//           busy lanes on the narrow z-bands), Phi_x / Phi_z carried where both
//           sigmas vanish as in the reference.
// Waits are bounded: on expiry the kernel sets the plan's error word, waits (again
// bounded) for the copies it issued, and carries on.
#include "tma.cuh"
#include "wave.cuh"

namespace pgb {
namespace {

constexpr int kWarps = 4;  // warps per block
constexpr uint32_t kPolls = 1u << 22;
#ifndef PGB_RING_AHEAD
#define PGB_RING_AHEAD 4   // rows whose copies are in flight ahead of the computation
#endif

template <typename T, int N> struct VecT;
template <> struct VecT<float, 4> { using type = float4; };
template <> struct VecT<float, 2> { using type = float2; };
template <> struct VecT<float, 1> { using type = float; };
template <> struct VecT<double, 2> { using type = double2; };
template <> struct VecT<double, 1> { using type = double; };

template <typename T, int N>
struct alignas(sizeof(T) * N) Vec {
    T v[N];
};
template <typename T, int N>
__device__ __forceinline__ Vec<T, N> lds(const T* p) {
    Vec<T, N> r;
    *reinterpret_cast<typename VecT<T, N>::type*>(r.v) = *reinterpret_cast<const typename VecT<T, N>::type*>(p);
    return r;
}
template <typename T, int N>
__device__ __forceinline__ void stg(T* p, const Vec<T, N>& r) {
    *reinterpret_cast<typename VecT<T, N>::type*>(p) = *reinterpret_cast<const typename VecT<T, N>::type*>(r.v);
}
template <typename T, int N>
__device__ __forceinline__ void stg_cs(T* p, const Vec<T, N>& r) {
    __stcs(reinterpret_cast<typename VecT<T, N>::type*>(p), *reinterpret_cast<const typename VecT<T, N>::type*>(r.v));
}

// Ring geometry of one task kind.  All slot widths are whole 16-byte units, so
// every bulk copy starts and ends 16-byte aligned (task z-bounds are multiples
// of 4 cells, rows start 128-byte aligned).
template <typename T, int R, int MODE, int KIND>
struct Ring {
    static constexpr int AL = 16 / (int)sizeof(T);              // elements per 16 bytes
    static constexpr int V = KIND == 0 ? AL : (AL > 1 ? AL / 2 : 1);  // cells per lane
    static constexpr int HZ = (R + AL - 1) / AL * AL;            // z-halo cells per side
    static constexpr int NB = HZ / V;                            // halo vectors per side
    static constexpr int SEG = 32 * V;                           // cells a task owns at most
    static constexpr int WS = SEG + 2 * HZ;                      // slot with halo (elements)
    static constexpr int A = MODE == kAdj && PGB_RING_AHEAD > 2 ? PGB_RING_AHEAD - 1 : PGB_RING_AHEAD;
    static constexpr int NU = 2 * R + A;                         // x-ring slots
    static constexpr bool PML = KIND == 1;
    static constexpr int NPF = MODE == kAdj ? 4 : 2;             // centre rows per stage
    static constexpr int PST = NPF * SEG + (PML ? WS : 0);       // stage (elements)
    static constexpr int ELEMS = NU * WS + (PML ? NU * SEG : 0) + A * PST;
    static_assert(A >= 1 && A <= 16, "the barrier block holds 16 mbarriers");
};

template <typename T, int R, int MODE>
struct WarpSmem {
    static constexpr int e0 = Ring<T, R, MODE, 0>::ELEMS, e1 = Ring<T, R, MODE, 1>::ELEMS;
    static constexpr size_t per_warp = 128 + sizeof(T) * (size_t)(e0 > e1 ? e0 : e1);  // barriers + rings
    static constexpr size_t bytes = kWarps * per_warp;
    static_assert(per_warp % 16 == 0, "warp regions stay 16-byte aligned");
};

// Pipeline position of a warp, carried across its tasks: the stage the next row
// uses and that stage's mbarrier phase parity.
struct Pipe {
    int s;
    uint32_t ph;
};

template <typename T, int R, int MODE, int KIND>
__device__ __forceinline__ void sweep(const WaveParams<T>& p, unsigned char* wsm, Pipe& pp, const int shot,
                                      const int x0, const int x1, const int zs, const int ze, bool& bad,
                                      bool& late) {
    using G = Ring<T, R, MODE, KIND>;
    constexpr int V = G::V, HZ = G::HZ, NB = G::NB, SEG = G::SEG, WS = G::WS, A = G::A, NU = G::NU;
    constexpr bool PML = G::PML;
    constexpr int NW = (2 * NB + 1) * V;  // z-window of a lane
    constexpr int C0 = NB * V;            // its centre
    uint64_t* bar = reinterpret_cast<uint64_t*>(wsm);
    T* uring = reinterpret_cast<T*>(wsm + 128);
    T* xring = uring + NU * WS;           // Phi_x rows (PML tasks)
    T* pring = xring + (PML ? NU * SEG : 0);
    const int lane = threadIdx.x & 31;
    const int niter = x1 - x0;
    const int zl = zs + lane * V;
    const bool own = zl < ze;
    const long long sh = (long long)shot * p.fstride;
    const T* ucur = p.u_cur + sh;
    T* uprev = p.u_prev + sh;
    const bool img = MODE == kAdj && p.image;
    auto rowoff = [&](int x) { return (long long)(x + kHalo) * p.ldz + kOZ; };
    const int ncen = (ze - zs + G::AL - 1) / G::AL * G::AL;
    const uint32_t bu = (uint32_t)(ncen + 2 * HZ) * sizeof(T);
    const uint32_t bc = (uint32_t)ncen * sizeof(T);
    const uint32_t bstage = bu + 2 * bc + (img ? 2 * bc : 0) + (PML ? bc + bu : 0);

    // copies for row x0 + i: u_k row x+R into x-ring slot `slot`, centre rows into stage s
    auto issue = [&](int i, int s, int slot, uint32_t extra) {
        const int x = x0 + i;
        T* st = pring + s * G::PST;
        mbar_arrive_expect_tx(&bar[s], bstage + extra);
        bulk_g2s(uring + slot * WS, ucur + rowoff(x + R) + zs - HZ, bu, &bar[s]);
        bulk_g2s(st, uprev + rowoff(x) + zs, bc, &bar[s]);
        bulk_g2s(st + SEG, p.c2 + rowoff(x) + zs, bc, &bar[s]);
        if (img) {
            bulk_g2s(st + 2 * SEG, p.dw_in + sh + rowoff(x) + zs, bc, &bar[s]);
            bulk_g2s(st + 3 * SEG, p.ic + sh + rowoff(x) + zs, bc, &bar[s]);
        }
        if (PML) {
            bulk_g2s(xring + slot * SEG, p.phx_in + sh + rowoff(x + R) + zs, bc, &bar[s]);
            bulk_g2s(st + G::NPF * SEG, p.phz_in + sh + rowoff(x) + zs - HZ, bu, &bar[s]);
        }
    };
    if (lane == 0) {
        fence_proxy_async();  // earlier generic reads of the rings before the new copies
        // rows x0-R .. x0+R-1 ride on the first row's stage
        issue(0, pp.s, 2 * R, 2 * R * (bu + (PML ? bc : 0)));
        for (int j = 0; j < 2 * R; ++j) {
            bulk_g2s(uring + j * WS, ucur + rowoff(x0 - R + j) + zs - HZ, bu, &bar[pp.s]);
            if (PML) bulk_g2s(xring + j * SEG, p.phx_in + sh + rowoff(x0 - R + j) + zs, bc, &bar[pp.s]);
        }
        int s = pp.s;
        for (int i = 1; i < min(A, niter); ++i) {
            if (++s == A) s = 0;
            issue(i, s, 2 * R + i, 0);
        }
    }

    // per-lane constants
    bool zok[V];
    T sgz[V], mgz[V];
#pragma unroll
    for (int v = 0; v < V; ++v) {
        const int z = zl + v;
        zok[v] = z > 0 && z < p.nz - 1;
        sgz[v] = (PML && z < p.nz) ? __ldg(p.sgz + z) : T(0);
        mgz[v] = (PML && MODE == kRecomp && z < p.nz) ? __ldg(p.mgz + z) : T(0);
    }
    T cx[R + 1], cz[R + 1];  // second-derivative weights with the grid spacing folded in
#pragma unroll
    for (int m = 0; m <= R; ++m) {
        cx[m] = T(d2w(R, m)) * p.idx2;
        cz[m] = T(d2w(R, m)) * p.idz2;
    }
    const int* bx = p.inj.box + shot * 6;
    const bool inj_task = p.inj.on && bx[0] < x1 && bx[1] > x0 && bx[4] < ze && bx[5] > zs;

    int b = 0;  // x-ring slot of row x - R
    for (int i = 0; i < niter; ++i) {
        const int x = x0 + i;
        const int s = pp.s;
        if (!mbar_wait_bounded(&bar[s], pp.ph, kPolls)) late = true;
        const T* st = pring + s * G::PST;
        auto slot = [&](int j) {  // x-ring slot of row x - R + j
            const int t = b + j;
            return t >= NU ? t - NU : t;
        };

        // ---- every shared-memory read of this row --------------------------------
        T w[NW];  // u_k row x around the lane's cells
        {
            const T* r = uring + slot(R) * WS + lane * V;
#pragma unroll
            for (int j = 0; j <= 2 * NB; ++j) {
                const Vec<T, V> a = lds<T, V>(r + j * V);
#pragma unroll
                for (int v = 0; v < V; ++v) w[j * V + v] = a.v[v];
            }
        }
        Vec<T, V> ux[2 * R];  // u_k rows x-R..x-1, x+1..x+R at the lane's cells
#pragma unroll
        for (int m = 1; m <= R; ++m) {
            ux[R - m] = lds<T, V>(uring + slot(R - m) * WS + HZ + lane * V);
            ux[R + m - 1] = lds<T, V>(uring + slot(R + m) * WS + HZ + lane * V);
        }
        const Vec<T, V> um = lds<T, V>(st + lane * V);
        const Vec<T, V> cc = lds<T, V>(st + SEG + lane * V);
        Vec<T, V> dwi, ici;
        if (MODE == kAdj && img) {
            dwi = lds<T, V>(st + 2 * SEG + lane * V);
            ici = lds<T, V>(st + 3 * SEG + lane * V);
        }
        Vec<T, V> px[2 * R + 1];  // Phi_x rows x-R..x+R (PML tasks)
        T wp[NW];                 // Phi_z row x around the lane's cells (PML tasks)
        if (PML) {
#pragma unroll
            for (int j = 0; j <= 2 * R; ++j) px[j] = lds<T, V>(xring + slot(j) * SEG + lane * V);
            const T* r = st + G::NPF * SEG + lane * V;
#pragma unroll
            for (int j = 0; j <= 2 * NB; ++j) {
                const Vec<T, V> a = lds<T, V>(r + j * V);
#pragma unroll
                for (int v = 0; v < V; ++v) wp[j * V + v] = a.v[v];
            }
        }
        __syncwarp();  // every lane has read stage s and row x-R: lane 0 may refill them
        if (lane == 0 && i + A < niter) {
            fence_proxy_async();
            issue(i + A, s, b, 0);
        }
        if (++pp.s == A) { pp.s = 0; pp.ph ^= 1u; }
        if (++b == NU) b = 0;

        // ---- the update -------------------------------------------------------------
        const bool xok = x > 0 && x < p.nx - 1;
        const bool inj_row = inj_task && own && x >= bx[0] && x < bx[1];
        T sgx = T(0), mgx = T(0);
        if (PML) {
            sgx = __ldg(p.sgx + x);
            if (MODE == kRecomp) mgx = __ldg(p.mgx + x);
        }
        Vec<T, V> un, dwo, pxo, pzo, ico;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const int z = zl + v;
            const T uc = w[C0 + v];
            // Laplacian in difference form: sum_m w_m ((u_+m - u_0) + (u_-m - u_0)),
            // equal to the central stencil because the weights sum to zero, and free
            // of the large cancellation of w_0 u_0 (the FP32 path depends on this)
            T F = T(0);
#pragma unroll
            for (int m = 1; m <= R; ++m) {
                F += cx[m] * ((ux[R + m - 1].v[v] - uc) + (ux[R - m].v[v] - uc));
                F += cz[m] * ((w[C0 + v + m] - uc) + (w[C0 + v - m] - uc));
            }
            if (inj_row && z < p.nz) F += inject_rhs(p.inj, bx, shot, x, z);
            const T uo = um.v[v], c2 = cc.v[v];
            const bool ok = xok && zok[v];
            T unew;
            if (PML) {
                T dpx = T(0), dpz = T(0), dx1 = T(0), dz1 = T(0);
#pragma unroll
                for (int m = 1; m <= R; ++m) {
                    const T a = T(d1w(R, m));
                    dpx += a * (px[R + m].v[v] - px[R - m].v[v]);
                    dpz += a * (wp[C0 + v + m] - wp[C0 + v - m]);
                    dx1 += a * (ux[R + m - 1].v[v] - ux[R - m].v[v]);
                    dz1 += a * (w[C0 + v + m] - w[C0 + v - m]);
                }
                F += dpx * p.idx + dpz * p.idz;
                const T sx = sgx, sz = sgz[v];
                const T phx = px[R].v[v], phz = wp[C0 + v];
                T ph_x = phx, ph_z = phz;  // carried where both sigmas vanish (_2D.h:172-176)
                if (sx != T(0) || sz != T(0)) {
                    const T dudx = dx1 * p.idx, dudz = dz1 * p.idz;
                    ph_x = phx - p.dt * sx * phx + p.dt * (sz - sx) * dudx;
                    ph_z = phz - p.dt * sz * phz + p.dt * (sx - sz) * dudz;
                    const T fac1 = T(2) * p.dt2 / (T(2) + p.dt * (sx + sz));
                    const T fac2 = c2 * F - (uo - T(2) * uc) * p.idt2 + (sx + sz) * uo * p.i2dt - (sx * sz) * uc;
                    unew = fac1 * fac2;
                } else {
                    unew = p.dt2 * c2 * F - (uo - T(2) * uc);
                }
                if (!ok) { unew = T(0); ph_x = T(0); ph_z = T(0); }
                pxo.v[v] = ph_x;
                pzo.v[v] = ph_z;
                if (MODE == kRecomp) {
                    const T mz = mgz[v];
                    const T d = c2 * F + ((mgx + mz) - (sx + sz)) * (unew - uo) * p.i2dt + (mgx * mz - sx * sz) * uc;
                    dwo.v[v] = ok ? d : T(0);
                }
            } else {
                unew = ok ? p.dt2 * c2 * F - (uo - T(2) * uc) : T(0);
                if (MODE == kRecomp) dwo.v[v] = ok ? c2 * F : T(0);
            }
            un.v[v] = unew;
            if (MODE == kFwd) bad |= own && !isfinite(unew);
            if (MODE == kAdj) ico.v[v] = ici.v[v] + uc * dwi.v[v];
        }
        if (own) {
            const long long o = rowoff(x) + zl;
            stg<T, V>(uprev + o, un);
            if (PML) {
                stg<T, V>(p.phx_out + sh + o, pxo);
                stg<T, V>(p.phz_out + sh + o, pzo);
            }
            if (MODE == kRecomp && p.dw_out) stg_cs<T, V>(p.dw_out + sh + o, dwo);
            if (MODE == kAdj && img) stg<T, V>(p.ic + sh + o, ico);
        }
    }
}

template <typename T, int R, int MODE>
__global__ void __launch_bounds__(kWarps * 32) wave2d_warp_kernel(const WaveParams<T> p, const int* __restrict__ tasks,
                                                                  int ntasks, int rec_blocks) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    if ((int)blockIdx.x < rec_blocks) {
        if (MODE == kFwd) record_block(p, blockIdx.x);
        return;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* wsm = smem_raw + warp * WarpSmem<T, R, MODE>::per_warp;
    uint64_t* bar = reinterpret_cast<uint64_t*>(wsm);
    constexpr int A = Ring<T, R, MODE, 0>::A;
    static_assert(A == Ring<T, R, MODE, 1>::A, "both kinds share the stage barriers");
    if (lane == 0) {
        for (int s = 0; s < A; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
    }
    __syncwarp();
    const unsigned long long total = (unsigned long long)ntasks * (unsigned)p.nshot;
    Pipe pp{0, 0u};
    int issued[A];  // rows issued per stage (for the drain after an expired wait)
    (void)issued;
    bool bad = false, late = false;
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(p.task_ctr, 1ull) - p.task_base;
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= total) break;
        const int shot = (int)(t / (unsigned)ntasks);
        const int* tk = tasks + 5 * (int)(t - (unsigned long long)shot * ntasks);
        const int x0 = __ldg(tk), x1 = __ldg(tk + 1), zs = __ldg(tk + 2), ze = __ldg(tk + 3), kind = __ldg(tk + 4);
        if (kind == 0)
            sweep<T, R, MODE, 0>(p, wsm, pp, shot, x0, x1, zs, ze, bad, late);
        else
            sweep<T, R, MODE, 1>(p, wsm, pp, shot, x0, x1, zs, ze, bad, late);
    }
    late = __any_sync(0xffffffffu, late);
    if (late) {
        // a stage whose wait expired may still have copies in flight: wait for the
        // last phase of every stage (bounded) before the shared memory is released
        // pp.s is the next stage to use; stage j's last armed phase has parity
        // pp.ph for j < pp.s and pp.ph ^ 1 otherwise
        for (int j = 0; j < A; ++j) mbar_wait_bounded(&bar[j], j < pp.s ? pp.ph : (pp.ph ^ 1u), kPolls);
    }
    if (p.err) {
        if (MODE == kFwd && bad) atomicOr(p.err, PGB_ERR_NONFINITE);
        if (late && lane == 0) atomicOr(p.err, PGB_ERR_TIMEOUT);
    }
}

template <typename T, int R>
void prep_warp() {
    cudaFuncSetAttribute(wave2d_warp_kernel<T, R, kFwd>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)WarpSmem<T, R, kFwd>::bytes);
    cudaFuncSetAttribute(wave2d_warp_kernel<T, R, kRecomp>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)WarpSmem<T, R, kRecomp>::bytes);
    cudaFuncSetAttribute(wave2d_warp_kernel<T, R, kAdj>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)WarpSmem<T, R, kAdj>::bytes);
}

template <typename T, int R, int MODE>
int occupancy() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, wave2d_warp_kernel<T, R, MODE>, kWarps * 32,
                                                      WarpSmem<T, R, MODE>::bytes) != cudaSuccess)
        n = 1;
    return n > 0 ? n : 1;
}

}  // namespace

template <typename T, int R, int MODE>
long long launch_wave2d_warp_tasks(const WaveParams<T>& p, const int* tasks, int ntasks, int blocks,
                                   cudaStream_t s) {
    const int rec = MODE == kFwd ? p.rec.blocks : 0;
    wave2d_warp_kernel<T, R, MODE><<<rec + blocks, kWarps * 32, WarpSmem<T, R, MODE>::bytes, s>>>(p, tasks, ntasks,
                                                                                                 rec);
    // counter values the launch consumes: one per task plus one final fetch per warp
    return (long long)ntasks * p.nshot + (long long)blocks * kWarps;
}

void wave2d_warp_prepare() {
    prep_warp<float, 1>(); prep_warp<float, 2>(); prep_warp<float, 3>(); prep_warp<float, 4>();
    prep_warp<double, 1>(); prep_warp<double, 2>(); prep_warp<double, 3>(); prep_warp<double, 4>();
}

int wave2d_warp_threads() { return kWarps * 32; }

// persistent blocks of one launch: resident blocks per SM x SMs, no more than the tasks need
int wave2d_warp_blocks(int dtype_bytes, int order, int mode, long long tasks) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int R = order / 2;
    int occ = 1;
#define PGB_OCC(TT, RR)                                                  \
    occ = mode == kFwd ? occupancy<TT, RR, kFwd>()                       \
        : mode == kRecomp ? occupancy<TT, RR, kRecomp>() : occupancy<TT, RR, kAdj>()
    if (dtype_bytes == 4) {
        switch (R) { case 1: PGB_OCC(float, 1); break; case 2: PGB_OCC(float, 2); break;
                     case 3: PGB_OCC(float, 3); break; default: PGB_OCC(float, 4); break; }
    } else {
        switch (R) { case 1: PGB_OCC(double, 1); break; case 2: PGB_OCC(double, 2); break;
                     case 3: PGB_OCC(double, 3); break; default: PGB_OCC(double, 4); break; }
    }
#undef PGB_OCC
    const long long need = (tasks + kWarps - 1) / kWarps;
    const long long have = (long long)occ * sms;
    return (int)(need < have ? need : have);
}

// widest z-range a task of each kind may own: 32 lanes x V cells (same rule as Ring)
int wave2d_warp_seg(int dtype_bytes, int order, int pml) {
    (void)order;
    const int AL = 16 / dtype_bytes;
    const int V = pml ? (AL > 1 ? AL / 2 : 1) : AL;
    return 32 * V;
}

#define PGB_INSTW(T, R)                                                                                          \
    template long long launch_wave2d_warp_tasks<T, R, kFwd>(const WaveParams<T>&, const int*, int, int,          \
                                                            cudaStream_t);                                       \
    template long long launch_wave2d_warp_tasks<T, R, kRecomp>(const WaveParams<T>&, const int*, int, int,       \
                                                               cudaStream_t);                                    \
    template long long launch_wave2d_warp_tasks<T, R, kAdj>(const WaveParams<T>&, const int*, int, int, cudaStream_t);
PGB_INSTW(float, 1)
PGB_INSTW(float, 2)
PGB_INSTW(float, 3)
PGB_INSTW(float, 4)
PGB_INSTW(double, 1)
PGB_INSTW(double, 2)
PGB_INSTW(double, 3)
PGB_INSTW(double, 4)

}  // namespace pgb
