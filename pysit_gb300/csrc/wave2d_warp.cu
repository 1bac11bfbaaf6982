// Batched 2D leapfrog step, warp-independent sweep (forward, recompute, adjoint).
//
// Same maths as the reference step cda_time_scalar_2D (pysit/solvers/
// constant_density_acoustic/time/scalar/constant_density_acoustic_time_scalar_2D.h:88-179)
// with the fusions of the batched pipeline:
//   kFwd    trace recording of u_k (appended recorder blocks, receivers.py:462-510);
//   kRecomp the imaging operand dWaveOp_k (constant_density_acoustic_base.py:24-40)
//           from the stencil's own bracket F: C^2 F where the step and mesh
//           sigmas agree, plus the sigma differences elsewhere (the right PML,
//           whose step profile is read one node further out, _2D.h:143-157);
//   kAdj    the time-reversed adjoint step with ic += q_k * dWaveOp_k fused
//           (temporal_modeling.py:312-365).
//
// Work decomposition: a table of warp tasks (x0, x1, zs, ze, kind) covers the
// padded grid once and serves every shot.  A warp owns cells z in [zs, ze) and
// sweeps rows x0..x1-1.  Lanes hold VV consecutive cells; the HL lanes at each
// end only carry the z-halo.  Per row:
//   * lane 0 streams the rows the warp needs D iterations ahead into the warp's
//     own shared-memory ring with 1-D bulk copies (cp.async.bulk), one mbarrier
//     per stage; every lane reads its 16-byte vector back (no global-load latency
//     on the critical path, no block barrier, warps never wait for each other);
//   * the 2R+1 rows of u_k the x-derivatives need live in a register queue that
//     rotates by renaming (the row loop is unrolled by 2R+1);
//   * z-neighbours come from the adjacent lanes with warp shuffles.
// Task kinds (warp-uniform branch):
//   kind 0  interior: at least R cells away from the padding, 16-byte vectors,
//           no PML state;
//   kind 1  PML shell: the padding and its R-wide rim, 8-byte vectors, Phi_x in a
//           register queue, Phi_z through shuffles.
// Waits are bounded: on expiry the kernel sets the plan's error word and goes on.
#include "tma.cuh"
#include "wave.cuh"

namespace pgb {
namespace {

constexpr int kWarps = 4;   // warps per block
constexpr int kStages = 3;  // rows in flight ahead of the computation
constexpr uint32_t kPolls = 1u << 22;

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

// per-kind geometry
template <typename T, int R, int KIND>
struct Geo {
    static constexpr int V = V16<T>::N;
    static constexpr int VV = KIND == 0 ? V : (V > 1 ? V / 2 : 1);
    // halo lanes per side: enough for R cells, and a whole number of 16-byte
    // vectors so every bulk copy starts 16-byte aligned
    static constexpr int A = V / VV;
    static constexpr int HL = ((R + VV - 1) / VV + A - 1) / A * A;
    static constexpr int W = 32 * VV;                 // cells held by the warp (with halo lanes)
    static constexpr int SEG = (32 - 2 * HL) * VV;    // cells owned by the warp at most
    static constexpr int Q = 2 * R + 1;
    // ring layout per warp (elements): prologue rows of u (and Phi_x), then stages
    static constexpr int NF = KIND == 0 ? 5 : 7;      // u_head, u_prev, c2, dw, ic, [phx_head, phz]
    static constexpr int PRO = (KIND == 0 ? 1 : 2) * 2 * R * W;
    static constexpr int STAGE = NF * W;
    static constexpr int ELEMS = PRO + kStages * STAGE;
};

template <typename T, int R>
struct WarpSmem {
    static constexpr int e0 = Geo<T, R, 0>::ELEMS, e1 = Geo<T, R, 1>::ELEMS;
    static constexpr int ELEMS = e0 > e1 ? e0 : e1;
    static constexpr size_t per_warp = 128 + sizeof(T) * (size_t)ELEMS;  // barriers + ring
    static constexpr size_t bytes = kWarps * per_warp;
};

template <typename T, int VV, int HL>
__device__ __forceinline__ void zwindow(const Vec<T, VV>& c, T (&w)[(2 * HL + 1) * VV]) {
#pragma unroll
    for (int v = 0; v < VV; ++v) w[HL * VV + v] = c.v[v];
#pragma unroll
    for (int d = 1; d <= HL; ++d) {
#pragma unroll
        for (int v = 0; v < VV; ++v) {
            w[(HL - d) * VV + v] = __shfl_up_sync(0xffffffffu, c.v[v], d);
            w[(HL + d) * VV + v] = __shfl_down_sync(0xffffffffu, c.v[v], d);
        }
    }
}

template <typename T, int R, int MODE, int KIND>
__device__ __forceinline__ void sweep(const WaveParams<T>& p, unsigned char* wsm, const int shot, const int x0,
                                      const int x1, const int zs, const int ze) {
    using G = Geo<T, R, KIND>;
    constexpr int VV = G::VV, HL = G::HL, W = G::W, Q = G::Q;
    constexpr bool PML = KIND == 1;
    constexpr int NWIN = (2 * HL + 1) * VV;
    uint64_t* bar = reinterpret_cast<uint64_t*>(wsm);
    T* ring = reinterpret_cast<T*>(wsm + 128);
    T* pro = ring;                    // 2R rows of u (then 2R rows of Phi_x)
    T* stg0 = ring + G::PRO;          // stage s at stg0 + s*STAGE, field f at + f*W
    const int lane = threadIdx.x & 31;
    const int niter = x1 - x0;
    const int zw0 = zs - HL * VV;                         // first cell held by lane 0
    const int zl = zw0 + lane * VV;                       // first cell of this lane's vector
    const bool own = lane >= HL && lane < 32 - HL && zl < ze;
    const long long sh = (long long)shot * p.fstride;
    const T* ucur = p.u_cur + sh;
    T* uprev = p.u_prev + sh;
    const bool zpad = PML && (zl < p.pzl || zl + VV - 1 >= p.nz - p.pzr);
    auto xpad = [&](int x) { return x < p.pxl || x >= p.nx - p.pxr; };
    auto rowoff = [&](int x) { return (long long)(x + kHalo) * p.ldz + kOZ; };

    // copy extents (elements): full lane range for u / Phi_z (clamped to the row
    // storage), owned range for the rest; both multiples of 4 elements (16 bytes)
    const int nfull = min(W, (p.ldz - kOZ - zw0) / 4 * 4);
    const int own0 = HL * VV;                              // lane HL's offset in a slot
    const int nown = ((min(ze, zs + G::SEG) - zs) + 3) / 4 * 4;

    if (lane == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
    }
    __syncwarp();

    auto issue = [&](int i) {  // copies of iteration i (row x0 + i) into stage i % kStages
        const int x = x0 + i;
        const int s = i % kStages;
        T* st = stg0 + s * G::STAGE;
        uint32_t bytes = (uint32_t)(nfull + 2 * nown) * sizeof(T);
        if (MODE == kAdj && p.image) bytes += 2u * nown * sizeof(T);
        if (PML) bytes += (uint32_t)(nown + nfull) * sizeof(T);
        if (i == 0) bytes += (uint32_t)(2 * R * nfull * (PML ? 2 : 1)) * sizeof(T);
        mbar_arrive_expect_tx(&bar[s], bytes);
        if (i == 0)
            for (int j = 0; j < 2 * R; ++j) {
                bulk_g2s(pro + j * W, ucur + rowoff(x0 - R + j) + zw0, nfull * sizeof(T), &bar[s]);
                if (PML) bulk_g2s(pro + (2 * R + j) * W, p.phx_in + sh + rowoff(x0 - R + j) + zw0,
                                  nfull * sizeof(T), &bar[s]);
            }
        bulk_g2s(st, ucur + rowoff(x + R) + zw0, nfull * sizeof(T), &bar[s]);
        bulk_g2s(st + W + own0, uprev + rowoff(x) + zs, nown * sizeof(T), &bar[s]);
        bulk_g2s(st + 2 * W + own0, p.c2 + rowoff(x) + zs, nown * sizeof(T), &bar[s]);
        if (MODE == kAdj && p.image) {
            bulk_g2s(st + 3 * W + own0, p.dw_in + sh + rowoff(x) + zs, nown * sizeof(T), &bar[s]);
            bulk_g2s(st + 4 * W + own0, p.ic + sh + rowoff(x) + zs, nown * sizeof(T), &bar[s]);
        }
        if (PML) {
            bulk_g2s(st + 5 * W + own0, p.phx_in + sh + rowoff(x + R) + zs, nown * sizeof(T), &bar[s]);
            bulk_g2s(st + 6 * W, p.phz_in + sh + rowoff(x) + zw0, nfull * sizeof(T), &bar[s]);
        }
    };
    if (lane == 0) {
        fence_proxy_async();
        for (int i = 0; i < min(kStages, niter); ++i) issue(i);
    }

    // per-lane constants
    T sgz[VV], mgz[VV];
    bool zok[VV], zpe[VV];
#pragma unroll
    for (int v = 0; v < VV; ++v) {
        const int z = zl + v;
        zok[v] = z > 0 && z < p.nz - 1;
        zpe[v] = z < p.pzl || z >= p.nz - p.pzr;
        sgz[v] = (PML && z >= 0 && z < p.nz) ? __ldg(p.sgz + z) : T(0);
        mgz[v] = (PML && MODE == kRecomp && z >= 0 && z < p.nz) ? __ldg(p.mgz + z) : T(0);
    }
    bool zpw[NWIN];  // padding test of each z-window element (PML tasks)
#pragma unroll
    for (int j = 0; j < NWIN; ++j) {
        const int z = zl - HL * VV + j;
        zpw[j] = z < p.pzl || z >= p.nz - p.pzr;
    }
    // combined Laplacian weights
    T cx[R + 1], cz[R + 1];
#pragma unroll
    for (int m = 0; m <= R; ++m) {
        cx[m] = T(d2w(R, m)) * p.idx2;
        cz[m] = T(d2w(R, m)) * p.idz2;
    }
    const int* bx = p.inj.box + shot * 6;
    const bool inj_task = p.inj.on && bx[0] < x1 && bx[1] > x0 && bx[4] < ze && bx[5] > zs;
    bool bad = false;
    bool late = false;

    Vec<T, VV> q[Q];
    Vec<T, VV> qx[Q];  // Phi_x queue (PML tasks)

    for (int ib = 0; ib < niter; ib += Q) {
#pragma unroll
        for (int so = 0; so < Q; ++so) {
            const int i = ib + so;
            if (i >= niter) break;
            const int x = x0 + i;
            const int s = i % kStages;
            const T* st = stg0 + s * G::STAGE;
            if (!mbar_wait_bounded(&bar[s], (uint32_t)((i / kStages) & 1), kPolls)) late = true;
            if (i == 0) {
#pragma unroll
                for (int j = 0; j < 2 * R; ++j) {
                    q[(so + j) % Q] = lds<T, VV>(pro + j * W + lane * VV);
                    if (PML) {
                        Vec<T, VV> a = lds<T, VV>(pro + (2 * R + j) * W + lane * VV);
                        const bool use = zpad || xpad(x0 - R + j);
#pragma unroll
                        for (int v = 0; v < VV; ++v) a.v[v] = use ? a.v[v] : T(0);
                        qx[(so + j) % Q] = a;
                    }
                }
            }
            q[(so + 2 * R) % Q] = lds<T, VV>(st + lane * VV);
            const Vec<T, VV> um = lds<T, VV>(st + W + lane * VV);
            const Vec<T, VV> cc = lds<T, VV>(st + 2 * W + lane * VV);
            Vec<T, VV> dwi, ici, pzc;
            if (MODE == kAdj && p.image) {
                dwi = lds<T, VV>(st + 3 * W + lane * VV);
                ici = lds<T, VV>(st + 4 * W + lane * VV);
            }
            if (PML) {
                Vec<T, VV> a = lds<T, VV>(st + 5 * W + lane * VV);
                const bool use = zpad || xpad(x + R);
#pragma unroll
                for (int v = 0; v < VV; ++v) a.v[v] = use ? a.v[v] : T(0);
                qx[(so + 2 * R) % Q] = a;
                pzc = lds<T, VV>(st + 6 * W + lane * VV);
            }
            __syncwarp();  // every lane has read stage s: lane 0 may refill it
            if (lane == 0 && i + kStages < niter) {
                fence_proxy_async();
                issue(i + kStages);
            }

            const Vec<T, VV>& qc = q[(so + R) % Q];
            T w[NWIN];
            zwindow<T, VV, HL>(qc, w);
            T wp[NWIN];  // Phi_z window (PML tasks)
            if (PML) {
                zwindow<T, VV, HL>(pzc, wp);
                const bool xp = xpad(x);
#pragma unroll
                for (int j = 0; j < NWIN; ++j) wp[j] = (xp || zpw[j]) ? wp[j] : T(0);
            }
            const bool xok = x > 0 && x < p.nx - 1;
            const bool inj_row = inj_task && x >= bx[0] && x < bx[1];
            Vec<T, VV> un, dwo, pxo, pzo, ico;
            T sgx = T(0), mgx = T(0);
            if (PML) {
                sgx = __ldg(p.sgx + x);
                if (MODE == kRecomp) mgx = __ldg(p.mgx + x);
            }
#pragma unroll
            for (int v = 0; v < VV; ++v) {
                const int z = zl + v;
                const T uc = w[HL * VV + v];
                // Laplacian in difference form: sum_m w_m ((u_+m - u_0) + (u_-m - u_0)),
                // equal to the central stencil because the weights sum to zero, and free
                // of the large cancellation of w_0 u_0 (the FP32 path depends on this)
                T F = T(0);
#pragma unroll
                for (int m = 1; m <= R; ++m) {
                    F += cx[m] * ((q[(so + R + m) % Q].v[v] - uc) + (q[(so + R - m) % Q].v[v] - uc));
                    F += cz[m] * ((w[HL * VV + v + m] - uc) + (w[HL * VV + v - m] - uc));
                }
                if (inj_row && own && z < p.nz) F += inject_rhs(p.inj, bx, shot, x, z);
                const T uo = um.v[v], c2 = cc.v[v];
                const bool ok = xok && zok[v];
                T unew;
                if (PML) {
                    T dpx = T(0), dpz = T(0), dx1 = T(0), dz1 = T(0);
#pragma unroll
                    for (int m = 1; m <= R; ++m) {
                        const T a = T(d1w(R, m));
                        dpx += a * (qx[(so + R + m) % Q].v[v] - qx[(so + R - m) % Q].v[v]);
                        dpz += a * (wp[HL * VV + v + m] - wp[HL * VV + v - m]);
                        dx1 += a * (q[(so + R + m) % Q].v[v] - q[(so + R - m) % Q].v[v]);
                        dz1 += a * (w[HL * VV + v + m] - w[HL * VV + v - m]);
                    }
                    F += dpx * p.idx + dpz * p.idz;
                    const T sx = sgx, sz = sgz[v];
                    T ph_x = T(0), ph_z = T(0);
                    if (sx != T(0) || sz != T(0)) {
                        const T dudx = dx1 * p.idx, dudz = dz1 * p.idz;
                        const T phx = qx[(so + R) % Q].v[v], phz = wp[HL * VV + v];
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
                if (MODE == kFwd) bad |= !isfinite(unew);
                if (MODE == kAdj) ico.v[v] = ici.v[v] + uc * dwi.v[v];
            }
            if (own) {
                const long long o = rowoff(x) + zl;
                stg<T, VV>(uprev + o, un);
                if (PML && (zpad || xpad(x))) {
                    stg<T, VV>(p.phx_out + sh + o, pxo);
                    stg<T, VV>(p.phz_out + sh + o, pzo);
                }
                if (MODE == kRecomp && p.dw_out) stg_cs<T, VV>(p.dw_out + sh + o, dwo);
                if (MODE == kAdj && p.image) stg<T, VV>(p.ic + sh + o, ico);
            }
        }
    }
    if (p.err) {
        if (MODE == kFwd && bad && own) atomicOr(p.err, PGB_ERR_NONFINITE);
        if (late && lane == 0) atomicOr(p.err, PGB_ERR_TIMEOUT);
    }
}

template <typename T, int R, int MODE>
__global__ void __launch_bounds__(kWarps * 32) wave2d_warp_kernel(const WaveParams<T> p, const int* __restrict__ tasks,
                                                                  int ntasks, int task_blocks) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    if ((int)blockIdx.x >= task_blocks) {
        if (MODE == kFwd) record_block(p, blockIdx.x - task_blocks);
        return;
    }
    const int warp = threadIdx.x >> 5;
    const int gw = blockIdx.x * kWarps + warp;
    if (gw >= ntasks * p.nshot) return;  // warp-uniform
    const int shot = gw / ntasks;
    const int* tk = tasks + 5 * (gw - shot * ntasks);
    const int x0 = __ldg(tk), x1 = __ldg(tk + 1), zs = __ldg(tk + 2), ze = __ldg(tk + 3), kind = __ldg(tk + 4);
    unsigned char* wsm = smem_raw + warp * WarpSmem<T, R>::per_warp;
    if (kind == 0)
        sweep<T, R, MODE, 0>(p, wsm, shot, x0, x1, zs, ze);
    else
        sweep<T, R, MODE, 1>(p, wsm, shot, x0, x1, zs, ze);
}

template <typename T, int R>
void prep_warp() {
    const int b = (int)WarpSmem<T, R>::bytes;
    cudaFuncSetAttribute(wave2d_warp_kernel<T, R, kFwd>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    cudaFuncSetAttribute(wave2d_warp_kernel<T, R, kRecomp>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    cudaFuncSetAttribute(wave2d_warp_kernel<T, R, kAdj>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
}

}  // namespace

template <typename T, int R, int MODE>
void launch_wave2d_warp_tasks(const WaveParams<T>& p, const int* tasks, int ntasks, cudaStream_t s) {
    const int task_blocks = (ntasks * p.nshot + kWarps - 1) / kWarps;
    const int grid = task_blocks + (MODE == kFwd ? p.rec.blocks : 0);
    wave2d_warp_kernel<T, R, MODE><<<grid, kWarps * 32, WarpSmem<T, R>::bytes, s>>>(p, tasks, ntasks, task_blocks);
}

void wave2d_warp_prepare() {
    prep_warp<float, 1>(); prep_warp<float, 2>(); prep_warp<float, 3>(); prep_warp<float, 4>();
    prep_warp<double, 1>(); prep_warp<double, 2>(); prep_warp<double, 3>(); prep_warp<double, 4>();
}

int wave2d_warp_threads() { return kWarps * 32; }

// widest z-range a task of each kind may own: (32 - 2*HL) * VV cells (same rule as Geo)
int wave2d_warp_seg(int dtype_bytes, int order, int pml) {
    const int V = 16 / dtype_bytes;
    const int VV = pml ? (V > 1 ? V / 2 : 1) : V;
    const int R = order / 2;
    const int A = V / VV;
    const int HL = ((R + VV - 1) / VV + A - 1) / A * A;
    return (32 - 2 * HL) * VV;
}

#define PGB_INSTW(T, R)                                                                                   \
    template void launch_wave2d_warp_tasks<T, R, kFwd>(const WaveParams<T>&, const int*, int, cudaStream_t);    \
    template void launch_wave2d_warp_tasks<T, R, kRecomp>(const WaveParams<T>&, const int*, int, cudaStream_t); \
    template void launch_wave2d_warp_tasks<T, R, kAdj>(const WaveParams<T>&, const int*, int, cudaStream_t);
PGB_INSTW(float, 1)
PGB_INSTW(float, 2)
PGB_INSTW(float, 3)
PGB_INSTW(float, 4)
PGB_INSTW(double, 1)
PGB_INSTW(double, 2)
PGB_INSTW(double, 3)
PGB_INSTW(double, 4)

}  // namespace pgb
