// Batched 2D leapfrog step: persistent warps fed by per-warp shared-memory row
// rings (forward, recompute, adjoint, Born scattered field).
//
// Same maths as the reference step cda_time_scalar_2D (pysit/solvers/
// constant_density_acoustic/time/scalar/constant_density_acoustic_time_scalar_2D.h:88-179)
// with the fusions of the batched pipeline:
//   kFwd    (with kRecomp and kBorn: leading blocks of the interior kernel record the
//           traces of u_k);
//   kRecomp the imaging operand dWaveOp_k (constant_density_acoustic_base.py:24-40)
//           from the stencil's own bracket F: C^2 F where the step and mesh
//           sigmas agree, plus the sigma differences elsewhere (the right PML,
//           whose step profile is read one node further out, _2D.h:143-157);
//   kAdj    the time-reversed adjoint step with ic += q_k * dWaveOp_k fused
//           (temporal_modeling.py:312-365);
//   kBorn   the scattered field u1 of linearised modelling, its source -m1 dWaveOp0_k
//           read from the stage like the adjoint's operands and added inside the bracket
//           (linear_forward_model, temporal_modeling.py:520-535).
//
// Work decomposition: a table of warp tasks (x0, x1, zs, ze, kind) covers the
// padded grid of one shot once.  The warps of the launch are persistent: each
// takes the next (shot, task) from a global counter until the launch's tasks
// are used up, so no wave of blocks runs half empty at the end.  A task owns the
// cells z in [zs, ze) of the rows x0..x1-1; lane L holds the V consecutive cells
// from zs + L*V.  Per row x, the warp has already asked (A rows ahead) for
//   * row x+R of u_k, with an R-cell z-halo each side, into the warp's x-ring
//     of 2R+A rows (the x-derivatives read rows x-R..x+R from it);
//   * the centre rows of u_{k-1}, C^2 (and dWaveOp, ic for the adjoint; Phi_z
//     with its halo, row x+R of Phi_x for the PML) into one of A stages,
// with 1-D bulk copies (cp.async.bulk) completing on the stage's mbarrier.  Every
// operand then comes from shared memory with aligned vector loads; the loop body
// is one row (no unrolling), which keeps the kernel small enough for the
// instruction cache.  Warps never wait for each other.
// Task kinds (warp-uniform branch):
//   kind 0  interior: at least R cells away from the padding and off the outer
//           (Dirichlet) ring, 16-byte lane vectors, no PML state, no masks;
//   kind 1  PML shell: the padding and its R-wide rim, 2-cell lane vectors (more
//           busy lanes on the narrow z-bands), Phi_x / Phi_z carried where both
//           sigmas vanish as in the reference.
// Injection (_2D.h:165): the source taps of the cells of a row, inline; the
// caller may instead switch the injection off here and add it after the step.
// Each lane issues at most one of a row's bulk copies (per-lane copy descriptors),
// and the arithmetic runs on cell pairs (packed f32x2 instructions in FP32).
// Waits are bounded (2^22 blocking tries of the stage's mbarrier, or WaveParams::polls
// non-blocking tests when the plan sets a limit; WaveParams::wait_fault adds a wait that
// always runs out, for tests): on expiry the
// warp waits, with the full limit, for every copy it still has in flight, sets the
// plan's error word, and takes no further task of the launch (it still draws them from
// the counter, so the counter stays in step with the later launches of the run).
#include "tma.cuh"
#include "wave.cuh"

namespace pgb {
namespace {

constexpr int kWarps = 4;  // warps per block
constexpr uint32_t kPolls = 1u << 22;  // tries of a drain wait (and the default of WaveParams::polls)
constexpr int kSpareBar = 15;          // the last of a warp's 16 mbarrier slots: never armed (test aid)
#ifndef PGB_RING_AHEAD
#define PGB_RING_AHEAD 4   // rows whose copies are in flight ahead of the computation
#endif
#ifndef PGB_RING_RB
#define PGB_RING_RB 2      // rows per iteration of the FP32 interior sweep
#endif
#ifndef PGB_SHELL_RB
#define PGB_SHELL_RB 1     // rows per iteration of the FP32 PML-shell sweep
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
    static constexpr int V = KIND == 0 ? AL : 2;                 // cells per lane (pairs)
    static constexpr int HZ = (R + AL - 1) / AL * AL;            // z-halo cells per side
    static constexpr int NB = HZ / V;                            // halo vectors per side
    static constexpr int SEG = 32 * V;                           // cells a task owns at most
    static constexpr int WS = SEG + 2 * HZ;                      // slot with halo (elements)
    // rows per iteration: the FP32 interior sweeps two rows at a time (the per-row
    // bookkeeping is shared, and the 2R+2 rows of the window are read once)
    static constexpr int RB = sizeof(T) == 4 ? (KIND == 0 ? PGB_RING_RB : PGB_SHELL_RB) : 1;
    static constexpr int AR = (MODE == kAdj || MODE == kBorn) && PGB_RING_AHEAD > 2 ? PGB_RING_AHEAD - 1 : PGB_RING_AHEAD;
    static constexpr int A = (AR + RB - 1) / RB < 2 ? 2 : (AR + RB - 1) / RB;  // iterations in flight
    static constexpr int NU = 2 * R + RB * A;                    // x-ring slots
    static constexpr bool PML = KIND == 1;
    static constexpr int NPF = MODE == kAdj || MODE == kBorn ? 4 : 2;  // centre fields per row
    static constexpr int PST = RB * (NPF * SEG + (PML ? WS : 0));  // stage (elements)
    // u ring, Phi_x ring (same slot stride, centre at +HZ, so one row offset serves both), stages
    static constexpr int ELEMS = NU * WS * (PML ? 2 : 1) + A * PST;
    static constexpr size_t per_warp = 128 + sizeof(T) * (size_t)ELEMS;  // barriers + rings
    static constexpr size_t bytes = kWarps * per_warp;
    static_assert(A >= 2 && A <= 15, "the barrier block holds 16 mbarriers, the last one spare");
    static_assert(V % 2 == 0 && HZ % V == 0, "lanes hold whole pairs; halo in whole vectors");
    static_assert(per_warp % 16 == 0, "warp regions stay 16-byte aligned");
    static_assert(RB == 1 || RB == 2, "one or two rows per iteration");
};

// Pair arithmetic: two neighbouring cells per operation.  FP32 uses the packed
// f32x2 instructions (one issue slot for two cells, each lane rounded exactly
// like the scalar operation); FP64 spells the pair out.
template <typename T> struct PairOps;
template <> struct PairOps<float> {
    using P = float2;
    static __device__ __forceinline__ P mk(float a, float b) { return make_float2(a, b); }
    static __device__ __forceinline__ P dup(float a) { return make_float2(a, a); }
    static __device__ __forceinline__ P add(P a, P b) { return __fadd2_rn(a, b); }
    static __device__ __forceinline__ P sub(P a, P b) {
        unsigned long long d;
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(*reinterpret_cast<unsigned long long*>(&a)),
            "l"(*reinterpret_cast<unsigned long long*>(&b)));
        return *reinterpret_cast<P*>(&d);
    }
    static __device__ __forceinline__ P mul(P a, P b) { return __fmul2_rn(a, b); }
    static __device__ __forceinline__ P fma(P a, P b, P c) { return __ffma2_rn(a, b, c); }
};
template <> struct PairOps<double> {
    using P = double2;
    static __device__ __forceinline__ P mk(double a, double b) { return make_double2(a, b); }
    static __device__ __forceinline__ P dup(double a) { return make_double2(a, a); }
    static __device__ __forceinline__ P add(P a, P b) { return make_double2(a.x + b.x, a.y + b.y); }
    static __device__ __forceinline__ P sub(P a, P b) { return make_double2(a.x - b.x, a.y - b.y); }
    static __device__ __forceinline__ P mul(P a, P b) { return make_double2(a.x * b.x, a.y * b.y); }
    static __device__ __forceinline__ P fma(P a, P b, P c) {
        return make_double2(::fma(a.x, b.x, c.x), ::fma(a.y, b.y, c.y));
    }
};

// Pipeline position of a warp, carried across its tasks: the stage the next row
// uses and that stage's mbarrier phase parity.
struct Pipe {
    int s;
    uint32_t ph;
};

template <typename T> __device__ __forceinline__ T rcp_(T x);
// FP32: the fast reciprocal (within ~1 ulp; the FP32 path's tolerances are 1e-4 / 1e-3);
// FP64 keeps the exact division of the reference
template <> __device__ __forceinline__ float rcp_(float x) { return __fdividef(1.0f, x); }
template <> __device__ __forceinline__ double rcp_(double x) { return 1.0 / x; }

// Waits (full limit) for the `armed` stages from stage s on (phase parity ph, flipped past
// the ring's end): the drain after an expired wait.
__device__ __noinline__ void drain_stages(unsigned char* wsm, int s, uint32_t ph, int A, int armed) {
    for (int j = 0; j < armed; ++j) {
        const int sj = s + j < A ? s + j : s + j - A;
        mbar_wait_bounded(reinterpret_cast<uint64_t*>(wsm) + sj, s + j < A ? ph : (ph ^ 1u), kPolls);
    }
}

template <typename T, int R, int MODE, int KIND>
__device__ __forceinline__ void sweep(const WaveParams<T>& p, unsigned char* wsm, Pipe& pp, const int shot,
                                      const int x0, const int x1, const int zs, const int ze, bool& bad,
                                      bool& late) {
    using G = Ring<T, R, MODE, KIND>;
    using O = PairOps<T>;
    using P = typename O::P;
    constexpr int V = G::V, HZ = G::HZ, NB = G::NB, SEG = G::SEG, WS = G::WS, A = G::A, NU = G::NU;
    constexpr int RB = G::RB, NPF = G::NPF;
    constexpr bool PML = G::PML;
    constexpr int NW = (2 * NB + 1) * V;  // z-window of a lane
    constexpr int C0 = NB * V;            // its centre
    constexpr int NR = 2 * R + RB;        // rows an iteration reads: x-R .. x+RB-1+R
    constexpr int TB = (int)sizeof(T);
    // byte layout of the warp region: barriers | u ring | Phi_x ring (PML) | stages
    constexpr int SLOT = WS * TB, STG = G::PST * TB;
    constexpr int OFF_U = 128, OFF_X = OFF_U + NU * SLOT, OFF_P = OFF_X + (PML ? NU * SLOT : 0);
    constexpr int OFF_PZ = NPF * RB * SEG * TB;  // Phi_z rows inside a stage
    const uint32_t bar0 = smem_u32(wsm);
    const int lane = threadIdx.x & 31;
    const unsigned char* lb = wsm + lane * V * TB;  // this lane's first cell in any slot
    const int niter = x1 - x0;                      // rows
    const int nit = (niter + RB - 1) / RB;          // iterations
    const int zl = zs + lane * V;
    const bool own = zl < ze;
    const long long sh = (long long)shot * p.fstride;
    T* uprev = p.u_prev + sh;
    const bool img = MODE == kAdj && p.image;
    const bool ext = img || MODE == kBorn;  // fields 3 and 4 (dWaveOp, ic or m1) ride in the stage
    auto rowoff = [&](int x) { return (long long)(x + kHalo) * p.ldz + kOZ; };
    const int ncen = (ze - zs + G::AL - 1) / G::AL * G::AL;
    const uint32_t bu = (uint32_t)(ncen + 2 * HZ) * TB;
    const uint32_t bc = (uint32_t)ncen * TB;
    const uint32_t brow = bu + 2 * bc + (ext ? 2 * bc : 0) + (PML ? bc + bu : 0);  // bytes per row
    auto bytes_it = [&](int it) { return (uint32_t)min(RB, niter - RB * it) * brow; };

    // One bulk copy per lane and iteration: lane c copies row r = c % RB of field
    // f = c / RB (field, row offset R for the x-ring fields, halo or centre, and
    // destination: x-ring slot or stage).
    //   0 u_k -> u ring; 1 u_{k-1}, 2 C^2 -> stage; [3 dWaveOp, 4 ic -> stage];
    //   [PML: Phi_x -> Phi_x ring; Phi_z (halo) -> stage]
    const int nfield = 3 + (ext ? 2 : 0) + (PML ? 2 : 0);
    const int ncp = nfield * RB;
    const int cf = lane / RB, cr = lane - cf * RB;
    const T* csrc = nullptr;  // element of row cr (x-ring fields: row cr + R)
    uint32_t cdst = 0, cstep = 0, cbytes = 0;
    bool cring = false;
    {
        const int cpml = 3 + (ext ? 2 : 0);
        const uint32_t w0 = smem_u32(wsm);
        if (cf == 0) {
            csrc = p.u_cur + sh + rowoff(cr + R) + zs - HZ; cdst = w0 + OFF_U; cstep = SLOT; cbytes = bu; cring = true;
        } else if (cf == 1 || cf == 2 || (ext && (cf == 3 || cf == 4))) {
            const T* f = cf == 1   ? (const T*)uprev
                         : cf == 2 ? p.c2
                         : cf == 3 ? p.dw_in + sh
                                   : (MODE == kBorn ? p.m1 : (const T*)p.ic + sh);
            csrc = f + rowoff(cr) + zs;
            cdst = w0 + OFF_P + ((cf - 1) * RB + cr) * SEG * TB; cstep = STG; cbytes = bc;
        } else if (PML && cf == cpml) {
            csrc = p.phx_in + sh + rowoff(cr + R) + zs; cdst = w0 + OFF_X + HZ * TB; cstep = SLOT; cbytes = bc;
            cring = true;
        } else if (PML && cf == cpml + 1) {
            csrc = p.phz_in + sh + rowoff(cr) + zs - HZ; cdst = w0 + OFF_P + OFF_PZ + cr * SLOT; cstep = STG;
            cbytes = bu;
        }
    }
    // the rows of iteration `it` into stage s; their x-ring slots follow the rows
    auto copy_iter = [&](int it, int s) {
        if (lane < ncp && RB * it + cr < niter) {
            int slot = RB * it + 2 * R + cr;
            slot -= slot / NU * NU;
            bulk_g2s_s(cdst + (uint32_t)(cring ? slot : s) * cstep, csrc + (long long)(x0 + RB * it) * p.ldz,
                       cbytes, bar0 + 8u * s);
        }
    };
    fence_proxy_async();  // earlier generic reads of the rings before the new copies
    {
        // the 2R leading rows x0-R .. x0+R-1 of u_k (and Phi_x) ride on the first stage
        const uint32_t pro = 2 * R * (bu + (PML ? bc : 0));
        if (lane == 0) mbar_arrive_expect_tx_s(bar0 + 8u * pp.s, bytes_it(0) + pro);
        if (lane < (PML ? 4 * R : 2 * R)) {
            const int j = lane < 2 * R ? lane : lane - 2 * R;
            const bool u = lane < 2 * R;
            const T* src = (u ? p.u_cur + sh - HZ : p.phx_in + sh) + rowoff(x0 - R + j) + zs;
            const uint32_t dst = smem_u32(wsm) + (u ? OFF_U : OFF_X + HZ * TB) + j * SLOT;
            bulk_g2s_s(dst, src, u ? bu : bc, bar0 + 8u * pp.s);
        }
        copy_iter(0, pp.s);
        int s = pp.s;
        for (int it = 1; it < min(A, nit); ++it) {
            if (++s == A) s = 0;
            if (lane == 0) mbar_arrive_expect_tx_s(bar0 + 8u * s, bytes_it(it));
            copy_iter(it, s);
        }
    }

    // test aid (WaveParams::wait_fault): a bounded wait on the warp's spare mbarrier, on which
    // nothing ever arrives, runs out and takes the expiry path with this task's copies in flight
    bool expired = p.wait_fault && !__all_sync(0xffffffffu, mbar_test_bounded(reinterpret_cast<uint64_t*>(wsm) + kSpareBar,
                                                                               0u, p.polls ? p.polls : 64u));

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
    // the box is read only when the step injects (its table may be absent otherwise)
    const int* bx = p.inj.box + shot * 6;
    const int bx0 = p.inj.on ? __ldg(bx) : 0, bx1 = p.inj.on ? __ldg(bx + 1) : 0;
    const bool inj_task = p.inj.on && bx0 < x1 && bx1 > x0 && __ldg(bx + 4) < ze && __ldg(bx + 5) > zs;
    // weight pairs, built once per task
    P wx[R + 1], wz[R + 1], a1[R + 1];
#pragma unroll
    for (int m = 1; m <= R; ++m) {
        wx[m] = O::dup(T(d2w(R, m)) * p.idx2);
        wz[m] = O::dup(T(d2w(R, m)) * p.idz2);
        a1[m] = O::dup(T(d1w(R, m)));
    }

    // byte offsets of the slots holding rows x-R .. x+RB-1+R (shifted by RB every iteration)
    int ra[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) ra[j] = j * SLOT;
    int nxs = (NR) % NU;             // x-ring slot of the first row entering next
    long long o = rowoff(x0) + zl;   // element of the lane's first cell in row x
    // sigma_x (and the mesh sigma_x) of the shell rows, loaded one iteration ahead
    T sx_n = PML ? __ldg(p.sgx + x0) : T(0);
    T mx_n = PML && MODE == kRecomp ? __ldg(p.mgx + x0) : T(0);
    int it = 0;
    for (; it < (expired ? 0 : nit); ++it, o += (long long)RB * p.ldz) {
        const int x = x0 + RB * it;
        const int s = pp.s;
        const bool ok = p.polls ? mbar_test_bounded(reinterpret_cast<uint64_t*>(wsm) + s, pp.ph, p.polls)
                                : mbar_wait_bounded(reinterpret_cast<uint64_t*>(wsm) + s, pp.ph, kPolls);
        if (!__all_sync(0xffffffffu, ok)) {
            expired = true;
            break;
        }
        const unsigned char* sb = lb + OFF_P + s * STG;  // this lane in stage s

        // ---- the shared-memory reads of this iteration ---------------------------------
        Vec<T, V> cv[NR];  // u_k rows x-R .. x+RB-1+R at the lane's cells
#pragma unroll
        for (int j = 0; j < NR; ++j) cv[j] = lds<T, V>(reinterpret_cast<const T*>(lb + OFF_U + ra[j] + HZ * TB));
        const T sx = sx_n, mgx = mx_n;
        if (PML && it + 1 < nit) {
            sx_n = __ldg(p.sgx + x + 1);
            if (MODE == kRecomp) mx_n = __ldg(p.mgx + x + 1);
        }
        (void)sx; (void)mgx;

#pragma unroll
        for (int r = 0; r < RB; ++r) {
            const int xr = x + r;
            const bool valid = RB == 1 || RB * it + r < niter;  // an odd last row has no partner
            T w[NW];  // u_k row xr around the lane's cells
#pragma unroll
            for (int j = 0; j <= 2 * NB; ++j) {
                const Vec<T, V> a = j == NB ? cv[R + r]
                                            : lds<T, V>(reinterpret_cast<const T*>(lb + OFF_U + ra[R + r] + j * V * TB));
#pragma unroll
                for (int v = 0; v < V; ++v) w[j * V + v] = a.v[v];
            }
            const Vec<T, V> um = lds<T, V>(reinterpret_cast<const T*>(sb + (0 * RB + r) * SEG * TB));
            const Vec<T, V> cc = lds<T, V>(reinterpret_cast<const T*>(sb + (1 * RB + r) * SEG * TB));
            Vec<T, V> dwi, ici;
            if ((MODE == kAdj && img) || MODE == kBorn) {  // for kBorn: dWaveOp0 and m1
                dwi = lds<T, V>(reinterpret_cast<const T*>(sb + (2 * RB + r) * SEG * TB));
                ici = lds<T, V>(reinterpret_cast<const T*>(sb + (3 * RB + r) * SEG * TB));
            }
            Vec<T, V> px[2 * R + 1];  // Phi_x rows xr-R..xr+R (PML tasks)
            T wp[NW];                 // Phi_z row xr around the lane's cells (PML tasks)
            if (PML) {
#pragma unroll
                for (int j = 0; j <= 2 * R; ++j)
                    px[j] = lds<T, V>(reinterpret_cast<const T*>(lb + OFF_X + ra[r + j] + HZ * TB));
#pragma unroll
                for (int j = 0; j <= 2 * NB; ++j) {
                    const Vec<T, V> a = lds<T, V>(reinterpret_cast<const T*>(sb + OFF_PZ + r * SLOT + j * V * TB));
#pragma unroll
                    for (int v = 0; v < V; ++v) wp[j * V + v] = a.v[v];
                }
            }

            // ---- the update of row xr, two cells at a time ----------------------------------
            const bool xok = xr > 0 && xr < p.nx - 1;
            const bool inj_row = inj_task && own && xr >= bx0 && xr < bx1;
            Vec<T, V> un, dwo, pxo, pzo, ico;
#pragma unroll
            for (int k = 0; k < V / 2; ++k) {
                const int v0 = 2 * k;
                auto pr = [&](const Vec<T, V>& a) { return O::mk(a.v[v0], a.v[v0 + 1]); };
                auto pw = [&](const T* a, int d) { return O::mk(a[C0 + v0 + d], a[C0 + v0 + 1 + d]); };
                const P uc = pw(w, 0);
                // Laplacian in difference form: sum_m w_m ((u_+m - u_0) + (u_-m - u_0)),
                // equal to the central stencil because the weights sum to zero, and free
                // of the large cancellation of w_0 u_0 (the FP32 path depends on this)
                // (x and z accumulate separately: two short dependency chains)
                P Fx = O::dup(T(0)), Fz = Fx;
#pragma unroll
                for (int m = 1; m <= R; ++m) {
                    Fx = O::fma(wx[m], O::add(O::sub(pr(cv[R + r + m]), uc), O::sub(pr(cv[R + r - m]), uc)), Fx);
                    Fz = O::fma(wz[m], O::add(O::sub(pw(w, m), uc), O::sub(pw(w, -m), uc)), Fz);
                }
                P F = O::add(Fx, Fz);
                if (inj_row) {
                    F.x += inject_rhs(p.inj, bx, shot, xr, zl + v0);
                    F.y += inject_rhs(p.inj, bx, shot, xr, zl + v0 + 1);
                }
                if (MODE == kBorn) F = O::sub(F, O::mul(pr(ici), pr(dwi)));  // rhs = -m1 dWaveOp0
                const P uo = pr(um), c2 = pr(cc);
                // interior tasks never touch the outer (Dirichlet) ring: no masks there
                const bool ok0 = !PML || (xok && zok[v0]), ok1 = !PML || (xok && zok[v0 + 1]);
                P unew;
                if (PML) {
                    P dpx = O::dup(T(0)), dpz = dpx, dx1 = dpx, dz1 = dpx;
#pragma unroll
                    for (int m = 1; m <= R; ++m) {
                        const P a = a1[m];
                        dpx = O::fma(a, O::sub(pr(px[R + m]), pr(px[R - m])), dpx);
                        dpz = O::fma(a, O::sub(pw(wp, m), pw(wp, -m)), dpz);
                        dx1 = O::fma(a, O::sub(pr(cv[R + r + m]), pr(cv[R + r - m])), dx1);
                        dz1 = O::fma(a, O::sub(pw(w, m), pw(w, -m)), dz1);
                    }
                    F = O::add(F, O::fma(dpx, O::dup(p.idx), O::mul(dpz, O::dup(p.idz))));
                    // split-field PML update (_2D.h:157-170), branch-free: with both sigmas
                    // zero it reduces to the plain leapfrog update and carries Phi unchanged
                    const P szp = O::mk(sgz[v0], sgz[v0 + 1]);
                    const P dsx = O::dup(p.dt * sx), dsz = O::mul(O::dup(p.dt), szp);
                    const P S = O::add(O::dup(sx), szp);  // sx + sz
                    const P phx = pr(px[R]), phz = pw(wp, 0);
                    // Phi' = Phi - dt s Phi + dt (s_other - s) du/dn
                    P ph_x = O::fma(O::mul(O::sub(dsz, dsx), O::dup(p.idx)), dx1, O::fma(dsx, O::mul(phx, O::dup(T(-1))), phx));
                    P ph_z = O::fma(O::mul(O::sub(dsx, dsz), O::dup(p.idz)), dz1, O::fma(dsz, O::mul(phz, O::dup(T(-1))), phz));
                    // u' = 2 dt^2 / (2 + dt S) * (C^2 F - (u_{k-1} - 2u)/dt^2 + S u_{k-1}/(2dt) - sx sz u)
                    const P den = O::fma(O::dup(p.dt), S, O::dup(T(2)));
                    const P fac1 = O::mul(O::dup(T(2) * p.dt2), O::mk(rcp_(den.x), rcp_(den.y)));
                    const P c2F = O::mul(c2, F);
                    P fac2 = O::fma(O::fma(O::dup(T(-2)), uc, uo), O::dup(-p.idt2), c2F);
                    fac2 = O::fma(O::mul(S, O::dup(p.i2dt)), uo, fac2);
                    fac2 = O::fma(O::mul(O::dup(-sx), szp), uc, fac2);
                    unew = O::mul(fac1, fac2);
                    if (!ok0) { unew.x = T(0); ph_x.x = T(0); ph_z.x = T(0); }
                    if (!ok1) { unew.y = T(0); ph_x.y = T(0); ph_z.y = T(0); }
                    pxo.v[v0] = ph_x.x; pxo.v[v0 + 1] = ph_x.y;
                    pzo.v[v0] = ph_z.x; pzo.v[v0 + 1] = ph_z.y;
                    if (MODE == kRecomp) {
                        // dWaveOp = C^2 F + (sm - s)(u' - u_{k-1})/(2dt) + (smx smz - sx sz) u
                        const P mzp = O::mk(mgz[v0], mgz[v0 + 1]);
                        const P dS = O::sub(O::add(O::dup(mgx), mzp), S);
                        const P dP = O::sub(O::mul(O::dup(mgx), mzp), O::mul(O::dup(sx), szp));
                        P d = O::fma(O::mul(dS, O::dup(p.i2dt)), O::sub(unew, uo), c2F);
                        d = O::fma(dP, uc, d);
                        dwo.v[v0] = ok0 ? d.x : T(0);
                        dwo.v[v0 + 1] = ok1 ? d.y : T(0);
                    }
                } else {
                    // u_{k+1} = dt^2 C^2 F - (u_{k-1} - 2 u_k)
                    const P q = O::fma(O::dup(T(-2)), uc, uo);
                    unew = O::fma(O::mul(O::dup(p.dt2), c2), F, O::mul(q, O::dup(T(-1))));
                    if (MODE == kRecomp) {
                        const P d = O::mul(c2, F);
                        dwo.v[v0] = d.x;
                        dwo.v[v0 + 1] = d.y;
                    }
                }
                un.v[v0] = unew.x;
                un.v[v0 + 1] = unew.y;
                if (MODE == kAdj) {
                    const P ic = O::fma(uc, pr(dwi), pr(ici));
                    ico.v[v0] = ic.x;
                    ico.v[v0 + 1] = ic.y;
                }
            }
            if (MODE == kFwd || MODE == kBorn || (MODE == kRecomp && p.nan_check)) {  // a NaN or Inf anywhere in the lane's cells survives the sum
                T sum = T(0);
#pragma unroll
                for (int v = 0; v < V; ++v) sum += un.v[v];
                bad |= own && valid && !isfinite(sum);
            }
            if (own && valid) {
                const long long orow = o + (long long)r * p.ldz;
                stg<T, V>(uprev + orow, un);
                if (PML) {
                    stg<T, V>(p.phx_out + sh + orow, pxo);
                    stg<T, V>(p.phz_out + sh + orow, pzo);
                }
                if (MODE == kRecomp && p.dw_out) stg_cs<T, V>(p.dw_out + sh + orow, dwo);
                if (MODE == kAdj && img) stg<T, V>(p.ic + sh + orow, ico);
            }
        }

        // ---- refill: every lane is done with stage s and rows x-R .. x-R+RB-1 ---------------
        __syncwarp();
        if (it + A < nit) {
            fence_proxy_async();
            if (lane == 0) mbar_arrive_expect_tx_s(bar0 + 8u * s, bytes_it(it + A));
            copy_iter(it + A, s);
        }
        if (++pp.s == A) { pp.s = 0; pp.ph ^= 1u; }
#pragma unroll
        for (int j = 0; j < 2 * R; ++j) ra[j] = ra[j + RB];
#pragma unroll
        for (int q = 0; q < RB; ++q) {
            const int t = nxs + q;
            ra[2 * R + q] = (t >= NU ? t - NU : t) * SLOT;
        }
        nxs += RB;
        if (nxs >= NU) nxs -= NU;
    }
    if (expired) {
        // every stage armed for iterations it .. it+A-1 may still receive bytes: wait for those
        // phases with the full limit before the warp leaves its tasks
        late = true;
        drain_stages(wsm, pp.s, pp.ph, A, min(A, nit - it));
    }
}

// Resident blocks per SM the register budget aims at (FP32): four 4-warp blocks
// (128 registers); a one-row interior sweep fits five (96 registers).
#ifndef PGB_SHELL_MINB
#define PGB_SHELL_MINB 4   // resident 4-warp blocks per SM the FP32 PML-shell kernel aims at
#endif
template <typename T, int KIND>
struct MinBlocks {
    static constexpr int value = sizeof(T) == 4 ? (KIND == 0 ? (PGB_RING_RB == 1 ? 5 : 4) : PGB_SHELL_MINB) : 1;
};

template <typename T, int R, int MODE, int KIND>
__global__ void __launch_bounds__(kWarps * 32, (MinBlocks<T, KIND>::value))
    wave2d_warp_kernel(const WaveParams<T> p, const int* __restrict__ tasks, int ntasks, int rec_blocks) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    if ((int)blockIdx.x < rec_blocks) {
        if (MODE != kAdj) record_block(p, blockIdx.x);
        return;
    }
    using G = Ring<T, R, MODE, KIND>;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* wsm = smem_raw + warp * G::per_warp;
    uint64_t* bar = reinterpret_cast<uint64_t*>(wsm);
    constexpr int A = G::A;
    if (lane == 0) {
        for (int s = 0; s < A; ++s) mbar_init(&bar[s], 1);
        if (p.wait_fault) mbar_init(&bar[kSpareBar], 1);  // one arrival expected, none ever made
        fence_mbar_init();
    }
    __syncwarp();
    unsigned long long* ctr = p.task_ctr + KIND;
    const unsigned long long base = KIND == 0 ? p.task_base : p.task_base2;
    const unsigned long long total = (unsigned long long)ntasks * (unsigned)p.nshot;
    Pipe pp{0, 0u};
    bool bad = false, late = false;
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(ctr, 1ull) - base;
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= total) break;
        if (late) continue;  // an expired wait: the remaining tasks are drawn, not run
        const int shot = (int)(t / (unsigned)ntasks);
        const int* tk = tasks + 5 * (int)(t - (unsigned long long)shot * ntasks);
        sweep<T, R, MODE, KIND>(p, wsm, pp, shot, __ldg(tk), __ldg(tk + 1), __ldg(tk + 2), __ldg(tk + 3), bad, late);
    }
    if (p.err) {
        if (MODE != kAdj && bad) atomicOr(p.err, PGB_ERR_NONFINITE);
        if (late && lane == 0) atomicOr(p.err, PGB_ERR_TIMEOUT);
    }
}

template <typename T, int R, int MODE, int KIND>
void prep_one() {
    using G = Ring<T, R, MODE, KIND>;
    cudaFuncSetAttribute(wave2d_warp_kernel<T, R, MODE, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)G::bytes);
    // all of the unified L1 / shared storage as shared memory: the rings are the working set
    cudaFuncSetAttribute(wave2d_warp_kernel<T, R, MODE, KIND>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         (int)cudaSharedmemCarveoutMaxShared);
}
template <typename T, int R>
void prep_warp() {
    prep_one<T, R, kFwd, 0>(); prep_one<T, R, kRecomp, 0>(); prep_one<T, R, kAdj, 0>(); prep_one<T, R, kBorn, 0>();
    prep_one<T, R, kFwd, 1>(); prep_one<T, R, kRecomp, 1>(); prep_one<T, R, kAdj, 1>(); prep_one<T, R, kBorn, 1>();
}

template <typename T, int R, int MODE, int KIND>
int occupancy() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, wave2d_warp_kernel<T, R, MODE, KIND>, kWarps * 32,
                                                      Ring<T, R, MODE, KIND>::bytes) != cudaSuccess)
        n = 1;
    return n > 0 ? n : 1;
}

}  // namespace

template <typename T, int R, int MODE, int KIND>
long long launch_wave2d_warp_tasks(const WaveParams<T>& p, const int* tasks, int ntasks, int blocks,
                                   cudaStream_t s) {
    const int rec = MODE != kAdj && KIND == 0 ? p.rec.blocks : 0;
    wave2d_warp_kernel<T, R, MODE, KIND>
        <<<rec + blocks, kWarps * 32, Ring<T, R, MODE, KIND>::bytes, s>>>(p, tasks, ntasks, rec);
    // counter values the launch consumes: one per task plus one final fetch per warp
    return (long long)ntasks * p.nshot + (long long)blocks * kWarps;
}

void wave2d_warp_prepare() {
    prep_warp<float, 1>(); prep_warp<float, 2>(); prep_warp<float, 3>(); prep_warp<float, 4>();
    prep_warp<double, 1>(); prep_warp<double, 2>(); prep_warp<double, 3>(); prep_warp<double, 4>();
}

int wave2d_warp_threads() { return kWarps * 32; }

// persistent blocks of one launch: resident blocks per SM x SMs
int wave2d_warp_blocks(int dtype_bytes, int order, int mode, int kind) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int R = order / 2;
    int occ = 1;
#define PGB_OCC(TT, RR)                                                                          \
    occ = kind == 0 ? (mode == kFwd ? occupancy<TT, RR, kFwd, 0>()                               \
                       : mode == kRecomp ? occupancy<TT, RR, kRecomp, 0>()                       \
                       : mode == kAdj ? occupancy<TT, RR, kAdj, 0>() : occupancy<TT, RR, kBorn, 0>()) \
                    : (mode == kFwd ? occupancy<TT, RR, kFwd, 1>()                               \
                       : mode == kRecomp ? occupancy<TT, RR, kRecomp, 1>()                       \
                       : mode == kAdj ? occupancy<TT, RR, kAdj, 1>() : occupancy<TT, RR, kBorn, 1>())
    if (dtype_bytes == 4) {
        switch (R) { case 1: PGB_OCC(float, 1); break; case 2: PGB_OCC(float, 2); break;
                     case 3: PGB_OCC(float, 3); break; default: PGB_OCC(float, 4); break; }
    } else {
        switch (R) { case 1: PGB_OCC(double, 1); break; case 2: PGB_OCC(double, 2); break;
                     case 3: PGB_OCC(double, 3); break; default: PGB_OCC(double, 4); break; }
    }
#undef PGB_OCC
    return occ * sms;
}

// widest z-range a task of each kind may own: 32 lanes x V cells (same rule as Ring)
int wave2d_warp_seg(int dtype_bytes, int order, int pml) {
    (void)order;
    const int V = pml ? 2 : 16 / dtype_bytes;
    return 32 * V;
}

#define PGB_INSTW1(T, R, K)                                                                                     \
    template long long launch_wave2d_warp_tasks<T, R, kFwd, K>(const WaveParams<T>&, const int*, int, int,       \
                                                               cudaStream_t);                                    \
    template long long launch_wave2d_warp_tasks<T, R, kRecomp, K>(const WaveParams<T>&, const int*, int, int,    \
                                                                  cudaStream_t);                                 \
    template long long launch_wave2d_warp_tasks<T, R, kAdj, K>(const WaveParams<T>&, const int*, int, int,       \
                                                               cudaStream_t);                                    \
    template long long launch_wave2d_warp_tasks<T, R, kBorn, K>(const WaveParams<T>&, const int*, int, int,      \
                                                                cudaStream_t);
#define PGB_INSTW(T, R) PGB_INSTW1(T, R, 0) PGB_INSTW1(T, R, 1)
PGB_INSTW(float, 1)
PGB_INSTW(float, 2)
PGB_INSTW(float, 3)
PGB_INSTW(float, 4)
PGB_INSTW(double, 1)
PGB_INSTW(double, 2)
PGB_INSTW(double, 3)
PGB_INSTW(double, 4)

}  // namespace pgb
