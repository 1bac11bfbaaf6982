// Batched 1D and 3D leapfrog steps (forward, recompute, adjoint modes) on the
// internal zero-halo layout of wave.cuh, for cda_time_scalar_1D (pysit/solvers/
// constant_density_acoustic/time/scalar/constant_density_acoustic_time_scalar_1D.h:78-130)
// and cda_time_scalar_3D (..._3D.h:107-235).
//
// 3D: a table of block tasks covers the padded grid once (interior: R cells
// clear of the padding and off the outer ring; PML shell: the rest).  Each kind
// is its own kernel; both sweep along x with the neighbour planes in L1, V cells
// (one 16-byte vector) per lane.
// 1D: one thread per cell.
//
// 3D auxiliary state: Phi_x/y/z is non-zero only inside the padding; psi
// (integrated on every cell by the reference, _3D.h:216,230) only influences
// the outputs through products of two or three sigmas, so the batched path
// integrates it only where at least two axes are inside the padding.
#include "wave.cuh"

namespace pgb {
namespace {

template <typename T>
__device__ __forceinline__ T inject_rhs3(const Inject<T>& inj, const int* bx, int shot, int x,
                                         int y, int z) {
    if (x < bx[0] || x >= bx[1] || y < bx[2] || y >= bx[3] || z < bx[4] || z >= bx[5]) return T(0);
    long long c = ((long long)(x - bx[0]) * (bx[3] - bx[2]) + (y - bx[2])) * (bx[5] - bx[4]) + (z - bx[4]);
    const int* rp = inj.rowptr + inj.rpbase[shot];
    int e0 = __ldg(rp + c), e1 = __ldg(rp + c + 1);
    const T* amp = inj.amp + shot * inj.amp_sstride;
    T acc = T(0);
    for (int e = e0; e < e1; ++e) acc += __ldg(inj.w + e) * __ldg(amp + __ldg(inj.pt + e));
    return acc;
}

template <typename T>
__device__ __forceinline__ void record3(const WaveParams<T>& p, long long id) {
    long long total = (long long)p.nshot * p.rec.nrec;
    if (id >= total) return;
    int shot = (int)(id / p.rec.nrec), r = (int)(id - (long long)shot * p.rec.nrec);
    int e0 = __ldg(p.rec.rowptr + id), e1 = __ldg(p.rec.rowptr + id + 1);
    const T* u = p.u_cur + (long long)shot * p.fstride;
    T acc = T(0);
    for (int e = e0; e < e1; ++e) acc += __ldg(p.rec.w + e) * u[__ldg(p.rec.off + e)];
    p.rec.traces[shot * p.rec.tr_sstride + r] = acc;
}

// derivative taps around v (a cell's address) along a 32-bit stride s (a field of one
// shot has fewer than 2^31 elements): first derivative sum_m a_m (v_+m - v_-m) ...
template <typename T, int R>
__device__ __forceinline__ T dd1(const T* __restrict__ v, int s) {
    T a = T(0);
#pragma unroll
    for (int m = 1; m <= R; ++m) a += T(d1w(R, m)) * (v[m * s] - v[-m * s]);
    return a;
}
// ... and second derivative in difference form: sum_m w_m ((v_+m - v_0) + (v_-m - v_0)),
// equal to the central stencil (the weights sum to zero) with far less FP32
// cancellation than w_0 v_0 + sum_m w_m (v_+m + v_-m)
template <typename T, int R>
__device__ __forceinline__ T dd2(const T* __restrict__ v, int s) {
    const T c = v[0];
    T a = T(0);
#pragma unroll
    for (int m = 1; m <= R; ++m) a += T(d2w(R, m)) * ((v[m * s] - c) + (v[-m * s] - c));
    return a;
}

// ---- task sweeps ---------------------------------------------------------------
// A task (x0, x1, y0, y1, zs, ze) is handled by one block: warp w owns y-row
// y0 + w and sweeps x0..x1-1 over the z-range [zs, ze).  The block's rows of the
// 2R+1 planes around x stay in L1 while it marches, so u_k comes from DRAM
// about once; the x- and y-neighbours are constant offsets from the centre row.
constexpr int kW3 = 8;  // warps (y-rows) per block
#ifndef PGB_3D_AHEAD
#define PGB_3D_AHEAD 1     // interior: rows ahead whose operands are prefetched into L1 (0: none)
#endif
#ifndef PGB_3D_SHELL_AHEAD
#define PGB_3D_SHELL_AHEAD 1  // the same for the PML shell
#endif

// L1 prefetch of the line holding q (the addresses used are rows the task reads)
__device__ __forceinline__ void pf_l1(const void* q) { asm volatile("prefetch.global.L1 [%0];" ::"l"(q)); }

// the operands of row (i, j) that are not in L1 yet when the sweep gets there:
// the new x-neighbour plane, the y-neighbour rows, u_{k-1}, C^2 (and the PML
// state / adjoint operands); o is the element offset of the row's first cell
template <typename T, int R, int MODE, bool PML>
__device__ __forceinline__ void prefetch_row(const WaveParams<T>& p, long long sh, long long o) {
    const long long ys = p.ldz, xs = (long long)p.rows_y * p.ldz;
    pf_l1(p.u_cur + sh + o + R * xs);
#pragma unroll
    for (int m = 1; m <= R; ++m) {
        pf_l1(p.u_cur + sh + o - m * ys);
        pf_l1(p.u_cur + sh + o + m * ys);
    }
    pf_l1(p.u_prev + sh + o);
    pf_l1(p.c2 + o);
    if (MODE == kAdj && p.image) {
        pf_l1(p.dw_in + sh + o);
        pf_l1(p.ic + sh + o);
    }
    if (PML) {
        pf_l1(p.phx_in + sh + o + R * xs);
        pf_l1(p.phz_in + sh + o);
#pragma unroll
        for (int m = 1; m <= R; ++m) {
            pf_l1(p.phy_in + sh + o - m * ys);
            pf_l1(p.phy_in + sh + o + m * ys);
        }
    }
}

template <typename T> struct Vec3;
template <> struct Vec3<float> { using type = float4; static constexpr int N = 4; };
template <> struct Vec3<double> { using type = double2; static constexpr int N = 2; };

template <typename T> struct Pair3;
template <> struct Pair3<float> {
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
template <> struct Pair3<double> {
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

template <typename T>
__device__ __forceinline__ typename Vec3<T>::type ldv(const T* q) {
    return __ldg(reinterpret_cast<const typename Vec3<T>::type*>(q));
}
template <typename T>
__device__ __forceinline__ typename Vec3<T>::type ldv_plain(const T* q) {
    return *reinterpret_cast<const typename Vec3<T>::type*>(q);
}

// Interior: 16-byte vectors (V cells per lane), arithmetic on cell pairs, no PML
// state (every tap is off the padding), no masks (off the outer ring).  Task
// z-bounds are multiples of 4 cells, so every vector load is aligned; a task whose
// z-range is at most 16 vectors gives a warp several y-rows (wave3d_task_rows).
#ifndef PGB_3D_INT_MINB
#define PGB_3D_INT_MINB 2  // resident interior blocks per SM the register budget aims at (FP32)
#endif
template <typename T, int R, int MODE>
__global__ void __launch_bounds__(kW3 * 32, (sizeof(T) == 4 ? PGB_3D_INT_MINB : 1))
    wave3d_interior_kernel(const WaveParams<T> p, const int* __restrict__ tasks, int ntasks) {
    using O = Pair3<T>;
    using P = typename O::P;
    using VT = typename Vec3<T>::type;
    constexpr int V = Vec3<T>::N;
    constexpr int AL = 16 / (int)sizeof(T);
    constexpr int HZ = (R + AL - 1) / AL * AL;
    constexpr int NB = HZ / V;
    constexpr int NW = (2 * NB + 1) * V;
    constexpr int C0 = NB * V;
    const int shot = blockIdx.x / ntasks;
    const int* tk = tasks + 6 * (blockIdx.x - shot * ntasks);
    // the task's z-range takes nzv lanes of a y-row and a warp 32 / nzv rows
    const int zs = __ldg(tk + 4), nzv = (__ldg(tk + 5) - zs) / V, rpw = 32 / nzv;
    const int lane = threadIdx.x & 31, r = lane / nzv;
    const int j = __ldg(tk + 2) + (threadIdx.x >> 5) * rpw + r;
    if (r >= rpw || j >= __ldg(tk + 3)) return;
    const int zl = zs + (lane - r * nzv) * V;
    const int x0 = __ldg(tk), x1 = __ldg(tk + 1);
    const long long sh = (long long)shot * p.fstride;
    const long long ys = p.ldz, xs = (long long)p.rows_y * p.ldz;
    P wx[R + 1], wy[R + 1], wz[R + 1];
#pragma unroll
    for (int m = 1; m <= R; ++m) {
        wx[m] = O::dup(T(d2w(R, m)) * p.idx2);
        wy[m] = O::dup(T(d2w(R, m)) * p.idy2);
        wz[m] = O::dup(T(d2w(R, m)) * p.idz2);
    }
    const int* bx = p.inj.box + shot * 6;
    const bool inj_col = p.inj.on && j >= bx[2] && j < bx[3] && zl + V > bx[4] && zl < bx[5];
    bool bad = false;
    long long o = ((long long)(x0 + p.hx) * p.rows_y + (j + p.hy)) * p.ldz + kOZ + zl;
    for (int i = x0; i < x1; ++i, o += xs) {
        if (PGB_3D_AHEAD > 0)
            prefetch_row<T, R, MODE, false>(p, sh, o + (long long)(min(i + PGB_3D_AHEAD, x1 - 1) - i) * xs);
        const T* u = p.u_cur + sh + o;
        T w[NW];
#pragma unroll
        for (int q = 0; q <= 2 * NB; ++q) {
            const VT a = ldv(u + (q - NB) * V);
            const T* av = reinterpret_cast<const T*>(&a);
#pragma unroll
            for (int v = 0; v < V; ++v) w[q * V + v] = av[v];
        }
        VT xa[2 * R], ya[2 * R];
#pragma unroll
        for (int m = 1; m <= R; ++m) {
            xa[R - m] = ldv(u - m * xs);
            xa[R + m - 1] = ldv(u + m * xs);
            ya[R - m] = ldv(u - m * ys);
            ya[R + m - 1] = ldv(u + m * ys);
        }
        const VT uo_v = ldv_plain(p.u_prev + sh + o);
        const VT c2_v = ldv(p.c2 + o);
        VT dw_v, ic_v;
        if (MODE == kAdj && p.image) {
            dw_v = __ldcs(reinterpret_cast<const VT*>(p.dw_in + sh + o));
            ic_v = ldv_plain(p.ic + sh + o);
        }
        const T* uov = reinterpret_cast<const T*>(&uo_v);
        const T* c2v = reinterpret_cast<const T*>(&c2_v);
        const T* dwv = reinterpret_cast<const T*>(&dw_v);
        const T* icv = reinterpret_cast<const T*>(&ic_v);
        T un[V], dwo[V], ico[V];
#pragma unroll
        for (int k2 = 0; k2 < V / 2; ++k2) {
            const int v0 = 2 * k2;
            auto pv = [&](const VT& a) {
                const T* t = reinterpret_cast<const T*>(&a);
                return O::mk(t[v0], t[v0 + 1]);
            };
            const P uc = O::mk(w[C0 + v0], w[C0 + v0 + 1]);
            // Laplacian in difference form (the FP32 path depends on it), one chain per axis
            P Fx = O::dup(T(0)), Fy = Fx, Fz = Fx;
#pragma unroll
            for (int m = 1; m <= R; ++m) {
                Fx = O::fma(wx[m], O::add(O::sub(pv(xa[R + m - 1]), uc), O::sub(pv(xa[R - m]), uc)), Fx);
                Fy = O::fma(wy[m], O::add(O::sub(pv(ya[R + m - 1]), uc), O::sub(pv(ya[R - m]), uc)), Fy);
                const P zp = O::mk(w[C0 + v0 + m], w[C0 + v0 + 1 + m]);
                const P zm = O::mk(w[C0 + v0 - m], w[C0 + v0 + 1 - m]);
                Fz = O::fma(wz[m], O::add(O::sub(zp, uc), O::sub(zm, uc)), Fz);
            }
            P F = O::add(O::add(Fx, Fy), Fz);
            if (inj_col) {
                F.x += inject_rhs3(p.inj, bx, shot, i, j, zl + v0);
                F.y += inject_rhs3(p.inj, bx, shot, i, j, zl + v0 + 1);
            }
            const P uo = O::mk(uov[v0], uov[v0 + 1]), c2 = O::mk(c2v[v0], c2v[v0 + 1]);
            // u_{k+1} = dt^2 C^2 F - (u_{k-1} - 2 u_k)
            const P q = O::fma(O::dup(T(-2)), uc, uo);
            const P unew = O::fma(O::mul(O::dup(p.dt2), c2), F, O::mul(q, O::dup(T(-1))));
            un[v0] = unew.x; un[v0 + 1] = unew.y;
            if (MODE == kRecomp) {
                const P d = O::mul(c2, F);
                dwo[v0] = d.x; dwo[v0 + 1] = d.y;
            }
            if (MODE == kAdj) {
                const P ic = O::fma(uc, O::mk(dwv[v0], dwv[v0 + 1]), O::mk(icv[v0], icv[v0 + 1]));
                ico[v0] = ic.x; ico[v0 + 1] = ic.y;
            }
        }
        *reinterpret_cast<VT*>(p.u_prev + sh + o) = *reinterpret_cast<const VT*>(un);
        if (MODE == kRecomp && p.dw_out) __stcs(reinterpret_cast<VT*>(p.dw_out + sh + o), *reinterpret_cast<const VT*>(dwo));
        if (MODE == kAdj && p.image) *reinterpret_cast<VT*>(p.ic + sh + o) = *reinterpret_cast<const VT*>(ico);
        if (MODE == kFwd || (MODE == kRecomp && p.nan_check)) {
            T sum = T(0);
#pragma unroll
            for (int v = 0; v < V; ++v) sum += un[v];
            bad |= !isfinite(sum);
        }
    }
    if (MODE != kAdj && bad && p.err) atomicOr(p.err, PGB_ERR_NONFINITE);
}

// a lane's V cells as an array (the components of a vector load)
template <typename T>
__device__ __forceinline__ T vc(const typename Vec3<T>::type& a, int v) {
    return reinterpret_cast<const T*>(&a)[v];
}

// store the first n of a lane's V cells: one vector store when all belong to the task
template <typename T, bool STREAM>
__device__ __forceinline__ void st_lane(T* q, const T* a, int n) {
    using VT = typename Vec3<T>::type;
    constexpr int V = Vec3<T>::N;
    if (n == V) {
        if constexpr (STREAM) __stcs(reinterpret_cast<VT*>(q), *reinterpret_cast<const VT*>(a));
        else *reinterpret_cast<VT*>(q) = *reinterpret_cast<const VT*>(a);
    } else {
#pragma unroll
        for (int v = 0; v < V; ++v)
            if (v < n) {
                if constexpr (STREAM) __stcs(q + v, a[v]);
                else q[v] = a[v];
            }
    }
}

// first derivative sum_m a_m (v_+m - v_-m) of each of a lane's cells along x or y
// from the 2R tap vectors t (t[R - m] at -m, t[R + m - 1] at +m), scaled by h
template <typename T, int R>
__device__ __forceinline__ void dd1_taps(const typename Vec3<T>::type (&t)[2 * R], T h, T* out) {
#pragma unroll
    for (int v = 0; v < Vec3<T>::N; ++v) {
        T a = T(0);
#pragma unroll
        for (int m = 1; m <= R; ++m) a += T(d1w(R, m)) * (vc<T>(t[R + m - 1], v) - vc<T>(t[R - m], v));
        out[v] = a * h;
    }
}
template <typename T, int R>
__device__ __forceinline__ void load_taps(const T* q, int s, typename Vec3<T>::type (&t)[2 * R]) {
#pragma unroll
    for (int m = 1; m <= R; ++m) {
        t[R - m] = ldv(q - m * s);
        t[R + m - 1] = ldv(q + m * s);
    }
}
// the centre window along z: the lane's V cells with HZ cells on either side
template <typename T, int NB>
__device__ __forceinline__ void load_window(const T* q, T* w) {
    constexpr int V = Vec3<T>::N;
#pragma unroll
    for (int b = 0; b <= 2 * NB; ++b) {
        const typename Vec3<T>::type a = ldv(q + (b - NB) * V);
#pragma unroll
        for (int v = 0; v < V; ++v) w[b * V + v] = vc<T>(a, v);
    }
}

// PML shell: V cells per lane along z (16-byte vectors), each with the general
// update of the reference's 3D step (_3D.h:107-235) and the batched fusions.  A
// task's z-range [zs, ze) (zs a multiple of 4, at most 32 vectors) takes nzv
// lanes of a y-row and a warp 32 / nzv rows; cells of a vector at or past ze are
// read (zero padding) but not written.  Operand groups no cell of the lane needs
// are skipped: Phi taps that can only meet zero state, psi away from the bands
// where two axes are in the padding, the PML terms where no sigma is set.  Cells
// of the outer ring get zero.
#ifndef PGB_3D_SHELL_WARPS
#define PGB_3D_SHELL_WARPS 8  // warps of a shell block
#endif
#ifndef PGB_3D_SHELL_MINB
#define PGB_3D_SHELL_MINB (16 / PGB_3D_SHELL_WARPS)  // resident shell blocks per SM (FP32): 128 registers
#endif
constexpr int kW3S = PGB_3D_SHELL_WARPS;
template <typename T, int R, int MODE>
__global__ void __launch_bounds__(kW3S * 32, (sizeof(T) == 4 ? PGB_3D_SHELL_MINB : 1))
    wave3d_shell_kernel(const WaveParams<T> p, const int* __restrict__ tasks, int ntasks) {
    using VT = typename Vec3<T>::type;
    constexpr int V = Vec3<T>::N;
    constexpr int AL = 16 / (int)sizeof(T);
    constexpr int HZ = (R + AL - 1) / AL * AL;
    constexpr int NB = HZ / V;
    constexpr int NW = (2 * NB + 1) * V;
    constexpr int C0 = NB * V;
    const int shot = blockIdx.x / ntasks;
    const int* tk = tasks + 6 * (blockIdx.x - shot * ntasks);
    const int zs = __ldg(tk + 4), ze = __ldg(tk + 5);
    const int nzv = (ze - zs + V - 1) / V, rpw = 32 / nzv;
    const int lane = threadIdx.x & 31, r = lane / nzv;
    const int j = __ldg(tk + 2) + (threadIdx.x >> 5) * rpw + r;
    if (r >= rpw || j >= __ldg(tk + 3)) return;
    const int zl = zs + (lane - r * nzv) * V;
    const int nv = min(V, ze - zl);  // cells of the lane's vector inside the task
    const int x0 = __ldg(tk), x1 = __ldg(tk + 1);
    const long long sh = (long long)shot * p.fstride;
    const int ys = p.ldz, xs = p.rows_y * p.ldz;  // a field of one shot has fewer than 2^31 elements
    // what the x sweep does not change: y and z sigmas and masks
    const T sy = __ldg(p.sgy + j);
    const T my = MODE == kRecomp ? __ldg(p.mgy + j) : T(0);
    const bool py = j < p.pyl || j >= p.ny - p.pyr;
    const bool neary = j - R < p.pyl || j + R >= p.ny - p.pyr;
    T sz[V], mz[V];
    bool okz[V], pz[V];
    bool any_sz = false, any_pz = false, any_nearz = false;
#pragma unroll
    for (int v = 0; v < V; ++v) {
        const int k = zl + v;
        const bool in = v < nv;
        sz[v] = in ? __ldg(p.sgz + k) : T(0);
        mz[v] = in && MODE == kRecomp ? __ldg(p.mgz + k) : T(0);
        okz[v] = in && j > 0 && j < p.ny - 1 && k > 0 && k < p.nz - 1;
        pz[v] = in && (k < p.pzl || k >= p.nz - p.pzr);
        any_sz |= sz[v] != T(0);
        any_pz |= pz[v];
        any_nearz |= in && (k - R < p.pzl || k + R >= p.nz - p.pzr);
    }
    const int* bx = p.inj.box + shot * 6;
    const bool inj_col = p.inj.on && j >= bx[2] && j < bx[3] && zl + V > bx[4] && zl < bx[5];
    bool bad = false;
    long long o = ((long long)(x0 + p.hx) * p.rows_y + (j + p.hy)) * p.ldz + kOZ + zl;
    for (int i = x0; i < x1; ++i, o += xs) {
        if (PGB_3D_SHELL_AHEAD > 0)
            prefetch_row<T, R, MODE, true>(p, sh, o + (long long)(min(i + PGB_3D_SHELL_AHEAD, x1 - 1) - i) * xs);
        const T sx = __ldg(p.sgx + i);
        const bool px = i < p.pxl || i >= p.nx - p.pxr;
        const bool nearx = i - R < p.pxl || i + R >= p.nx - p.pxr;
        const bool okx = i > 0 && i < p.nx - 1;
        const T* u = p.u_cur + sh + o;
        // u: Laplacian in difference form per axis and the first derivatives
        T w[NW];
        load_window<T, NB>(u, w);
        T uc[V], F[V], dux[V], duy[V], duz[V];
        {
            VT t[2 * R];
            load_taps<T, R>(u, xs, t);
#pragma unroll
            for (int v = 0; v < V; ++v) {
                uc[v] = w[C0 + v];
                T a2 = T(0), a1 = T(0);
#pragma unroll
                for (int m = 1; m <= R; ++m) {
                    const T up = vc<T>(t[R + m - 1], v), um = vc<T>(t[R - m], v);
                    a2 += T(d2w(R, m)) * ((up - uc[v]) + (um - uc[v]));
                    a1 += T(d1w(R, m)) * (up - um);
                }
                F[v] = a2 * p.idx2;
                dux[v] = a1 * p.idx;
            }
            load_taps<T, R>(u, ys, t);
#pragma unroll
            for (int v = 0; v < V; ++v) {
                T a2 = T(0), a1 = T(0);
#pragma unroll
                for (int m = 1; m <= R; ++m) {
                    const T up = vc<T>(t[R + m - 1], v), um = vc<T>(t[R - m], v);
                    a2 += T(d2w(R, m)) * ((up - uc[v]) + (um - uc[v]));
                    a1 += T(d1w(R, m)) * (up - um);
                }
                F[v] += a2 * p.idy2;
                duy[v] = a1 * p.idy;
            }
        }
#pragma unroll
        for (int v = 0; v < V; ++v) {
            T a2 = T(0), a1 = T(0);
#pragma unroll
            for (int m = 1; m <= R; ++m) {
                const T up = w[C0 + v + m], um = w[C0 + v - m];
                a2 += T(d2w(R, m)) * ((up - uc[v]) + (um - uc[v]));
                a1 += T(d1w(R, m)) * (up - um);
            }
            F[v] += a2 * p.idz2;
            duz[v] = a1 * p.idz;
        }
        // Phi derivatives: the state is zero outside the padding; a tap group no cell can
        // see non-zero is skipped (one that some cells need adds exact zeros to the others)
        if (nearx || py || any_pz) {
            VT t[2 * R];
            T d[V];
            load_taps<T, R>(p.phx_in + sh + o, xs, t);
            dd1_taps<T, R>(t, p.idx, d);
#pragma unroll
            for (int v = 0; v < V; ++v) F[v] += d[v];
        }
        if (neary || px || any_pz) {
            VT t[2 * R];
            T d[V];
            load_taps<T, R>(p.phy_in + sh + o, ys, t);
            dd1_taps<T, R>(t, p.idy, d);
#pragma unroll
            for (int v = 0; v < V; ++v) F[v] += d[v];
        }
        if (any_nearz || px || py) {
            load_window<T, NB>(p.phz_in + sh + o, w);
#pragma unroll
            for (int v = 0; v < V; ++v) {
                T a = T(0);
#pragma unroll
                for (int m = 1; m <= R; ++m) a += T(d1w(R, m)) * (w[C0 + v + m] - w[C0 + v - m]);
                F[v] += a * p.idz;
            }
        }
        if (inj_col) {
#pragma unroll
            for (int v = 0; v < V; ++v) F[v] += inject_rhs3(p.inj, bx, shot, i, j, zl + v);
        }
        bool psireg[V];
        bool any_ps = false;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            psireg[v] = (int)px + (int)py + (int)pz[v] >= 2;
            any_ps |= psireg[v];
        }
        T ps[V];
        if (any_ps) {
            const VT a = ldv(p.psi_in + sh + o);
#pragma unroll
            for (int v = 0; v < V; ++v) ps[v] = psireg[v] ? vc<T>(a, v) : T(0);
        } else {
#pragma unroll
            for (int v = 0; v < V; ++v) ps[v] = T(0);
        }
        const VT uo_v = ldv_plain(p.u_prev + sh + o);
        const VT c2_v = ldv(p.c2 + o);
        alignas(16) T un[V];
        if (sx != T(0) || sy != T(0) || any_sz) {
            // psi derivatives where two sigmas meet (zero elsewhere, as the products they enter)
            T dpx[V], dpy[V], dpz[V];
#pragma unroll
            for (int v = 0; v < V; ++v) dpx[v] = dpy[v] = dpz[v] = T(0);
            if (sy != T(0) && any_sz) {
                VT t[2 * R];
                load_taps<T, R>(p.psi_in + sh + o, xs, t);
                dd1_taps<T, R>(t, p.idx, dpx);
            }
            if (sx != T(0) && any_sz) {
                VT t[2 * R];
                load_taps<T, R>(p.psi_in + sh + o, ys, t);
                dd1_taps<T, R>(t, p.idy, dpy);
            }
            if (sx != T(0) && sy != T(0)) {
                load_window<T, NB>(p.psi_in + sh + o, w);
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    T a = T(0);
#pragma unroll
                    for (int m = 1; m <= R; ++m) a += T(d1w(R, m)) * (w[C0 + v + m] - w[C0 + v - m]);
                    dpz[v] = a * p.idz;
                }
            }
            const VT phx_v = ldv(p.phx_in + sh + o), phy_v = ldv(p.phy_in + sh + o), phz_v = ldv(p.phz_in + sh + o);
            alignas(16) T nxo[V], nyo[V], nzo[V];
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const T szv = sz[v], uo = vc<T>(uo_v, v), c2 = vc<T>(c2_v, v);
                const T phx = vc<T>(phx_v, v), phy = vc<T>(phy_v, v), phz = vc<T>(phz_v, v);
                const bool pml = sx != T(0) || sy != T(0) || szv != T(0);
                const bool ok = okx && okz[v];
                const T psx = sy != T(0) && szv != T(0) ? dpx[v] : T(0);
                const T psy = szv != T(0) && sx != T(0) ? dpy[v] : T(0);
                const T psz = sx != T(0) && sy != T(0) ? dpz[v] : T(0);
                const T nx_ = phx - p.dt * sx * phx + p.dt * (sy + szv - sx) * dux[v] + p.dt * (sy * szv * psx);
                const T ny_ = phy - p.dt * sy * phy + p.dt * (szv + sx - sy) * duy[v] + p.dt * (szv * sx * psy);
                const T nz_ = phz - p.dt * szv * phz + p.dt * (sx + sy - szv) * duz[v] + p.dt * (sx * sy * psz);
                const T fac1 = T(2) * p.dt2 / (T(2) + p.dt * (sx + sy + szv));
                // the reference multiplies sigma_x sigma_y sigma_z psi by C^2 (_3D.h:219); the
                // consistent form (psi_c2 = 0) leaves it out, as the matrix operator does
                const T src = p.psi_c2 ? c2 * (F[v] - (sx * sy * szv) * ps[v]) : c2 * F[v] - (sx * sy * szv) * ps[v];
                const T fac2 = src - (uo - T(2) * uc[v]) * p.idt2 + (sx + sy + szv) * uo * p.i2dt -
                               (sx * sy + sy * szv + szv * sx) * uc[v];
                const T upml = fac1 * fac2, uplain = p.dt2 * c2 * F[v] - (uo - T(2) * uc[v]);
                un[v] = ok ? (pml ? upml : uplain) : T(0);
                // cells outside the padding keep their zero state
                nxo[v] = ok && pml ? nx_ : T(0);
                nyo[v] = ok && pml ? ny_ : T(0);
                nzo[v] = ok && pml ? nz_ : T(0);
            }
            st_lane<T, false>(p.phx_out + sh + o, nxo, nv);
            st_lane<T, false>(p.phy_out + sh + o, nyo, nv);
            st_lane<T, false>(p.phz_out + sh + o, nzo, nv);
        } else {
#pragma unroll
            for (int v = 0; v < V; ++v)
                un[v] = okx && okz[v] ? p.dt2 * vc<T>(c2_v, v) * F[v] - (vc<T>(uo_v, v) - T(2) * uc[v]) : T(0);
        }
        if (any_ps) {
            alignas(16) T pso[V];
#pragma unroll
            for (int v = 0; v < V; ++v) pso[v] = psireg[v] && okx && okz[v] ? ps[v] + p.dt * uc[v] : T(0);
            st_lane<T, false>(p.psi_out + sh + o, pso, nv);
        }
        st_lane<T, false>(p.u_prev + sh + o, un, nv);
        if (MODE == kRecomp && p.dw_out) {
            const T mx = __ldg(p.mgx + i);
            alignas(16) T dwo[V];
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const T szv = sz[v], mzv = mz[v], c2 = vc<T>(c2_v, v), sxyz = sx * sy * szv;
                T d = p.psi_c2 ? c2 * (F[v] - sxyz * ps[v]) : c2 * F[v] - sxyz * ps[v];
                d += ((mx + my + mzv) - (sx + sy + szv)) * (un[v] - vc<T>(uo_v, v)) * p.i2dt +
                     ((mx * my + my * mzv + mzv * mx) - (sx * sy + sy * szv + szv * sx)) * uc[v] + (mx * my * mzv) * ps[v];
                dwo[v] = okx && okz[v] ? d : T(0);
            }
            st_lane<T, true>(p.dw_out + sh + o, dwo, nv);
        }
        if (MODE == kAdj && p.image) {
            const VT dw_v = __ldcs(reinterpret_cast<const VT*>(p.dw_in + sh + o));
            const VT ic_v = ldv_plain(p.ic + sh + o);
            alignas(16) T ico[V];
#pragma unroll
            for (int v = 0; v < V; ++v) ico[v] = vc<T>(ic_v, v) + uc[v] * vc<T>(dw_v, v);
            st_lane<T, false>(p.ic + sh + o, ico, nv);
        }
        if (MODE == kFwd || (MODE == kRecomp && p.nan_check)) {
#pragma unroll
            for (int v = 0; v < V; ++v) bad |= v < nv && !isfinite(un[v]);
        }
    }
    if (MODE != kAdj && bad && p.err) atomicOr(p.err, PGB_ERR_NONFINITE);
}

// 1D: one axis (z), Phi_z only (_1D.h:117-129).
template <typename T, int R, int MODE>
__global__ void __launch_bounds__(256) wave1d_kernel(const WaveParams<T> p, int ntile) {
    const int b = blockIdx.x;
    if (b >= ntile * p.nshot) {
        if (MODE != kAdj) record3(p, (long long)(b - ntile * p.nshot) * blockDim.x + threadIdx.x);
        return;
    }
    const int shot = b / ntile;
    const int k = (b - shot * ntile) * blockDim.x + threadIdx.x;
    if (k >= p.nz) return;
    const long long sh = (long long)shot * p.fstride;
    const long long o = kOZ + k;
    const T* __restrict__ u = p.u_cur + sh;
    const bool ok = k > 0 && k < p.nz - 1;
    const T sz = __ldg(p.sgz + k);
    const T uc = u[o], uo = p.u_prev[sh + o], c2 = __ldg(p.c2 + o);
    T F = dd2<T, R>(u + o, 1) * p.idz2 + dd1<T, R>(p.phz_in + sh + o, 1) * p.idz;
    const int* bx = p.inj.box + shot * 6;
    if (p.inj.on) F += inject_rhs3(p.inj, bx, shot, 0, 0, k);
    T unew;
    if (sz != T(0)) {
        const T dudz = dd1<T, R>(u + o, 1) * p.idz;
        const T phz = p.phz_in[sh + o];
        T nz_ = phz - p.dt * sz * (phz + dudz);
        const T fac1 = T(2) * p.dt2 / (T(2) + p.dt * sz);
        const T fac2 = c2 * F - (uo - T(2) * uc) * p.idt2 + sz * uo * p.i2dt;
        unew = fac1 * fac2;
        if (!ok) { unew = T(0); nz_ = T(0); }
        p.phz_out[sh + o] = nz_;
    } else {
        unew = p.dt2 * c2 * F - (uo - T(2) * uc);
        if (!ok) unew = T(0);
    }
    p.u_prev[sh + o] = unew;
    if (MODE == kRecomp && p.dw_out) {
        const T mz = __ldg(p.mgz + k);
        T d = c2 * F + (mz - sz) * (unew - uo) * p.i2dt;
        __stcs(p.dw_out + sh + o, ok ? d : T(0));
    }
    if (MODE == kAdj && p.image) p.ic[sh + o] += uc * __ldcs(p.dw_in + sh + o);
}

}  // namespace

template <typename T, int R, int MODE, int KIND>
void launch_wave3d_tasks(const WaveParams<T>& p, const int* tasks, int ntasks, cudaStream_t s) {
    if (ntasks <= 0) return;
    const int grid = ntasks * p.nshot;
    if (KIND == 0)
        wave3d_interior_kernel<T, R, MODE><<<grid, kW3 * 32, 0, s>>>(p, tasks, ntasks);
    else
        wave3d_shell_kernel<T, R, MODE><<<grid, kW3S * 32, 0, s>>>(p, tasks, ntasks);
}

int wave3d_seg(int dtype_bytes, int kind) {
    (void)kind;
    return 32 * (16 / dtype_bytes);
}
int wave3d_task_rows(int dtype_bytes, int kind, int zcells) {
    const int V = 16 / dtype_bytes;
    return (kind == 0 ? kW3 : kW3S) * (32 / ((zcells + V - 1) / V));
}

template <typename T, int R, int MODE>
void launch_wave1d(const WaveParams<T>& p, int bz, cudaStream_t s) {
    (void)bz;
    const int tb = 128;
    int ntile = ceil_div(p.nz, tb);
    int grid = ntile * p.nshot;
    if (MODE != kAdj && p.rec.nrec > 0 && p.rec.traces) grid += ceil_div((long long)p.nshot * p.rec.nrec, tb);
    wave1d_kernel<T, R, MODE><<<grid, tb, 0, s>>>(p, ntile);
}

#define PGB_INST3K(T, R, M)                                                                            \
    template void launch_wave3d_tasks<T, R, M, 0>(const WaveParams<T>&, const int*, int, cudaStream_t); \
    template void launch_wave3d_tasks<T, R, M, 1>(const WaveParams<T>&, const int*, int, cudaStream_t);
#define PGB_INST13(T, R)                                                                    \
    PGB_INST3K(T, R, kFwd) PGB_INST3K(T, R, kRecomp) PGB_INST3K(T, R, kAdj)                 \
    template void launch_wave1d<T, R, kFwd>(const WaveParams<T>&, int, cudaStream_t);    \
    template void launch_wave1d<T, R, kRecomp>(const WaveParams<T>&, int, cudaStream_t); \
    template void launch_wave1d<T, R, kAdj>(const WaveParams<T>&, int, cudaStream_t);
PGB_INST13(float, 1)
PGB_INST13(float, 2)
PGB_INST13(float, 3)
PGB_INST13(float, 4)
PGB_INST13(double, 1)
PGB_INST13(double, 2)
PGB_INST13(double, 3)
PGB_INST13(double, 4)

}  // namespace pgb
