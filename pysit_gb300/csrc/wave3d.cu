// Batched 1D and 3D leapfrog steps (forward, recompute, adjoint modes) on the
// internal zero-halo layout of wave.cuh, for cda_time_scalar_1D (pysit/solvers/
// constant_density_acoustic/time/scalar/constant_density_acoustic_time_scalar_1D.h:78-130)
// and cda_time_scalar_3D (..._3D.h:107-235).
//
// 3D: a table of block tasks covers the padded grid once (interior: R cells
// clear of the padding and off the outer ring; PML shell: the rest).  Each kind
// is its own kernel; both sweep along x with the neighbour planes in L1.
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

// One cell of the reference's 3D step (_3D.h:107-235) with the batched fusions:
// the general path, PML included.  Cells of the outer ring get zero.
template <typename T, int R, int MODE>
__device__ __forceinline__ void cell3d(const WaveParams<T>& p, const int shot, const int i, const int j,
                                       const int k) {
    // every operand is addressed from the cell's own offset (64-bit once) with 32-bit taps
    const long long base = (long long)shot * p.fstride +
                           ((long long)(i + p.hx) * p.rows_y + (j + p.hy)) * p.ldz + kOZ + k;
    const long long o = base - (long long)shot * p.fstride;  // the cell in the shared C^2 field
    const int ys = p.ldz, xs = p.rows_y * p.ldz;
    const T* __restrict__ u = p.u_cur + base;
    const bool ok = i > 0 && i < p.nx - 1 && j > 0 && j < p.ny - 1 && k > 0 && k < p.nz - 1;
    const bool px = i < p.pxl || i >= p.nx - p.pxr;
    const bool py = j < p.pyl || j >= p.ny - p.pyr;
    const bool pz = k < p.pzl || k >= p.nz - p.pzr;
    const bool psireg = (int)px + (int)py + (int)pz >= 2;
    const T sx = __ldg(p.sgx + i), sy = __ldg(p.sgy + j), sz = __ldg(p.sgz + k);
    const T uc = u[0], uo = p.u_prev[base], c2 = __ldg(p.c2 + o);
    T F = dd2<T, R>(u, xs) * p.idx2 + dd2<T, R>(u, ys) * p.idy2 + dd2<T, R>(u, 1) * p.idz2;
    // Phi derivatives: state is zero outside the padding, skip the reads where no tap can reach it
    const bool nearx = i - R < p.pxl || i + R >= p.nx - p.pxr;
    const bool neary = j - R < p.pyl || j + R >= p.ny - p.pyr;
    const bool nearz = k - R < p.pzl || k + R >= p.nz - p.pzr;
    if (nearx || py || pz) F += dd1<T, R>(p.phx_in + base, xs) * p.idx;
    if (neary || px || pz) F += dd1<T, R>(p.phy_in + base, ys) * p.idy;
    if (nearz || px || py) F += dd1<T, R>(p.phz_in + base, 1) * p.idz;
    const int* bx = p.inj.box + shot * 6;
    if (p.inj.on) F += inject_rhs3(p.inj, bx, shot, i, j, k);
    const T ps = psireg ? p.psi_in[base] : T(0);
    T unew;
    const bool pmlc = sx != T(0) || sy != T(0) || sz != T(0);
    if (pmlc) {
        const T dudx = dd1<T, R>(u, xs) * p.idx, dudy = dd1<T, R>(u, ys) * p.idy, dudz = dd1<T, R>(u, 1) * p.idz;
        T dpsx = T(0), dpsy = T(0), dpsz = T(0);
        if (sy != T(0) && sz != T(0)) dpsx = dd1<T, R>(p.psi_in + base, xs) * p.idx;
        if (sz != T(0) && sx != T(0)) dpsy = dd1<T, R>(p.psi_in + base, ys) * p.idy;
        if (sx != T(0) && sy != T(0)) dpsz = dd1<T, R>(p.psi_in + base, 1) * p.idz;
        const T phx = p.phx_in[base], phy = p.phy_in[base], phz = p.phz_in[base];
        T nx_ = phx - p.dt * sx * phx + p.dt * (sy + sz - sx) * dudx + p.dt * (sy * sz * dpsx);
        T ny_ = phy - p.dt * sy * phy + p.dt * (sz + sx - sy) * dudy + p.dt * (sz * sx * dpsy);
        T nz_ = phz - p.dt * sz * phz + p.dt * (sx + sy - sz) * dudz + p.dt * (sx * sy * dpsz);
        const T fac1 = T(2) * p.dt2 / (T(2) + p.dt * (sx + sy + sz));
        // the reference multiplies sigma_x sigma_y sigma_z psi by C^2 (_3D.h:219); the
        // consistent form (psi_c2 = 0) leaves it out, as the matrix operator does
        const T src = p.psi_c2 ? c2 * (F - (sx * sy * sz) * ps) : c2 * F - (sx * sy * sz) * ps;
        const T fac2 = src - (uo - T(2) * uc) * p.idt2 + (sx + sy + sz) * uo * p.i2dt -
                       (sx * sy + sy * sz + sz * sx) * uc;
        unew = fac1 * fac2;
        if (!ok) { nx_ = ny_ = nz_ = unew = T(0); }
        p.phx_out[base] = nx_;
        p.phy_out[base] = ny_;
        p.phz_out[base] = nz_;
    } else {
        unew = p.dt2 * c2 * F - (uo - T(2) * uc);
        if (!ok) unew = T(0);
    }
    if (psireg) p.psi_out[base] = ok ? ps + p.dt * uc : T(0);
    p.u_prev[base] = unew;
    if (MODE == kRecomp && p.dw_out) {
        T d = p.psi_c2 ? c2 * (F - (sx * sy * sz) * ps) : c2 * F - (sx * sy * sz) * ps;
        const T mx = __ldg(p.mgx + i), my = __ldg(p.mgy + j), mz = __ldg(p.mgz + k);
        d += ((mx + my + mz) - (sx + sy + sz)) * (unew - uo) * p.i2dt +
             ((mx * my + my * mz + mz * mx) - (sx * sy + sy * sz + sz * sx)) * uc + (mx * my * mz) * ps;
        __stcs(p.dw_out + base, ok ? d : T(0));
    }
    if (MODE == kAdj && p.image) p.ic[base] += uc * __ldcs(p.dw_in + base);
    if ((MODE == kFwd || (MODE == kRecomp && p.nan_check)) && p.err && !isfinite(unew))
        atomicOr(p.err, PGB_ERR_NONFINITE);
}

// ---- task sweeps ---------------------------------------------------------------
// A task (x0, x1, y0, y1, zs, ze) is handled by one block: warp w owns y-row
// y0 + w and sweeps x0..x1-1 over the z-range [zs, ze).  The block's rows of the
// 2R+1 planes around x stay in L1 while it marches, so u_k comes from DRAM
// about once; the x- and y-neighbours are constant offsets from the centre row.
constexpr int kW3 = 8;  // warps (y-rows) per block
#ifndef PGB_3D_AHEAD
#define PGB_3D_AHEAD 2     // rows ahead whose operands are prefetched into L1
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

// PML shell: one cell per lane, the general per-cell update
#ifndef PGB_3D_SHELL_MINB
#define PGB_3D_SHELL_MINB 4  // resident shell blocks per SM the register budget aims at (64 registers)
#endif
template <typename T, int R, int MODE>
__global__ void __launch_bounds__(kW3 * 32, PGB_3D_SHELL_MINB) wave3d_shell_kernel(const WaveParams<T> p, const int* __restrict__ tasks,
                                                               int ntasks) {
    const int shot = blockIdx.x / ntasks;
    const int* tk = tasks + 6 * (blockIdx.x - shot * ntasks);
    const int j = __ldg(tk + 2) + (threadIdx.x >> 5);
    const int k = __ldg(tk + 4) + (threadIdx.x & 31);
    if (j >= __ldg(tk + 3) || k >= __ldg(tk + 5)) return;
    const int x1 = __ldg(tk + 1);
    const long long sh = (long long)shot * p.fstride;
    const long long xs = (long long)p.rows_y * p.ldz;
    const long long o0 = ((long long)(p.hx) * p.rows_y + (j + p.hy)) * p.ldz + kOZ + k;  // row x = 0
    for (int i = __ldg(tk); i < x1; ++i) {
        prefetch_row<T, R, MODE, true>(p, sh, o0 + (long long)min(i + PGB_3D_AHEAD, x1 - 1) * xs);
        cell3d<T, R, MODE>(p, shot, i, j, k);
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
// z-bounds are multiples of 4 cells, so every vector load is aligned.
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
    const int j = __ldg(tk + 2) + (threadIdx.x >> 5);
    const int zl = __ldg(tk + 4) + (threadIdx.x & 31) * V;
    if (j >= __ldg(tk + 3) || zl >= __ldg(tk + 5)) return;
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
        wave3d_shell_kernel<T, R, MODE><<<grid, kW3 * 32, 0, s>>>(p, tasks, ntasks);
}

int wave3d_rows_per_block() { return kW3; }
int wave3d_seg(int dtype_bytes, int kind) { return kind == 0 ? 32 * (16 / dtype_bytes) : 32; }

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
