// Batched 2D leapfrog step, warp-independent sweep (forward, recompute, adjoint).
//
// Same maths as the reference step cda_time_scalar_2D (pysit/solvers/
// constant_density_acoustic/time/scalar/constant_density_acoustic_time_scalar_2D.h:88-179)
// with the mode-specific fusions described in wave2d.cu (trace recording,
// dWaveOp from the stencil bracket, adjoint imaging).
//
// Work decomposition: a table of warp tasks (x0, x1, zs, ze, kind) covers the
// padded grid once; the same table serves every shot.  A warp owns the cells
// z in [zs, ze) and sweeps rows x0..x1-1.  Its lanes hold VV consecutive cells
// each; the HL lanes at each end only load the z-halo.  Per row a lane
//   * keeps the 2R+1 rows of u_k its x-derivatives need in a register queue,
//   * gets its z-neighbours from the adjacent lanes with warp shuffles,
//   * prefetches the next row (u_k head, u_{k-1}, C^2, [dWaveOp, ic]) before
//     computing the current one, so loads overlap arithmetic,
// with no shared memory and no block barrier: warps never wait for each other.
// Two task kinds, selected per warp (warp-uniform branch):
//   kind 0  interior: cells at least R away from the padding; 16-byte vectors,
//           no PML state at all;
//   kind 1  PML shell: the padding and its R-wide rim; 8-byte vectors (half the
//           register queue), Phi_x in a register queue, Phi_z by shuffles, PML
//           state loaded only for vectors inside the padding.
#include "wave.cuh"

namespace pgb {
namespace {

constexpr int kWarps = 4;  // warps per block

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
__device__ __forceinline__ Vec<T, N> zvec() {
    Vec<T, N> r;
#pragma unroll
    for (int i = 0; i < N; ++i) r.v[i] = T(0);
    return r;
}
template <typename T, int N>
__device__ __forceinline__ Vec<T, N> ldv(const T* p) {
    Vec<T, N> r;
    *reinterpret_cast<typename VecT<T, N>::type*>(r.v) = *reinterpret_cast<const typename VecT<T, N>::type*>(p);
    return r;
}
template <typename T, int N>
__device__ __forceinline__ Vec<T, N> ldv_ro(const T* p) {
    Vec<T, N> r;
    *reinterpret_cast<typename VecT<T, N>::type*>(r.v) = __ldg(reinterpret_cast<const typename VecT<T, N>::type*>(p));
    return r;
}
template <typename T, int N>
__device__ __forceinline__ Vec<T, N> ldv_cs(const T* p) {
    Vec<T, N> r;
    *reinterpret_cast<typename VecT<T, N>::type*>(r.v) = __ldcs(reinterpret_cast<const typename VecT<T, N>::type*>(p));
    return r;
}
template <typename T, int N>
__device__ __forceinline__ void stv(T* p, const Vec<T, N>& r) {
    *reinterpret_cast<typename VecT<T, N>::type*>(p) = *reinterpret_cast<const typename VecT<T, N>::type*>(r.v);
}
template <typename T, int N>
__device__ __forceinline__ void stv_cs(T* p, const Vec<T, N>& r) {
    __stcs(reinterpret_cast<typename VecT<T, N>::type*>(p), *reinterpret_cast<const typename VecT<T, N>::type*>(r.v));
}

// window of the row held by lanes lane-HL .. lane+HL (HL*VV cells of halo per side)
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

template <typename T, int R, int MODE, int VV, bool PML>
__device__ __forceinline__ void sweep(const WaveParams<T>& p, const int shot, const int x0, const int x1,
                                      const int zs, const int ze) {
    constexpr int HL = (R + VV - 1) / VV;
    constexpr int Q = 2 * R + 1;
    constexpr int NWIN = (2 * HL + 1) * VV;
    const int lane = threadIdx.x & 31;
    const int zl = zs + (lane - HL) * VV;                 // first cell of this lane's vector
    const bool ldz = zl < p.nz;                            // vector holds grid cells (else zeros)
    const bool own = lane >= HL && lane < 32 - HL && zl < ze;
    const long long sh = (long long)shot * p.fstride;
    const T* __restrict__ ucur = p.u_cur + sh;
    T* __restrict__ uprev = p.u_prev + sh;
    const T* __restrict__ phx_in = p.phx_in + sh;
    const T* __restrict__ phz_in = p.phz_in + sh;
    const bool zpad = PML && (zl < p.pzl || zl + VV - 1 >= p.nz - p.pzr);
    auto xpad = [&](int x) { return x < p.pxl || x >= p.nx - p.pxr; };
    auto off = [&](int x) { return (long long)(x + kHalo) * p.ldz + kOZ + zl; };
    const int* bx = p.inj.box + shot * 6;
    const bool inj_task = p.inj.on && bx[0] < x1 && bx[1] > x0 && bx[4] < ze && bx[5] > zs;

    T sgz[VV], mgz[VV];
    bool zok[VV];
#pragma unroll
    for (int v = 0; v < VV; ++v) {
        const int z = zl + v;
        zok[v] = z > 0 && z < p.nz - 1;
        sgz[v] = (PML && z >= 0 && z < p.nz) ? __ldg(p.sgz + z) : T(0);
        mgz[v] = (PML && MODE == kRecomp && z >= 0 && z < p.nz) ? __ldg(p.mgz + z) : T(0);
    }

    Vec<T, VV> q[Q];
    Vec<T, VV> qx[Q];  // used by PML tasks only
#pragma unroll
    for (int j = 0; j < Q - 1; ++j) {
        const int x = x0 - R + j;
        q[j] = ldz ? ldv_ro<T, VV>(ucur + off(x)) : zvec<T, VV>();
        if (PML) qx[j] = (ldz && (zpad || xpad(x))) ? ldv_ro<T, VV>(phx_in + off(x)) : zvec<T, VV>();
    }
    // prefetch registers of the first row
    Vec<T, VV> nq = ldz ? ldv_ro<T, VV>(ucur + off(x0 + R)) : zvec<T, VV>();
    Vec<T, VV> nqx;
    if (PML) nqx = (ldz && (zpad || xpad(x0 + R))) ? ldv_ro<T, VV>(phx_in + off(x0 + R)) : zvec<T, VV>();
    Vec<T, VV> num = ldz ? ldv<T, VV>(uprev + off(x0)) : zvec<T, VV>();
    Vec<T, VV> ncc = ldz ? ldv_ro<T, VV>(p.c2 + off(x0)) : zvec<T, VV>();
    Vec<T, VV> npz;
    if (PML) npz = (ldz && (zpad || xpad(x0))) ? ldv_ro<T, VV>(phz_in + off(x0)) : zvec<T, VV>();
    Vec<T, VV> ndw, nic;
    if (MODE == kAdj && p.image) {
        ndw = own ? ldv_cs<T, VV>(p.dw_in + sh + off(x0)) : zvec<T, VV>();
        nic = own ? ldv<T, VV>(p.ic + sh + off(x0)) : zvec<T, VV>();
    }
    bool bad = false;

    for (int x = x0; x < x1; ++x) {
        q[Q - 1] = nq;
        if (PML) qx[Q - 1] = nqx;
        const Vec<T, VV> um = num, cc = ncc;
        Vec<T, VV> pzc;
        if (PML) pzc = npz;
        Vec<T, VV> dwi, ici;
        if (MODE == kAdj && p.image) { dwi = ndw; ici = nic; }
        // prefetch row x + 1
        if (x + 1 < x1) {
            const int xn = x + 1;
            nq = ldz ? ldv_ro<T, VV>(ucur + off(xn + R)) : zvec<T, VV>();
            if (PML) nqx = (ldz && (zpad || xpad(xn + R))) ? ldv_ro<T, VV>(phx_in + off(xn + R)) : zvec<T, VV>();
            num = ldz ? ldv<T, VV>(uprev + off(xn)) : zvec<T, VV>();
            ncc = ldz ? ldv_ro<T, VV>(p.c2 + off(xn)) : zvec<T, VV>();
            if (PML) npz = (ldz && (zpad || xpad(xn))) ? ldv_ro<T, VV>(phz_in + off(xn)) : zvec<T, VV>();
            if (MODE == kAdj && p.image) {
                ndw = own ? ldv_cs<T, VV>(p.dw_in + sh + off(xn)) : zvec<T, VV>();
                nic = own ? ldv<T, VV>(p.ic + sh + off(xn)) : zvec<T, VV>();
            }
        }
        T w[NWIN];
        zwindow<T, VV, HL>(q[R], w);
        T wp[NWIN];  // Phi_z window, PML tasks only
        if (PML) zwindow<T, VV, HL>(pzc, wp);
        const bool xok = x > 0 && x < p.nx - 1;
        const bool xp = PML && xpad(x);
        const T sgx = PML ? __ldg(p.sgx + x) : T(0);
        const T mgx = (PML && MODE == kRecomp) ? __ldg(p.mgx + x) : T(0);
        const bool inj_row = inj_task && x >= bx[0] && x < bx[1];
        Vec<T, VV> un, dwo, pxo, pzo, ico;
#pragma unroll
        for (int v = 0; v < VV; ++v) {
            const int z = zl + v;
            const T uc = w[HL * VV + v];
            T lz = T(d2w(R, 0)) * uc, lx = T(d2w(R, 0)) * uc, dz1 = T(0), dx1 = T(0);
#pragma unroll
            for (int m = 1; m <= R; ++m) {
                const T zp = w[HL * VV + v + m], zm = w[HL * VV + v - m];
                const T xpv = q[R + m].v[v], xmv = q[R - m].v[v];
                lz += T(d2w(R, m)) * (zp + zm);
                lx += T(d2w(R, m)) * (xpv + xmv);
                if (PML) {
                    dz1 += T(d1w(R, m)) * (zp - zm);
                    dx1 += T(d1w(R, m)) * (xpv - xmv);
                }
            }
            T F = lx * p.idx2 + lz * p.idz2;
            if (inj_row && own && z < p.nz) F += inject_rhs(p.inj, bx, shot, x, z);
            const T uo = um.v[v], c2 = cc.v[v];
            const bool ok = xok && zok[v];
            T unew;
            if (PML) {
                T dpx = T(0), dpz = T(0);
#pragma unroll
                for (int m = 1; m <= R; ++m) {
                    dpx += T(d1w(R, m)) * (qx[R + m].v[v] - qx[R - m].v[v]);
                    dpz += T(d1w(R, m)) * (wp[HL * VV + v + m] - wp[HL * VV + v - m]);
                }
                F += dpx * p.idx + dpz * p.idz;
                const T sx = sgx, sz = sgz[v];
                T ph_x = T(0), ph_z = T(0);
                if (sx != T(0) || sz != T(0)) {
                    const T dudx = dx1 * p.idx, dudz = dz1 * p.idz;
                    const T phx = qx[R].v[v], phz = wp[HL * VV + v];
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
                    T d = c2 * F + ((mgx + mz) - (sx + sz)) * (unew - uo) * p.i2dt + (mgx * mz - sx * sz) * uc;
                    dwo.v[v] = ok ? d : T(0);
                }
            } else {
                unew = p.dt2 * c2 * F - (uo - T(2) * uc);
                if (!ok) unew = T(0);
                if (MODE == kRecomp) dwo.v[v] = ok ? c2 * F : T(0);
            }
            un.v[v] = unew;
            if (MODE == kFwd) bad |= !isfinite(unew);
            if (MODE == kAdj) ico.v[v] = ici.v[v] + uc * dwi.v[v];
        }
        if (own) {
            const long long o = off(x);
            stv<T, VV>(uprev + o, un);
            if (PML && (xp || zpad)) {
                stv<T, VV>(p.phx_out + sh + o, pxo);
                stv<T, VV>(p.phz_out + sh + o, pzo);
            }
            if (MODE == kRecomp && p.dw_out) stv_cs<T, VV>(p.dw_out + sh + o, dwo);
            if (MODE == kAdj && p.image) stv<T, VV>(p.ic + sh + o, ico);
        }
#pragma unroll
        for (int j = 0; j < Q - 1; ++j) {
            q[j] = q[j + 1];
            if (PML) qx[j] = qx[j + 1];
        }
    }
    if (MODE == kFwd && bad && own && p.err) atomicOr(p.err, PGB_ERR_NONFINITE);
}

template <typename T, int R, int MODE>
__global__ void __launch_bounds__(kWarps * 32) wave2d_warp_kernel(const WaveParams<T> p, const int* __restrict__ tasks,
                                                                  int ntasks, int task_blocks) {
    if ((int)blockIdx.x >= task_blocks) {
        if (MODE == kFwd) record_block(p, blockIdx.x - task_blocks);
        return;
    }
    const int gw = blockIdx.x * kWarps + (threadIdx.x >> 5);
    if (gw >= ntasks * p.nshot) return;  // warp-uniform
    const int shot = gw / ntasks;
    const int* tk = tasks + 5 * (gw - shot * ntasks);
    const int x0 = __ldg(tk), x1 = __ldg(tk + 1), zs = __ldg(tk + 2), ze = __ldg(tk + 3), kind = __ldg(tk + 4);
    constexpr int V = V16<T>::N;
    if (kind == 0)
        sweep<T, R, MODE, V, false>(p, shot, x0, x1, zs, ze);
    else
        sweep<T, R, MODE, (V > 1 ? V / 2 : 1), true>(p, shot, x0, x1, zs, ze);
}

}  // namespace

// The task table of a launch sits in p.rec-independent storage: the plan passes it
// through p.inj-free fields below (tasks pointer and count are launch arguments).
template <typename T, int R, int MODE>
void launch_wave2d_warp_tasks(const WaveParams<T>& p, const int* tasks, int ntasks, cudaStream_t s) {
    const int task_blocks = (ntasks * p.nshot + kWarps - 1) / kWarps;
    const int grid = task_blocks + (MODE == kFwd ? p.rec.blocks : 0);
    wave2d_warp_kernel<T, R, MODE><<<grid, kWarps * 32, 0, s>>>(p, tasks, ntasks, task_blocks);
}

int wave2d_warp_threads() { return kWarps * 32; }

// widest z-range a task of each kind may cover: (32 - 2*HL) * VV cells
int wave2d_warp_seg(int dtype_bytes, int order, int pml) {
    const int V = 16 / dtype_bytes;
    const int VV = pml ? (V > 1 ? V / 2 : 1) : V;
    const int R = order / 2;
    const int HL = (R + VV - 1) / VV;
    return (32 - 2 * HL) * VV;
}
int wave2d_warp_vec(int dtype_bytes, int pml) {
    const int V = 16 / dtype_bytes;
    return pml ? (V > 1 ? V / 2 : 1) : V;
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
