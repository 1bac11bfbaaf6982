// Batched 1D and 3D leapfrog steps (forward, recompute, adjoint modes) on the
// internal zero-halo layout of wave.cuh.  Same maths as wave2d.cu for
// cda_time_scalar_1D (pysit/solvers/constant_density_acoustic/time/scalar/
// constant_density_acoustic_time_scalar_1D.h:78-130) and cda_time_scalar_3D
// (..._3D.h:107-235), one thread per cell, z on threadIdx.x.
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

template <typename T, int R>
__device__ __forceinline__ T dd1(const T* __restrict__ v, long long o, long long s) {
    T a = T(0);
#pragma unroll
    for (int m = 1; m <= R; ++m) a += T(d1w(R, m)) * (v[o + m * s] - v[o - m * s]);
    return a;
}
// second derivative in difference form: sum_m w_m ((v_+m - v_0) + (v_-m - v_0)),
// equal to the central stencil (the weights sum to zero) with far less FP32
// cancellation than w_0 v_0 + sum_m w_m (v_+m + v_-m)
template <typename T, int R>
__device__ __forceinline__ T dd2(const T* __restrict__ v, long long o, long long s) {
    const T c = v[o];
    T a = T(0);
#pragma unroll
    for (int m = 1; m <= R; ++m) a += T(d2w(R, m)) * ((v[o + m * s] - c) + (v[o - m * s] - c));
    return a;
}

// grid: x = cells along z (blockDim.x), y = y index, z = x index * nshot;
// recorder blocks use blockIdx.y == gridDim.y - 1 beyond the tile range.
template <typename T, int R, int MODE>
__global__ void __launch_bounds__(256) wave3d_cell_kernel(const WaveParams<T> p, int nrecblk) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    int xi = blockIdx.z;
    if (xi >= p.nx * p.nshot) {
        if (MODE == kFwd) {
            long long id = ((long long)(xi - p.nx * p.nshot) * gridDim.y + j) * gridDim.x * blockDim.x +
                           (long long)blockIdx.x * blockDim.x + threadIdx.x;
            record3(p, id);
        }
        return;
    }
    const int shot = xi / p.nx;
    const int i = xi - shot * p.nx;
    if (k >= p.nz || j >= p.ny) return;
    const long long sh = (long long)shot * p.fstride;
    const long long ys = p.ldz, xs = (long long)p.rows_y * p.ldz;
    const long long o = ((long long)(i + p.hx) * p.rows_y + (j + p.hy)) * p.ldz + kOZ + k;
    const T* __restrict__ u = p.u_cur + sh;
    const bool ok = i > 0 && i < p.nx - 1 && j > 0 && j < p.ny - 1 && k > 0 && k < p.nz - 1;
    const bool px = i < p.pxl || i >= p.nx - p.pxr;
    const bool py = j < p.pyl || j >= p.ny - p.pyr;
    const bool pz = k < p.pzl || k >= p.nz - p.pzr;
    const bool psireg = (int)px + (int)py + (int)pz >= 2;
    const T sx = __ldg(p.sgx + i), sy = __ldg(p.sgy + j), sz = __ldg(p.sgz + k);
    const T uc = u[o], uo = p.u_prev[sh + o], c2 = __ldg(p.c2 + o);
    T F = dd2<T, R>(u, o, xs) * p.idx2 + dd2<T, R>(u, o, ys) * p.idy2 + dd2<T, R>(u, o, 1) * p.idz2;
    // Phi derivatives: state is zero outside the padding, skip the reads where no tap can reach it
    const bool nearx = i - R < p.pxl || i + R >= p.nx - p.pxr;
    const bool neary = j - R < p.pyl || j + R >= p.ny - p.pyr;
    const bool nearz = k - R < p.pzl || k + R >= p.nz - p.pzr;
    if (nearx || py || pz) F += dd1<T, R>(p.phx_in + sh, o, xs) * p.idx;
    if (neary || px || pz) F += dd1<T, R>(p.phy_in + sh, o, ys) * p.idy;
    if (nearz || px || py) F += dd1<T, R>(p.phz_in + sh, o, 1) * p.idz;
    const int* bx = p.inj.box + shot * 6;
    if (p.inj.on) F += inject_rhs3(p.inj, bx, shot, i, j, k);
    const T ps = psireg ? p.psi_in[sh + o] : T(0);
    T unew;
    const bool pmlc = sx != T(0) || sy != T(0) || sz != T(0);
    if (pmlc) {
        const T dudx = dd1<T, R>(u, o, xs) * p.idx, dudy = dd1<T, R>(u, o, ys) * p.idy,
                dudz = dd1<T, R>(u, o, 1) * p.idz;
        T dpsx = T(0), dpsy = T(0), dpsz = T(0);
        if (sy != T(0) && sz != T(0)) dpsx = dd1<T, R>(p.psi_in + sh, o, xs) * p.idx;
        if (sz != T(0) && sx != T(0)) dpsy = dd1<T, R>(p.psi_in + sh, o, ys) * p.idy;
        if (sx != T(0) && sy != T(0)) dpsz = dd1<T, R>(p.psi_in + sh, o, 1) * p.idz;
        const T phx = p.phx_in[sh + o], phy = p.phy_in[sh + o], phz = p.phz_in[sh + o];
        T nx_ = phx - p.dt * sx * phx + p.dt * (sy + sz - sx) * dudx + p.dt * (sy * sz * dpsx);
        T ny_ = phy - p.dt * sy * phy + p.dt * (sz + sx - sy) * dudy + p.dt * (sz * sx * dpsy);
        T nz_ = phz - p.dt * sz * phz + p.dt * (sx + sy - sz) * dudz + p.dt * (sx * sy * dpsz);
        const T fac1 = T(2) * p.dt2 / (T(2) + p.dt * (sx + sy + sz));
        const T fac2 = c2 * (F - (sx * sy * sz) * ps) - (uo - T(2) * uc) * p.idt2 +
                       (sx + sy + sz) * uo * p.i2dt - (sx * sy + sy * sz + sz * sx) * uc;
        unew = fac1 * fac2;
        if (!ok) { nx_ = ny_ = nz_ = unew = T(0); }
        p.phx_out[sh + o] = nx_;
        p.phy_out[sh + o] = ny_;
        p.phz_out[sh + o] = nz_;
    } else {
        unew = p.dt2 * c2 * F - (uo - T(2) * uc);
        if (!ok) unew = T(0);
    }
    if (psireg) p.psi_out[sh + o] = ok ? ps + p.dt * uc : T(0);
    p.u_prev[sh + o] = unew;
    if (MODE == kRecomp && p.dw_out) {
        T d = c2 * (F - (sx * sy * sz) * ps);
        const T mx = __ldg(p.mgx + i), my = __ldg(p.mgy + j), mz = __ldg(p.mgz + k);
        d += ((mx + my + mz) - (sx + sy + sz)) * (unew - uo) * p.i2dt +
             ((mx * my + my * mz + mz * mx) - (sx * sy + sy * sz + sz * sx)) * uc + (mx * my * mz) * ps;
        __stcs(p.dw_out + sh + o, ok ? d : T(0));
    }
    if (MODE == kAdj && p.image) p.ic[sh + o] += uc * __ldcs(p.dw_in + sh + o);
}

// 1D: one axis (z), Phi_z only (_1D.h:117-129).
template <typename T, int R, int MODE>
__global__ void __launch_bounds__(256) wave1d_kernel(const WaveParams<T> p, int ntile) {
    const int b = blockIdx.x;
    if (b >= ntile * p.nshot) {
        if (MODE == kFwd) record3(p, (long long)(b - ntile * p.nshot) * blockDim.x + threadIdx.x);
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
    T F = dd2<T, R>(u, o, 1) * p.idz2 + dd1<T, R>(p.phz_in + sh, o, 1) * p.idz;
    const int* bx = p.inj.box + shot * 6;
    if (p.inj.on) F += inject_rhs3(p.inj, bx, shot, 0, 0, k);
    T unew;
    if (sz != T(0)) {
        const T dudz = dd1<T, R>(u, o, 1) * p.idz;
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

template <typename T, int R, int MODE>
void launch_wave3d(const WaveParams<T>& p, int bz, cudaStream_t s) {
    (void)bz;
    const int tb = 64;
    dim3 grd(ceil_div(p.nz, tb), p.ny, p.nx * p.nshot);
    int recblk = 0;
    if (MODE == kFwd && p.rec.nrec > 0) {
        long long per = (long long)grd.x * tb * grd.y;
        recblk = ceil_div((long long)p.nshot * p.rec.nrec, per);
        grd.z += recblk;
    }
    wave3d_cell_kernel<T, R, MODE><<<grd, tb, 0, s>>>(p, recblk);
}

template <typename T, int R, int MODE>
void launch_wave1d(const WaveParams<T>& p, int bz, cudaStream_t s) {
    (void)bz;
    const int tb = 128;
    int ntile = ceil_div(p.nz, tb);
    int grid = ntile * p.nshot;
    if (MODE == kFwd && p.rec.nrec > 0) grid += ceil_div((long long)p.nshot * p.rec.nrec, tb);
    wave1d_kernel<T, R, MODE><<<grid, tb, 0, s>>>(p, ntile);
}

#define PGB_INST13(T, R)                                                                    \
    template void launch_wave3d<T, R, kFwd>(const WaveParams<T>&, int, cudaStream_t);    \
    template void launch_wave3d<T, R, kRecomp>(const WaveParams<T>&, int, cudaStream_t); \
    template void launch_wave3d<T, R, kAdj>(const WaveParams<T>&, int, cudaStream_t);    \
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
