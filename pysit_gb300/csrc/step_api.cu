// Per-step leapfrog kernels with the exact semantics of the reference step
// templates (one launch = one time step over the whole padded grid):
//   cda_time_scalar_1D  pysit/solvers/constant_density_acoustic/time/scalar/
//                       constant_density_acoustic_time_scalar_1D.h:44-131
//   cda_time_scalar_2D  ..._2D.h:43-180
//   cda_time_scalar_3D  ..._3D.h:46-236
// Zero-extended stencils (fd_manual.hpp:5-70), Dirichlet outer ring, right PML
// profile read at r[n_r - ((n-1) - i)] (_2D.h:143-157), psi integrated on every
// non-ring cell in 3D.  These kernels serve the per-step API (time_step) and the
// plain per-shot path; the batched pipeline lives in wave2d_warp.cu / wave3d.cu.
//
// One thread per cell, z (the contiguous axis) on threadIdx.x.  Taps outside
// [0, n) are skipped, which is the zero extension of the reference.
#include "common.cuh"

namespace pgb {
namespace {

template <typename T>
struct Prof {  // one axis: left / right PML profile
    const T* l; int nl;
    const T* r; int nr;
    __device__ __forceinline__ T at(int i, int n) const {
        if (nl > 0 && i < nl) return l[i];
        if (nr > 0 && i >= n - nr) return r[nr - ((n - 1) - i)];
        return T(0);
    }
};

// first derivative, second derivative of v along one axis at position p of n,
// element stride s; out-of-range taps contribute zero.
template <typename T, int R>
__device__ __forceinline__ void derivs(const T* __restrict__ v, long long idx, long long s, int p,
                                       int n, T& d1, T& d2) {
    T a = 0, b = 0;
#pragma unroll
    for (int m = -R; m <= R; ++m) {
        if (p + m < 0 || p + m >= n) continue;
        T x = v[idx + m * s];
        a += T(d1tap(R, m)) * x;
        b += T(d2tap(R, m)) * x;
    }
    d1 = a;
    d2 = b;
}

template <typename T, int R>
__device__ __forceinline__ T deriv1(const T* __restrict__ v, long long idx, long long s, int p,
                                    int n) {
    T a = 0;
#pragma unroll
    for (int m = -R; m <= R; ++m) {
        if (m == 0 || p + m < 0 || p + m >= n) continue;
        a += T(d1tap(R, m)) * v[idx + m * s];
    }
    return a;
}

template <typename T>
struct Step1DArgs {
    const T *km1_u, *k_phiz, *k_u, *C, *rhs;
    Prof<T> pz;
    T dt, dt2, idz, idz2;
    int nz;
    T *kp1_phiz, *kp1_u;
};

template <typename T, int R>
__global__ void __launch_bounds__(256) step1d_kernel(Step1DArgs<T> a) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.nz) return;
    if (k == 0 || k == a.nz - 1) {
        a.kp1_phiz[k] = 0;
        a.kp1_u[k] = 0;
        return;
    }
    T dudz, lap;
    derivs<T, R>(a.k_u, k, 1, k, a.nz, dudz, lap);
    dudz *= a.idz;
    lap *= a.idz2;
    T dphiz = deriv1<T, R>(a.k_phiz, k, 1, k, a.nz) * a.idz;
    T sz = a.pz.at(k, a.nz);
    T c2 = a.C[k] * a.C[k];
    T um = a.km1_u[k], uc = a.k_u[k], ph = a.k_phiz[k];
    T F = a.rhs[k] + lap + dphiz;
    if (sz != T(0)) {
        a.kp1_phiz[k] = ph - a.dt * sz * (ph + dudz);
        T fac1 = T(2) * a.dt2 / (T(2) + a.dt * sz);
        T fac2 = c2 * F - (um - T(2) * uc) / a.dt2 + sz * um / (T(2) * a.dt);
        a.kp1_u[k] = fac1 * fac2;
    } else {
        a.kp1_phiz[k] = ph;
        a.kp1_u[k] = a.dt2 * c2 * F - (um - T(2) * uc);
    }
}

template <typename T>
struct Step2DArgs {
    const T *km1_u, *k_phix, *k_phiz, *k_u, *C, *rhs;
    Prof<T> px, pz;
    T dt, dt2, idx_, idx2, idz, idz2;
    int nx, nz;
    T *kp1_phix, *kp1_phiz, *kp1_u;
};

template <typename T, int R>
__global__ void __launch_bounds__(256) step2d_kernel(Step2DArgs<T> a) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (k >= a.nz || i >= a.nx) return;
    long long idx = (long long)i * a.nz + k;
    if (i == 0 || i == a.nx - 1 || k == 0 || k == a.nz - 1) {
        a.kp1_phix[idx] = 0;
        a.kp1_phiz[idx] = 0;
        a.kp1_u[idx] = 0;
        return;
    }
    T dudx, lapx, dudz, lapz;
    derivs<T, R>(a.k_u, idx, a.nz, i, a.nx, dudx, lapx);
    derivs<T, R>(a.k_u, idx, 1, k, a.nz, dudz, lapz);
    dudx *= a.idx_;
    dudz *= a.idz;
    T lap = lapx * a.idx2 + lapz * a.idz2;
    T dphix = deriv1<T, R>(a.k_phix, idx, a.nz, i, a.nx) * a.idx_;
    T dphiz = deriv1<T, R>(a.k_phiz, idx, 1, k, a.nz) * a.idz;
    T sx = a.px.at(i, a.nx), sz = a.pz.at(k, a.nz);
    T c2 = a.C[idx] * a.C[idx];
    T um = a.km1_u[idx], uc = a.k_u[idx];
    T phx = a.k_phix[idx], phz = a.k_phiz[idx];
    T F = a.rhs[idx] + lap + dphix + dphiz;
    if (sz != T(0) || sx != T(0)) {
        a.kp1_phix[idx] = phx - a.dt * sx * phx + a.dt * (sz - sx) * dudx;
        a.kp1_phiz[idx] = phz - a.dt * sz * phz + a.dt * (sx - sz) * dudz;
        T fac1 = T(2) * a.dt2 / (T(2) + a.dt * (sx + sz));
        T fac2 = c2 * F - (um - T(2) * uc) / a.dt2 + (sx + sz) * um / (T(2) * a.dt) - (sx * sz) * uc;
        a.kp1_u[idx] = fac1 * fac2;
    } else {
        a.kp1_phix[idx] = phx;
        a.kp1_phiz[idx] = phz;
        a.kp1_u[idx] = a.dt2 * c2 * F - (um - T(2) * uc);
    }
}

template <typename T>
struct Step3DArgs {
    const T *km1_u, *k_phix, *k_phiy, *k_phiz, *k_psi, *k_u, *C, *rhs;
    Prof<T> px, py, pz;
    T dt, dt2, idx_, idx2, idy, idy2, idz, idz2;
    int nx, ny, nz;
    T *kp1_phix, *kp1_phiy, *kp1_phiz, *kp1_psi, *kp1_u;
};

template <typename T, int R>
__global__ void __launch_bounds__(256) step3d_kernel(Step3DArgs<T> a) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int i = blockIdx.z;
    if (k >= a.nz || j >= a.ny) return;
    long long ys = a.nz, xs = (long long)a.ny * a.nz;
    long long idx = (long long)i * xs + (long long)j * ys + k;
    if (i == 0 || i == a.nx - 1 || j == 0 || j == a.ny - 1 || k == 0 || k == a.nz - 1) {
        a.kp1_u[idx] = 0;
        a.kp1_phix[idx] = 0;
        a.kp1_phiy[idx] = 0;
        a.kp1_phiz[idx] = 0;
        a.kp1_psi[idx] = 0;
        return;
    }
    T dudx, lapx, dudy, lapy, dudz, lapz;
    derivs<T, R>(a.k_u, idx, xs, i, a.nx, dudx, lapx);
    derivs<T, R>(a.k_u, idx, ys, j, a.ny, dudy, lapy);
    derivs<T, R>(a.k_u, idx, 1, k, a.nz, dudz, lapz);
    dudx *= a.idx_;
    dudy *= a.idy;
    dudz *= a.idz;
    T lap = lapx * a.idx2 + lapy * a.idy2 + lapz * a.idz2;
    T dphix = deriv1<T, R>(a.k_phix, idx, xs, i, a.nx) * a.idx_;
    T dphiy = deriv1<T, R>(a.k_phiy, idx, ys, j, a.ny) * a.idy;
    T dphiz = deriv1<T, R>(a.k_phiz, idx, 1, k, a.nz) * a.idz;
    T sx = a.px.at(i, a.nx), sy = a.py.at(j, a.ny), sz = a.pz.at(k, a.nz);
    T c2 = a.C[idx] * a.C[idx];
    T um = a.km1_u[idx], uc = a.k_u[idx], ps = a.k_psi[idx];
    a.kp1_psi[idx] = ps + a.dt * uc;
    T F = a.rhs[idx] + lap + dphix + dphiy + dphiz;
    if (sz != T(0) || sy != T(0) || sx != T(0)) {
        T dpsx = deriv1<T, R>(a.k_psi, idx, xs, i, a.nx) * a.idx_;
        T dpsy = deriv1<T, R>(a.k_psi, idx, ys, j, a.ny) * a.idy;
        T dpsz = deriv1<T, R>(a.k_psi, idx, 1, k, a.nz) * a.idz;
        T phx = a.k_phix[idx], phy = a.k_phiy[idx], phz = a.k_phiz[idx];
        a.kp1_phix[idx] = phx - a.dt * sx * phx + a.dt * (sy + sz - sx) * dudx + a.dt * (sy * sz * dpsx);
        a.kp1_phiy[idx] = phy - a.dt * sy * phy + a.dt * (sz + sx - sy) * dudy + a.dt * (sz * sx * dpsy);
        a.kp1_phiz[idx] = phz - a.dt * sz * phz + a.dt * (sx + sy - sz) * dudz + a.dt * (sx * sy * dpsz);
        T fac1 = T(2) * a.dt2 / (T(2) + a.dt * (sx + sy + sz));
        T fac2 = c2 * (F - (sx * sy * sz) * ps) - (um - T(2) * uc) / a.dt2 +
                 (sx + sy + sz) * um / (T(2) * a.dt) - (sx * sy + sy * sz + sz * sx) * uc;
        a.kp1_u[idx] = fac1 * fac2;
    } else {
        a.kp1_phix[idx] = a.k_phix[idx];
        a.kp1_phiy[idx] = a.k_phiy[idx];
        a.kp1_phiz[idx] = a.k_phiz[idx];
        a.kp1_u[idx] = a.dt2 * c2 * F - (um - T(2) * uc);
    }
}

// dWaveOp = (u+ - 2u + u-)/dt^2 + S1 (u+ - u-)/(2dt) + S2 u + S3 psi
template <typename T>
__global__ void __launch_bounds__(256) dwaveop_kernel(int dim, const T* __restrict__ um,
                                                      const T* __restrict__ uc,
                                                      const T* __restrict__ up,
                                                      const T* __restrict__ psi,
                                                      const T* __restrict__ sgx,
                                                      const T* __restrict__ sgy,
                                                      const T* __restrict__ sgz, int nx, int ny,
                                                      int nz, T idt2, T i2dt, T* __restrict__ out) {
    long long n = (long long)nx * ny * nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        int k = (int)(c % nz);
        long long r = c / nz;
        int j = (int)(r % ny);
        int i = (int)(r / ny);
        T sx = sgx ? sgx[i] : T(0), sy = sgy ? sgy[j] : T(0), sz = sgz ? sgz[k] : T(0);
        T a = um[c], b = uc[c], d = up[c];
        T v = (d - T(2) * b + a) * idt2;
        T s1 = sx + sy + sz;
        T s2 = sx * sy + sx * sz + sy * sz;
        v += s1 * (d - a) * i2dt + s2 * b;
        if (dim == 3 && psi) v += (sx * sy * sz) * psi[c];
        out[c] = v;
    }
}

template <typename T>
Prof<T> prof(const void* l, int nl, const void* r, int nr) {
    return Prof<T>{static_cast<const T*>(l), nl, static_cast<const T*>(r), nr};
}

template <typename T>
int launch1d(int order, const void* km1_u, const void* k_phiz, const void* k_u, const void* C,
             const void* rhs, const void* zl, int nzl, const void* zr, int nzr, double dt,
             double dz, int nz, void* kp1_phiz, void* kp1_u, cudaStream_t s) {
    Step1DArgs<T> a{(const T*)km1_u, (const T*)k_phiz, (const T*)k_u, (const T*)C, (const T*)rhs,
                    prof<T>(zl, nzl, zr, nzr), T(dt), T(T(dt) * T(dt)), T(1.0 / dz),
                    T(1.0 / (T(dz) * T(dz))), nz, (T*)kp1_phiz, (T*)kp1_u};
    dim3 blk(256), grd(ceil_div(nz, 256));
    switch (order) {
        case 2: step1d_kernel<T, 1><<<grd, blk, 0, s>>>(a); break;
        case 4: step1d_kernel<T, 2><<<grd, blk, 0, s>>>(a); break;
        case 6: step1d_kernel<T, 3><<<grd, blk, 0, s>>>(a); break;
        case 8: step1d_kernel<T, 4><<<grd, blk, 0, s>>>(a); break;
    }
    PGB_CHECK_CUDA(cudaGetLastError());
    return PYSIT_OK;
}

template <typename T>
int launch2d(int order, const void* km1_u, const void* k_phix, const void* k_phiz,
             const void* k_u, const void* C, const void* rhs, const void* xl, int nxl,
             const void* xr, int nxr, const void* zl, int nzl, const void* zr, int nzr,
             double dt, double dx, double dz, int nx, int nz, void* kp1_phix, void* kp1_phiz,
             void* kp1_u, cudaStream_t s) {
    Step2DArgs<T> a{(const T*)km1_u, (const T*)k_phix, (const T*)k_phiz, (const T*)k_u,
                    (const T*)C, (const T*)rhs, prof<T>(xl, nxl, xr, nxr), prof<T>(zl, nzl, zr, nzr),
                    T(dt), T(T(dt) * T(dt)), T(1.0 / dx), T(1.0 / (T(dx) * T(dx))), T(1.0 / dz),
                    T(1.0 / (T(dz) * T(dz))), nx, nz, (T*)kp1_phix, (T*)kp1_phiz, (T*)kp1_u};
    dim3 blk(32, 8), grd(ceil_div(nz, 32), ceil_div(nx, 8));
    switch (order) {
        case 2: step2d_kernel<T, 1><<<grd, blk, 0, s>>>(a); break;
        case 4: step2d_kernel<T, 2><<<grd, blk, 0, s>>>(a); break;
        case 6: step2d_kernel<T, 3><<<grd, blk, 0, s>>>(a); break;
        case 8: step2d_kernel<T, 4><<<grd, blk, 0, s>>>(a); break;
    }
    PGB_CHECK_CUDA(cudaGetLastError());
    return PYSIT_OK;
}

template <typename T>
int launch3d(int order, const void* km1_u, const void* k_phix, const void* k_phiy,
             const void* k_phiz, const void* k_psi, const void* k_u, const void* C,
             const void* rhs, const void* xl, int nxl, const void* xr, int nxr, const void* yl,
             int nyl, const void* yr, int nyr, const void* zl, int nzl, const void* zr, int nzr,
             double dt, double dx, double dy, double dz, int nx, int ny, int nz, void* kp1_phix,
             void* kp1_phiy, void* kp1_phiz, void* kp1_psi, void* kp1_u, cudaStream_t s) {
    Step3DArgs<T> a{(const T*)km1_u, (const T*)k_phix, (const T*)k_phiy, (const T*)k_phiz,
                    (const T*)k_psi, (const T*)k_u, (const T*)C, (const T*)rhs,
                    prof<T>(xl, nxl, xr, nxr), prof<T>(yl, nyl, yr, nyr), prof<T>(zl, nzl, zr, nzr),
                    T(dt), T(T(dt) * T(dt)), T(1.0 / dx), T(1.0 / (T(dx) * T(dx))), T(1.0 / dy),
                    T(1.0 / (T(dy) * T(dy))), T(1.0 / dz), T(1.0 / (T(dz) * T(dz))), nx, ny, nz,
                    (T*)kp1_phix, (T*)kp1_phiy, (T*)kp1_phiz, (T*)kp1_psi, (T*)kp1_u};
    dim3 blk(32, 8), grd(ceil_div(nz, 32), ceil_div(ny, 8), nx);
    switch (order) {
        case 2: step3d_kernel<T, 1><<<grd, blk, 0, s>>>(a); break;
        case 4: step3d_kernel<T, 2><<<grd, blk, 0, s>>>(a); break;
        case 6: step3d_kernel<T, 3><<<grd, blk, 0, s>>>(a); break;
        case 8: step3d_kernel<T, 4><<<grd, blk, 0, s>>>(a); break;
    }
    PGB_CHECK_CUDA(cudaGetLastError());
    return PYSIT_OK;
}

int check_common(int dtype, int order) {
    PGB_REQUIRE(dtype == PYSIT_F32 || dtype == PYSIT_F64, "dtype must be PYSIT_F32 or PYSIT_F64 (got %d)", dtype);
    PGB_REQUIRE(order == 2 || order == 4 || order == 6 || order == 8,
                "spatial_accuracy_order must be one of 2, 4, 6, 8 (got %d)", order);
    return PYSIT_OK;
}

int check_sigma(const void* l, int nl, const void* r, int nr, int n, const char* ax) {
    PGB_REQUIRE(nl >= 0 && nr >= 0, "negative PML profile length on axis %s", ax);
    PGB_REQUIRE(nl == 0 || l, "NULL left PML profile on axis %s", ax);
    PGB_REQUIRE(nr == 0 || r, "NULL right PML profile on axis %s", ax);
    PGB_REQUIRE(nl <= n && nr <= n, "PML profile longer than the axis %s (n=%d)", ax, n);
    return PYSIT_OK;
}

}  // namespace
}  // namespace pgb

using namespace pgb;

extern "C" int pysit_cda_step_1d(int dtype, int order, const void* km1_u, const void* k_phiz,
                                 const void* k_u, const void* C, const void* rhs,
                                 const void* zlpml, int n_zlpml, const void* zrpml, int n_zrpml,
                                 double dt, double dz, int nz, void* kp1_phiz, void* kp1_u,
                                 void* stream) {
    int rc = check_common(dtype, order);
    if (rc) return rc;
    PGB_REQUIRE(nz >= 3, "nz must be >= 3 (got %d)", nz);
    PGB_REQUIRE(km1_u && k_phiz && k_u && C && rhs && kp1_phiz && kp1_u, "NULL array argument");
    rc = check_sigma(zlpml, n_zlpml, zrpml, n_zrpml, nz, "z");
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (dtype == PYSIT_F64)
        return launch1d<double>(order, km1_u, k_phiz, k_u, C, rhs, zlpml, n_zlpml, zrpml, n_zrpml,
                                dt, dz, nz, kp1_phiz, kp1_u, s);
    return launch1d<float>(order, km1_u, k_phiz, k_u, C, rhs, zlpml, n_zlpml, zrpml, n_zrpml, dt,
                           dz, nz, kp1_phiz, kp1_u, s);
}

extern "C" int pysit_cda_step_2d(int dtype, int order, const void* km1_u, const void* k_phix,
                                 const void* k_phiz, const void* k_u, const void* C,
                                 const void* rhs, const void* xlpml, int n_xlpml,
                                 const void* xrpml, int n_xrpml, const void* zlpml, int n_zlpml,
                                 const void* zrpml, int n_zrpml, double dt, double dx, double dz,
                                 int nx, int nz, void* kp1_phix, void* kp1_phiz, void* kp1_u,
                                 void* stream) {
    int rc = check_common(dtype, order);
    if (rc) return rc;
    PGB_REQUIRE(nx >= 3 && nz >= 3, "grid must be at least 3x3 (got %dx%d)", nx, nz);
    PGB_REQUIRE(km1_u && k_phix && k_phiz && k_u && C && rhs && kp1_phix && kp1_phiz && kp1_u,
                "NULL array argument");
    if ((rc = check_sigma(xlpml, n_xlpml, xrpml, n_xrpml, nx, "x"))) return rc;
    if ((rc = check_sigma(zlpml, n_zlpml, zrpml, n_zrpml, nz, "z"))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (dtype == PYSIT_F64)
        return launch2d<double>(order, km1_u, k_phix, k_phiz, k_u, C, rhs, xlpml, n_xlpml, xrpml,
                                n_xrpml, zlpml, n_zlpml, zrpml, n_zrpml, dt, dx, dz, nx, nz,
                                kp1_phix, kp1_phiz, kp1_u, s);
    return launch2d<float>(order, km1_u, k_phix, k_phiz, k_u, C, rhs, xlpml, n_xlpml, xrpml,
                           n_xrpml, zlpml, n_zlpml, zrpml, n_zrpml, dt, dx, dz, nx, nz, kp1_phix,
                           kp1_phiz, kp1_u, s);
}

extern "C" int pysit_cda_step_3d(int dtype, int order, const void* km1_u, const void* k_phix,
                                 const void* k_phiy, const void* k_phiz, const void* k_psi,
                                 const void* k_u, const void* C, const void* rhs,
                                 const void* xlpml, int n_xlpml, const void* xrpml, int n_xrpml,
                                 const void* ylpml, int n_ylpml, const void* yrpml, int n_yrpml,
                                 const void* zlpml, int n_zlpml, const void* zrpml, int n_zrpml,
                                 double dt, double dx, double dy, double dz, int nx, int ny,
                                 int nz, void* kp1_phix, void* kp1_phiy, void* kp1_phiz,
                                 void* kp1_psi, void* kp1_u, void* stream) {
    int rc = check_common(dtype, order);
    if (rc) return rc;
    PGB_REQUIRE(nx >= 3 && ny >= 3 && nz >= 3, "grid must be at least 3x3x3 (got %dx%dx%d)", nx, ny, nz);
    PGB_REQUIRE(ny <= 65535 * 8 && nx <= 65535, "grid too large for the per-step 3D kernel");
    PGB_REQUIRE(km1_u && k_phix && k_phiy && k_phiz && k_psi && k_u && C && rhs && kp1_phix &&
                    kp1_phiy && kp1_phiz && kp1_psi && kp1_u,
                "NULL array argument");
    if ((rc = check_sigma(xlpml, n_xlpml, xrpml, n_xrpml, nx, "x"))) return rc;
    if ((rc = check_sigma(ylpml, n_ylpml, yrpml, n_yrpml, ny, "y"))) return rc;
    if ((rc = check_sigma(zlpml, n_zlpml, zrpml, n_zrpml, nz, "z"))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (dtype == PYSIT_F64)
        return launch3d<double>(order, km1_u, k_phix, k_phiy, k_phiz, k_psi, k_u, C, rhs, xlpml,
                                n_xlpml, xrpml, n_xrpml, ylpml, n_ylpml, yrpml, n_yrpml, zlpml,
                                n_zlpml, zrpml, n_zrpml, dt, dx, dy, dz, nx, ny, nz, kp1_phix,
                                kp1_phiy, kp1_phiz, kp1_psi, kp1_u, s);
    return launch3d<float>(order, km1_u, k_phix, k_phiy, k_phiz, k_psi, k_u, C, rhs, xlpml,
                           n_xlpml, xrpml, n_xrpml, ylpml, n_ylpml, yrpml, n_yrpml, zlpml, n_zlpml,
                           zrpml, n_zrpml, dt, dx, dy, dz, nx, ny, nz, kp1_phix, kp1_phiy,
                           kp1_phiz, kp1_psi, kp1_u, s);
}

extern "C" int pysit_cda_dwaveop(int dtype, int dim, const void* km1_u, const void* k_u,
                                 const void* kp1_u, const void* psi_k, const void* sig_x,
                                 const void* sig_y, const void* sig_z, int nx, int ny, int nz,
                                 double dt, void* out, void* stream) {
    PGB_REQUIRE(dtype == PYSIT_F32 || dtype == PYSIT_F64, "bad dtype %d", dtype);
    PGB_REQUIRE(dim >= 1 && dim <= 3, "dim must be 1, 2 or 3 (got %d)", dim);
    PGB_REQUIRE(nx >= 1 && ny >= 1 && nz >= 1, "bad grid size");
    PGB_REQUIRE(km1_u && k_u && kp1_u && out, "NULL array argument");
    PGB_REQUIRE(dim < 3 || psi_k, "3D dWaveOp needs psi_k");
    long long n = (long long)nx * ny * nz;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 32) blocks = 152 * 32;
    cudaStream_t s = (cudaStream_t)stream;
    if (dtype == PYSIT_F64) {
        dwaveop_kernel<double><<<blocks, 256, 0, s>>>(
            dim, (const double*)km1_u, (const double*)k_u, (const double*)kp1_u,
            (const double*)psi_k, (const double*)sig_x, (const double*)sig_y, (const double*)sig_z,
            nx, ny, nz, 1.0 / (dt * dt), 1.0 / (2.0 * dt), (double*)out);
    } else {
        dwaveop_kernel<float><<<blocks, 256, 0, s>>>(
            dim, (const float*)km1_u, (const float*)k_u, (const float*)kp1_u, (const float*)psi_k,
            (const float*)sig_x, (const float*)sig_y, (const float*)sig_z, nx, ny, nz,
            (float)(1.0 / (dt * dt)), (float)(1.0 / (2.0 * dt)), (float*)out);
    }
    PGB_CHECK_CUDA(cudaGetLastError());
    return PYSIT_OK;
}
