/*
 * oracle/cda_oracle.c -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * CPU restatement of PySIT's constant-density acoustic leapfrog step with
 * split-field PML, used only as the checker: by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  The product
 * path (pysit_gb300) never links or calls this file.
 *
 * Parity pin: tests/test_oracle_pin.py compares these functions with the
 * reference's own templates (compiled from pysit/solvers/constant_density_acoustic/
 * time/scalar/ headers into oracle/_ref by oracle/Makefile) on random inputs, and
 * tests/golden/ holds traces and gradients produced by the reference package.
 *
 * Semantics restated (reference file:line, paths inside the pysit project):
 *  - one call = one time step over the whole padded grid, z is the fastest axis
 *    (constant_density_acoustic_time_scalar_2D.h:81-92, _3D.h:98-113);
 *  - every output is zeroed, the outer ring of cells is never updated
 *    (homogeneous Dirichlet; _2D.h:94-100, _3D.h:115-124, _1D.h:81-87);
 *  - derivative taps that fall outside [0,n) contribute zero: the "shifted"
 *    stencils of pysit/solvers/fd_tools/fd_manual.hpp:5-70 are exactly a
 *    zero-extension of the field for n >= order;
 *  - first/second derivative weights are the standard central-difference
 *    weights of orders 2..8 (fd_manual.hpp:8-69);
 *  - PML sigma: left profile l[i] for i < nl, else right profile
 *    r[nr-((n-1)-i)] for i >= n-nr (_2D.h:137-157) -- note the right index is
 *    shifted one node relative to the mesh's own sigma map;
 *  - PML branch when any sigma != 0, update formulas of _2D.h:159-174,
 *    _3D.h:210-232, _1D.h:117-129; psi' = psi + dt*u on every non-ring cell
 *    in 3D (_3D.h:216,230).
 *
 * Both double and float instantiations exist (the reference instantiates both,
 * constant_density_acoustic_time_scalar.i:57-84).  Scalars dt/dx/... are
 * double, as in the reference signature.
 */
#include <stddef.h>
#include "cda_oracle.h"

/* antisymmetric first-derivative weights a_m (m = 1..R) and symmetric
 * second-derivative weights b_m (m = 0..R) of the central stencils of
 * order 2R, R = 1..4 (standard Fornberg weights). */
static const double D1W[5][5] = {
    {0, 0, 0, 0, 0},
    {0, 1.0 / 2.0, 0, 0, 0},
    {0, 2.0 / 3.0, -1.0 / 12.0, 0, 0},
    {0, 3.0 / 4.0, -3.0 / 20.0, 1.0 / 60.0, 0},
    {0, 4.0 / 5.0, -1.0 / 5.0, 4.0 / 105.0, -1.0 / 280.0},
};
static const double D2W[5][5] = {
    {0, 0, 0, 0, 0},
    {-2.0, 1.0, 0, 0, 0},
    {-5.0 / 2.0, 4.0 / 3.0, -1.0 / 12.0, 0, 0},
    {-49.0 / 18.0, 3.0 / 2.0, -3.0 / 20.0, 1.0 / 90.0, 0},
    {-205.0 / 72.0, 8.0 / 5.0, -1.0 / 5.0, 8.0 / 315.0, -1.0 / 560.0},
};

/* The arithmetic is written once as a macro body and instantiated for double
 * and float, mirroring the two reference template instantiations. */
#define DEFINE_ORACLE(T, SUF)                                                          \
                                                                                       \
static inline __attribute__((always_inline))                                          \
T d1_##SUF(const T* v, ptrdiff_t idx, ptrdiff_t s, int pos, int n, const int R, T del) \
{                                                                                      \
    /* taps summed from -R to +R, out-of-range taps are zero; a cell R or more from    \
     * both ends takes every tap, so its loop drops the range test and sums the same   \
     * terms in the same order */                                                      \
    T acc = 0;                                                                         \
    if (pos >= R && pos < n - R) {                                                     \
        for (int m = -R; m <= R; ++m) {                                                \
            if (m == 0) continue;                                                      \
            T w = (T)(m > 0 ? D1W[R][m] : -D1W[R][-m]);                                \
            acc += w * v[idx + (ptrdiff_t)m * s];                                      \
        }                                                                              \
        return acc / del;                                                              \
    }                                                                                  \
    for (int m = -R; m <= R; ++m) {                                                    \
        if (m == 0) continue;                                                          \
        int p = pos + m;                                                               \
        if (p < 0 || p >= n) continue;                                                 \
        T w = (T)(m > 0 ? D1W[R][m] : -D1W[R][-m]);                                    \
        acc += w * v[idx + (ptrdiff_t)m * s];                                          \
    }                                                                                  \
    return acc / del;                                                                  \
}                                                                                      \
                                                                                       \
static inline __attribute__((always_inline))                                          \
T d2_##SUF(const T* v, ptrdiff_t idx, ptrdiff_t s, int pos, int n, const int R, T del2) \
{                                                                                      \
    T acc = 0;                                                                         \
    if (pos >= R && pos < n - R) {                                                     \
        for (int m = -R; m <= R; ++m) {                                                \
            T w = (T)D2W[R][m < 0 ? -m : m];                                           \
            acc += w * v[idx + (ptrdiff_t)m * s];                                      \
        }                                                                              \
        return acc / del2;                                                             \
    }                                                                                  \
    for (int m = -R; m <= R; ++m) {                                                    \
        int p = pos + m;                                                               \
        if (p < 0 || p >= n) continue;                                                 \
        T w = (T)D2W[R][m < 0 ? -m : m];                                               \
        acc += w * v[idx + (ptrdiff_t)m * s];                                          \
    }                                                                                  \
    return acc / del2;                                                                 \
}                                                                                      \
                                                                                       \
static T sig_##SUF(const T* l, int nl, const T* r, int nr, int i, int n)              \
{                                                                                      \
    if (nl > 0 && i < nl) return l[i];                                                 \
    if (nr > 0 && i >= n - nr) return r[nr - ((n - 1) - i)];                           \
    return (T)0;                                                                       \
}                                                                                      \
                                                                                       \
int oracle_cda1d_step_##SUF(int order, const T* km1_u, const T* k_phiz, const T* k_u,  \
                            const T* C, const T* rhs, const T* zl, int nzl,            \
                            const T* zr, int nzr, double dt, double dz, int nz,        \
                            T* kp1_phiz, T* kp1_u)                                     \
{                                                                                      \
    int R = order / 2;                                                                 \
    if (order < 2 || order > 8 || (order & 1) || nz < 3) return -1;                    \
    T dt2 = (T)(dt * dt);                                                              \
    T tdz = (T)dz, tdz2 = tdz * tdz;                                                   \
    for (int k = 0; k < nz; ++k) {                                                     \
        kp1_phiz[k] = 0; kp1_u[k] = 0;                                                 \
        if (k == 0 || k == nz - 1) continue;                                           \
        T dudz = d1_##SUF(k_u, k, 1, k, nz, R, tdz);                                   \
        T dphizdz = d1_##SUF(k_phiz, k, 1, k, nz, R, tdz);                             \
        T lap = d2_##SUF(k_u, k, 1, k, nz, R, tdz2);                                   \
        T sz = sig_##SUF(zl, nzl, zr, nzr, k, nz);                                     \
        T c2 = C[k] * C[k];                                                            \
        if (sz != 0) {                                                                 \
            kp1_phiz[k] = k_phiz[k] - dt * sz * (k_phiz[k] + dudz);                    \
            T fac1 = (T)(2.0 * dt2 / (2.0 + dt * sz));                                 \
            T fac2 = c2 * (rhs[k] + lap + dphizdz) - (km1_u[k] - 2.0 * k_u[k]) / dt2   \
                     + sz * km1_u[k] / (2.0 * dt);                                     \
            kp1_u[k] = fac1 * fac2;                                                    \
        } else {                                                                       \
            kp1_phiz[k] = k_phiz[k];                                                   \
            kp1_u[k] = dt2 * c2 * (rhs[k] + lap + dphizdz) - (km1_u[k] - 2.0 * k_u[k]); \
        }                                                                              \
    }                                                                                  \
    return 0;                                                                          \
}                                                                                      \
                                                                                       \
/* the step body, inlined once per stencil radius R (1..4) so that the tap loops   \
 * unroll; the public entry below picks the instance */                               \
static inline __attribute__((always_inline))                                          \
void step2d_##SUF(const int R, const T* km1_u, const T* k_phix,                       \
                  const T* k_phiz, const T* k_u, const T* C, const T* rhs,             \
                  const T* xl, int nxl, const T* xr, int nxr,                          \
                  const T* zl, int nzl, const T* zr, int nzr,                          \
                  double dt, double dx, double dz, int nx, int nz,                     \
                  T* kp1_phix, T* kp1_phiz, T* kp1_u)                                  \
{                                                                                      \
    T dt2 = (T)(dt * dt);                                                              \
    T tdx = (T)dx, tdx2 = tdx * tdx, tdz = (T)dz, tdz2 = tdz * tdz;                    \
    ptrdiff_t xs = nz;                                                                 \
    for (int i = 0; i < nx; ++i) {                                                     \
        for (int k = 0; k < nz; ++k) {                                                 \
            ptrdiff_t idx = (ptrdiff_t)i * xs + k;                                     \
            kp1_phix[idx] = 0; kp1_phiz[idx] = 0; kp1_u[idx] = 0;                      \
            if (i == 0 || i == nx - 1 || k == 0 || k == nz - 1) continue;              \
            T dudx = d1_##SUF(k_u, idx, xs, i, nx, R, tdx);                            \
            T dphixdx = d1_##SUF(k_phix, idx, xs, i, nx, R, tdx);                      \
            T lap = d2_##SUF(k_u, idx, xs, i, nx, R, tdx2);                            \
            T dudz = d1_##SUF(k_u, idx, 1, k, nz, R, tdz);                             \
            T dphizdz = d1_##SUF(k_phiz, idx, 1, k, nz, R, tdz);                       \
            lap += d2_##SUF(k_u, idx, 1, k, nz, R, tdz2);                              \
            T sx = sig_##SUF(xl, nxl, xr, nxr, i, nx);                                 \
            T sz = sig_##SUF(zl, nzl, zr, nzr, k, nz);                                 \
            T c2 = C[idx] * C[idx];                                                    \
            T um = km1_u[idx], uc = k_u[idx];                                          \
            if (sz != 0 || sx != 0) {                                                  \
                kp1_phix[idx] = k_phix[idx] - dt * sx * k_phix[idx]                    \
                                + dt * (sz - sx) * dudx;                               \
                kp1_phiz[idx] = k_phiz[idx] - dt * sz * k_phiz[idx]                    \
                                + dt * (sx - sz) * dudz;                               \
                T fac1 = (T)(2.0 * dt2 / (2.0 + dt * (sx + sz)));                      \
                T fac2 = c2 * (rhs[idx] + lap + dphixdx + dphizdz)                     \
                         - (um - 2.0 * uc) / dt2 + (sx + sz) * um / (2.0 * dt)         \
                         - (sx * sz) * uc;                                             \
                kp1_u[idx] = fac1 * fac2;                                              \
            } else {                                                                   \
                kp1_phix[idx] = k_phix[idx];                                           \
                kp1_phiz[idx] = k_phiz[idx];                                           \
                kp1_u[idx] = dt2 * c2 * (rhs[idx] + lap + dphixdx + dphizdz)           \
                             - (um - 2.0 * uc);                                        \
            }                                                                          \
        }                                                                              \
    }                                                                                  \
}                                                                                      \
                                                                                       \
int oracle_cda2d_step_##SUF(int order, const T* km1_u, const T* k_phix,                \
                            const T* k_phiz, const T* k_u, const T* C, const T* rhs,   \
                            const T* xl, int nxl, const T* xr, int nxr,                \
                            const T* zl, int nzl, const T* zr, int nzr,                \
                            double dt, double dx, double dz, int nx, int nz,           \
                            T* kp1_phix, T* kp1_phiz, T* kp1_u)                        \
{                                                                                      \
    if (order < 2 || order > 8 || (order & 1) || nx < 3 || nz < 3) return -1;          \
    switch (order / 2) {                                                               \
    case 1: step2d_##SUF(1, km1_u, k_phix, k_phiz, k_u, C, rhs, xl, nxl, xr, nxr, zl,  \
                         nzl, zr, nzr, dt, dx, dz, nx, nz, kp1_phix, kp1_phiz, kp1_u); \
            break;                                                                     \
    case 2: step2d_##SUF(2, km1_u, k_phix, k_phiz, k_u, C, rhs, xl, nxl, xr, nxr, zl,  \
                         nzl, zr, nzr, dt, dx, dz, nx, nz, kp1_phix, kp1_phiz, kp1_u); \
            break;                                                                     \
    case 3: step2d_##SUF(3, km1_u, k_phix, k_phiz, k_u, C, rhs, xl, nxl, xr, nxr, zl,  \
                         nzl, zr, nzr, dt, dx, dz, nx, nz, kp1_phix, kp1_phiz, kp1_u); \
            break;                                                                     \
    default: step2d_##SUF(4, km1_u, k_phix, k_phiz, k_u, C, rhs, xl, nxl, xr, nxr, zl, \
                          nzl, zr, nzr, dt, dx, dz, nx, nz, kp1_phix, kp1_phiz,        \
                          kp1_u);                                                      \
    }                                                                                  \
    return 0;                                                                          \
}                                                                                      \
                                                                                       \
static inline __attribute__((always_inline))                                          \
void step3d_##SUF(const int R, const T* km1_u, const T* k_phix,                       \
                  const T* k_phiy, const T* k_phiz, const T* k_psi,                    \
                  const T* k_u, const T* C, const T* rhs,                              \
                  const T* xl, int nxl, const T* xr, int nxr,                          \
                  const T* yl, int nyl, const T* yr, int nyr,                          \
                  const T* zl, int nzl, const T* zr, int nzr,                          \
                  double dt, double dx, double dy, double dz,                          \
                  int nx, int ny, int nz,                                              \
                  T* kp1_phix, T* kp1_phiy, T* kp1_phiz, T* kp1_psi, T* kp1_u)         \
{                                                                                      \
    T dt2 = (T)(dt * dt);                                                              \
    T tdx = (T)dx, tdx2 = tdx * tdx, tdy = (T)dy, tdy2 = tdy * tdy;                    \
    T tdz = (T)dz, tdz2 = tdz * tdz;                                                   \
    ptrdiff_t ys = nz, xs = (ptrdiff_t)ny * nz;                                        \
    for (int i = 0; i < nx; ++i)                                                       \
    for (int j = 0; j < ny; ++j)                                                       \
    for (int k = 0; k < nz; ++k) {                                                     \
        ptrdiff_t idx = (ptrdiff_t)i * xs + (ptrdiff_t)j * ys + k;                     \
        kp1_u[idx] = 0; kp1_phix[idx] = 0; kp1_phiy[idx] = 0; kp1_phiz[idx] = 0;       \
        kp1_psi[idx] = 0;                                                              \
        if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || k == 0 || k == nz - 1)   \
            continue;                                                                  \
        T dudx = d1_##SUF(k_u, idx, xs, i, nx, R, tdx);                                \
        T dphixdx = d1_##SUF(k_phix, idx, xs, i, nx, R, tdx);                          \
        T dpsidx = d1_##SUF(k_psi, idx, xs, i, nx, R, tdx);                            \
        T lap = d2_##SUF(k_u, idx, xs, i, nx, R, tdx2);                                \
        T dudy = d1_##SUF(k_u, idx, ys, j, ny, R, tdy);                                \
        T dphiydy = d1_##SUF(k_phiy, idx, ys, j, ny, R, tdy);                          \
        T dpsidy = d1_##SUF(k_psi, idx, ys, j, ny, R, tdy);                            \
        lap += d2_##SUF(k_u, idx, ys, j, ny, R, tdy2);                                 \
        T dudz = d1_##SUF(k_u, idx, 1, k, nz, R, tdz);                                 \
        T dphizdz = d1_##SUF(k_phiz, idx, 1, k, nz, R, tdz);                           \
        T dpsidz = d1_##SUF(k_psi, idx, 1, k, nz, R, tdz);                             \
        lap += d2_##SUF(k_u, idx, 1, k, nz, R, tdz2);                                  \
        T sx = sig_##SUF(xl, nxl, xr, nxr, i, nx);                                     \
        T sy = sig_##SUF(yl, nyl, yr, nyr, j, ny);                                     \
        T sz = sig_##SUF(zl, nzl, zr, nzr, k, nz);                                     \
        T c2 = C[idx] * C[idx];                                                        \
        T um = km1_u[idx], uc = k_u[idx];                                              \
        kp1_psi[idx] = k_psi[idx] + dt * uc;                                           \
        if (sz != 0 || sy != 0 || sx != 0) {                                           \
            kp1_phix[idx] = k_phix[idx] - dt * sx * k_phix[idx]                        \
                            + dt * (sy + sz - sx) * dudx + dt * (sy * sz * dpsidx);    \
            kp1_phiy[idx] = k_phiy[idx] - dt * sy * k_phiy[idx]                        \
                            + dt * (sz + sx - sy) * dudy + dt * (sz * sx * dpsidy);    \
            kp1_phiz[idx] = k_phiz[idx] - dt * sz * k_phiz[idx]                        \
                            + dt * (sx + sy - sz) * dudz + dt * (sx * sy * dpsidz);    \
            T fac1 = (T)(2.0 * dt2 / (2.0 + dt * (sx + sy + sz)));                     \
            T src = g_psi_consistent                                                   \
                ? c2 * (rhs[idx] + lap + dphixdx + dphiydy + dphizdz)                  \
                      - (sx * sy * sz) * k_psi[idx]                                    \
                : c2 * (rhs[idx] + lap + dphixdx + dphiydy + dphizdz                   \
                        - (sx * sy * sz) * k_psi[idx]);                                \
            T fac2 = src                                                               \
                     - (um - 2.0 * uc) / dt2 + (sx + sy + sz) * um / (2.0 * dt)        \
                     - (sx * sy + sy * sz + sz * sx) * uc;                             \
            kp1_u[idx] = fac1 * fac2;                                                  \
        } else {                                                                       \
            kp1_phix[idx] = k_phix[idx];                                               \
            kp1_phiy[idx] = k_phiy[idx];                                               \
            kp1_phiz[idx] = k_phiz[idx];                                               \
            kp1_u[idx] = dt2 * c2 * (rhs[idx] + lap + dphixdx + dphiydy + dphizdz)     \
                         - (um - 2.0 * uc);                                            \
        }                                                                              \
    }                                                                                  \
}                                                                                      \
                                                                                       \
int oracle_cda3d_step_##SUF(int order, const T* km1_u, const T* k_phix,                \
                            const T* k_phiy, const T* k_phiz, const T* k_psi,          \
                            const T* k_u, const T* C, const T* rhs,                    \
                            const T* xl, int nxl, const T* xr, int nxr,                \
                            const T* yl, int nyl, const T* yr, int nyr,                \
                            const T* zl, int nzl, const T* zr, int nzr,                \
                            double dt, double dx, double dy, double dz,                \
                            int nx, int ny, int nz,                                    \
                            T* kp1_phix, T* kp1_phiy, T* kp1_phiz, T* kp1_psi,         \
                            T* kp1_u)                                                  \
{                                                                                      \
    if (order < 2 || order > 8 || (order & 1) || nx < 3 || ny < 3 || nz < 3)           \
        return -1;                                                                     \
    switch (order / 2) {                                                               \
    case 1: step3d_##SUF(1, km1_u, k_phix, k_phiy, k_phiz, k_psi, k_u, C, rhs, xl, nxl, \
                         xr, nxr, yl, nyl, yr, nyr, zl, nzl, zr, nzr, dt, dx, dy, dz,  \
                         nx, ny, nz, kp1_phix, kp1_phiy, kp1_phiz, kp1_psi, kp1_u);    \
            break;                                                                     \
    case 2: step3d_##SUF(2, km1_u, k_phix, k_phiy, k_phiz, k_psi, k_u, C, rhs, xl, nxl, \
                         xr, nxr, yl, nyl, yr, nyr, zl, nzl, zr, nzr, dt, dx, dy, dz,  \
                         nx, ny, nz, kp1_phix, kp1_phiy, kp1_phiz, kp1_psi, kp1_u);    \
            break;                                                                     \
    case 3: step3d_##SUF(3, km1_u, k_phix, k_phiy, k_phiz, k_psi, k_u, C, rhs, xl, nxl, \
                         xr, nxr, yl, nyl, yr, nyr, zl, nzl, zr, nzr, dt, dx, dy, dz,  \
                         nx, ny, nz, kp1_phix, kp1_phiy, kp1_phiz, kp1_psi, kp1_u);    \
            break;                                                                     \
    default: step3d_##SUF(4, km1_u, k_phix, k_phiy, k_phiz, k_psi, k_u, C, rhs, xl,    \
                          nxl, xr, nxr, yl, nyl, yr, nyr, zl, nzl, zr, nzr, dt, dx,    \
                          dy, dz, nx, ny, nz, kp1_phix, kp1_phiy, kp1_phiz, kp1_psi,   \
                          kp1_u);                                                      \
    }                                                                                  \
    return 0;                                                                          \
}

/* 3D: 0 (default) = the reference's step (_3D.h:219, C^2 on sigma_x sigma_y sigma_z psi);
 * 1 = that term without C^2, the form of the reference's matrix operator */
int g_psi_consistent = 0;
void oracle_set_psi_consistent(int on) { g_psi_consistent = on ? 1 : 0; }

DEFINE_ORACLE(double, f64)
DEFINE_ORACLE(float, f32)
