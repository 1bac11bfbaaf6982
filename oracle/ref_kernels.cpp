/*
 * oracle/ref_kernels.cpp -- TEST INFRASTRUCTURE (builds the reference itself as a checker).
 *
 * Instantiates the reference's own step templates, included at build time from
 * the reference tree (pysit/solvers/constant_density_acoustic/time/scalar/
 * constant_density_acoustic_time_scalar_{1D,2D,3D}.h and the OpenMP variants
 * _{1D,2D,3D}_{4,6}.h), and exposes them with the oracle's C signature
 * (oracle/cda_oracle.h) under the prefix ref_.  Nothing of the reference is
 * copied here: oracle/Makefile compiles this file with -I pointing into the
 * read-only reference tree and writes the library to oracle/_ref/.
 *
 * The OpenMP variants read OMP_NUM_THREADS with getenv/atoi
 * (constant_density_acoustic_time_scalar_2D_4.h:57-58); the wrappers set it
 * when it is missing so that the reference code does not dereference NULL.
 */
#include <cstdlib>
#include "constant_density_acoustic_time_scalar_1D.h"
#include "constant_density_acoustic_time_scalar_2D.h"
#include "constant_density_acoustic_time_scalar_3D.h"
#include "constant_density_acoustic_time_scalar_1D_4.h"
#include "constant_density_acoustic_time_scalar_1D_6.h"
#include "constant_density_acoustic_time_scalar_2D_4.h"
#include "constant_density_acoustic_time_scalar_2D_6.h"
#include "constant_density_acoustic_time_scalar_3D_4.h"
#include "constant_density_acoustic_time_scalar_3D_6.h"

#define CC(p) const_cast<T*>(p)

namespace {

template <typename T, int O>
void step1(const T* km1_u, const T* k_phiz, const T* k_u, const T* C, const T* rhs,
           const T* zl, int nzl, const T* zr, int nzr, double dt, double dz, int nz,
           T* kp1_phiz, T* kp1_u, bool omp)
{
    int n = nz;
    if (omp) {
        if (O == 4)
            cda_time_scalar_1D_4<T, 4>(CC(km1_u), n, 1, CC(k_phiz), n, 1, CC(k_u), n, 1, CC(C), n, 1,
                                       CC(rhs), n, 1, CC(zl), nzl, CC(zr), nzr, dt, dz, nz,
                                       kp1_phiz, n, 1, kp1_u, n, 1);
        else
            cda_time_scalar_1D_6<T, 6>(CC(km1_u), n, 1, CC(k_phiz), n, 1, CC(k_u), n, 1, CC(C), n, 1,
                                       CC(rhs), n, 1, CC(zl), nzl, CC(zr), nzr, dt, dz, nz,
                                       kp1_phiz, n, 1, kp1_u, n, 1);
        return;
    }
    cda_time_scalar_1D<T, O>(CC(km1_u), n, 1, CC(k_phiz), n, 1, CC(k_u), n, 1, CC(C), n, 1,
                             CC(rhs), n, 1, CC(zl), nzl, CC(zr), nzr, dt, dz, nz,
                             kp1_phiz, n, 1, kp1_u, n, 1);
}

template <typename T, int O>
void step2(const T* km1_u, const T* k_phix, const T* k_phiz, const T* k_u, const T* C,
           const T* rhs, const T* xl, int nxl, const T* xr, int nxr, const T* zl, int nzl,
           const T* zr, int nzr, double dt, double dx, double dz, int nx, int nz,
           T* kp1_phix, T* kp1_phiz, T* kp1_u, bool omp)
{
    int n = nx * nz;
#define ARGS2 CC(km1_u), n, 1, CC(k_phix), n, 1, CC(k_phiz), n, 1, CC(k_u), n, 1, CC(C), n, 1, \
              CC(rhs), n, 1, CC(xl), nxl, CC(xr), nxr, CC(zl), nzl, CC(zr), nzr, dt, dx, dz, nx, nz, \
              kp1_phix, n, 1, kp1_phiz, n, 1, kp1_u, n, 1
    if (omp) {
        if (O == 4) cda_time_scalar_2D_4<T, 4>(ARGS2);
        else cda_time_scalar_2D_6<T, 6>(ARGS2);
        return;
    }
    cda_time_scalar_2D<T, O>(ARGS2);
#undef ARGS2
}

template <typename T, int O>
void step3(const T* km1_u, const T* k_phix, const T* k_phiy, const T* k_phiz, const T* k_psi,
           const T* k_u, const T* C, const T* rhs, const T* xl, int nxl, const T* xr, int nxr,
           const T* yl, int nyl, const T* yr, int nyr, const T* zl, int nzl, const T* zr, int nzr,
           double dt, double dx, double dy, double dz, int nx, int ny, int nz, T* kp1_phix,
           T* kp1_phiy, T* kp1_phiz, T* kp1_psi, T* kp1_u, bool omp)
{
    int n = nx * ny * nz;
#define ARGS3 CC(km1_u), n, 1, CC(k_phix), n, 1, CC(k_phiy), n, 1, CC(k_phiz), n, 1, CC(k_psi), n, 1, \
              CC(k_u), n, 1, CC(C), n, 1, CC(rhs), n, 1, CC(xl), nxl, CC(xr), nxr, CC(yl), nyl,        \
              CC(yr), nyr, CC(zl), nzl, CC(zr), nzr, dt, dx, dy, dz, nx, ny, nz, kp1_phix, n, 1,       \
              kp1_phiy, n, 1, kp1_phiz, n, 1, kp1_psi, n, 1, kp1_u, n, 1
    if (omp) {
        if (O == 4) cda_time_scalar_3D_4<T, 4>(ARGS3);
        else cda_time_scalar_3D_6<T, 6>(ARGS3);
        return;
    }
    cda_time_scalar_3D<T, O>(ARGS3);
#undef ARGS3
}

void ensure_omp_env() { setenv("OMP_NUM_THREADS", "1", 0); }

}  // namespace

#define DISPATCH(ORDER_VAR, CALL)          \
    switch (ORDER_VAR) {                   \
    case 2: CALL(2); break;                \
    case 4: CALL(4); break;                \
    case 6: CALL(6); break;                \
    case 8: CALL(8); break;                \
    default: return -1;                    \
    }

#define DEFINE_REF(T, SUF)                                                                        \
extern "C" int ref_cda1d_step_##SUF(int order, const T* km1_u, const T* k_phiz, const T* k_u,    \
                                    const T* C, const T* rhs, const T* zl, int nzl, const T* zr,  \
                                    int nzr, double dt, double dz, int nz, T* kp1_phiz, T* kp1_u, \
                                    int omp)                                                      \
{                                                                                                 \
    if (omp && order != 4 && order != 6) return -1;                                               \
    ensure_omp_env();                                                                             \
    DISPATCH(order, CALL1_##SUF)                                                                  \
    return 0;                                                                                     \
}                                                                                                 \
extern "C" int ref_cda2d_step_##SUF(int order, const T* km1_u, const T* k_phix, const T* k_phiz, \
                                    const T* k_u, const T* C, const T* rhs, const T* xl, int nxl, \
                                    const T* xr, int nxr, const T* zl, int nzl, const T* zr,      \
                                    int nzr, double dt, double dx, double dz, int nx, int nz,     \
                                    T* kp1_phix, T* kp1_phiz, T* kp1_u, int omp)                  \
{                                                                                                 \
    if (omp && order != 4 && order != 6) return -1;                                               \
    ensure_omp_env();                                                                             \
    DISPATCH(order, CALL2_##SUF)                                                                  \
    return 0;                                                                                     \
}                                                                                                 \
extern "C" int ref_cda3d_step_##SUF(int order, const T* km1_u, const T* k_phix, const T* k_phiy, \
                                    const T* k_phiz, const T* k_psi, const T* k_u, const T* C,    \
                                    const T* rhs, const T* xl, int nxl, const T* xr, int nxr,     \
                                    const T* yl, int nyl, const T* yr, int nyr, const T* zl,      \
                                    int nzl, const T* zr, int nzr, double dt, double dx,          \
                                    double dy, double dz, int nx, int ny, int nz, T* kp1_phix,    \
                                    T* kp1_phiy, T* kp1_phiz, T* kp1_psi, T* kp1_u, int omp)      \
{                                                                                                 \
    if (omp && order != 4 && order != 6) return -1;                                               \
    ensure_omp_env();                                                                             \
    DISPATCH(order, CALL3_##SUF)                                                                  \
    return 0;                                                                                     \
}

#define CALL1_IMPL(T, O) step1<T, O>(km1_u, k_phiz, k_u, C, rhs, zl, nzl, zr, nzr, dt, dz, nz, \
                                     kp1_phiz, kp1_u, omp != 0)
#define CALL2_IMPL(T, O) step2<T, O>(km1_u, k_phix, k_phiz, k_u, C, rhs, xl, nxl, xr, nxr, zl, nzl, \
                                     zr, nzr, dt, dx, dz, nx, nz, kp1_phix, kp1_phiz, kp1_u, omp != 0)
#define CALL3_IMPL(T, O) step3<T, O>(km1_u, k_phix, k_phiy, k_phiz, k_psi, k_u, C, rhs, xl, nxl, xr, \
                                     nxr, yl, nyl, yr, nyr, zl, nzl, zr, nzr, dt, dx, dy, dz, nx, ny, \
                                     nz, kp1_phix, kp1_phiy, kp1_phiz, kp1_psi, kp1_u, omp != 0)
#define CALL1_f64(O) CALL1_IMPL(double, O)
#define CALL2_f64(O) CALL2_IMPL(double, O)
#define CALL3_f64(O) CALL3_IMPL(double, O)
#define CALL1_f32(O) CALL1_IMPL(float, O)
#define CALL2_f32(O) CALL2_IMPL(float, O)
#define CALL3_f32(O) CALL3_IMPL(float, O)

DEFINE_REF(double, f64)
DEFINE_REF(float, f32)
