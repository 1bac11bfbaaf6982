/*
 * oracle/cda_oracle.h -- TEST INFRASTRUCTURE (checker only, never product code).
 * Declarations of the CPU restatement in cda_oracle.c.  Argument order follows
 * the reference templates cda_time_scalar_{1D,2D,3D}
 * (pysit/solvers/constant_density_acoustic/time/scalar/
 *  constant_density_acoustic_time_scalar_{1D.h:45-56,2D.h:44-61,3D.h:47-72})
 * without SWIG's per-array (rows, cols) pairs.  Return 0 on success, -1 on a
 * bad order or a grid smaller than 3 cells along an axis.
 */
#ifndef PYSIT_GB300_CDA_ORACLE_H
#define PYSIT_GB300_CDA_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_DECL(T, SUF)                                                            \
int oracle_cda1d_step_##SUF(int order, const T* km1_u, const T* k_phiz, const T* k_u,  \
                            const T* C, const T* rhs, const T* zl, int nzl,            \
                            const T* zr, int nzr, double dt, double dz, int nz,        \
                            T* kp1_phiz, T* kp1_u);                                    \
int oracle_cda2d_step_##SUF(int order, const T* km1_u, const T* k_phix,                \
                            const T* k_phiz, const T* k_u, const T* C, const T* rhs,   \
                            const T* xl, int nxl, const T* xr, int nxr,                \
                            const T* zl, int nzl, const T* zr, int nzr,                \
                            double dt, double dx, double dz, int nx, int nz,           \
                            T* kp1_phix, T* kp1_phiz, T* kp1_u);                       \
int oracle_cda3d_step_##SUF(int order, const T* km1_u, const T* k_phix,                \
                            const T* k_phiy, const T* k_phiz, const T* k_psi,          \
                            const T* k_u, const T* C, const T* rhs,                    \
                            const T* xl, int nxl, const T* xr, int nxr,                \
                            const T* yl, int nyl, const T* yr, int nyr,                \
                            const T* zl, int nzl, const T* zr, int nzr,                \
                            double dt, double dx, double dy, double dz,                \
                            int nx, int ny, int nz,                                    \
                            T* kp1_phix, T* kp1_phiy, T* kp1_phiz, T* kp1_psi,         \
                            T* kp1_u);

ORACLE_DECL(double, f64)
ORACLE_DECL(float, f32)

/* 3D psi term: 0 (default) = C^2 multiplies sigma_x sigma_y sigma_z psi, as the
 * reference's step does (_3D.h:219); 1 = it does not (the matrix operator's form). */
void oracle_set_psi_consistent(int on);

#ifdef __cplusplus
}
#endif
#endif
