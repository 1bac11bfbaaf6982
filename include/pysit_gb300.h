/*
 * pysit_gb300.h -- C ABI of libpysit_gb300.so, the GB300 (sm_103a) engine for
 * PySIT's time-domain constant-density acoustic solver with PML and its
 * adjoint-state FWI gradient.
 *
 * Conventions for every entry point:
 *   - plain pointers and sizes only; array pointers marked "dev" are device
 *     pointers (e.g. torch.Tensor.data_ptr()), "host" are host pointers;
 *   - all wavefield arrays are C-contiguous with z the fastest axis, exactly the
 *     reference layout (idx = i*nz + k in 2D, (i*ny + j)*nz + k in 3D);
 *   - dtype is PYSIT_F32 or PYSIT_F64 and applies to every array argument of a
 *     kernel call (the reference's SWIG typemaps also demand one dtype,
 *     constant_density_acoustic_time_scalar.i:16-42);
 *   - `stream` is a cudaStream_t (0 = legacy default stream);
 *   - the return value is PYSIT_OK (0) or a negative PYSIT_E* code, and
 *     pysit_cuda_last_error() returns a message for the calling thread;
 *   - no C++ exception crosses the ABI; the library holds no host threads.
 */
#ifndef PYSIT_GB300_H
#define PYSIT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PYSIT_OK          0
#define PYSIT_EINVAL     -1  /* bad argument (shape, order, dtype, alignment, size) */
#define PYSIT_ECUDA      -2  /* CUDA runtime error */
#define PYSIT_ENONFINITE -3  /* NaN/Inf found in a wavefield (unstable CFL) */
#define PYSIT_ESTATE     -4  /* call out of order (e.g. no workspace bound) */
#define PYSIT_EHOST      -5  /* host-side failure inside the library (a host allocation) */
#define PYSIT_ETIMEOUT   -6  /* a bounded device wait expired: the results of the run are invalid
                                (reported by the host layer from bit 0 of pysit_plan_status) */

#define PYSIT_F32 0
#define PYSIT_F64 1

/* Message describing the last error on the calling thread ("" if none). */
const char* pysit_cuda_last_error(void);
/* ABI version of this header (major*1000 + minor); pysit_cuda_version() returns the
 * library's, so a client can check that the two match. */
#define PYSIT_ABI_VERSION 1001
int pysit_cuda_version(void);

/* ------------------------------------------------------------------------
 * Per-step kernels: one leapfrog step over the whole padded grid.
 * Same argument order and meaning as the reference templates, minus SWIG's
 * (rows, cols) pairs:
 *   pysit_cda_step_1d  <- cda_time_scalar_1D  (pysit/solvers/constant_density_acoustic/
 *                         time/scalar/constant_density_acoustic_time_scalar_1D.h:44-56)
 *   pysit_cda_step_2d  <- cda_time_scalar_2D  (..._2D.h:43-61)
 *   pysit_cda_step_3d  <- cda_time_scalar_3D  (..._3D.h:46-72)
 * bound through SWIG at constant_density_acoustic_time_scalar.i:57-84 and
 * called from ConstantDensityAcousticTimeScalar_{1,2,3}D_cpp.time_step
 * (..._1D.py:138-158, _2D.py:166-190, _3D.py:194-227).
 * The sigma arrays are the per-side PML profiles (length n_*l / n_*r, may be 0
 * for a Dirichlet side).  Outputs must not alias inputs.
 * ------------------------------------------------------------------------ */
int pysit_cda_step_1d(int dtype, int order,
                      const void* km1_u, const void* k_phiz, const void* k_u,
                      const void* C, const void* rhs,
                      const void* zlpml, int n_zlpml, const void* zrpml, int n_zrpml,
                      double dt, double dz, int nz,
                      void* kp1_phiz, void* kp1_u, void* stream);

int pysit_cda_step_2d(int dtype, int order,
                      const void* km1_u, const void* k_phix, const void* k_phiz,
                      const void* k_u, const void* C, const void* rhs,
                      const void* xlpml, int n_xlpml, const void* xrpml, int n_xrpml,
                      const void* zlpml, int n_zlpml, const void* zrpml, int n_zrpml,
                      double dt, double dx, double dz, int nx, int nz,
                      void* kp1_phix, void* kp1_phiz, void* kp1_u, void* stream);

int pysit_cda_step_3d(int dtype, int order,
                      const void* km1_u, const void* k_phix, const void* k_phiy,
                      const void* k_phiz, const void* k_psi, const void* k_u,
                      const void* C, const void* rhs,
                      const void* xlpml, int n_xlpml, const void* xrpml, int n_xrpml,
                      const void* ylpml, int n_ylpml, const void* yrpml, int n_yrpml,
                      const void* zlpml, int n_zlpml, const void* zrpml, int n_zrpml,
                      double dt, double dx, double dy, double dz, int nx, int ny, int nz,
                      void* kp1_phix, void* kp1_phiy, void* kp1_phiz, void* kp1_psi,
                      void* kp1_u, void* stream);

/* Imaging-condition operand of one step (the reference's dWaveOp,
 * ConstantDensityAcousticBase._compute_dWaveOp_time,
 * pysit/solvers/constant_density_acoustic/constant_density_acoustic_base.py:24-40):
 *   out = (u_kp1 - 2 u_k + u_km1)/dt^2 + S1 (u_kp1 - u_km1)/(2 dt) + S2 u_k [+ S3 psi_k]
 * with S1 = sum of the mesh sigma maps, S2 = sum of their pairwise products and
 * S3 = their triple product (3D).  sig_x/sig_y/sig_z are the full-length
 * per-axis sigma maps (length nx/ny/nz; pass NULL for an absent axis) of the
 * mesh (StructuredPML.eval_on_mesh, pysit/core/mesh.py:784-831).  psi_k may be
 * NULL in 1D/2D.  All arrays have nx*ny*nz entries. */
int pysit_cda_dwaveop(int dtype, int dim, const void* km1_u, const void* k_u,
                      const void* kp1_u, const void* psi_k,
                      const void* sig_x, const void* sig_y, const void* sig_z,
                      int nx, int ny, int nz, double dt, void* out, void* stream);

/* ------------------------------------------------------------------------
 * Batched, checkpointed forward / gradient pipeline ("plan").
 * Replaces the per-shot Python loops of TemporalModeling.forward_model
 * (pysit/modeling/temporal_modeling.py:60-169), adjoint_model (:228-387),
 * migrate_shot (:171-214) and TemporalLeastSquares._gradient_helper /
 * compute_gradient / evaluate (pysit/objective_functions/
 * temporal_least_squares.py:27-198) by one call per gradient for a whole
 * batch of shots.  The library allocates no device memory: the caller asks
 * for the workspace size and binds a buffer it owns.
 * ------------------------------------------------------------------------ */
typedef struct pysit_plan pysit_plan;

typedef struct {
    int dim;               /* 1, 2 or 3 */
    int order;             /* spatial accuracy order 2, 4, 6, 8 */
    int dtype;             /* PYSIT_F32 or PYSIT_F64 */
    int n[3];              /* padded grid sizes (x, y, z); unused axes = 1, 1D uses n[2] */
    double delta[3];       /* grid spacings (x, y, z) */
    int pad_lo[3];         /* padding cells on the low / high side of each axis, used */
    int pad_hi[3];         /*   to fold the PML strips of the gradient (add_padding)   */
    double dt;             /* time step */
    int nsteps;            /* number of time steps */
    int imaging_period;    /* image every p-th step (TemporalLeastSquares.imaging_period) */
    int checkpoint_every;  /* segment length S of the checkpoint / recompute schedule */
    int shots_per_launch;  /* shots advanced together by one kernel launch (<= nshots) */
    int nshots;            /* shots in the batch */
    /* PML profiles in the step kernels' convention (host, FP64): per axis the left
     * and right arrays that time_step passes to the reference kernel. */
    const double* sig_l[3]; int nsig_l[3];
    const double* sig_r[3]; int nsig_r[3];
    /* Full-length per-axis sigma maps of the mesh (host, FP64, length n[a]), the
     * convention of the imaging operand dWaveOp; NULL for an axis without PML. */
    const double* sigmap[3];
    /* Sources: per shot a list of taps (padded flat cell, source point, weight);
     * rhs_k(cell) = sum_taps weight * src_amp[shot][k][point]. */
    int nsrc;                      /* source points per shot */
    const int64_t* src_tap_ptr;    /* host [nshots+1] offsets into the tap arrays */
    const int64_t* src_tap_cell;   /* host */
    const int32_t* src_tap_point;  /* host */
    const double* src_tap_w;       /* host */
    const double* src_amp;         /* host [nshots][nsteps][nsrc] */
    /* Receivers: per shot a list of taps (padded flat cell, receiver, sampling
     * weight, injection weight).  trace[k][r] = sum w_sample * u_k(cell);
     * adjoint rhs_k(cell) = sum w_inject * resid[k][r]. */
    int nrec;                      /* receivers per shot */
    const int64_t* rec_tap_ptr;    /* host [nshots+1] */
    const int64_t* rec_tap_cell;   /* host */
    const int32_t* rec_tap_point;  /* host */
    const double* rec_tap_wsample; /* host */
    const double* rec_tap_winject; /* host */
    int use_graph;                 /* capture the time loops in CUDA graphs (1) or launch eagerly (0) */
    int psi_consistent;            /* 3D PML: 0 = the reference's step, which multiplies sigma_x sigma_y
                                      sigma_z psi by C^2 (_3D.h:219; unstable at realistic PML amplitudes);
                                      1 = that term without C^2, as in the reference's matrix operator */
    int tile_x;                    /* 2D/3D task length along x in rows; 0 = the default (32 in 2D, 64 in 3D);
                                      pysit_plan_autotune chooses it by timing */
    const int32_t* shot_nsteps;    /* host [nshots] or NULL: the record length of each shot in steps
                                      (1..nsteps); the residual of a shot is zero from its length on, so
                                      its misfit and gradient are those of a run of that many steps */
    int store_dwaveop;             /* 0 = checkpointed gradient (forward, recompute, adjoint sweeps);
                                      1 = the forward sweep keeps dWaveOp of every imaged step in the
                                      workspace and the adjoint reads it back (no checkpoints, no
                                      recompute; about ceil(nsteps / imaging_period) fields per shot of
                                      a launch).  Same results; needs imaging_period 1 for the Hessian */
    int forward_only;              /* 1 = only forward modelling (pysit_plan_forward): no adjoint,
                                      checkpoint or imaging buffers; other runs return PYSIT_EINVAL */
    double shell_share[3];         /* 2D, per step mode (forward, recompute, adjoint): share of the GPU's
                                      resident blocks given to the PML-shell kernel, in (0, 1), so that it
                                      runs beside the interior kernel from the start; 0 = each kernel sized
                                      for the whole GPU (the default: inside the CUDA graph of a sweep
                                      that balanced the two kernels best in measurements) */
    int lanes;                     /* >= 2: the shots are split into that many contiguous ranges whose
                                      launch sequences run side by side on their own streams (each lane
                                      with its own buffers: lanes x the workspace of its shots); 0 or 1 =
                                      one sequence.  Results are the lanes' sums, in lane order */
    uint32_t wait_polls;           /* 0 = a step kernel's wait for a bulk copy into shared memory makes
                                      up to 2^22 blocking tries (far beyond any copy's latency); n > 0 =
                                      at most n non-blocking tests before the wait counts as expired.
                                      An expired wait sets bit 0 of the status word; the warp waits
                                      (with the full limit) for the copies it has in flight and runs
                                      no further task, so the run's results are invalid */
    int wait_fault;                /* test aid, 0 in normal use.  1 = every task of the 2D step kernels
                                      first waits (bounded: wait_polls non-blocking tests, 64 when
                                      wait_polls is 0) on an mbarrier on which nothing ever arrives;
                                      the wait runs out and takes the expiry path above with the
                                      task's bulk copies in flight.  Lets a test check that path and
                                      the status report without any GPU fault */
    int tile_z;                    /* 2D/3D: z extent of an interior task at most, in cells (a multiple of
                                      4, >= 16); 0 = the kernel's full width (32 lanes x the lane vector:
                                      128 cells in FP32, 64 in FP64).  Narrower tasks leave lanes idle but
                                      make more tasks; pysit_plan_autotune_tiles chooses it by timing */
} pysit_plan_desc;

int pysit_plan_create(const pysit_plan_desc* desc, pysit_plan** out);
int pysit_plan_destroy(pysit_plan* plan);
/* Device workspace the plan needs, in bytes (256-byte aligned buffer). */
int pysit_plan_workspace_bytes(const pysit_plan* plan, uint64_t* bytes);
/* Binds (and initialises) the caller-owned workspace; uploads acquisition data. */
int pysit_plan_bind_workspace(pysit_plan* plan, void* workspace_dev, uint64_t bytes,
                              void* stream);
/* Sets the padded wave speed C (dev, FP64, n[0]*n[1]*n[2] cells, z fastest). */
int pysit_plan_set_model(pysit_plan* plan, const double* C_padded_dev, void* stream);
/* Forward modelling of every shot: traces_dev (plan dtype) receives
 * [nshots][nsteps][nrec] samples u_k at the receivers, k = 0..nsteps-1
 * (TemporalModeling.forward_model 'simdata', temporal_modeling.py:123-125). */
int pysit_plan_forward(pysit_plan* plan, void* traces_dev, void* stream);
/* Misfit and gradient of the batch.  dobs_dev (plan dtype, [nshots][nsteps][nrec])
 * holds the observed data already resampled to this plan's time axis
 * (ReceiverSet.interpolate_data).  Outputs (dev, FP64):
 *   grad_dev    [prod(n - pad_lo - pad_hi)] unpadded gradient with respect to
 *               m = C^-2, PML strips folded onto the boundary (= the reference's
 *               compute_gradient result);
 *   rnorm2_dev  [1] sum over shots of ||dobs - dsim||^2 (objective = 0.5*dt*rnorm2);
 *   traces_dev  optional (may be NULL) simulated traces as in pysit_plan_forward. */
int pysit_plan_gradient(pysit_plan* plan, const void* dobs_dev, double* grad_dev,
                        double* rnorm2_dev, void* traces_dev, void* stream);
/* Migration F* of a data-space operand (TemporalModeling.migrate_shot,
 * temporal_modeling.py:171-214, for every shot of the batch, summed):
 * operand_dev (plan dtype, [nshots][nsteps][nrec]) drives the adjoint directly;
 * image_dev (FP64, unpadded) = sum over shots of -dt*p*sum_k q_k*dWaveOp_k with
 * the strips folded; norm2_dev [1] = ||operand||^2. */
int pysit_plan_migrate(pysit_plan* plan, const void* operand_dev, double* image_dev,
                       double* norm2_dev, void* stream);
/* Misfit only (TemporalLeastSquares.evaluate without the 0.5*dt factor). */
int pysit_plan_misfit(pysit_plan* plan, const void* dobs_dev, double* rnorm2_dev,
                      void* traces_dev, void* stream);
/* Linearised (Born) modelling of every shot about the plan's model:
 * TemporalModeling.linear_forward_model(shot, m0, m1, ['simdata'])
 * (pysit/modeling/temporal_modeling.py:389-546).  m1_dev: model perturbation
 * (m = C^-2 space, FP64, device) on the unpadded grid in PySIT's flat order; it is
 * edge-padded on the device as the reference does (:434).  traces_dev: device
 * [nshots][nsteps][nrec] of the plan's dtype, u1 sampled before each step. */
int pysit_plan_born(pysit_plan* plan, const double* m1_dev, void* traces_dev, void* stream);
/* Gauss-Newton Hessian application summed over the shots:
 * TemporalLeastSquares.apply_hessian(shots, m0, m1, 'approximate')
 * (pysit/objective_functions/temporal_least_squares.py:200-249), i.e. the sum over
 * shots of migrate_shot(F_s m1) imaging every step: out_dev (FP64, unpadded) =
 * sum_s -dt sum_k q_k dWaveOp0_k with the strips folded, q driven by the Born
 * traces d1.  d1norm2_dev [1] (may be NULL) = ||d1||^2.  'levenberg' adds mu*m1,
 * which the caller does.  Each shot group runs one Born sweep (saving the background
 * checkpoints) and one checkpointed migration. */
int pysit_plan_hessian(pysit_plan* plan, const double* m1_dev, double* out_dev, double* d1norm2_dev,
                       void* stream);
/* Reads and clears the plan's device status word (synchronises `stream`):
 * bit 0 (1) = a bounded wait for a bulk copy expired (results invalid),
 * bit 1 (2) = a non-finite wavefield value appeared (unstable time step). */
int pysit_plan_status(pysit_plan* plan, int* flags, void* stream);
/* ------------------------------------------------------------------------
 * Allocation-free per-shot misfit.  No counterpart in the reference: it exists
 * for callers that cannot allocate device memory (applications that reserve all
 * device memory in their own pool up front, C/Fortran codes that link no
 * allocator).  Inputs dobs, dsim and output resid (may be NULL) are
 * [nshots][per_shot] arrays of `dtype`; resid may be the same array as dobs or
 * dsim (an in-place residual).  rnorm2 (FP64, dev) receives
 * sum_i (dobs - dsim)^2 per shot over every one of the per_shot samples: unlike
 * the plan's misfit, which stops each shot at its own record length, nothing here
 * knows record lengths, so a caller with uneven records zeroes the samples past
 * each shot's end in both arrays first.  No allocation: the reduction scratch is a
 * fixed 128 KiB device array (nshots <= 256, larger counts are rejected).  Its
 * address differs per CUDA context; the first call made in each context looks it
 * up (make that call before any stream capture), later calls in the same context
 * reuse it, and a new context (another one the host made current, or the one
 * rebuilt after cudaDeviceReset) gets its own lookup.  All calls share the array:
 * calls that overlap on the GPU race.
 * ------------------------------------------------------------------------ */
int pysit_misfit_per_shot_noalloc(int dtype, const void* dobs, const void* dsim, int nshots,
                                  int64_t per_shot, void* resid, double* rnorm2, void* stream);
/* Number of kernel launches the last forward/gradient/misfit call issued. */
int pysit_plan_last_launch_count(const pysit_plan* plan, int64_t* launches);

/* Benchmarking aid, no counterpart in the reference: enqueues `nsteps` launches
 * of one step kernel (mode 0 forward, 1 forward recompute writing dWaveOp,
 * 2 adjoint with imaging) of the first shot group on the plan's own buffers, so
 * that a caller can time one kernel with events on `stream`.  The wavefield
 * buffers keep evolving from whatever the previous run left; nothing is
 * returned and the next forward/gradient call starts from scratch. */
int pysit_plan_step_loop(pysit_plan* plan, int mode, int nsteps, void* stream);

/* Autotuner, no counterpart in the reference (its kernels have no tiles): times
 * `nsteps` forward and `nsteps` adjoint steps (as pysit_plan_step_loop does) for
 * each of the `ncand` task lengths along x in `candidates` (8..4096 rows), twice (the
 * second pass in reverse order), keeps the fastest, writes it to *chosen and the
 * better of each candidate's two times in milliseconds to ms[ncand] (may be NULL).  Needs a bound workspace and a model; 2D and 3D plans.
 * It drops the plan's captured graphs (they hold the old task tables); the
 * wavefield buffers are left in an arbitrary state, as after step_loop. */
int pysit_plan_autotune(pysit_plan* plan, const int* candidates, int ncand, int nsteps, int* chosen,
                        double* ms, void* stream);
/* The autotuner over both tile dimensions, no counterpart in the reference: as
 * pysit_plan_autotune for every pair of a task length along x in cand_x[ncx] (8..4096) and a
 * z extent of the interior tasks in cand_z[ncz] (0 = the full width, else >= 16 cells);
 * writes the fastest pair to *chosen_x / *chosen_z and the better of each pair's two times
 * to ms[ix * ncz + iz] (may be NULL). */
int pysit_plan_autotune_tiles(pysit_plan* plan, const int* cand_x, int ncx, const int* cand_z, int ncz,
                              int nsteps, int* chosen_x, int* chosen_z, double* ms, void* stream);
/* The plan's current task length along x and z extent of its interior tasks (0: full width). */
int pysit_plan_get_tiles(const pysit_plan* plan, int* tile_x, int* tile_z);
/* A host copy of the plan's current task table, no counterpart in the reference (diagnostics
 * and tests; needs no device).  2D: rows of 5 ints (x0, x1, zs, ze, kind: 0 interior, 1 PML
 * shell), the warp tasks of one shot; 3D: rows of 6 ints (x0, x1, y0, y1, zs, ze), one block of
 * 8 warps each, a warp taking 32 / ceil((ze - zs) / V) y-rows (V = 4 FP32, 2 FP64 cells a lane);
 * 1D: none.  The interior tasks come first, *n_interior of them.  *n_ints receives the table's
 * size in ints; at most cap ints are written to out (which may be NULL). */
int pysit_plan_task_table(const pysit_plan* plan, int32_t* out, uint64_t cap, uint64_t* n_ints,
                          int32_t* n_interior);
/* The plan's current tuning: task length along x and the three 2D shell block shares
 * (pysit_plan_desc.shell_share).  Either output may be NULL. */
int pysit_plan_get_tuning(const pysit_plan* plan, int* tile_x, double* shell_share);

/* ------------------------------------------------------------------------
 * Plan groups, no counterpart in the reference (it runs shots one after the
 * other): several plans (different grids, orders or record lengths) whose
 * gradients run concurrently, captured together in one CUDA graph - each plan
 * on a stream of its own forked from the caller's stream and joined back.
 * The plans stay owned by the caller and must outlive the group.
 * ------------------------------------------------------------------------ */
typedef struct pysit_group pysit_group;
int pysit_group_create(pysit_plan* const* plans, int nplans, pysit_group** out);
int pysit_group_destroy(pysit_group* group);
/* Misfit and gradient of every plan: dobs[i], grad[i], rnorm2[i] as for
 * pysit_plan_gradient of plan i.  The graph is cached per set of pointers. */
int pysit_group_gradient(pysit_group* group, const void* const* dobs, double* const* grad,
                         double* const* rnorm2, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PYSIT_GB300_H */
