// Batched forward / gradient pipeline ("plan") behind pysit_plan_* of the C ABI.
//
// Schedule of one gradient for a group of shots (all shots of a group advance
// together in every launch):
//   forward sweep   k = 0..n-1: record traces of u_k, step to u_{k+1}; every S
//                   steps save the step inputs (u_{k-1}, u_k, PML state) as a
//                   checkpoint            (TemporalModeling.forward_model,
//                   pysit/modeling/temporal_modeling.py:115-161, without the
//                   per-step dWaveOp list of :146-148)
//   residual        r = dobs - dsim and ||r||^2 in FP64
//                   (TemporalLeastSquares._residual / evaluate,
//                   pysit/objective_functions/temporal_least_squares.py:27-82)
//   backward sweep  segments from last to first: restore the checkpoint,
//                   recompute the segment writing dWaveOp_k into a replay
//                   buffer, then run the adjoint steps k = k1..k0 with
//                   ic += q_k * dWaveOp_k  (adjoint_model, :312-365)
//   reduction       grad += dt * p * sum_shots ic_shot (FP64)   (:367-369 and
//                   compute_gradient's grad -= g, temporal_least_squares.py:167)
//   fold            PML strips summed onto the boundary rows/columns
//                   (ModelPerturbationBase.add_padding,
//                   pysit/solvers/model_parameter.py:537-594).
// The whole schedule of a call is captured once in a CUDA graph and replayed.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <set>
#include <tuple>
#include <vector>

#include "wave.cuh"

#ifndef PGB_REC_BLOCKS_PER_SM
#define PGB_REC_BLOCKS_PER_SM 1  // 2D recorder blocks per SM (leading blocks of the interior kernel)
#endif

namespace pgb {
namespace {

// Runs `enqueue` while `cap` captures a graph.  A C++ exception thrown meanwhile ends the
// capture (dropping the partial graph) before it propagates, so the stream stays usable.
template <typename F>
void capture_into(cudaStream_t cap, F&& enqueue) {
    try {
        enqueue();
    } catch (...) {
        cudaGraph_t partial = nullptr;
        cudaStreamEndCapture(cap, &partial);
        if (partial) cudaGraphDestroy(partial);
        throw;
    }
}

// ---------------------------------------------------------------------------
// small kernels
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long ioff(int i, int j, int k, int hx, int hy, int rows_y,
                                          int ldz) {
    return ((long long)(i + hx) * rows_y + (j + hy)) * ldz + kOZ + k;
}

template <typename T>
__global__ void set_c2_kernel(const double* __restrict__ C, int nx, int ny, int nz, int hx,
                              int hy, int rows_y, int ldz, T* __restrict__ c2) {
    long long n = (long long)nx * ny * nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        int k = (int)(c % nz);
        long long r = c / nz;
        int j = (int)(r % ny), i = (int)(r / ny);
        T v = T(C[c]);
        c2[ioff(i, j, k, hx, hy, rows_y, ldz)] = v * v;
    }
}

// Injection term of one 2D step added after the stencil kernels:
//     u_{k+1} += fac C^2 rhs,   fac = dt^2, or 2 dt^2 / (2 + dt (sx + sz)) where a sigma is nonzero,
// the factor the reference's update applies to C^2 (rhs + ...) (_2D.h:157-179); the update is
// linear in rhs, so adding it afterwards equals injecting it inside the stencil.  One thread per
// (shot, cell of the shot's injection box); cells of the outer ring are left alone, as the
// reference skips them.  Used for wide operators (the adjoint source at every receiver), whose
// per-cell tap walk would stall the stencil's row loop.
template <typename T>
__global__ void inject_scatter2d_kernel(const WaveParams<T> p, int cells_max) {
    const long long n = (long long)p.nshot * cells_max;
    for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < n;
         id += (long long)gridDim.x * blockDim.x) {
        const int shot = (int)(id / cells_max), c = (int)(id - (long long)shot * cells_max);
        const int* bx = p.inj.box + shot * 6;
        const int bzw = bx[5] - bx[4];
        if (bzw <= 0 || c >= (bx[1] - bx[0]) * bzw) continue;
        const int x = bx[0] + c / bzw, z = bx[4] + c % bzw;
        if (x <= 0 || x >= p.nx - 1 || z <= 0 || z >= p.nz - 1) continue;
        const T rhs = inject_rhs(p.inj, bx, shot, x, z);
        const T sx = p.sgx[x], sz = p.sgz[z];
        const T fac = (sx != T(0) || sz != T(0)) ? T(2) * p.dt2 / (T(2) + p.dt * (sx + sz)) : p.dt2;
        const long long o = foff2(p, x, z);
        p.u_prev[(long long)shot * p.fstride + o] += fac * p.c2[o] * rhs;
    }
}

// The same for a 3D step: fac = 2 dt^2 / (2 + dt (sx + sy + sz)) where a sigma is
// nonzero (_3D.h:220-226).
template <typename T>
__global__ void inject_scatter3d_kernel(const WaveParams<T> p, int cells_max) {
    const long long n = (long long)p.nshot * cells_max;
    for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < n;
         id += (long long)gridDim.x * blockDim.x) {
        const int shot = (int)(id / cells_max), c = (int)(id - (long long)shot * cells_max);
        const int* bx = p.inj.box + shot * 6;
        const int byw = bx[3] - bx[2], bzw = bx[5] - bx[4];
        if (byw <= 0 || bzw <= 0 || c >= (bx[1] - bx[0]) * byw * bzw) continue;
        const int x = bx[0] + c / (byw * bzw), r = c % (byw * bzw);
        const int y = bx[2] + r / bzw, z = bx[4] + r % bzw;
        if (x <= 0 || x >= p.nx - 1 || y <= 0 || y >= p.ny - 1 || z <= 0 || z >= p.nz - 1) continue;
        // the tap sum of the cell, as inject_rhs does in 2D
        const long long cell = ((long long)(x - bx[0]) * byw + (y - bx[2])) * bzw + (z - bx[4]);
        const int* rp = p.inj.rowptr + p.inj.rpbase[shot];
        const T* amp = p.inj.amp + shot * p.inj.amp_sstride;
        T rhs = T(0);
        for (int e = rp[cell]; e < rp[cell + 1]; ++e) rhs += p.inj.w[e] * amp[p.inj.pt[e]];
        const T sx = p.sgx[x], sy = p.sgy[y], sz = p.sgz[z];
        const T fac = (sx != T(0) || sy != T(0) || sz != T(0)) ? T(2) * p.dt2 / (T(2) + p.dt * (sx + sy + sz))
                                                               : p.dt2;
        const long long o = ((long long)(x + p.hx) * p.rows_y + (y + p.hy)) * p.ldz + kOZ + z;
        p.u_prev[(long long)shot * p.fstride + o] += fac * p.c2[o] * rhs;
    }
}

// Born source of one step added after the stencil kernels of the scattered field u1:
//     u1_{k+1} += fac C^2 rhs1,   rhs1 = -m1 dWaveOp0_k
// (TemporalModeling.linear_forward_model, pysit/modeling/temporal_modeling.py:520-525; the
// step is linear in rhs, fac as in inject_scatter2d/3d_kernel).  One block per row
// (shot, x, y) of the padded grid, threads along z; cells of the outer ring are skipped as
// the reference's step skips them.  m1 and C^2 are shared by the shots; dw holds dWaveOp0_k
// of every shot of the launch.
template <typename T>
__global__ void __launch_bounds__(128) born_source_kernel(const WaveParams<T> p, int dim, const T* __restrict__ m1,
                                                          const T* __restrict__ dw) {
    const long long rows = (long long)p.nshot * p.nx * p.ny;
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
        const int shot = (int)(r / ((long long)p.nx * p.ny));
        const int xy = (int)(r - (long long)shot * p.nx * p.ny);
        const int x = xy / p.ny, y = xy - x * p.ny;
        if (dim >= 2 && (x == 0 || x == p.nx - 1)) continue;
        if (dim == 3 && (y == 0 || y == p.ny - 1)) continue;
        const T sxy = p.sgx[x] + p.sgy[y];
        const long long row = ((long long)(x + p.hx) * p.rows_y + (y + p.hy)) * p.ldz + kOZ;
        const long long sh = (long long)shot * p.fstride;
        for (int z = 1 + threadIdx.x; z < p.nz - 1; z += blockDim.x) {
            const T s = sxy + p.sgz[z];
            const bool pml = p.sgx[x] != T(0) || p.sgy[y] != T(0) || p.sgz[z] != T(0);
            const T fac = pml ? T(2) * p.dt2 / (T(2) + p.dt * s) : p.dt2;
            const long long o = row + z;
            p.u_prev[sh + o] -= fac * __ldg(p.c2 + o) * (__ldg(m1 + o) * __ldcs(dw + sh + o));
        }
    }
}

// m1 of the unpadded grid (FP64, PySIT's flat order) -> the padded internal layout with
// numpy.pad(mode='edge') semantics: every padding cell takes the value of the nearest
// physical cell (m1.with_padding(padding_mode='edge'), temporal_modeling.py:434).
template <typename T>
__global__ void edge_pad_kernel(const double* __restrict__ m, int nx, int ny, int nz, int lx, int ly, int lz,
                                int px, int py, int pz, int hx, int hy, int rows_y, int ldz, T* __restrict__ out) {
    const long long n = (long long)nx * ny * nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(c % nz);
        const long long r = c / nz;
        const int j = (int)(r % ny), i = (int)(r / ny);
        const int ii = min(max(i - lx, 0), px - 1), jj = min(max(j - ly, 0), py - 1), kk = min(max(k - lz, 0), pz - 1);
        out[ioff(i, j, k, hx, hy, rows_y, ldz)] = T(m[((long long)ii * py + jj) * pz + kk]);
    }
}

// trace recorder as a kernel of its own (runs beside the stencil kernels: it only reads u_k)
template <typename T>
__global__ void record_kernel(const WaveParams<T> p) {
    record_block(p, blockIdx.x);
}

constexpr int kRedBlocks = 1024;
constexpr int kRedThreads = 256;

// resid = dobs - dsim (in place over the trace buffer); per-block FP64 partial
// sums of resid^2 in a fixed order (deterministic).  operand = 1: resid = dobs (a
// migration operand); dobs = NULL: the operand is already in the trace buffer.
template <typename T>
__global__ void __launch_bounds__(kRedThreads) residual_kernel(const T* __restrict__ dobs,
                                                               T* __restrict__ tr, long long n,
                                                               double* __restrict__ partial,
                                                               int operand, const int* __restrict__ shot_steps,
                                                               int nsteps, int nrec) {
    double acc = 0.0;
    const long long per_shot = (long long)nsteps * nrec;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        T r = !dobs ? tr[c] : operand ? dobs[c] : dobs[c] - tr[c];
        // a shot's record ends at its own length: no residual after it
        if (shot_steps) {
            const long long sh = c / per_shot;
            if ((c - sh * per_shot) / nrec >= shot_steps[sh]) r = T(0);
        }
        tr[c] = r;
        acc += (double)r * (double)r;
    }
    __shared__ double s[kRedThreads];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kRedThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

// out[0] (+)= sum of partial[0..n) in a fixed order, one block.
__global__ void __launch_bounds__(kRedThreads) sum_partials_kernel(const double* __restrict__ partial,
                                                                   int n, double* __restrict__ out,
                                                                   int accumulate) {
    __shared__ double s[kRedThreads];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += partial[i];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kRedThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = (accumulate ? out[0] : 0.0) + s[0];
}

// grad_pad[c] += scale * sum_s ic[s](c) in FP64, shots summed in order.
template <typename T>
__global__ void reduce_ic_kernel(const T* __restrict__ ic, long long fstride, int nshot, int nx,
                                 int ny, int nz, int hx, int hy, int rows_y, int ldz, double scale,
                                 double* __restrict__ gpad) {
    long long n = (long long)nx * ny * nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        int k = (int)(c % nz);
        long long r = c / nz;
        int j = (int)(r % ny), i = (int)(r / ny);
        long long o = ioff(i, j, k, hx, hy, rows_y, ldz);
        double acc = 0.0;
        for (int s = 0; s < nshot; ++s) acc += (double)ic[s * fstride + o];
        gpad[c] += scale * acc;
    }
}

// Unpadded gradient: each physical cell collects the padded cells that
// add_padding folds onto it (strips beyond a boundary row/column fold onto it).
__global__ void fold_kernel(const double* __restrict__ gpad, int nx, int ny, int nz, int lx,
                            int hxp, int ly, int hyp, int lz, int hzp, double* __restrict__ out) {
    const int px = nx - lx - hxp, py = ny - ly - hyp, pz = nz - lz - hzp;
    long long n = (long long)px * py * pz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        int k = (int)(c % pz);
        long long r = c / pz;
        int j = (int)(r % py), i = (int)(r / py);
        int i0 = lx + i, i1 = lx + i, j0 = ly + j, j1 = ly + j, k0 = lz + k, k1 = lz + k;
        if (i == 0) i0 = 0;
        if (i == px - 1) i1 = nx - 1;
        if (j == 0) j0 = 0;
        if (j == py - 1) j1 = ny - 1;
        if (k == 0) k0 = 0;
        if (k == pz - 1) k1 = nz - 1;
        double acc = 0.0;
        for (int a = i0; a <= i1; ++a)
            for (int b = j0; b <= j1; ++b)
                for (int d = k0; d <= k1; ++d) acc += gpad[((long long)a * ny + b) * nz + d];
        out[c] = acc;
    }
}

int grid_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    return (int)std::max<long long>(1, std::min<long long>(b, 152LL * 16));
}

// ---------------------------------------------------------------------------
// host-side plan
// ---------------------------------------------------------------------------
struct CSRBox {  // injection operator of one shot: box + CSR over box cells
    int box[6];
    std::vector<int> rowptr;  // relative entry indices
    std::vector<int> pt;
    std::vector<double> w;
};

}  // namespace
}  // namespace pgb

struct pysit_plan {
    virtual ~pysit_plan() = default;
    virtual int workspace_bytes(uint64_t* b) const = 0;
    virtual int bind(void* ws, uint64_t bytes, cudaStream_t s) = 0;
    virtual int set_model(const double* C, cudaStream_t s) = 0;
    virtual int forward(void* traces, cudaStream_t s) = 0;
    virtual int gradient(const void* dobs, double* grad, double* rnorm2, void* traces,
                         cudaStream_t s, bool with_grad, bool migrate) = 0;
    virtual int status(int* flags, cudaStream_t s) = 0;
    virtual int step_loop(int mode, int nsteps, cudaStream_t s) = 0;
    virtual int autotune(const int* cand, int ncand, int nsteps, int* chosen, double* ms, cudaStream_t s) = 0;
    virtual int tuning(int* tile, double* share) const = 0;
    // autotune over task lengths along x and z extents of the interior tasks (0: full width)
    virtual int autotune2(const int* cx, int ncx, const int* cz, int ncz, int nsteps, int* chosen_x,
                          int* chosen_z, double* ms, cudaStream_t s) = 0;
    virtual int tiles(int* tile_x, int* tile_z) const = 0;
    // host copy of the current task table (interior tasks first)
    virtual int task_table(int32_t* out, uint64_t cap, uint64_t* n_ints, int32_t* n_interior) const = 0;
    // enqueue misfit + gradient on s without graph handling (for a group's capture)
    virtual int enqueue_grad_raw(const void* dobs, double* grad, double* rnorm2, cudaStream_t s) = 0;
    // linearised modelling / Gauss-Newton Hessian application for a model perturbation
    virtual int born(const double* m1, void* traces, cudaStream_t s) = 0;
    virtual int hessian(const double* m1, double* out, double* d1norm2, cudaStream_t s) = 0;
    int64_t last_launches = 0;
};

namespace pgb {
namespace {

template <typename T>
struct PlanT final : public pysit_plan {
    // ---- description -------------------------------------------------------
    int dim, order, R, nx, ny, nz, nsteps, p_img, S, G, nshots, nsrc, nrec, use_graph, psi_consistent;
    int store_all = 0;           // the forward sweep keeps every imaged dWaveOp (no checkpoints, no recompute)
    int fwd_only = 0;            // forward modelling only: no adjoint, imaging or checkpoint buffers
    int nslots = 1;              // replay slots: S (checkpointed) or ceil(nsteps / p_img) (kept)
    int tile_req = 0;            // requested task length along x (0: default)
    int tz = 0;                  // z extent of an interior task at most (0: the kernel's full width)
    unsigned wait_polls = 0;     // tries of a step kernel's bulk-copy wait (0: the kernels' default)
    int wait_fault = 0;          // test aid: the 2D step kernels' waits run out (pysit_plan_desc.wait_fault)
    std::vector<int> shot_steps; // record length of each shot in steps (empty: all nsteps)
    size_t task_cap = 0;         // ints the task buffer holds (enough for any tile the tuner may set)
    double dx, dy, dz, dt;
    int pad_lo[3], pad_hi[3];
    int pl[3], pr[3];  // PML-state widths (kernel profile lengths)
    std::vector<double> sg[3], mg[3];
    // ---- layout --------------------------------------------------------------
    int hx, hy, rows_y, ldz;
    long long fstride;  // elements per field per shot (256-byte multiple)
    int bz, tx, ntz, ntx;
    int nseg;
    std::vector<int> tasks2d;    // [ntasks][5] warp tasks of the 2D sweep: interior first, then shell
    int ntask2d[2] = {0, 0};     // tasks of each kind
    std::vector<int> tasks3d;    // [ntasks][6] block tasks of the 3D sweep: interior first, then shell
    int ntask3d[2] = {0, 0};
    int blocks2d[4][2] = {{1, 1}, {1, 1}, {1, 1}, {1, 1}};  // resident task blocks per mode and kind (whole GPU)
    unsigned long long ctr_next[2] = {0, 0};  // task-counter values the next 2D launch starts at
    double shell_frac[4] = {0.0, 0.0, 0.0, 0.0};  // 2D, per mode: share of the resident blocks given to the
                                 // PML-shell kernel (0: each kernel is sized for the whole GPU and they
                                 // overlap only where one runs out)
    cudaStream_t aux = nullptr;  // second stream of the 2D step (shell kernel beside the interior one)
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // ---- acquisition (host) ----------------------------------------------------
    std::vector<CSRBox> src_inj, rec_inj;
    int rec_box_max = 0;              // largest receiver injection box (cells) over the shots
    bool rec_in_shell = false;        // 2D: every receiver box lies in cells of PML-shell tasks only
    std::vector<int> rec_rows;        // [nshots*nrec+1]
    int rec_lanes = 1;                // recorder threads per (shot, receiver)
    mutable int rec_cap = 0;          // 2D: recorder blocks at most (a share of the block slots; 0: not yet known)
    std::vector<long long> rec_off;   // internal offsets
    std::vector<double> rec_ws;       // sampling weights
    std::vector<double> src_amp;      // [nshots][nsteps][nsrc]
    // ---- workspace -------------------------------------------------------------
    char* ws = nullptr;
    uint64_t ws_need = 0;
    struct Off {
        size_t c2, sgx, sgy, sgz, mgx, mgy, mgz;
        size_t U[2], PX[2], PY[2], PZ[2], PS[2];   // forward state
        size_t A[2], AX[2], AY[2], AZ[2], AS[2];   // adjoint state
        size_t ic, replay, ckpt, traces, srcamp, m1;
        size_t sbox, srpb, srow, spt, sw;          // source injection
        size_t rbox, rrpb, rrow, rpt, rw;          // receiver injection
        size_t recrow, recoff, recw;               // recording
        size_t gpad, partial, rnorm, err, tasks, ctr, shsteps;
    } off{};
    size_t field_bytes = 0;      // one field for G shots
    int ckpt_fields = 0;         // fields per checkpoint
    bool model_set = false;
    // ---- graphs ----------------------------------------------------------------
    cudaStream_t cap = nullptr;
    struct GraphKey {
        int kind;
        const void *a, *b, *c, *d;
        bool operator<(const GraphKey& o) const {
            if (kind != o.kind) return kind < o.kind;
            if (a != o.a) return a < o.a;
            if (b != o.b) return b < o.b;
            if (c != o.c) return c < o.c;
            return d < o.d;
        }
    };
    struct GraphRec {
        cudaGraphExec_t exec = nullptr;
        int64_t launches = 0;
    };
    std::map<GraphKey, GraphRec> graphs;
    std::set<GraphKey> seen;  // run sequences used once so far: eager; captured on their second use
    int64_t launches = 0;

    ~PlanT() override {
        for (auto& kv : graphs)
            if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
        if (cap) cudaStreamDestroy(cap);
        if (aux) cudaStreamDestroy(aux);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
    }

    template <typename U>
    U* at(size_t o) const { return reinterpret_cast<U*>(ws + o); }
    T* fld(size_t o, int shot = 0) const { return at<T>(o) + (long long)shot * fstride; }

    // ---- creation --------------------------------------------------------------
    int init(const pysit_plan_desc& d) {
        dim = d.dim; order = d.order; R = order / 2;
        nx = d.n[0]; ny = d.n[1]; nz = d.n[2];
        if (dim == 1) { nx = 1; ny = 1; }
        if (dim == 2) ny = 1;
        dx = d.delta[0]; dy = d.delta[1]; dz = d.delta[2];
        dt = d.dt; nsteps = d.nsteps; p_img = d.imaging_period;
        S = std::min(d.checkpoint_every, d.nsteps);  // an interval past the record is one segment
        nshots = d.nshots; G = std::min(d.shots_per_launch, d.nshots); nsrc = d.nsrc; nrec = d.nrec;
        use_graph = d.use_graph;
        psi_consistent = d.psi_consistent ? 1 : 0;
        store_all = d.store_dwaveop ? 1 : 0;
        fwd_only = d.forward_only ? 1 : 0;
        tile_req = d.tile_x > 0 ? d.tile_x : 0;
        PGB_REQUIRE(d.tile_z == 0 || d.tile_z >= kMinTileZ, "tile_z %d below %d cells", d.tile_z, kMinTileZ);
        tz = d.tile_z > 0 ? d.tile_z / 4 * 4 : 0;
        wait_polls = d.wait_polls;
        wait_fault = d.wait_fault ? 1 : 0;
        for (int m = 0; m < 3; ++m)
            shell_frac[m] = d.shell_share[m] > 0 && d.shell_share[m] < 1 ? d.shell_share[m] : 0.0;
        shot_steps.clear();
        if (d.shot_nsteps) {
            for (int s2 = 0; s2 < d.nshots; ++s2) {
                PGB_REQUIRE(d.shot_nsteps[s2] >= 1 && d.shot_nsteps[s2] <= d.nsteps,
                            "record length of shot %d (%d steps) outside [1, nsteps = %d]", s2, d.shot_nsteps[s2],
                            d.nsteps);
                shot_steps.push_back(d.shot_nsteps[s2]);
            }
        }
        for (int a = 0; a < 3; ++a) { pad_lo[a] = d.pad_lo[a]; pad_hi[a] = d.pad_hi[a]; }
        const int na[3] = {nx, ny, nz};
        for (int a = 0; a < 3; ++a) {
            pl[a] = d.sig_l[a] ? d.nsig_l[a] : 0;
            pr[a] = d.sig_r[a] ? d.nsig_r[a] : 0;
            PGB_REQUIRE(pl[a] >= 0 && pr[a] >= 0 && pl[a] <= na[a] && pr[a] <= na[a],
                        "bad PML profile length on axis %d", a);
            sg[a].assign(na[a], 0.0);
            mg[a].assign(na[a], 0.0);
            for (int i = 0; i < na[a]; ++i) {
                // profile lookup of the step kernels (_2D.h:137-157)
                if (pl[a] > 0 && i < pl[a]) sg[a][i] = d.sig_l[a][i];
                else if (pr[a] > 0 && i >= na[a] - pr[a] && i <= na[a] - 2)
                    sg[a][i] = d.sig_r[a][pr[a] - ((na[a] - 1) - i)];
                if (d.sigmap[a]) mg[a][i] = d.sigmap[a][i];
            }
        }
        // layout
        hx = dim >= 2 ? kHalo : 0;
        hy = dim == 3 ? kHalo : 0;
        rows_y = ny + 2 * hy;
        ldz = ((kOZ + nz + kTailZ) + 31) / 32 * 32;
        fstride = (long long)(nx + 2 * hx) * rows_y * ldz;
        fstride = (fstride + 63) / 64 * 64;
        // the 3D shell kernel addresses its taps with 32-bit offsets of up to R x-planes
        PGB_REQUIRE(dim < 3 || (long long)kHalo * rows_y * ldz < (1LL << 31),
                    "3D x-plane of %lld elements is too large (R planes must stay below 2^31 elements)",
                    (long long)rows_y * ldz);
        field_bytes = (size_t)fstride * G * sizeof(T);
        nseg = (nsteps + S - 1) / S;
        nslots = store_all ? (nsteps + p_img - 1) / p_img : S;
        ckpt_fields = dim == 1 ? 3 : dim == 2 ? 4 : 6;
        choose_tiling();
        // acquisition
        int rc = build_injection(d.src_tap_ptr, d.src_tap_cell, d.src_tap_point, d.src_tap_w, nsrc,
                                 src_inj, "source");
        if (rc) return rc;
        rc = build_injection(d.rec_tap_ptr, d.rec_tap_cell, d.rec_tap_point, d.rec_tap_winject, nrec,
                             rec_inj, "receiver");
        if (rc) return rc;
        rec_box_max = 0;
        for (auto& b : rec_inj)
            rec_box_max = std::max(rec_box_max, (b.box[1] - b.box[0]) * (b.box[3] - b.box[2]) * (b.box[5] - b.box[4]));
        if (dim == 2) {
            // the bounds of the interior tasks (as build_tasks2d_ draws them)
            const int xa = pl[0] > 0 ? pl[0] + R : 1, xb = pr[0] > 0 ? nx - pr[0] - R : nx - 1;
            const int za = ((pl[2] > 0 ? pl[2] + R : 1) + 3) / 4 * 4, zb = (pr[2] > 0 ? nz - pr[2] - R : nz - 1) / 4 * 4;
            rec_in_shell = !rec_inj.empty();
            for (auto& b : rec_inj) {
                if (b.box[1] <= b.box[0] || b.box[5] <= b.box[4]) continue;  // no taps
                const bool zout = b.box[5] <= za || b.box[4] >= zb, xout = b.box[1] <= xa || b.box[0] >= xb;
                if (!(zout || xout || xa >= xb || za >= zb)) rec_in_shell = false;
            }
        }
        rc = build_recording(d);
        if (rc) return rc;
        src_amp.assign(d.src_amp, d.src_amp + (size_t)nshots * nsteps * nsrc);
        carve();
        return PYSIT_OK;
    }

    void choose_tiling() {
        constexpr int V = V16<T>::N;
        if (dim == 2) {
            bz = wave2d_warp_threads();
            tx = tile_req ? tile_req : 32;
            build_tasks2d();
            ntz = ntx = 1;
            return;
        }
        if (dim == 3) {
            bz = 128;  // threads of the recorder blocks
            tx = tile_req ? tile_req : 64;
            build_tasks3d();
            ntz = ntx = 1;
            return;
        }
        // 1D: fewest loaded elements (tile + halo) per useful cell, bz >= 64
        double best = 1e30;
        for (int b : {64, 128, 256}) {
            int tiles = (nz + b * V - 1) / (b * V);
            double cost = (double)tiles * (b * V + 2 * kHalo) / nz;
            if (cost < best - 1e-9) { best = cost; bz = b; }
        }
        tx = 32;
        ntz = (nz + bz * V - 1) / (bz * V);
        ntx = (nx + tx - 1) / tx;
    }

    // Warp tasks covering the padded grid once.  Interior (kind 0): cells at least
    // R away from the padding; PML shell (kind 1): the rest.  z boundaries are
    // multiples of 4 cells (vectors never straddle two tasks) except the grid end.
    void split(int a, int b, int w, std::vector<std::pair<int, int>>& out) const {
        if (b <= a) return;
        int n = (b - a + w - 1) / w;
        int width = ((b - a + n - 1) / n + 3) / 4 * 4;
        for (int z = a; z < b; z += width) out.push_back({z, std::min(b, z + width)});
    }
    // 3D z segments of at most w cells (w a multiple of 4 and of V): the even split, or
    // full w-wide segments and a remainder, whichever leaves fewer lanes idle.  A warp
    // takes 32 / nv rows of a segment of nv vectors, so a narrow remainder fills a warp
    // with several rows.
    void split3d(int a, int b, int w, std::vector<std::pair<int, int>>& out) const {
        constexpr int V = V16<T>::N;
        auto eff = [&](const std::vector<std::pair<int, int>>& seg) {
            double used = 0, slots = 0;
            for (auto& z : seg) {
                const int nv = (z.second - z.first + V - 1) / V;
                used += nv;
                slots += 32.0 / (32 / nv);  // lane slots one row of the segment takes
            }
            return slots > 0 ? used / slots : 0.0;
        };
        std::vector<std::pair<int, int>> even, full;
        split(a, b, w, even);
        for (int z = a; z < b; z += w) full.push_back({z, std::min(b, z + w)});
        const auto& pick = eff(full) > eff(even) + 1e-9 ? full : even;
        out.insert(out.end(), pick.begin(), pick.end());
    }
    void add_tasks(int xa, int xb, int za, int zb, int kind) {
        if (xb <= xa || zb <= za) return;
        std::vector<std::pair<int, int>> zs;
        int w = wave2d_warp_seg((int)sizeof(T), order, kind);
        if (kind == 0 && tz > 0) w = std::min(w, tz);
        split(za, zb, w, zs);
        const int nxc = (xb - xa + tx - 1) / tx, wx = (xb - xa + nxc - 1) / nxc;  // even x chunks
        for (int x = xa; x < xb; x += wx)
            for (auto& z : zs) {
                int t[5] = {x, std::min(xb, x + wx), z.first, z.second, kind};
                tasks2d.insert(tasks2d.end(), t, t + 5);
            }
    }
    void build_tasks2d() {
        tasks2d.clear();
        build_tasks2d_();
        // interior tasks were added first
        ntask2d[0] = ntask2d[1] = 0;
        for (size_t t = 0; t < tasks2d.size(); t += 5) ++ntask2d[tasks2d[t + 4] ? 1 : 0];
    }
    void build_tasks2d_() {
        // interior: R cells clear of the padding and off the outer (Dirichlet) ring
        const int xa = pl[0] > 0 ? pl[0] + R : 1;
        const int xb = pr[0] > 0 ? nx - pr[0] - R : nx - 1;
        int za = ((pl[2] > 0 ? pl[2] + R : 1) + 3) / 4 * 4;
        int zb = (pr[2] > 0 ? nz - pr[2] - R : nz - 1) / 4 * 4;
        if (xa >= xb || za >= zb) {  // no interior: the whole grid is shell
            add_tasks(0, nx, 0, nz, 1);
            return;
        }
        add_tasks(xa, xb, za, zb, 0);   // interior
        add_tasks(0, xa, 0, nz, 1);     // low-x band
        add_tasks(xb, nx, 0, nz, 1);    // high-x band
        add_tasks(xa, xb, 0, za, 1);    // low-z band
        add_tasks(xa, xb, zb, nz, 1);   // high-z band
    }

    // 3D block tasks: the interior box (R cells clear of the padding, off the outer
    // ring, z-bounds multiples of 4) and the six slabs of the shell around it; x in
    // chunks of about tx rows, z in segments, y in groups of the rows one block
    // covers (a shell warp takes several rows of a narrow z segment).
    // Consecutive tasks are neighbouring y-groups (their halo rows meet in L2).
    void add_tasks3d(int xa, int xb, int ya, int yb, int za, int zb, int kind) {
        if (xb <= xa || yb <= ya || zb <= za) return;
        std::vector<std::pair<int, int>> zs;
        int w = wave3d_seg((int)sizeof(T), kind);
        if (kind == 0 && tz > 0) w = std::min(w, tz);
        split3d(za, zb, w, zs);
        const int nxc = (xb - xa + tx - 1) / tx, wx = (xb - xa + nxc - 1) / nxc;
        for (int x = xa; x < xb; x += wx)
            for (auto& z : zs)
                for (int y = ya, rows = wave3d_task_rows((int)sizeof(T), kind, z.second - z.first); y < yb;
                     y += rows) {
                    int t[6] = {x, std::min(xb, x + wx), y, std::min(yb, y + rows), z.first, z.second};
                    tasks3d.insert(tasks3d.end(), t, t + 6);
                }
    }
    void build_tasks3d() {
        tasks3d.clear();
        const int xa = pl[0] > 0 ? pl[0] + R : 1, xb = pr[0] > 0 ? nx - pr[0] - R : nx - 1;
        const int ya = pl[1] > 0 ? pl[1] + R : 1, yb = pr[1] > 0 ? ny - pr[1] - R : ny - 1;
        const int za = ((pl[2] > 0 ? pl[2] + R : 1) + 3) / 4 * 4;
        const int zb = (pr[2] > 0 ? nz - pr[2] - R : nz - 1) / 4 * 4;
        ntask3d[0] = ntask3d[1] = 0;
        if (xa >= xb || ya >= yb || za >= zb) {
            add_tasks3d(0, nx, 0, ny, 0, nz, 1);
        } else {
            add_tasks3d(xa, xb, ya, yb, za, zb, 0);
            ntask3d[0] = (int)(tasks3d.size() / 6);
            add_tasks3d(0, xa, 0, ny, 0, nz, 1);    // low-x slab
            add_tasks3d(xb, nx, 0, ny, 0, nz, 1);   // high-x slab
            add_tasks3d(xa, xb, 0, ya, 0, nz, 1);   // low-y slab
            add_tasks3d(xa, xb, yb, ny, 0, nz, 1);  // high-y slab
            add_tasks3d(xa, xb, ya, yb, 0, za, 1);  // low-z slab
            add_tasks3d(xa, xb, ya, yb, zb, nz, 1); // high-z slab
        }
        ntask3d[1] = (int)(tasks3d.size() / 6) - ntask3d[0];
    }

    // ints of the task table for a task length tx_try and z extent tz_try (the current table is kept)
    static constexpr int kMinTileX = 8;
    static constexpr int kMinTileZ = 16;
    size_t task_ints(int tx_try, int tz_try) {
        if (dim == 1) return 0;
        const int keep = tx, keepz = tz;
        tx = tx_try;
        tz = tz_try;
        size_t n;
        if (dim == 2) { build_tasks2d(); n = tasks2d.size(); } else { build_tasks3d(); n = tasks3d.size(); }
        tx = keep;
        tz = keepz;
        if (dim == 2) build_tasks2d(); else build_tasks3d();
        return n;
    }

    long long internal_offset(long long cell) const {
        int k = (int)(cell % nz);
        long long r = cell / nz;
        int j = (int)(r % ny), i = (int)(r / ny);
        return ((long long)(i + hx) * rows_y + (j + hy)) * ldz + kOZ + k;
    }

    int build_injection(const int64_t* ptr, const int64_t* cell, const int32_t* pt, const double* w,
                        int npts, std::vector<CSRBox>& out, const char* what) {
        out.assign(nshots, CSRBox{});
        const long long ncell = (long long)nx * ny * nz;
        for (int s = 0; s < nshots; ++s) {
            CSRBox& b = out[s];
            long long e0 = ptr ? ptr[s] : 0, e1 = ptr ? ptr[s + 1] : 0;
            PGB_REQUIRE(e1 >= e0, "%s tap pointers must be non-decreasing", what);
            int lo[3] = {nx, ny, nz}, hi[3] = {0, 0, 0};
            for (long long e = e0; e < e1; ++e) {
                PGB_REQUIRE(cell[e] >= 0 && cell[e] < ncell, "%s tap cell %lld out of the grid", what,
                            (long long)cell[e]);
                PGB_REQUIRE(pt[e] >= 0 && pt[e] < npts, "%s tap point %d out of range", what, pt[e]);
                int k = (int)(cell[e] % nz);
                long long r = cell[e] / nz;
                int j = (int)(r % ny), i = (int)(r / ny);
                lo[0] = std::min(lo[0], i); hi[0] = std::max(hi[0], i + 1);
                lo[1] = std::min(lo[1], j); hi[1] = std::max(hi[1], j + 1);
                lo[2] = std::min(lo[2], k); hi[2] = std::max(hi[2], k + 1);
            }
            if (e1 == e0) { for (int a = 0; a < 3; ++a) { lo[a] = 0; hi[a] = 0; } }
            b.box[0] = lo[0]; b.box[1] = hi[0]; b.box[2] = lo[1]; b.box[3] = hi[1];
            b.box[4] = lo[2]; b.box[5] = hi[2];
            long long bw = (long long)(hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]);
            if (bw < 0) bw = 0;
            PGB_REQUIRE(bw < (1LL << 30), "%s footprint too large", what);
            std::vector<int> cnt(bw + 1, 0);
            auto boxcell = [&](long long c) {
                int k = (int)(c % nz);
                long long r = c / nz;
                int j = (int)(r % ny), i = (int)(r / ny);
                return ((long long)(i - lo[0]) * (hi[1] - lo[1]) + (j - lo[1])) * (hi[2] - lo[2]) +
                       (k - lo[2]);
            };
            for (long long e = e0; e < e1; ++e) cnt[boxcell(cell[e]) + 1]++;
            b.rowptr.assign(bw + 1, 0);
            for (long long c = 0; c < bw; ++c) b.rowptr[c + 1] = b.rowptr[c] + cnt[c + 1];
            b.pt.assign(e1 - e0, 0);
            b.w.assign(e1 - e0, 0.0);
            std::vector<int> fill(b.rowptr.begin(), b.rowptr.begin() + bw);
            for (long long e = e0; e < e1; ++e) {  // stable: taps keep their order per cell
                long long c = boxcell(cell[e]);
                int pos = fill[c]++;
                b.pt[pos] = pt[e];
                b.w[pos] = w[e];
            }
        }
        return PYSIT_OK;
    }

    int build_recording(const pysit_plan_desc& d) {
        const long long ncell = (long long)nx * ny * nz;
        rec_rows.assign((size_t)nshots * nrec + 1, 0);
        std::vector<long long> cnt((size_t)nshots * nrec + 1, 0);
        long long total = d.rec_tap_ptr ? d.rec_tap_ptr[nshots] - d.rec_tap_ptr[0] : 0;
        PGB_REQUIRE(total < (1LL << 31), "too many receiver taps");
        for (int s = 0; s < nshots && d.rec_tap_ptr; ++s)
            for (long long e = d.rec_tap_ptr[s]; e < d.rec_tap_ptr[s + 1]; ++e) {
                PGB_REQUIRE(d.rec_tap_point[e] >= 0 && d.rec_tap_point[e] < nrec, "receiver index out of range");
                PGB_REQUIRE(d.rec_tap_cell[e] >= 0 && d.rec_tap_cell[e] < ncell, "receiver tap out of grid");
                cnt[(size_t)s * nrec + d.rec_tap_point[e] + 1]++;
            }
        for (size_t r = 0; r < (size_t)nshots * nrec; ++r) rec_rows[r + 1] = (int)(rec_rows[r] + cnt[r + 1]);
        // threads per receiver: about 8 taps a thread, at most a warp
        const double mean_taps = nshots * nrec > 0 ? (double)total / ((double)nshots * nrec) : 0.0;
        rec_lanes = 1;
        while (rec_lanes < 32 && rec_lanes * 8 < mean_taps) rec_lanes *= 2;
        rec_off.assign(total, 0);
        rec_ws.assign(total, 0.0);
        std::vector<int> fill(rec_rows.begin(), rec_rows.end() - 1);
        for (int s = 0; s < nshots && d.rec_tap_ptr; ++s)
            for (long long e = d.rec_tap_ptr[s]; e < d.rec_tap_ptr[s + 1]; ++e) {
                int pos = fill[(size_t)s * nrec + d.rec_tap_point[e]]++;
                rec_off[pos] = internal_offset(d.rec_tap_cell[e]);
                rec_ws[pos] = d.rec_tap_wsample[e];
            }
        return PYSIT_OK;
    }

    void carve() {
        size_t tot = 0;
        auto take = [&](size_t bytes) { size_t o = tot; tot += (bytes + 255) / 256 * 256; return o; };
        const size_t one = (size_t)fstride * sizeof(T);  // one field, one shot
        off.c2 = take(one);
        off.sgx = take(nx * sizeof(T)); off.sgy = take(ny * sizeof(T)); off.sgz = take(nz * sizeof(T));
        off.mgx = take(nx * sizeof(T)); off.mgy = take(ny * sizeof(T)); off.mgz = take(nz * sizeof(T));
        // a forward-only plan aliases the adjoint state onto the forward one and keeps
        // no imaging, replay or checkpoint storage
        const size_t adj_bytes = fwd_only ? 0 : field_bytes;
        for (int b = 0; b < 2; ++b) {
            off.U[b] = take(field_bytes); off.A[b] = fwd_only ? off.U[b] : take(adj_bytes);
            off.PZ[b] = take(field_bytes); off.AZ[b] = fwd_only ? off.PZ[b] : take(adj_bytes);
            off.PX[b] = dim >= 2 ? take(field_bytes) : off.PZ[b];
            off.AX[b] = fwd_only ? off.PX[b] : dim >= 2 ? take(adj_bytes) : off.AZ[b];
            off.PY[b] = dim == 3 ? take(field_bytes) : off.PZ[b];
            off.AY[b] = fwd_only ? off.PY[b] : dim == 3 ? take(adj_bytes) : off.AZ[b];
            off.PS[b] = dim == 3 ? take(field_bytes) : off.PZ[b];
            off.AS[b] = fwd_only ? off.PS[b] : dim == 3 ? take(adj_bytes) : off.AZ[b];
        }
        off.ic = take(adj_bytes);
        off.m1 = take(fwd_only ? 0 : one);
        off.replay = take(fwd_only ? 0 : field_bytes * (size_t)nslots);
        off.ckpt = take(fwd_only || store_all ? 0 : field_bytes * (size_t)ckpt_fields * nseg);
        off.traces = take((size_t)G * nsteps * nrec * sizeof(T));
        off.srcamp = take((size_t)nshots * nsteps * nsrc * sizeof(T));
        auto take_inj = [&](std::vector<CSRBox>& v, size_t& box, size_t& rpb, size_t& row, size_t& pt,
                            size_t& w) {
            size_t nrow = 0, nent = 0;
            for (auto& b : v) { nrow += b.rowptr.size(); nent += b.pt.size(); }
            box = take(v.size() * 6 * sizeof(int));
            rpb = take(v.size() * sizeof(long long));
            row = take(std::max<size_t>(nrow, 1) * sizeof(int));
            pt = take(std::max<size_t>(nent, 1) * sizeof(int));
            w = take(std::max<size_t>(nent, 1) * sizeof(T));
        };
        take_inj(src_inj, off.sbox, off.srpb, off.srow, off.spt, off.sw);
        take_inj(rec_inj, off.rbox, off.rrpb, off.rrow, off.rpt, off.rw);
        off.recrow = take(rec_rows.size() * sizeof(int));
        off.recoff = take(std::max<size_t>(rec_off.size(), 1) * sizeof(long long));
        off.recw = take(std::max<size_t>(rec_ws.size(), 1) * sizeof(T));
        off.gpad = take((size_t)nx * ny * nz * sizeof(double));
        off.err = take(sizeof(int));
        off.ctr = take(2 * sizeof(unsigned long long));
        off.shsteps = take(std::max<size_t>(shot_steps.size(), 1) * sizeof(int));
        // the largest table any tuning can ask for: the shortest x-chunk, and every z extent
        // (in 3D a narrower segment can give more tasks: its warps take several rows, but
        // not always enough to make up for the extra segments)
        task_cap = std::max<size_t>(task_ints(kMinTileX, 0), std::max(tasks2d.size(), tasks3d.size()));
        for (int z = kMinTileZ; z <= 32 * V16<T>::N; z += 4) task_cap = std::max(task_cap, task_ints(kMinTileX, z));
        off.tasks = take(std::max<size_t>(task_cap, 1) * sizeof(int));
        off.partial = take(kRedBlocks * sizeof(double));
        off.rnorm = take(sizeof(double));
        ws_need = tot;
    }

    int workspace_bytes(uint64_t* b) const override { *b = ws_need; return PYSIT_OK; }

    template <typename U>
    int upload(size_t o, const std::vector<U>& v, cudaStream_t s) {
        if (v.empty()) return PYSIT_OK;
        PGB_CHECK_CUDA(cudaMemcpyAsync(ws + o, v.data(), v.size() * sizeof(U), cudaMemcpyHostToDevice, s));
        return PYSIT_OK;
    }
    std::vector<T> toT(const std::vector<double>& v) { return std::vector<T>(v.begin(), v.end()); }

    int upload_inj(std::vector<CSRBox>& v, size_t box, size_t rpb, size_t row, size_t pt, size_t w,
                   cudaStream_t s) {
        std::vector<int> boxes, rows, pts;
        std::vector<long long> bases;
        std::vector<double> ws_;
        for (auto& b : v) {
            boxes.insert(boxes.end(), b.box, b.box + 6);
            bases.push_back((long long)rows.size());
            int base = (int)pts.size();
            for (int r : b.rowptr) rows.push_back(r + base);
            pts.insert(pts.end(), b.pt.begin(), b.pt.end());
            ws_.insert(ws_.end(), b.w.begin(), b.w.end());
        }
        int rc;
        if ((rc = upload(box, boxes, s)) || (rc = upload(rpb, bases, s)) || (rc = upload(row, rows, s)) ||
            (rc = upload(pt, pts, s)))
            return rc;
        std::vector<T> wt = toT(ws_);
        rc = upload(w, wt, s);
        if (rc) return rc;
        return cudaStreamSynchronize(s) == cudaSuccess ? PYSIT_OK : cuda_status(cudaGetLastError(), "upload");
    }

    int bind(void* w, uint64_t bytes, cudaStream_t s) override {
        PGB_REQUIRE(w != nullptr, "NULL workspace");
        PGB_REQUIRE(aligned(w, 256), "workspace must be 256-byte aligned");
        PGB_REQUIRE(bytes >= ws_need, "workspace too small: %llu < %llu bytes",
                    (unsigned long long)bytes, (unsigned long long)ws_need);
        for (auto& kv : graphs)
            if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
        graphs.clear();
        seen.clear();
        ws = static_cast<char*>(w);
        PGB_CHECK_CUDA(cudaMemsetAsync(ws, 0, ws_need, s));
        int rc;
        std::vector<T> tmp;
        if ((rc = upload(off.sgx, tmp = toT(sg[0]), s)) || (rc = upload(off.sgy, tmp = toT(sg[1]), s)) ||
            (rc = upload(off.sgz, tmp = toT(sg[2]), s)) || (rc = upload(off.mgx, tmp = toT(mg[0]), s)) ||
            (rc = upload(off.mgy, tmp = toT(mg[1]), s)) || (rc = upload(off.mgz, tmp = toT(mg[2]), s)))
            return rc;
        PGB_CHECK_CUDA(cudaStreamSynchronize(s));
        if ((rc = upload(off.srcamp, tmp = toT(src_amp), s))) return rc;
        PGB_CHECK_CUDA(cudaStreamSynchronize(s));
        if ((rc = upload_inj(src_inj, off.sbox, off.srpb, off.srow, off.spt, off.sw, s))) return rc;
        if ((rc = upload_inj(rec_inj, off.rbox, off.rrpb, off.rrow, off.rpt, off.rw, s))) return rc;
        if ((rc = upload(off.recrow, rec_rows, s)) || (rc = upload(off.recoff, rec_off, s))) return rc;
        if ((rc = upload(off.recw, tmp = toT(rec_ws), s))) return rc;
        if ((rc = upload(off.tasks, dim == 3 ? tasks3d : tasks2d, s))) return rc;
        if ((rc = upload(off.shsteps, shot_steps, s))) return rc;
        PGB_CHECK_CUDA(cudaStreamSynchronize(s));
        if (!cap) PGB_CHECK_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        if (dim == 2) {
            wave2d_warp_prepare();
            for (int m = 0; m < 4; ++m)
                for (int k = 0; k < 2; ++k) blocks2d[m][k] = wave2d_warp_blocks((int)sizeof(T), order, m, k);
        }
        if (dim >= 2) {
            if (!aux) PGB_CHECK_CUDA(cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking));
            if (!ev_fork) PGB_CHECK_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
            if (!ev_join) PGB_CHECK_CUDA(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
        }
        PGB_CHECK_CUDA(cudaGetLastError());
        model_set = false;
        return PYSIT_OK;
    }

    int status(int* flags, cudaStream_t s) override {
        PGB_REQUIRE(ws, "no workspace bound");
        int v = 0;
        PGB_CHECK_CUDA(cudaMemcpyAsync(&v, ws + off.err, sizeof(int), cudaMemcpyDeviceToHost, s));
        PGB_CHECK_CUDA(cudaStreamSynchronize(s));
        PGB_CHECK_CUDA(cudaMemsetAsync(ws + off.err, 0, sizeof(int), s));
        *flags = v;
        return PYSIT_OK;
    }

    int set_model(const double* C, cudaStream_t s) override {
        PGB_REQUIRE(ws, "no workspace bound");
        PGB_REQUIRE(C, "NULL model");
        long long n = (long long)nx * ny * nz;
        set_c2_kernel<T><<<grid_for(n, 256), 256, 0, s>>>(C, nx, ny, nz, hx, hy, rows_y, ldz, at<T>(off.c2));
        PGB_CHECK_CUDA(cudaGetLastError());
        model_set = true;
        return PYSIT_OK;
    }

    // ---- step launch -------------------------------------------------------------
    struct State {  // role-tracking pointers of one wavefield state (ping-pong)
        T *prev, *cur, *phx[2], *phy[2], *phz[2], *psi[2];
        int pb = 0;  // which PML buffer is the input
    };

    WaveParams<T> base_params(int g0, int gn) const {
        WaveParams<T> p{};
        p.nx = nx; p.ny = ny; p.nz = nz; p.ldz = ldz; p.rows_y = rows_y; p.fstride = fstride;
        p.hx = hx; p.hy = hy; p.tx = tx; p.ty = 1; p.ntz = ntz; p.nty = 1; p.ntx = ntx; p.nshot = gn;
        p.c2 = at<T>(off.c2);
        p.sgx = at<T>(off.sgx); p.sgy = at<T>(off.sgy); p.sgz = at<T>(off.sgz);
        p.mgx = at<T>(off.mgx); p.mgy = at<T>(off.mgy); p.mgz = at<T>(off.mgz);
        p.pxl = pl[0]; p.pxr = pr[0]; p.pyl = pl[1]; p.pyr = pr[1]; p.pzl = pl[2]; p.pzr = pr[2];
        p.dt = T(dt); p.dt2 = T(dt * dt); p.idt2 = T(1.0 / (dt * dt)); p.i2dt = T(1.0 / (2.0 * dt));
        p.idx = T(1.0 / dx); p.idx2 = T(1.0 / (T(dx) * T(dx)));
        p.idy = T(1.0 / dy); p.idy2 = T(1.0 / (T(dy) * T(dy)));
        p.idz = T(1.0 / dz); p.idz2 = T(1.0 / (T(dz) * T(dz)));
        p.err = ws ? at<int>(off.err) : nullptr;
        p.polls = wait_polls;
        p.wait_fault = wait_fault;
        p.psi_c2 = psi_consistent ? 0 : 1;
        p.task_ctr = ws ? at<unsigned long long>(off.ctr) : nullptr;
        (void)g0;
        return p;
    }

    void set_inject(WaveParams<T>& p, bool src, int g0, int k, const T* resid) const {
        Inject<T>& j = p.inj;
        if (src) {
            j.box = at<int>(off.sbox) + g0 * 6;
            j.rpbase = at<long long>(off.srpb) + g0;
            j.rowptr = at<int>(off.srow);
            j.pt = at<int>(off.spt);
            j.w = at<T>(off.sw);
            j.amp_sstride = (long long)nsteps * nsrc;
            j.amp = at<T>(off.srcamp) + (long long)g0 * j.amp_sstride + (long long)k * nsrc;
            j.on = nsrc > 0;
        } else {
            j.box = at<int>(off.rbox) + g0 * 6;
            j.rpbase = at<long long>(off.rrpb) + g0;
            j.rowptr = at<int>(off.rrow);
            j.pt = at<int>(off.rpt);
            j.w = at<T>(off.rw);
            j.amp_sstride = (long long)nsteps * nrec;
            j.amp = resid + (long long)k * nrec;
            j.on = nrec > 0;
        }
    }

    // One 2D step: the interior kernel on s and the PML-shell kernel on the
    // auxiliary stream, forked from and joined back into s (graph branches when
    // captured), each a persistent grid drawing (shot, task) pairs from its counter.
    template <int RR, int MODE>
    void launch2d(const WaveParams<T>& p, cudaStream_t s) {
        const int* tk = at<int>(off.tasks);
        const long long wpb = wave2d_warp_threads() / 32;
        WaveParams<T> q = p;
        q.task_base = ctr_next[0];
        q.task_base2 = ctr_next[1];
        int nb[2];
        // with a shell share the two kernels split the resident block slots (they run side by
        // side from the start); otherwise each is sized for the whole GPU
        const double fr = shell_frac[MODE];
        const int cap1 = fr > 0 ? std::max(1, (int)(fr * blocks2d[MODE][1] + 0.5)) : blocks2d[MODE][1];
        const int cap0 = fr > 0 ? std::max(1, blocks2d[MODE][0] - (int)(fr * blocks2d[MODE][0] + 0.5))
                                : blocks2d[MODE][0];
        for (int k = 0; k < 2; ++k) {
            const long long need = ((long long)ntask2d[k] * p.nshot + wpb - 1) / wpb;
            nb[k] = (int)std::min<long long>(need, k ? cap1 : cap0);
        }
        // the adjoint source covers every receiver: added by a scatter kernel after the step
        const bool scatter = MODE == kAdj && q.inj.on && rec_box_max > 0;
        if (scatter) q.inj.on = 0;
        const bool rec = MODE != kAdj && q.rec.blocks > 0;
        const int recb = q.rec.blocks;
        q.rec.blocks = 0;
        const bool fork = ntask2d[1] > 0 && ntask2d[0] > 0;
        cudaStream_t side = fork ? aux : s;
        if (fork) {
            cudaEventRecord(ev_fork, s);
            cudaStreamWaitEvent(aux, ev_fork, 0);
        }
#ifndef PGB_FUSED_REC
#define PGB_FUSED_REC 1
#endif
        // the recorder rides as extra leading blocks of the interior kernel (they read u_k,
        // which the step leaves alone, and exit at once); as a kernel of its own ahead of the
        // shell kernel it held the shell back until the interior kernel's blocks retired
        const bool fused_rec = PGB_FUSED_REC && rec && ntask2d[0] > 0;
        if (rec && !fused_rec) {
            record_kernel<T><<<recb, bz, 0, side>>>(q);
            ++launches;
        }
        if (ntask2d[1] > 0) {
            ctr_next[1] += launch_wave2d_warp_tasks<T, RR, MODE, 1>(q, tk + 5 * ntask2d[0], ntask2d[1], nb[1], side);
            ++launches;
        }
        if (ntask2d[0] > 0) {
            WaveParams<T> qi = q;
            qi.rec.blocks = fused_rec ? recb : 0;
            ctr_next[0] += launch_wave2d_warp_tasks<T, RR, MODE, 0>(qi, tk, ntask2d[0], nb[0], s);
            ++launches;
        }
        // the adjoint source adds to cells the shell kernel has written; when every receiver
        // box lies in shell cells it follows the shell kernel on its stream, overlapping the
        // interior kernel's tail, else it waits for both
        const bool scatter_side = scatter && fork && rec_in_shell;
        auto do_scatter = [&](cudaStream_t st) {
            q.inj.on = 1;
            const long long n = (long long)q.nshot * rec_box_max;
            inject_scatter2d_kernel<T><<<(int)std::min<long long>((n + 255) / 256, 4096), 256, 0, st>>>(q, rec_box_max);
            ++launches;
        };
        if (scatter_side) do_scatter(side);
        if (fork) {
            cudaEventRecord(ev_join, aux);
            cudaStreamWaitEvent(s, ev_join, 0);
        }
        if (scatter && !scatter_side) do_scatter(s);
    }

    // One 3D step: interior kernel on s, PML-shell kernel (and the trace recorder)
    // on the auxiliary stream, forked and joined as in 2D; the adjoint source is
    // added after the step by a scatter kernel.
    template <int RR, int MODE>
    void launch3d(const WaveParams<T>& p, cudaStream_t s) {
        const int* tk = at<int>(off.tasks);
        WaveParams<T> q = p;
        const bool scatter = MODE == kAdj && q.inj.on && rec_box_max > 0;
        if (scatter) q.inj.on = 0;
        const bool rec = MODE != kAdj && q.rec.blocks > 0;
        const bool fork = ntask3d[0] > 0 && (ntask3d[1] > 0 || rec);
        cudaStream_t side = fork ? aux : s;
        if (fork) {
            cudaEventRecord(ev_fork, s);
            cudaStreamWaitEvent(aux, ev_fork, 0);
        }
        if (rec) {
            record_kernel<T><<<q.rec.blocks, bz, 0, side>>>(q);
            ++launches;
        }
        if (ntask3d[1] > 0) {
            launch_wave3d_tasks<T, RR, MODE, 1>(q, tk + 6 * ntask3d[0], ntask3d[1], side);
            ++launches;
        }
        if (ntask3d[0] > 0) {
            launch_wave3d_tasks<T, RR, MODE, 0>(q, tk, ntask3d[0], s);
            ++launches;
        }
        if (fork) {
            cudaEventRecord(ev_join, aux);
            cudaStreamWaitEvent(s, ev_join, 0);
        }
        if (scatter) {
            q.inj.on = 1;
            const long long n = (long long)q.nshot * rec_box_max;
            inject_scatter3d_kernel<T><<<(int)std::min<long long>((n + 255) / 256, 4096), 256, 0, s>>>(q, rec_box_max);
            ++launches;
        }
    }

    void launch(const WaveParams<T>& p, int mode, cudaStream_t s) {
        if (dim == 1) ++launches;
#define PGB_L(RR)                                                              \
    do {                                                                       \
        if (dim == 2) {                                                        \
            if (mode == kFwd) launch2d<RR, kFwd>(p, s);                        \
            else if (mode == kRecomp) launch2d<RR, kRecomp>(p, s);             \
            else if (mode == kBorn) launch2d<RR, kBorn>(p, s);                 \
            else launch2d<RR, kAdj>(p, s);                                     \
        } else if (dim == 3) {                                                 \
            if (mode == kFwd) launch3d<RR, kFwd>(p, s);                        \
            else if (mode == kRecomp) launch3d<RR, kRecomp>(p, s);             \
            else launch3d<RR, kAdj>(p, s);                                     \
        } else {                                                               \
            if (mode == kFwd) launch_wave1d<T, RR, kFwd>(p, bz, s);            \
            else if (mode == kRecomp) launch_wave1d<T, RR, kRecomp>(p, bz, s); \
            else launch_wave1d<T, RR, kAdj>(p, bz, s);                         \
        }                                                                      \
    } while (0)
        switch (R) {
            case 1: PGB_L(1); break;
            case 2: PGB_L(2); break;
            case 3: PGB_L(3); break;
            default: PGB_L(4); break;
        }
#undef PGB_L
    }

    // fill the state pointers of a sweep from buffer sets
    State make_state(const size_t* U, const size_t* PX, const size_t* PY, const size_t* PZ,
                     const size_t* PS) const {
        State st{};
        st.prev = at<T>(U[0]); st.cur = at<T>(U[1]);
        for (int b = 0; b < 2; ++b) {
            st.phx[b] = at<T>(PX[b]); st.phy[b] = at<T>(PY[b]);
            st.phz[b] = at<T>(PZ[b]); st.psi[b] = at<T>(PS[b]);
        }
        st.pb = 0;
        return st;
    }

    void bind_state(WaveParams<T>& p, const State& st) const {
        p.u_prev = st.prev; p.u_cur = st.cur;
        p.phx_in = st.phx[st.pb]; p.phx_out = st.phx[st.pb ^ 1];
        p.phy_in = st.phy[st.pb]; p.phy_out = st.phy[st.pb ^ 1];
        p.phz_in = st.phz[st.pb]; p.phz_out = st.phz[st.pb ^ 1];
        p.psi_in = st.psi[st.pb]; p.psi_out = st.psi[st.pb ^ 1];
    }
    static void advance(State& st) { std::swap(st.prev, st.cur); st.pb ^= 1; }

    void zero_state(const size_t* U, const size_t* PX, const size_t* PY, const size_t* PZ,
                    const size_t* PS, cudaStream_t s) const {
        for (int b = 0; b < 2; ++b) {
            cudaMemsetAsync(ws + U[b], 0, field_bytes, s);
            cudaMemsetAsync(ws + PZ[b], 0, field_bytes, s);
            if (dim >= 2) cudaMemsetAsync(ws + PX[b], 0, field_bytes, s);
            if (dim == 3) {
                cudaMemsetAsync(ws + PY[b], 0, field_bytes, s);
                cudaMemsetAsync(ws + PS[b], 0, field_bytes, s);
            }
        }
    }

    // the arrays a checkpoint holds: prev, cur and the input PML state
    void ckpt_ptrs(const State& st, T** v) const {
        int n = 0;
        v[n++] = st.prev; v[n++] = st.cur; v[n++] = st.phz[st.pb];
        if (dim >= 2) v[n++] = st.phx[st.pb];
        if (dim == 3) { v[n++] = st.phy[st.pb]; v[n++] = st.psi[st.pb]; }
    }

    void copy_fields(T* const* dst, T* const* src, cudaStream_t s) const {
        for (int f = 0; f < ckpt_fields; ++f)
            if (dst[f] && src[f]) cudaMemcpyAsync(dst[f], src[f], field_bytes, cudaMemcpyDeviceToDevice, s);
    }

    T* replay_slot(long long i) const { return fld(off.replay) + (size_t)i * fstride * G; }

    T* ckpt_slot(int seg, int f) const {
        return reinterpret_cast<T*>(ws + off.ckpt + ((size_t)seg * ckpt_fields + f) * field_bytes);
    }

    // forward sweep of one group; with `checkpoints` (a gradient follows) it saves the
    // checkpoints, or with store_all writes dWaveOp of every imaged step instead
    void forward_sweep(int g0, int gn, bool checkpoints, cudaStream_t s) {
        zero_state(off.U, off.PX, off.PY, off.PZ, off.PS, s);
        State st = make_state(off.U, off.PX, off.PY, off.PZ, off.PS);
        WaveParams<T> p = base_params(g0, gn);
        T* tr = at<T>(off.traces);
        const bool keep = checkpoints && store_all;
        for (int k = 0; k < nsteps; ++k) {
            if (keep) {
                bind_state(p, st);
                set_inject(p, true, g0, k, nullptr);
                set_recording(p, g0, gn, tr + (long long)k * nrec);
                p.dw_out = (k % p_img == 0) ? replay_slot(k / p_img) : nullptr;
                p.nan_check = 1;
                launch(p, kRecomp, s);
                advance(st);
                continue;
            }
            if (checkpoints && k % S == 0) {
                T* src[6]; T* dst[6];
                ckpt_ptrs(st, src);
                for (int f = 0; f < ckpt_fields; ++f) dst[f] = ckpt_slot(k / S, f);
                copy_fields(dst, src, s);
            }
            bind_state(p, st);
            set_inject(p, true, g0, k, nullptr);
            set_recording(p, g0, gn, tr + (long long)k * nrec);
            launch(p, kFwd, s);
            advance(st);
        }
    }

    void backward_sweep(int g0, int gn, cudaStream_t s, int period = 0) {
        if (period <= 0) period = p_img;
        zero_state(off.A, off.AX, off.AY, off.AZ, off.AS, s);
        cudaMemsetAsync(ws + off.ic, 0, field_bytes, s);
        State adj = make_state(off.A, off.AX, off.AY, off.AZ, off.AS);
        const T* resid = at<T>(off.traces);
        if (store_all) {  // dWaveOp of every imaged step is in the replay buffer already
            WaveParams<T> q = base_params(g0, gn);
            for (int k = nsteps - 1; k >= 0; --k) {
                bind_state(q, adj);
                set_inject(q, false, g0, k, resid);
                q.image = (k % period == 0);
                q.dw_in = replay_slot(k / period);
                q.ic = fld(off.ic);
                launch(q, kAdj, s);
                advance(adj);
            }
            return;
        }
        for (int seg = nseg - 1; seg >= 0; --seg) {
            const int k0 = seg * S, k1 = std::min(k0 + S, nsteps) - 1;
            // restore the forward state at k0 into buffer set 0
            State fw = make_state(off.U, off.PX, off.PY, off.PZ, off.PS);
            {
                T* dst[6]; T* src[6];
                ckpt_ptrs(fw, dst);
                for (int f = 0; f < ckpt_fields; ++f) src[f] = ckpt_slot(seg, f);
                copy_fields(dst, src, s);
            }
            WaveParams<T> p = base_params(g0, gn);
            for (int k = k0; k <= k1; ++k) {
                bind_state(p, fw);
                set_inject(p, true, g0, k, nullptr);
                p.dw_out = (k % period == 0) ? fld(off.replay) + (size_t)(k - k0) * fstride * G : nullptr;
                launch(p, kRecomp, s);
                advance(fw);
            }
            WaveParams<T> q = base_params(g0, gn);
            for (int k = k1; k >= k0; --k) {
                bind_state(q, adj);
                set_inject(q, false, g0, k, resid);
                q.image = (k % period == 0);
                q.dw_in = fld(off.replay) + (size_t)(k - k0) * fstride * G;
                q.ic = fld(off.ic);
                launch(q, kAdj, s);
                advance(adj);
            }
        }
    }

    // Linearised (Born) sweep of one group: the background field u0 (forward buffers) steps in
    // recompute mode, writing dWaveOp0_k into replay slot 0; the scattered field u1 (adjoint
    // buffers) steps without a source, its traces recorded before each step, then takes the
    // Born source -m1 dWaveOp0_k (linear_forward_model, temporal_modeling.py:485-535).  With
    // `checkpoints` the u0 state is saved every S steps as the forward sweep does.
    void born_sweep(int g0, int gn, bool checkpoints, cudaStream_t s) {
        zero_state(off.U, off.PX, off.PY, off.PZ, off.PS, s);
        zero_state(off.A, off.AX, off.AY, off.AZ, off.AS, s);
        State u0 = make_state(off.U, off.PX, off.PY, off.PZ, off.PS);
        State u1 = make_state(off.A, off.AX, off.AY, off.AZ, off.AS);
        WaveParams<T> p0 = base_params(g0, gn), p1 = base_params(g0, gn);
        T* tr = at<T>(off.traces);
        const long long rows = (long long)gn * nx * ny;
        const int nb = (int)std::min<long long>(rows, 152LL * 16);
        for (int k = 0; k < nsteps; ++k) {
            // kept schedule: dWaveOp0 of every step stays for the migration (imaging every step)
            T* dw = checkpoints && store_all ? replay_slot(k) : replay_slot(0);
            if (checkpoints && !store_all && k % S == 0) {
                T* src[6]; T* dst[6];
                ckpt_ptrs(u0, src);
                for (int f = 0; f < ckpt_fields; ++f) dst[f] = ckpt_slot(k / S, f);
                copy_fields(dst, src, s);
            }
            bind_state(p0, u0);
            set_inject(p0, true, g0, k, nullptr);
            p0.dw_out = dw;
            launch(p0, kRecomp, s);
            bind_state(p1, u1);
            set_inject(p1, true, g0, k, nullptr);  // valid tables, switched off: u1 has no source
            p1.inj.on = 0;
            set_recording(p1, g0, gn, tr + (long long)k * nrec);
            if (dim == 2) {  // the Born source read inside the u1 step
                p1.dw_in = dw;
                p1.m1 = at<T>(off.m1);
                launch(p1, kBorn, s);
            } else {
                launch(p1, kFwd, s);
                born_source_kernel<T><<<nb, 128, 0, s>>>(p1, dim, at<T>(off.m1), dw);
                ++launches;
            }
            advance(u0);
            advance(u1);
        }
    }

    void pad_perturbation(const double* m1, cudaStream_t s) {
        const long long n = (long long)nx * ny * nz;
        const int px = nx - pad_lo[0] - pad_hi[0], py = ny - pad_lo[1] - pad_hi[1], pz = nz - pad_lo[2] - pad_hi[2];
        edge_pad_kernel<T><<<grid_for(n, 256), 256, 0, s>>>(m1, nx, ny, nz, pad_lo[0], pad_lo[1], pad_lo[2], px, py,
                                                            pz, hx, hy, rows_y, ldz, at<T>(off.m1));
        ++launches;
    }

    void enqueue_born(const double* m1, void* traces_out, cudaStream_t s) {
        reset_task_counter(s);
        pad_perturbation(m1, s);
        const size_t tr_group = (size_t)nsteps * nrec * sizeof(T);
        for (int g0 = 0; g0 < nshots; g0 += G) {
            const int gn = std::min(G, nshots - g0);
            born_sweep(g0, gn, false, s);
            if (nrec > 0)
                cudaMemcpyAsync(static_cast<char*>(traces_out) + (size_t)g0 * tr_group, ws + off.traces, tr_group * gn,
                                cudaMemcpyDeviceToDevice, s);
        }
    }

    // sum_s F_s* F_s m1: each group's Born traces d1 are migrated at once with the u0
    // checkpoints the Born sweep saved (apply_hessian 'approximate',
    // temporal_least_squares.py:209-217; migrate_shot images every step)
    void enqueue_hessian(const double* m1, double* out, double* d1norm2, cudaStream_t s) {
        reset_task_counter(s);
        pad_perturbation(m1, s);
        cudaMemsetAsync(ws + off.gpad, 0, (size_t)nx * ny * nz * sizeof(double), s);
        cudaMemsetAsync(ws + off.rnorm, 0, sizeof(double), s);
        for (int g0 = 0; g0 < nshots; g0 += G) {
            const int gn = std::min(G, nshots - g0);
            born_sweep(g0, gn, true, s);
            const long long n = (long long)gn * nsteps * nrec;
            if (n > 0) {  // ||d1||^2, and a shot's record ends at its own length
                residual_kernel<T><<<kRedBlocks, kRedThreads, 0, s>>>(
                    nullptr, at<T>(off.traces), n, at<double>(off.partial), 1,
                    shot_steps.empty() ? nullptr : at<int>(off.shsteps) + g0, nsteps, nrec);
                sum_partials_kernel<<<1, kRedThreads, 0, s>>>(at<double>(off.partial), kRedBlocks, at<double>(off.rnorm),
                                                              1);
                launches += 2;
            }
            backward_sweep(g0, gn, s, 1);
            const long long nc = (long long)nx * ny * nz;
            reduce_ic_kernel<T><<<grid_for(nc, 256), 256, 0, s>>>(fld(off.ic), fstride, gn, nx, ny, nz, hx, hy, rows_y,
                                                                  ldz, -dt, at<double>(off.gpad));
            ++launches;
        }
        const int px = nx - pad_lo[0] - pad_hi[0], py = ny - pad_lo[1] - pad_hi[1], pz = nz - pad_lo[2] - pad_hi[2];
        fold_kernel<<<grid_for((long long)px * py * pz, 256), 256, 0, s>>>(at<double>(off.gpad), nx, ny, nz, pad_lo[0],
                                                                           pad_hi[0], pad_lo[1], pad_hi[1], pad_lo[2],
                                                                           pad_hi[2], out);
        ++launches;
        if (d1norm2) cudaMemcpyAsync(d1norm2, ws + off.rnorm, sizeof(double), cudaMemcpyDeviceToDevice, s);
    }

    int born(const double* m1, void* traces, cudaStream_t s) override {
        PGB_REQUIRE(ws, "no workspace bound");
        PGB_REQUIRE(!fwd_only, "the plan was built for forward modelling only");
        PGB_REQUIRE(model_set, "pysit_plan_set_model must be called first");
        PGB_REQUIRE(m1, "NULL model perturbation");
        PGB_REQUIRE(traces || nrec == 0, "NULL traces output");
        return run(4, m1, traces, nullptr, nullptr, s, [&](cudaStream_t st) { enqueue_born(m1, traces, st); });
    }

    int hessian(const double* m1, double* out, double* d1norm2, cudaStream_t s) override {
        PGB_REQUIRE(ws, "no workspace bound");
        PGB_REQUIRE(!fwd_only, "the plan was built for forward modelling only");
        PGB_REQUIRE(!store_all || p_img == 1, "a plan that keeps dWaveOp applies the Hessian with imaging_period 1 only");
        PGB_REQUIRE(model_set, "pysit_plan_set_model must be called first");
        PGB_REQUIRE(m1 && out, "NULL argument");
        return run(5, m1, out, d1norm2, nullptr, s,
                   [&](cudaStream_t st) { enqueue_hessian(m1, out, d1norm2, st); });
    }

    // the 2D sweep's task counter restarts at zero with every run (eager or graph replay)
    void reset_task_counter(cudaStream_t s) {
        cudaMemsetAsync(ws + off.ctr, 0, 2 * sizeof(unsigned long long), s);
        ctr_next[0] = ctr_next[1] = 0;
    }

    // n launches of one step kernel on the first shot group's buffers, for timing
    // (the state keeps evolving from whatever the last run left; no output)
    int step_loop(int mode, int n, cudaStream_t s) override {
        PGB_REQUIRE(ws, "no workspace bound");
        PGB_REQUIRE(model_set, "pysit_plan_set_model must be called first");
        PGB_REQUIRE(mode >= kFwd && mode <= kAdj, "mode must be 0 (forward), 1 (recompute) or 2 (adjoint)");
        PGB_REQUIRE(!fwd_only || mode == kFwd, "the plan was built for forward modelling only");
        PGB_REQUIRE(n >= 0, "nsteps must be >= 0");
        launches = 0;
        reset_task_counter(s);
        const int gn = std::min(G, nshots);
        WaveParams<T> p = base_params(0, gn);
        State st = mode == kAdj ? make_state(off.A, off.AX, off.AY, off.AZ, off.AS)
                                : make_state(off.U, off.PX, off.PY, off.PZ, off.PS);
        for (int i = 0; i < n; ++i) {
            const int k = i % nsteps;
            bind_state(p, st);
            if (mode == kAdj) {
                set_inject(p, false, 0, k, at<T>(off.traces));
                p.image = 1;
                p.dw_in = replay_slot(k % nslots);
                p.ic = fld(off.ic);
            } else {
                set_inject(p, true, 0, k, nullptr);
                if (mode == kRecomp) p.dw_out = replay_slot(k % nslots);
                // the forward sweep records traces (the kept schedule's runs in recompute mode)
                if (mode == kFwd || store_all) set_recording(p, 0, gn, at<T>(off.traces) + (long long)k * nrec);
            }
            launch(p, mode, s);
            advance(st);
        }
        PGB_CHECK_CUDA(cudaGetLastError());
        last_launches = launches;
        return PYSIT_OK;
    }

    int autotune(const int* cand, int ncand, int n, int* chosen, double* ms_out, cudaStream_t s) override {
        int cz = tz, chosen_z = 0;
        return autotune2(cand, ncand, &cz, 1, n, chosen, &chosen_z, ms_out, s);
    }

    // Every (x length, z extent) pair is timed twice, the second pass in reverse order; each
    // keeps its faster time and the fastest pair stays.  ms_out[ix * ncz + iz].
    int autotune2(const int* cx, int ncx, const int* cz, int ncz, int n, int* chosen_x, int* chosen_z,
                  double* ms_out, cudaStream_t s) override {
        PGB_REQUIRE(ws, "no workspace bound");
        PGB_REQUIRE(model_set, "pysit_plan_set_model must be called first");
        PGB_REQUIRE(dim >= 2, "autotuning applies to the 2D and 3D task sweeps");
        PGB_REQUIRE(cx && ncx >= 1 && cz && ncz >= 1 && chosen_x && chosen_z, "need candidates and outputs");
        PGB_REQUIRE(n >= 1, "nsteps must be >= 1");
        for (int c = 0; c < ncx; ++c)
            PGB_REQUIRE(cx[c] >= kMinTileX && cx[c] <= 4096, "candidate task length %d outside [%d, 4096]", cx[c],
                        kMinTileX);
        for (int c = 0; c < ncz; ++c)
            PGB_REQUIRE(cz[c] == 0 || cz[c] >= kMinTileZ, "candidate z extent %d below %d (0: full width)", cz[c],
                        kMinTileZ);
        cudaEvent_t e0, e1;
        PGB_CHECK_CUDA(cudaEventCreate(&e0));
        PGB_CHECK_CUDA(cudaEventCreate(&e1));
        const int nc = ncx * ncz;
        int best = 0;
        float best_ms = 1e30f;
        int rc = PYSIT_OK;
        std::vector<float> t(nc, 1e30f);
        for (int pass = 0; pass < 2 && rc == PYSIT_OK; ++pass)
            for (int i = 0; i < nc && rc == PYSIT_OK; ++i) {
                const int c = pass == 0 ? i : nc - 1 - i;
                if ((rc = use_tile(cx[c / ncz], cz[c % ncz], s))) break;
                // the sweeps a gradient runs: forward (in recompute mode when dWaveOp is kept) and adjoint
                const int fmode = store_all ? kRecomp : kFwd;
                if ((rc = step_loop(fmode, 2, s))) break;  // warm-up
                cudaEventRecord(e0, s);
                if ((rc = step_loop(fmode, n, s)) || (!fwd_only && (rc = step_loop(kAdj, n, s)))) break;
                cudaEventRecord(e1, s);
                if (cudaEventSynchronize(e1) != cudaSuccess) { rc = cuda_status(cudaGetLastError(), "autotune"); break; }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                t[c] = std::min(t[c], ms);
            }
        for (int c = 0; c < nc && rc == PYSIT_OK; ++c) {
            if (ms_out) ms_out[c] = t[c];
            if (t[c] < best_ms) { best_ms = t[c]; best = c; }
        }
        if (rc == PYSIT_OK) rc = use_tile(cx[best / ncz], cz[best % ncz], s);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc) return rc;
        *chosen_x = cx[best / ncz];
        *chosen_z = cz[best % ncz];
        return PYSIT_OK;
    }

    int tiles(int* tile_x, int* tile_z) const override {
        if (tile_x) *tile_x = tx;
        if (tile_z) *tile_z = tz;
        return PYSIT_OK;
    }

    int task_table(int32_t* out, uint64_t cap, uint64_t* n_ints, int32_t* n_interior) const override {
        static const std::vector<int> none;
        const std::vector<int>& tab = dim == 3 ? tasks3d : dim == 2 ? tasks2d : none;
        if (n_ints) *n_ints = tab.size();
        if (n_interior) *n_interior = dim == 3 ? ntask3d[0] : dim == 2 ? ntask2d[0] : 0;
        if (out) std::copy_n(tab.begin(), std::min<size_t>((size_t)cap, tab.size()), out);
        return PYSIT_OK;
    }

    int tuning(int* tile, double* share) const override {
        if (tile) *tile = tx;
        if (share)
            for (int m = 0; m < 3; ++m) share[m] = shell_frac[m];
        return PYSIT_OK;
    }

    // rebuild and upload the task table for task length t and z extent z; captured graphs
    // hold the old table's counts, so they are dropped
    int use_tile(int t, int z, cudaStream_t s) {
        tx = t;
        tz = z > 0 ? z / 4 * 4 : 0;
        std::vector<int>& tab = dim == 3 ? (build_tasks3d(), tasks3d) : (build_tasks2d(), tasks2d);
        PGB_REQUIRE(tab.size() <= task_cap, "task table of %zu ints exceeds its buffer (%zu)", tab.size(), task_cap);
        PGB_CHECK_CUDA(cudaMemcpyAsync(ws + off.tasks, tab.data(), tab.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        PGB_CHECK_CUDA(cudaStreamSynchronize(s));
        for (auto& kv : graphs)
            if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
        graphs.clear();
        seen.clear();
        return PYSIT_OK;
    }

    void set_recording(WaveParams<T>& p, int g0, int gn, T* tr_k) const {
        p.rec.rowptr = at<int>(off.recrow) + (size_t)g0 * nrec;
        p.rec.off = at<long long>(off.recoff);
        p.rec.w = at<T>(off.recw);
        p.rec.traces = tr_k;
        p.rec.tr_sstride = (long long)nsteps * nrec;
        p.rec.nrec = nrec;
        p.rec.lanes = rec_lanes;
        // 2D: the recorder blocks lead the interior kernel's grid and hold one of its block
        // slots each while they run, so a few of them stride over the receivers and the step's
        // own blocks take the other slots from the start
        if (rec_cap == 0) {
            int dev = 0, sms = 0;
            if (cudaGetDevice(&dev) != cudaSuccess ||
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
                cudaGetLastError();
                sms = 1;
            }
            rec_cap = std::max(1, sms * PGB_REC_BLOCKS_PER_SM);
        }
        const long long need = nrec > 0 ? ceil_div((long long)gn * nrec * rec_lanes, bz) : 0;
        p.rec.blocks = (int)(dim == 2 ? std::min<long long>(need, (long long)rec_cap) : need);
    }

    void enqueue_forward(void* traces_out, cudaStream_t s) {
        reset_task_counter(s);
        const size_t tr_group = (size_t)nsteps * nrec * sizeof(T);
        for (int g0 = 0; g0 < nshots; g0 += G) {
            int gn = std::min(G, nshots - g0);
            forward_sweep(g0, gn, false, s);
            if (traces_out && nrec > 0)
                cudaMemcpyAsync(static_cast<char*>(traces_out) + (size_t)g0 * tr_group, ws + off.traces,
                                tr_group * gn, cudaMemcpyDeviceToDevice, s);
        }
    }

    void enqueue_gradient(const void* dobs, double* grad, double* rnorm2, void* traces_out, bool with_grad,
                          bool migrate, cudaStream_t s) {
        reset_task_counter(s);
        const size_t tr_group = (size_t)nsteps * nrec * sizeof(T);
        if (with_grad) cudaMemsetAsync(ws + off.gpad, 0, (size_t)nx * ny * nz * sizeof(double), s);
        cudaMemsetAsync(ws + off.rnorm, 0, sizeof(double), s);
        for (int g0 = 0; g0 < nshots; g0 += G) {
            int gn = std::min(G, nshots - g0);
            forward_sweep(g0, gn, with_grad, s);
            if (traces_out && nrec > 0)
                cudaMemcpyAsync(static_cast<char*>(traces_out) + (size_t)g0 * tr_group, ws + off.traces,
                                tr_group * gn, cudaMemcpyDeviceToDevice, s);
            long long n = (long long)gn * nsteps * nrec;
            if (n > 0) {
                residual_kernel<T><<<kRedBlocks, kRedThreads, 0, s>>>(
                    static_cast<const T*>(dobs) + (size_t)g0 * nsteps * nrec, at<T>(off.traces), n,
                    at<double>(off.partial), migrate ? 1 : 0, shot_steps.empty() ? nullptr : at<int>(off.shsteps) + g0,
                    nsteps, nrec);
                sum_partials_kernel<<<1, kRedThreads, 0, s>>>(at<double>(off.partial), kRedBlocks,
                                                              at<double>(off.rnorm), 1);
                launches += 2;
            }
            if (with_grad) {
                backward_sweep(g0, gn, s);
                long long nc = (long long)nx * ny * nz;
                // migration returns F* r = -dt p sum q dWaveOp (adjoint_model, :367-371);
                // the gradient is its negative (compute_gradient, :167)
                reduce_ic_kernel<T><<<grid_for(nc, 256), 256, 0, s>>>(
                    fld(off.ic), fstride, gn, nx, ny, nz, hx, hy, rows_y, ldz,
                    migrate ? -dt * p_img : dt * p_img, at<double>(off.gpad));
                ++launches;
            }
        }
        if (with_grad) {
            const int px = nx - pad_lo[0] - pad_hi[0], py = ny - pad_lo[1] - pad_hi[1],
                      pz = nz - pad_lo[2] - pad_hi[2];
            fold_kernel<<<grid_for((long long)px * py * pz, 256), 256, 0, s>>>(
                at<double>(off.gpad), nx, ny, nz, pad_lo[0], pad_hi[0], pad_lo[1], pad_hi[1], pad_lo[2],
                pad_hi[2], grad);
            ++launches;
        }
        cudaMemcpyAsync(rnorm2, ws + off.rnorm, sizeof(double), cudaMemcpyDeviceToDevice, s);
    }

    // run `enqueue` eagerly or through a cached CUDA graph keyed by the I/O pointers
    template <typename F>
    int run(int kind, const void* a, const void* b, const void* c, const void* d, cudaStream_t s, F enqueue) {
        if (!use_graph) {
            launches = 0;
            enqueue(s);
            PGB_CHECK_CUDA(cudaGetLastError());
            last_launches = launches;
            return PYSIT_OK;
        }
        GraphKey key{kind, a, b, c, d};
        auto it = graphs.find(key);
        if (it == graphs.end() && seen.insert(key).second) {
            // first use: launched as it is enqueued (a graph pays off from the second use on;
            // an optimiser's line search often calls a plan only once or twice)
            launches = 0;
            enqueue(s);
            PGB_CHECK_CUDA(cudaGetLastError());
            last_launches = launches;
            return PYSIT_OK;
        }
        if (it == graphs.end()) {
            launches = 0;
            cudaGraph_t graph = nullptr;
            PGB_CHECK_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
            capture_into(cap, [&] { enqueue(cap); });
            cudaError_t e = cudaStreamEndCapture(cap, &graph);
            if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture");
            GraphRec rec;
            e = cudaGraphInstantiate(&rec.exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return cuda_status(e, "cudaGraphInstantiate");
            rec.launches = launches;
            it = graphs.emplace(key, rec).first;
        }
        PGB_CHECK_CUDA(cudaGraphLaunch(it->second.exec, s));
        last_launches = it->second.launches;
        return PYSIT_OK;
    }

    int forward(void* traces, cudaStream_t s) override {
        PGB_REQUIRE(ws, "no workspace bound");
        PGB_REQUIRE(model_set, "pysit_plan_set_model must be called first");
        return run(0, traces, nullptr, nullptr, nullptr, s,
                   [&](cudaStream_t st) { enqueue_forward(traces, st); });
    }

    int gradient(const void* dobs, double* grad, double* rnorm2, void* traces, cudaStream_t s,
                 bool with_grad, bool migrate) override {
        PGB_REQUIRE(ws, "no workspace bound");
        PGB_REQUIRE(model_set, "pysit_plan_set_model must be called first");
        PGB_REQUIRE(dobs || nrec == 0, "NULL observed data");
        PGB_REQUIRE(rnorm2, "NULL misfit output");
        PGB_REQUIRE(!fwd_only || !with_grad, "the plan was built for forward modelling only");
        PGB_REQUIRE(!with_grad || grad, "NULL gradient output");
        return run(migrate ? 3 : with_grad ? 1 : 2, dobs, grad, rnorm2, traces, s, [&](cudaStream_t st) {
            enqueue_gradient(dobs, grad, rnorm2, traces, with_grad, migrate, st);
        });
    }

    int enqueue_grad_raw(const void* dobs, double* grad, double* rnorm2, cudaStream_t s) override {
        PGB_REQUIRE(ws, "no workspace bound");
        PGB_REQUIRE(model_set, "pysit_plan_set_model must be called first");
        PGB_REQUIRE((dobs || nrec == 0) && grad && rnorm2, "NULL argument");
        PGB_REQUIRE(!fwd_only, "the plan was built for forward modelling only");
        launches = 0;
        enqueue_gradient(dobs, grad, rnorm2, nullptr, true, false, s);
        last_launches = launches;
        return PYSIT_OK;
    }
};

// out[i] = sum over lanes of g[lane][i] (lanes in order: deterministic); rn_out = sum of rn
__global__ void lanes_sum_kernel(const double* __restrict__ g, int lanes, long long n, double* __restrict__ out,
                                 const double* __restrict__ rn, double* __restrict__ rn_out) {
    if (out)
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
             i += (long long)gridDim.x * blockDim.x) {
            double a = 0.0;
            for (int c = 0; c < lanes; ++c) a += g[(long long)c * n + i];
            out[i] = a;
        }
    if (rn_out && blockIdx.x == 0 && threadIdx.x == 0) {
        double a = 0.0;
        for (int c = 0; c < lanes; ++c) a += rn[c];
        *rn_out = a;
    }
}

// A plan whose shots are split into `lanes` contiguous ranges, each a plan of its own
// (own workspace slice, streams and task counters), whose launch sequences run side by side:
// forked from the caller's stream, joined back, captured in one graph.  The sequences never
// wait for each other, so one lane's step kernels fill the gaps at the other's step
// boundaries.  Gradients, images and misfits of the lanes are summed in a fixed order.
template <typename T>
struct LanesPlan final : public pysit_plan {
    std::vector<std::unique_ptr<PlanT<T>>> kids;
    std::vector<int> first;             // first shot of each lane
    std::vector<size_t> kid_off;        // workspace offset of each lane
    size_t off_g = 0, off_rn = 0;       // per-lane unpadded sums and misfits
    long long ndof = 0;                 // unpadded cells
    size_t tr_shot = 0;                 // bytes of one shot's traces
    uint64_t ws_need = 0;
    char* ws = nullptr;
    int use_graph = 1;
    std::vector<cudaStream_t> st;
    std::vector<cudaEvent_t> done;
    cudaEvent_t root = nullptr;
    cudaStream_t cap = nullptr;
    struct Key {
        int kind;
        const void *a, *b, *c, *d;
        bool operator<(const Key& o) const {
            return std::tie(kind, a, b, c, d) < std::tie(o.kind, o.a, o.b, o.c, o.d);
        }
    };
    std::map<Key, std::pair<cudaGraphExec_t, int64_t>> graphs;
    std::set<Key> seen;

    ~LanesPlan() override {
        for (auto& kv : graphs)
            if (kv.second.first) cudaGraphExecDestroy(kv.second.first);
        for (auto x : st) cudaStreamDestroy(x);
        for (auto e : done) cudaEventDestroy(e);
        if (root) cudaEventDestroy(root);
        if (cap) cudaStreamDestroy(cap);
    }

    int init(const pysit_plan_desc& d, int lanes) {
        use_graph = d.use_graph;
        for (int c = 0; c < lanes; ++c) {
            const int s0 = (int)((long long)c * d.nshots / lanes), s1 = (int)((long long)(c + 1) * d.nshots / lanes);
            first.push_back(s0);
            pysit_plan_desc k = d;  // the lane's shots: per-shot arrays re-based at s0
            std::vector<int64_t> sp, rp;
            k.nshots = s1 - s0;
            k.shots_per_launch = std::min(d.shots_per_launch, s1 - s0);
            k.lanes = 1;
            if (d.src_tap_ptr) {
                const int64_t b = d.src_tap_ptr[s0];
                for (int q = s0; q <= s1; ++q) sp.push_back(d.src_tap_ptr[q] - b);
                k.src_tap_ptr = sp.data();
                if (d.src_tap_cell) k.src_tap_cell = d.src_tap_cell + b;
                if (d.src_tap_point) k.src_tap_point = d.src_tap_point + b;
                if (d.src_tap_w) k.src_tap_w = d.src_tap_w + b;
            }
            if (d.src_amp) k.src_amp = d.src_amp + (size_t)s0 * d.nsteps * d.nsrc;
            if (d.rec_tap_ptr) {
                const int64_t b = d.rec_tap_ptr[s0];
                for (int q = s0; q <= s1; ++q) rp.push_back(d.rec_tap_ptr[q] - b);
                k.rec_tap_ptr = rp.data();
                if (d.rec_tap_cell) k.rec_tap_cell = d.rec_tap_cell + b;
                if (d.rec_tap_point) k.rec_tap_point = d.rec_tap_point + b;
                if (d.rec_tap_wsample) k.rec_tap_wsample = d.rec_tap_wsample + b;
                if (d.rec_tap_winject) k.rec_tap_winject = d.rec_tap_winject + b;
            }
            if (d.shot_nsteps) k.shot_nsteps = d.shot_nsteps + s0;
            auto kid = std::make_unique<PlanT<T>>();
            int rc = kid->init(k);  // copies everything it keeps: the re-based arrays may go
            if (rc) return rc;
            kids.push_back(std::move(kid));
        }
        const PlanT<T>& k0 = *kids[0];
        ndof = (long long)(k0.nx - k0.pad_lo[0] - k0.pad_hi[0]) * (k0.ny - k0.pad_lo[1] - k0.pad_hi[1]) *
               (k0.nz - k0.pad_lo[2] - k0.pad_hi[2]);
        tr_shot = (size_t)k0.nsteps * k0.nrec * sizeof(T);
        size_t tot = 0;
        auto take = [&](size_t bytes) { size_t o = tot; tot += (bytes + 255) / 256 * 256; return o; };
        for (auto& kid : kids) kid_off.push_back(take(kid->ws_need));
        off_g = take((size_t)lanes * ndof * sizeof(double));
        off_rn = take((size_t)lanes * sizeof(double));
        ws_need = tot;
        return PYSIT_OK;
    }

    int lanes() const { return (int)kids.size(); }
    double* g_lane(int c) const { return reinterpret_cast<double*>(ws + off_g) + (size_t)c * ndof; }
    double* rn_lane(int c) const { return reinterpret_cast<double*>(ws + off_rn) + c; }
    template <typename P> static P* shift(P* base, size_t bytes) {
        return base ? reinterpret_cast<P*>(reinterpret_cast<char*>(const_cast<void*>(static_cast<const void*>(base))) + bytes) : nullptr;
    }

    int workspace_bytes(uint64_t* b) const override { *b = ws_need; return PYSIT_OK; }

    int bind(void* w, uint64_t bytes, cudaStream_t s) override {
        PGB_REQUIRE(w != nullptr, "NULL workspace");
        PGB_REQUIRE(aligned(w, 256), "workspace must be 256-byte aligned");
        PGB_REQUIRE(bytes >= ws_need, "workspace too small: %llu < %llu bytes", (unsigned long long)bytes,
                    (unsigned long long)ws_need);
        for (auto& kv : graphs)
            if (kv.second.first) cudaGraphExecDestroy(kv.second.first);
        graphs.clear();
        seen.clear();
        ws = static_cast<char*>(w);
        for (int c = 0; c < lanes(); ++c) {
            int rc = kids[c]->bind(ws + kid_off[c], kids[c]->ws_need, s);
            if (rc) return rc;
        }
        PGB_CHECK_CUDA(cudaMemsetAsync(ws + off_g, 0, ws_need - off_g, s));
        if (!cap) {
            PGB_CHECK_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
            PGB_CHECK_CUDA(cudaEventCreateWithFlags(&root, cudaEventDisableTiming));
            for (int c = 0; c < lanes(); ++c) {
                cudaStream_t x;
                cudaEvent_t e;
                PGB_CHECK_CUDA(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
                st.push_back(x);
                PGB_CHECK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
                done.push_back(e);
            }
        }
        return PYSIT_OK;
    }

    int set_model(const double* C, cudaStream_t s) override {
        for (auto& kid : kids) {
            int rc = kid->set_model(C, s);
            if (rc) return rc;
        }
        return PYSIT_OK;
    }

    int status(int* flags, cudaStream_t s) override {
        int all = 0;
        for (auto& kid : kids) {
            int f = 0, rc = kid->status(&f, s);
            if (rc) return rc;
            all |= f;
        }
        *flags = all;
        return PYSIT_OK;
    }

    // every lane's sequence on its own stream, forked from s and joined back into s
    template <typename F>
    void fork(cudaStream_t s, F fn) {
        cudaEventRecord(root, s);
        for (int c = 0; c < lanes(); ++c) {
            cudaStreamWaitEvent(st[c], root, 0);
            fn(c, st[c]);
            cudaEventRecord(done[c], st[c]);
        }
        for (int c = 0; c < lanes(); ++c) cudaStreamWaitEvent(s, done[c], 0);
    }

    void sum(double* out, double* rn_out, cudaStream_t s) {
        lanes_sum_kernel<<<grid_for(ndof, 256), 256, 0, s>>>(reinterpret_cast<const double*>(ws + off_g), lanes(), ndof,
                                                            out, reinterpret_cast<const double*>(ws + off_rn), rn_out);
    }

    int64_t kid_launches() const {
        int64_t n = 0;
        for (auto& kid : kids) n += kid->launches;
        return n;
    }

    template <typename F>
    int run(int kind, const void* a, const void* b, const void* c, const void* d, cudaStream_t s, F enqueue) {
        for (auto& kid : kids) kid->launches = 0;
        if (!use_graph) {
            enqueue(s);
            PGB_CHECK_CUDA(cudaGetLastError());
            last_launches = kid_launches() + 1;
            return PYSIT_OK;
        }
        Key key{kind, a, b, c, d};
        auto it = graphs.find(key);
        if (it == graphs.end() && seen.insert(key).second) {  // first use: eager, as PlanT::run
            enqueue(s);
            PGB_CHECK_CUDA(cudaGetLastError());
            last_launches = kid_launches() + 1;
            return PYSIT_OK;
        }
        if (it == graphs.end()) {
            cudaGraph_t graph = nullptr;
            PGB_CHECK_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
            capture_into(cap, [&] { enqueue(cap); });
            cudaError_t e = cudaStreamEndCapture(cap, &graph);
            if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture");
            cudaGraphExec_t exec = nullptr;
            e = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return cuda_status(e, "cudaGraphInstantiate");
            it = graphs.emplace(key, std::make_pair(exec, kid_launches() + 1)).first;
        }
        PGB_CHECK_CUDA(cudaGraphLaunch(it->second.first, s));
        last_launches = it->second.second;
        return PYSIT_OK;
    }

    int ready() const {
        PGB_REQUIRE(ws, "no workspace bound");
        PGB_REQUIRE(kids[0]->model_set, "pysit_plan_set_model must be called first");
        return PYSIT_OK;
    }

    int forward(void* traces, cudaStream_t s) override {
        if (int rc = ready()) return rc;
        return run(0, traces, nullptr, nullptr, nullptr, s, [&](cudaStream_t q) {
            fork(q, [&](int c, cudaStream_t x) { kids[c]->enqueue_forward(shift(traces, first[c] * tr_shot), x); });
        });
    }

    void enqueue_grad(const void* dobs, double* grad, double* rnorm2, void* traces, bool with_grad, bool migrate,
                      cudaStream_t q) {
        fork(q, [&](int c, cudaStream_t x) {
            kids[c]->enqueue_gradient(shift(dobs, first[c] * tr_shot), with_grad ? g_lane(c) : nullptr, rn_lane(c),
                                      shift(traces, first[c] * tr_shot), with_grad, migrate, x);
        });
        sum(with_grad ? grad : nullptr, rnorm2, q);
    }

    int gradient(const void* dobs, double* grad, double* rnorm2, void* traces, cudaStream_t s, bool with_grad,
                 bool migrate) override {
        if (int rc = ready()) return rc;
        const PlanT<T>& k0 = *kids[0];
        PGB_REQUIRE(dobs || k0.nrec == 0, "NULL observed data");
        PGB_REQUIRE(rnorm2, "NULL misfit output");
        PGB_REQUIRE(!k0.fwd_only || !with_grad, "the plan was built for forward modelling only");
        PGB_REQUIRE(!with_grad || grad, "NULL gradient output");
        return run(migrate ? 3 : with_grad ? 1 : 2, dobs, grad, rnorm2, traces, s, [&](cudaStream_t q) {
            enqueue_grad(dobs, grad, rnorm2, traces, with_grad, migrate, q);
        });
    }

    int enqueue_grad_raw(const void* dobs, double* grad, double* rnorm2, cudaStream_t s) override {
        if (int rc = ready()) return rc;
        PGB_REQUIRE((dobs || kids[0]->nrec == 0) && grad && rnorm2, "NULL argument");
        PGB_REQUIRE(!kids[0]->fwd_only, "the plan was built for forward modelling only");
        for (auto& kid : kids) kid->launches = 0;
        enqueue_grad(dobs, grad, rnorm2, nullptr, true, false, s);
        last_launches = kid_launches() + 1;
        return PYSIT_OK;
    }

    int born(const double* m1, void* traces, cudaStream_t s) override {
        if (int rc = ready()) return rc;
        PGB_REQUIRE(!kids[0]->fwd_only, "the plan was built for forward modelling only");
        PGB_REQUIRE(m1, "NULL model perturbation");
        PGB_REQUIRE(traces || kids[0]->nrec == 0, "NULL traces output");
        return run(4, m1, traces, nullptr, nullptr, s, [&](cudaStream_t q) {
            fork(q, [&](int c, cudaStream_t x) { kids[c]->enqueue_born(m1, shift(traces, first[c] * tr_shot), x); });
        });
    }

    int hessian(const double* m1, double* out, double* d1norm2, cudaStream_t s) override {
        if (int rc = ready()) return rc;
        const PlanT<T>& k0 = *kids[0];
        PGB_REQUIRE(!k0.fwd_only, "the plan was built for forward modelling only");
        PGB_REQUIRE(!k0.store_all || k0.p_img == 1, "a plan that keeps dWaveOp applies the Hessian with imaging_period 1 only");
        PGB_REQUIRE(m1 && out, "NULL argument");
        return run(5, m1, out, d1norm2, nullptr, s, [&](cudaStream_t q) {
            fork(q, [&](int c, cudaStream_t x) { kids[c]->enqueue_hessian(m1, g_lane(c), rn_lane(c), x); });
            sum(out, d1norm2, q);
        });
    }

    // timing and tuning act on the first lane's buffers; the chosen task length goes to all
    int step_loop(int mode, int n, cudaStream_t s) override {
        int rc = kids[0]->step_loop(mode, n, s);
        last_launches = kids[0]->last_launches;
        return rc;
    }
    int autotune(const int* cand, int ncand, int n, int* chosen, double* ms, cudaStream_t s) override {
        int cz = 0, chosen_z = 0;
        kids[0]->tiles(nullptr, &cz);
        return autotune2(cand, ncand, &cz, 1, n, chosen, &chosen_z, ms, s);
    }
    int autotune2(const int* cx, int ncx, const int* cz, int ncz, int n, int* chosen_x, int* chosen_z, double* ms,
                  cudaStream_t s) override {
        int rc = kids[0]->autotune2(cx, ncx, cz, ncz, n, chosen_x, chosen_z, ms, s);
        for (int c = 1; c < lanes() && rc == PYSIT_OK; ++c) rc = kids[c]->use_tile(*chosen_x, *chosen_z, s);
        for (auto& kv : graphs)
            if (kv.second.first) cudaGraphExecDestroy(kv.second.first);
        graphs.clear();
        seen.clear();
        return rc;
    }
    int tuning(int* tile, double* share) const override { return kids[0]->tuning(tile, share); }
    int tiles(int* tile_x, int* tile_z) const override { return kids[0]->tiles(tile_x, tile_z); }
    int task_table(int32_t* out, uint64_t cap, uint64_t* n_ints, int32_t* n_interior) const override {
        return kids[0]->task_table(out, cap, n_ints, n_interior);
    }
};

}  // namespace
}  // namespace pgb

using namespace pgb;

extern "C" int pysit_plan_create(const pysit_plan_desc* d, pysit_plan** out) try {
    PGB_REQUIRE(d && out, "NULL argument");
    *out = nullptr;
    PGB_REQUIRE(d->dim >= 1 && d->dim <= 3, "dim must be 1, 2 or 3");
    PGB_REQUIRE(d->order == 2 || d->order == 4 || d->order == 6 || d->order == 8, "order must be 2/4/6/8");
    PGB_REQUIRE(d->dtype == PYSIT_F32 || d->dtype == PYSIT_F64, "bad dtype");
    PGB_REQUIRE(d->nsteps >= 1, "nsteps must be >= 1");
    PGB_REQUIRE(d->dt > 0, "dt must be positive");
    PGB_REQUIRE(d->nshots >= 1 && d->shots_per_launch >= 1, "need at least one shot");
    PGB_REQUIRE(d->imaging_period >= 1 && d->checkpoint_every >= 1, "imaging_period / checkpoint_every must be >= 1");
    PGB_REQUIRE(d->nsrc >= 0 && d->nrec >= 0, "negative point counts");
    PGB_REQUIRE(d->nsrc == 0 || (d->src_tap_ptr && d->src_amp), "source taps / amplitudes missing");
    PGB_REQUIRE(d->nrec == 0 || d->rec_tap_ptr, "receiver taps missing");
    for (int a = 0; a < 3; ++a) {
        bool used = (d->dim == 1 && a == 2) || (d->dim == 2 && a != 1) || d->dim == 3;
        if (!used) continue;
        PGB_REQUIRE(d->n[a] >= 3, "grid axis %d must have >= 3 cells", a);
        PGB_REQUIRE(d->delta[a] > 0, "grid spacing on axis %d must be positive", a);
        PGB_REQUIRE(d->pad_lo[a] >= 0 && d->pad_hi[a] >= 0 && d->pad_lo[a] + d->pad_hi[a] < d->n[a],
                    "bad padding on axis %d", a);
    }
    if (d->dim == 3) PGB_REQUIRE(d->n[1] >= 3, "3D needs ny >= 3");
    std::unique_ptr<pysit_plan> p;
    int rc;
    const int lanes = std::min(std::max(d->lanes, 1), d->nshots);
    if (lanes > 1 && d->dtype == PYSIT_F64) {
        auto q = std::make_unique<LanesPlan<double>>();
        rc = q->init(*d, lanes);
        p = std::move(q);
    } else if (lanes > 1) {
        auto q = std::make_unique<LanesPlan<float>>();
        rc = q->init(*d, lanes);
        p = std::move(q);
    } else if (d->dtype == PYSIT_F64) {
        auto q = std::make_unique<PlanT<double>>();
        rc = q->init(*d);
        p = std::move(q);
    } else {
        auto q = std::make_unique<PlanT<float>>();
        rc = q->init(*d);
        p = std::move(q);
    }
    if (rc) return rc;
    *out = p.release();
    return PYSIT_OK;
} PGB_API_CATCH("pysit_plan_create")

extern "C" int pysit_plan_destroy(pysit_plan* p) try {
    delete p;
    return PYSIT_OK;
} PGB_API_CATCH("pysit_plan_destroy")

extern "C" int pysit_plan_workspace_bytes(const pysit_plan* p, uint64_t* bytes) try {
    PGB_REQUIRE(p && bytes, "NULL argument");
    return p->workspace_bytes(bytes);
} PGB_API_CATCH("pysit_plan_workspace_bytes")

extern "C" int pysit_plan_bind_workspace(pysit_plan* p, void* ws, uint64_t bytes, void* stream) try {
    PGB_REQUIRE(p, "NULL plan");
    return p->bind(ws, bytes, (cudaStream_t)stream);
} PGB_API_CATCH("pysit_plan_bind_workspace")

extern "C" int pysit_plan_set_model(pysit_plan* p, const double* C, void* stream) try {
    PGB_REQUIRE(p, "NULL plan");
    return p->set_model(C, (cudaStream_t)stream);
} PGB_API_CATCH("pysit_plan_set_model")

extern "C" int pysit_plan_forward(pysit_plan* p, void* traces, void* stream) try {
    PGB_REQUIRE(p, "NULL plan");
    return p->forward(traces, (cudaStream_t)stream);
} PGB_API_CATCH("pysit_plan_forward")

extern "C" int pysit_plan_gradient(pysit_plan* p, const void* dobs, double* grad, double* rnorm2,
                                   void* traces, void* stream) try {
    PGB_REQUIRE(p, "NULL plan");
    return p->gradient(dobs, grad, rnorm2, traces, (cudaStream_t)stream, true, false);
} PGB_API_CATCH("pysit_plan_gradient")

extern "C" int pysit_plan_migrate(pysit_plan* p, const void* operand, double* image, double* norm2,
                                  void* stream) try {
    PGB_REQUIRE(p, "NULL plan");
    return p->gradient(operand, image, norm2, nullptr, (cudaStream_t)stream, true, true);
} PGB_API_CATCH("pysit_plan_migrate")

extern "C" int pysit_plan_misfit(pysit_plan* p, const void* dobs, double* rnorm2, void* traces,
                                 void* stream) try {
    PGB_REQUIRE(p, "NULL plan");
    return p->gradient(dobs, nullptr, rnorm2, traces, (cudaStream_t)stream, false, false);
} PGB_API_CATCH("pysit_plan_misfit")

extern "C" int pysit_plan_born(pysit_plan* p, const double* m1, void* traces, void* stream) try {
    PGB_REQUIRE(p, "NULL plan");
    return p->born(m1, traces, (cudaStream_t)stream);
} PGB_API_CATCH("pysit_plan_born")

extern "C" int pysit_plan_hessian(pysit_plan* p, const double* m1, double* out, double* d1norm2, void* stream) try {
    PGB_REQUIRE(p, "NULL plan");
    return p->hessian(m1, out, d1norm2, (cudaStream_t)stream);
} PGB_API_CATCH("pysit_plan_hessian")

extern "C" int pysit_plan_status(pysit_plan* p, int* flags, void* stream) try {
    PGB_REQUIRE(p && flags, "NULL argument");
    return p->status(flags, (cudaStream_t)stream);
} PGB_API_CATCH("pysit_plan_status")

extern "C" int pysit_plan_last_launch_count(const pysit_plan* p, int64_t* n) try {
    PGB_REQUIRE(p && n, "NULL argument");
    *n = p->last_launches;
    return PYSIT_OK;
} PGB_API_CATCH("pysit_plan_last_launch_count")

extern "C" int pysit_plan_step_loop(pysit_plan* p, int mode, int nsteps, void* stream) try {
    PGB_REQUIRE(p, "NULL plan");
    return p->step_loop(mode, nsteps, (cudaStream_t)stream);
} PGB_API_CATCH("pysit_plan_step_loop")

extern "C" int pysit_plan_get_tuning(const pysit_plan* p, int* tile_x, double* shell_share) try {
    PGB_REQUIRE(p, "NULL plan");
    return p->tuning(tile_x, shell_share);
} PGB_API_CATCH("pysit_plan_get_tuning")

extern "C" int pysit_plan_autotune(pysit_plan* p, const int* candidates, int ncand, int nsteps, int* chosen,
                                   double* ms, void* stream) try {
    PGB_REQUIRE(p, "NULL plan");
    return p->autotune(candidates, ncand, nsteps, chosen, ms, (cudaStream_t)stream);
} PGB_API_CATCH("pysit_plan_autotune")

extern "C" int pysit_plan_autotune_tiles(pysit_plan* p, const int* cand_x, int ncx, const int* cand_z, int ncz,
                                         int nsteps, int* chosen_x, int* chosen_z, double* ms, void* stream) try {
    PGB_REQUIRE(p, "NULL plan");
    return p->autotune2(cand_x, ncx, cand_z, ncz, nsteps, chosen_x, chosen_z, ms, (cudaStream_t)stream);
} PGB_API_CATCH("pysit_plan_autotune_tiles")

extern "C" int pysit_plan_get_tiles(const pysit_plan* p, int* tile_x, int* tile_z) try {
    PGB_REQUIRE(p, "NULL plan");
    return p->tiles(tile_x, tile_z);
} PGB_API_CATCH("pysit_plan_get_tiles")

extern "C" int pysit_plan_task_table(const pysit_plan* p, int32_t* out, uint64_t cap, uint64_t* n_ints,
                                     int32_t* n_interior) try {
    PGB_REQUIRE(p, "NULL plan");
    return p->task_table(out, cap, n_ints, n_interior);
} PGB_API_CATCH("pysit_plan_task_table")

// ---- plan groups ------------------------------------------------------------------------
struct pysit_group {
    std::vector<pysit_plan*> plans;
    std::vector<cudaStream_t> streams;  // one per plan
    std::vector<cudaEvent_t> done;      // one per plan
    cudaStream_t cap = nullptr;
    cudaEvent_t root = nullptr;
    std::map<std::vector<const void*>, cudaGraphExec_t> graphs;
    ~pysit_group() {
        for (auto& kv : graphs)
            if (kv.second) cudaGraphExecDestroy(kv.second);
        for (auto s : streams) cudaStreamDestroy(s);
        for (auto e : done) cudaEventDestroy(e);
        if (cap) cudaStreamDestroy(cap);
        if (root) cudaEventDestroy(root);
    }
};

extern "C" int pysit_group_create(pysit_plan* const* plans, int nplans, pysit_group** out) try {
    PGB_REQUIRE(plans && out && nplans >= 1, "need at least one plan and an output");
    for (int i = 0; i < nplans; ++i) PGB_REQUIRE(plans[i], "NULL plan %d", i);
    std::unique_ptr<pysit_group> g(new pysit_group());
    g->plans.assign(plans, plans + nplans);
    PGB_CHECK_CUDA(cudaStreamCreateWithFlags(&g->cap, cudaStreamNonBlocking));
    PGB_CHECK_CUDA(cudaEventCreateWithFlags(&g->root, cudaEventDisableTiming));
    for (int i = 0; i < nplans; ++i) {
        cudaStream_t s;
        cudaEvent_t e;
        PGB_CHECK_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        g->streams.push_back(s);
        PGB_CHECK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        g->done.push_back(e);
    }
    *out = g.release();
    return PYSIT_OK;
} PGB_API_CATCH("pysit_group_create")

extern "C" int pysit_group_destroy(pysit_group* g) try {
    delete g;
    return PYSIT_OK;
} PGB_API_CATCH("pysit_group_destroy")

extern "C" int pysit_group_gradient(pysit_group* g, const void* const* dobs, double* const* grad,
                                    double* const* rnorm2, void* stream) try {
    PGB_REQUIRE(g && dobs && grad && rnorm2, "NULL argument");
    const int n = (int)g->plans.size();
    std::vector<const void*> key;
    for (int i = 0; i < n; ++i) { key.push_back(dobs[i]); key.push_back(grad[i]); key.push_back(rnorm2[i]); }
    auto it = g->graphs.find(key);
    if (it == g->graphs.end()) {
        PGB_CHECK_CUDA(cudaStreamBeginCapture(g->cap, cudaStreamCaptureModeThreadLocal));
        cudaEventRecord(g->root, g->cap);
        int rc = PYSIT_OK;
        capture_into(g->cap, [&] {
            for (int i = 0; i < n && rc == PYSIT_OK; ++i) {
                cudaStreamWaitEvent(g->streams[i], g->root, 0);
                rc = g->plans[i]->enqueue_grad_raw(dobs[i], grad[i], rnorm2[i], g->streams[i]);
                cudaEventRecord(g->done[i], g->streams[i]);
                cudaStreamWaitEvent(g->cap, g->done[i], 0);
            }
        });
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(g->cap, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture (group)");
        cudaGraphExec_t exec = nullptr;
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return cuda_status(e, "cudaGraphInstantiate (group)");
        it = g->graphs.emplace(key, exec).first;
    }
    PGB_CHECK_CUDA(cudaGraphLaunch(it->second, (cudaStream_t)stream));
    return PYSIT_OK;
} PGB_API_CATCH("pysit_group_gradient")
