// Device-side data layout and kernel parameters of the batched wave pipeline.
//
// Internal field layout (per shot, per field): a zero halo of HX = 4 rows on
// both x sides (2D/3D), HY = 4 rows on both y sides (3D), and along z a row
// pitch `ldz` (multiple of 32 elements) with the grid starting at z offset
// OZ = 4.  Cell (i, j, k) of the padded PySIT grid lives at
//     ((i + HX) * (ny + 2*HY) + (j + HY)) * ldz + OZ + k.
// The halos are never written with non-zero values, so the stencils read the
// reference's zero extension without bounds tests, rows start 128-byte
// aligned and z-vectors of 16 bytes are aligned.
#pragma once

#include "common.cuh"

namespace pgb {

constexpr int kHalo = 4;  // x/y halo rows and smem z halo (max stencil radius)
constexpr int kOZ = 4;    // z offset of cell k = 0 inside a row
constexpr int kTailZ = 12;  // zero cells kept after the last cell of a row (>= halo + vector - 1)

// bits of the device error word of a plan
#define PGB_ERR_TIMEOUT 1    // a bounded wait for a bulk copy expired
#define PGB_ERR_NONFINITE 2  // a NaN / Inf wavefield value (unstable time step)

template <typename T> struct V16;
template <> struct V16<float> { using type = float4; static constexpr int N = 4; };
template <> struct V16<double> { using type = double2; static constexpr int N = 2; };

template <typename T>
struct alignas(16) VReg {
    T v[V16<T>::N];
};

template <typename T>
__device__ __forceinline__ VReg<T> vzero() {
    VReg<T> r;
#pragma unroll
    for (int i = 0; i < V16<T>::N; ++i) r.v[i] = T(0);
    return r;
}
template <typename T>
__device__ __forceinline__ VReg<T> vld_ro(const T* p) {  // read-only path
    VReg<T> r;
    *reinterpret_cast<typename V16<T>::type*>(r.v) =
        __ldg(reinterpret_cast<const typename V16<T>::type*>(p));
    return r;
}
template <typename T>
__device__ __forceinline__ VReg<T> vld(const T* p) {
    VReg<T> r;
    *reinterpret_cast<typename V16<T>::type*>(r.v) =
        *reinterpret_cast<const typename V16<T>::type*>(p);
    return r;
}
template <typename T>
__device__ __forceinline__ VReg<T> vld_stream(const T* p) {  // read once: evict-first
    VReg<T> r;
    *reinterpret_cast<typename V16<T>::type*>(r.v) =
        __ldcs(reinterpret_cast<const typename V16<T>::type*>(p));
    return r;
}
template <typename T>
__device__ __forceinline__ void vst(T* p, const VReg<T>& r) {
    *reinterpret_cast<typename V16<T>::type*>(p) = *reinterpret_cast<const typename V16<T>::type*>(r.v);
}
template <typename T>
__device__ __forceinline__ void vst_stream(T* p, const VReg<T>& r) {
    __stcs(reinterpret_cast<typename V16<T>::type*>(p), *reinterpret_cast<const typename V16<T>::type*>(r.v));
}

// Kernel modes of the batched step.
enum StepMode : int {
    kFwd = 0,     // forward step; records traces of u_k
    kRecomp = 1,  // forward recompute; writes the imaging operand dWaveOp_k
    kAdj = 2,     // adjoint step driven by the residual; accumulates ic += q_k * dWaveOp_k
    kBorn = 3,    // 2D: scattered-field step with the Born source -m1 dWaveOp0_k inside the stencil
};

// Injection operator of one step: per shot a box of cells [x0,x1) x [y0,y1) x [z0,z1)
// with CSR rows over the box cells (x-major, z fastest); entries (point, weight).
// rhs(cell) = sum_e w[e] * amp[shot * amp_sstride + pt[e]].
template <typename T>
struct Inject {
    const int* box;          // [nshot][6]: x0, x1, y0, y1, z0, z1 (grid coords)
    const long long* rpbase; // [nshot] offset of the shot's first row pointer
    const int* rowptr;       // CSR row pointers (absolute entry indices)
    const int* pt;           // entry point index
    const T* w;              // entry weight
    const T* amp;            // amplitudes of this step for shot 0
    long long amp_sstride;   // amplitude stride between shots
    int on;                  // 0: no injection this step
};

// Trace recording of u_k: per (shot, receiver) a CSR row of taps.
template <typename T>
struct Record {
    const int* rowptr;       // [nshot*nrec + 1] absolute tap index (shot-major)
    const long long* off;    // tap offset inside a field (internal layout)
    const T* w;              // tap weight (sampling operator)
    T* traces;               // trace sample k of shot 0 receiver 0
    long long tr_sstride;    // stride between shots in the trace array
    int nrec;
    int blocks;              // number of recorder blocks appended to the grid
    int lanes;               // threads per (shot, receiver): a power of two up to 32
};

template <typename T>
struct WaveParams {
    // geometry
    int nx, ny, nz;          // padded grid (ny = 1 in 2D)
    int ldz;                 // row pitch (elements)
    int rows_y;              // ny + 2*HY
    long long fstride;       // elements between consecutive shots of one field
    int hx, hy;              // halos (4 / 0 in 2D)
    // tiling
    int tx;                  // rows swept per block along x
    int ty;                  // 3D: y rows per block (blockDim.y)
    int ntz, nty, ntx;       // tiles per shot along z, y, x
    int nshot;               // shots in this launch
    // wavefields (shot 0 base)
    T* u_prev;               // in: u_{k-1}; out: u_{k+1} (same cell, in place)
    const T* u_cur;          // u_k
    const T* phx_in; T* phx_out;
    const T* phy_in; T* phy_out;
    const T* phz_in; T* phz_out;
    const T* psi_in; T* psi_out;
    const T* c2;             // C^2, shared by all shots (internal layout)
    // PML (kernel convention) and mesh sigma maps, full length per axis
    const T *sgx, *sgy, *sgz;
    const T *mgx, *mgy, *mgz;
    int pxl, pxr, pyl, pyr, pzl, pzr;  // padding widths holding PML state
    // scalars
    T dt, dt2, idt2, i2dt, idx, idx2, idy, idy2, idz, idz2;
    // injection / recording / imaging
    Inject<T> inj;
    Record<T> rec;
    T* dw_out;               // kRecomp: imaging operand of this step (shot 0 base)
    const T* dw_in;          // kAdj: imaging operand of this step
    T* ic;                   // kAdj: imaging accumulator (shot 0 base)
    int image;               // kAdj: accumulate this step
    const T* m1;             // kBorn: edge-padded model perturbation (internal layout, shared by the shots);
                             // dw_in holds dWaveOp0_k
    int* err;                // device error word (PGB_ERR_* bits), may be NULL
    unsigned polls;          // 0: a bulk-copy wait tries 2^22 times (each try may suspend); n: n non-blocking tests
    int wait_fault;          // test aid: each task first waits (bounded) on a barrier nothing arrives on
    int psi_c2;              // 3D: 1 = C^2 multiplies sigma_x sigma_y sigma_z psi (the reference), 0 = not
    int nan_check;           // kRecomp: flag non-finite u_{k+1} as kFwd does (a forward sweep that keeps dWaveOp)
    // 2D persistent sweep: task counters (interior, PML shell) shared by the
    // launches of one run; this launch's tasks of kind 0 are the counter values
    // task_base .. task_base + tasks - 1 of task_ctr[0], those of kind 1 start at
    // task_base2 on task_ctr[1]
    unsigned long long* task_ctr;
    unsigned long long task_base, task_base2;
};

// ---- helpers shared by the 2D kernels ---------------------------------------
template <typename T>
__device__ __forceinline__ long long foff2(const WaveParams<T>& p, int x, int z) {
    return (long long)(x + kHalo) * p.ldz + kOZ + z;
}

// rhs of one cell from the injection operator of its shot
template <typename T>
__device__ __forceinline__ T inject_rhs(const Inject<T>& inj, const int* bx, int shot, int x, int z) {
    if (x < bx[0] || x >= bx[1] || z < bx[4] || z >= bx[5]) return T(0);
    int c = (x - bx[0]) * (bx[5] - bx[4]) + (z - bx[4]);
    const int* rp = inj.rowptr + inj.rpbase[shot];
    int e0 = __ldg(rp + c), e1 = __ldg(rp + c + 1);
    const T* amp = inj.amp + shot * inj.amp_sstride;
    T acc = T(0);
    int e = e0;
    // taps in groups of 8: the point indices and weights first, then the amplitudes, so that
    // a group's dependent loads are in flight together (the sum keeps the taps' order)
    for (; e + 8 <= e1; e += 8) {
        int pt[8];
        T w[8], a[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) { pt[q] = __ldg(inj.pt + e + q); w[q] = __ldg(inj.w + e + q); }
#pragma unroll
        for (int q = 0; q < 8; ++q) a[q] = __ldg(amp + pt[q]);
#pragma unroll
        for (int q = 0; q < 8; ++q) acc += w[q] * a[q];
    }
    for (; e < e1; ++e) acc += __ldg(inj.w + e) * __ldg(amp + __ldg(inj.pt + e));
    return acc;
}

// trace recorder block: p.rec.lanes threads per (shot, receiver), the p.rec.blocks
// recorder blocks striding over the receivers.  Lane l sums taps l, l + lanes, ... in
// order, up to 8 of them with their loads in flight together; a fixed butterfly over the
// lanes adds the partial sums, so the result does not depend on scheduling.  Every thread
// of the block takes part (the butterfly shuffles over whole warps).
template <typename T>
__device__ __forceinline__ void record_block(const WaveParams<T>& p, int rb) {
    constexpr int kTaps = 8;
    const int G = p.rec.lanes;
    const long long t = (long long)rb * blockDim.x + threadIdx.x;
    const int l = (int)(t & (G - 1));
    const long long total = (long long)p.nshot * p.rec.nrec;
    const long long pass = (long long)p.rec.blocks * blockDim.x / G;  // receivers per pass
    for (long long base = 0; base < total; base += pass) {           // the same count on every lane
        const long long id = base + t / G;
        T acc = T(0);
        if (id < total) {
            const int shot = (int)(id / p.rec.nrec);
            const int e1 = __ldg(p.rec.rowptr + id + 1);
            const T* u = p.u_cur + (long long)shot * p.fstride;
            for (int e = __ldg(p.rec.rowptr + id) + l; e < e1; e += kTaps * G) {
                long long off[kTaps];
                T w[kTaps], v[kTaps];
#pragma unroll
                for (int q = 0; q < kTaps; ++q) {
                    const bool in = e + q * G < e1;
                    off[q] = in ? __ldg(p.rec.off + e + q * G) : 0;
                    w[q] = in ? __ldg(p.rec.w + e + q * G) : T(0);
                }
#pragma unroll
                for (int q = 0; q < kTaps; ++q) v[q] = e + q * G < e1 ? __ldg(u + off[q]) : T(0);
#pragma unroll
                for (int q = 0; q < kTaps; ++q)
                    if (e + q * G < e1) acc += w[q] * v[q];
            }
        }
        for (int m = G >> 1; m > 0; m >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, m);
        if (id < total && l == 0) {
            const int shot = (int)(id / p.rec.nrec), r = (int)(id - (long long)shot * p.rec.nrec);
            p.rec.traces[shot * p.rec.tr_sstride + r] = acc;
        }
    }
}

// persistent-warp 2D sweep fed by shared-memory row rings, one task kind per
// kernel (0 interior, 1 PML shell); tasks = [ntasks][5] ints (x0, x1, zs, ze,
// kind) of one shot, shared by all shots; `blocks` task blocks.  Returns the
// number of task-counter values the launch consumes.
template <typename T, int R, int MODE, int KIND>
long long launch_wave2d_warp_tasks(const WaveParams<T>& p, const int* tasks, int ntasks, int blocks,
                                   cudaStream_t s);
int wave2d_warp_threads();
int wave2d_warp_seg(int dtype_bytes, int order, int pml);
// resident task blocks of the whole GPU for one (dtype, order, mode, kind)
int wave2d_warp_blocks(int dtype_bytes, int order, int mode, int kind);
void wave2d_warp_prepare();
// 3D block tasks (x0, x1, y0, y1, zs, ze): one block per task and shot (KIND 0
// interior, 1 PML shell); a warp takes 32 / (vectors of the z-range) y-rows
template <typename T, int R, int MODE, int KIND>
void launch_wave3d_tasks(const WaveParams<T>& p, const int* tasks, int ntasks, cudaStream_t s);
int wave3d_seg(int dtype_bytes, int kind);  // widest z-range of a task of each kind
int wave3d_task_rows(int dtype_bytes, int kind, int zcells);  // y-rows of a task of zcells z-cells
template <typename T, int R, int MODE>
void launch_wave1d(const WaveParams<T>& p, int bz, cudaStream_t s);

}  // namespace pgb
