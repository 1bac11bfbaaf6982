// Batched 2D leapfrog step (forward, recompute and adjoint modes) over many
// shots at once, on the internal zero-halo layout of wave.cuh.
//
// Maths: one step of cda_time_scalar_2D (pysit/solvers/constant_density_acoustic/
// time/scalar/constant_density_acoustic_time_scalar_2D.h:88-179) per shot, with
// the rhs built in-kernel from the source / residual injection operator, plus
//   kFwd    trace recording of u_k (ReceiverSet.sample_data_from_array,
//           pysit/core/receivers.py:462-510; TemporalModeling.forward_model
//           records u_k before stepping, temporal_modeling.py:123-125);
//   kRecomp the imaging operand dWaveOp_k (constant_density_acoustic_base.py:24-40)
//           computed from the stencil's own bracket F (no (u+ - 2u + u-)/dt^2
//           cancellation): in a cell whose step sigmas equal the mesh sigmas it is
//           exactly C^2 F; elsewhere (the right PML, whose step profile is read one
//           node further out, _2D.h:143-157) the sigma differences are added;
//   kAdj    the time-reversed adjoint step of adjoint_model (:312-365) with the
//           zero-lag imaging ic += q_k * dWaveOp_k fused (:329-337).
//
// Thread mapping (memory-bound stencil, no tensor cores): a block covers a tile
// of TZ = blockDim.x * V cells along z (V = 16 bytes of T per thread, vector
// loads) and sweeps `tx` rows along x.  Each thread keeps the 2R+1 rows of u_k
// (and of Phi_x in PML tiles) that its x-derivatives need in a register queue;
// the z-neighbours come from a double-buffered shared-memory copy of the centre
// row (one __syncthreads per row).  Tiles whose halo does not reach the padding
// never touch the PML state; in PML tiles the PML state is loaded only for
// vectors inside the padding (elsewhere it is identically zero).
#include "wave.cuh"

namespace pgb {
namespace {

template <typename T>
__device__ __forceinline__ long long foff2(const WaveParams<T>& p, int x, int z) {
    return (long long)(x + kHalo) * p.ldz + kOZ + z;
}

template <typename T>
__device__ __forceinline__ T inject_rhs(const Inject<T>& inj, const int* bx, int shot, int x,
                                        int z) {
    if (x < bx[0] || x >= bx[1] || z < bx[4] || z >= bx[5]) return T(0);
    int c = (x - bx[0]) * (bx[5] - bx[4]) + (z - bx[4]);
    const int* rp = inj.rowptr + inj.rpbase[shot];
    int e0 = __ldg(rp + c), e1 = __ldg(rp + c + 1);
    const T* amp = inj.amp + shot * inj.amp_sstride;
    T acc = T(0);
    for (int e = e0; e < e1; ++e) acc += __ldg(inj.w + e) * __ldg(amp + __ldg(inj.pt + e));
    return acc;
}

template <typename T>
__device__ __forceinline__ void record_block(const WaveParams<T>& p, int rb) {
    int id = rb * blockDim.x + threadIdx.x;
    int total = p.nshot * p.rec.nrec;
    if (id >= total) return;
    int shot = id / p.rec.nrec, r = id - shot * p.rec.nrec;
    int e0 = __ldg(p.rec.rowptr + id), e1 = __ldg(p.rec.rowptr + id + 1);
    const T* u = p.u_cur + (long long)shot * p.fstride;
    T acc = T(0);
    for (int e = e0; e < e1; ++e) acc += __ldg(p.rec.w + e) * u[__ldg(p.rec.off + e)];
    p.rec.traces[shot * p.rec.tr_sstride + r] = acc;
}

template <typename T, int R, int MODE, bool PML>
__device__ __forceinline__ void sweep2d(const WaveParams<T>& p, const int shot, const int x0,
                                        const int x1, const int z0, T* __restrict__ smem) {
    constexpr int V = V16<T>::N;
    constexpr int H = kHalo;
    constexpr int HV = H / V;            // halo vectors per side
    constexpr int NW = (V + 2 * H) / V;  // z-window vectors per thread
    constexpr int Q = 2 * R + 1;
    const int t = threadIdx.x;
    const int TZ = blockDim.x * V;
    const int SROW = TZ + 2 * H;
    const int zc = z0 + t * V;
    const bool zin = zc < p.nz;
    const long long sh = (long long)shot * p.fstride;
    const T* __restrict__ ucur = p.u_cur + sh;
    T* __restrict__ uprev = p.u_prev + sh;
    const T* __restrict__ phx_in = p.phx_in + sh;
    const T* __restrict__ phz_in = p.phz_in + sh;

    // vectors of this thread that may hold non-zero PML state
    const bool zpad = PML && (zc < p.pzl || zc + V - 1 >= p.nz - p.pzr);
    const int* bx = p.inj.box + shot * 6;
    const bool inj_blk = p.inj.on && bx[0] < x1 && bx[1] > x0 && bx[4] < z0 + TZ && bx[5] > z0;

    // per-thread z-axis data
    T sgz[V], mgz[V];
    bool zok[V];
#pragma unroll
    for (int v = 0; v < V; ++v) {
        int z = zc + v;
        zok[v] = z > 0 && z < p.nz - 1;
        sgz[v] = (PML && z < p.nz) ? __ldg(p.sgz + z) : T(0);
        mgz[v] = (PML && MODE == kRecomp && z < p.nz) ? __ldg(p.mgz + z) : T(0);
    }

    VReg<T> q[Q];
    VReg<T> qx[PML ? Q : 1];
#pragma unroll
    for (int j = 0; j < Q; ++j) {
        const int x = x0 - R + j;
        q[j] = zin ? vld_ro(ucur + foff2(p, x, zc)) : vzero<T>();
        if (PML) {
            const bool xp = x < p.pxl || x >= p.nx - p.pxr;
            qx[j] = (zin && (zpad || xp)) ? vld_ro(phx_in + foff2(p, x, zc)) : vzero<T>();
        }
    }

    int buf = 0;
    for (int x = x0; x < x1; ++x) {
        T* su = smem + buf * SROW;
        T* sp = smem + (2 + buf) * SROW;
        const long long o = foff2(p, x, zc);
        const bool xp = PML && (x < p.pxl || x >= p.nx - p.pxr);
        const bool padv = PML && zin && (zpad || xp);

        // loads of this row issued before the barrier
        VReg<T> um = zin ? vld(uprev + o) : vzero<T>();
        VReg<T> cc = zin ? vld_ro(p.c2 + o) : vzero<T>();
        VReg<T> pzc = padv ? vld_ro(phz_in + o) : vzero<T>();
        VReg<T> dwi;
        if (MODE == kAdj) dwi = (zin && p.image) ? vld_stream(p.dw_in + sh + o) : vzero<T>();

        vst(su + H + t * V, q[R]);
        if (PML) vst(sp + H + t * V, pzc);
        if (t < HV) {
            const int zh = z0 - H + t * V;
            vst(su + t * V, vld_ro(ucur + foff2(p, x, zh)));
            if (PML) vst(sp + t * V, vld_ro(phz_in + foff2(p, x, zh)));
        } else if (t < 2 * HV) {
            const int zh = z0 + TZ + (t - HV) * V;
            const bool in = zh < p.nz;
            vst(su + H + TZ + (t - HV) * V, in ? vld_ro(ucur + foff2(p, x, zh)) : vzero<T>());
            if (PML) vst(sp + H + TZ + (t - HV) * V, in ? vld_ro(phz_in + foff2(p, x, zh)) : vzero<T>());
        }
        __syncthreads();

        T w[NW * V];
        T wp[PML ? NW * V : 1];
#pragma unroll
        for (int i = 0; i < NW; ++i) {
            VReg<T> r = vld(su + t * V + i * V);
#pragma unroll
            for (int v = 0; v < V; ++v) w[i * V + v] = r.v[v];
            if (PML) {
                VReg<T> rp = vld(sp + t * V + i * V);
#pragma unroll
                for (int v = 0; v < V; ++v) wp[i * V + v] = rp.v[v];
            }
        }

        const T sgx = PML ? __ldg(p.sgx + x) : T(0);
        const T mgx = (PML && MODE == kRecomp) ? __ldg(p.mgx + x) : T(0);
        const bool xok = x > 0 && x < p.nx - 1;
        const bool inj_row = inj_blk && x >= bx[0] && x < bx[1];

        VReg<T> un, dwo, pxo, pzo, ico;
        bool any_pml = false;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const int z = zc + v;
            const T uc = q[R].v[v];
            // second derivatives and first derivatives along z (smem window) and x (queue)
            T lz = T(d2w(R, 0)) * uc, dz1 = T(0);
            T lx = T(d2w(R, 0)) * uc, dx1 = T(0);
#pragma unroll
            for (int m = 1; m <= R; ++m) {
                const T zp = w[H + v + m], zm = w[H + v - m];
                const T xpv = q[R + m].v[v], xmv = q[R - m].v[v];
                lz += T(d2w(R, m)) * (zp + zm);
                lx += T(d2w(R, m)) * (xpv + xmv);
                dz1 += T(d1w(R, m)) * (zp - zm);
                dx1 += T(d1w(R, m)) * (xpv - xmv);
            }
            T F = lx * p.idx2 + lz * p.idz2;
            if (inj_row && z < p.nz) F += inject_rhs(p.inj, bx, shot, x, z);
            T sx = T(0), sz = T(0);
            if (PML) {
                T dpx = T(0), dpz = T(0);
#pragma unroll
                for (int m = 1; m <= R; ++m) {
                    dpx += T(d1w(R, m)) * (qx[R + m].v[v] - qx[R - m].v[v]);
                    dpz += T(d1w(R, m)) * (wp[H + v + m] - wp[H + v - m]);
                }
                F += dpx * p.idx + dpz * p.idz;
                sx = sgx;
                sz = sgz[v];
            }
            const T uo = um.v[v];
            const T c2 = cc.v[v];
            const bool ok = xok && zok[v];
            T unew;
            T ph_x = T(0), ph_z = T(0);
            if (PML && (sx != T(0) || sz != T(0))) {
                const T dudx = dx1 * p.idx, dudz = dz1 * p.idz;
                const T phx = qx[R].v[v], phz = pzc.v[v];
                ph_x = phx - p.dt * sx * phx + p.dt * (sz - sx) * dudx;
                ph_z = phz - p.dt * sz * phz + p.dt * (sx - sz) * dudz;
                const T fac1 = T(2) * p.dt2 / (T(2) + p.dt * (sx + sz));
                const T fac2 = c2 * F - (uo - T(2) * uc) * p.idt2 + (sx + sz) * uo * p.i2dt -
                               (sx * sz) * uc;
                unew = fac1 * fac2;
                any_pml = true;
            } else {
                unew = p.dt2 * c2 * F - (uo - T(2) * uc);
            }
            if (!ok) { unew = T(0); ph_x = T(0); ph_z = T(0); }
            un.v[v] = unew;
            pxo.v[v] = ph_x;
            pzo.v[v] = ph_z;
            if (MODE == kRecomp) {
                T d = c2 * F;
                if (PML) {
                    const T mz = mgz[v];
                    d += ((mgx + mz) - (sx + sz)) * (unew - uo) * p.i2dt + (mgx * mz - sx * sz) * uc;
                }
                dwo.v[v] = ok ? d : T(0);
            }
            if (MODE == kAdj) ico.v[v] = uc * dwi.v[v];
        }

        if (zin) {
            vst(uprev + o, un);
            if (PML && padv) {
                vst(p.phx_out + sh + o, pxo);
                vst(p.phz_out + sh + o, pzo);
            }
            if (MODE == kRecomp && p.dw_out) vst_stream(p.dw_out + sh + o, dwo);
            if (MODE == kAdj && p.image) {
                VReg<T> a = vld(p.ic + sh + o);
#pragma unroll
                for (int v = 0; v < V; ++v) a.v[v] += ico.v[v];
                vst(p.ic + sh + o, a);
            }
        }
        (void)any_pml;

        // advance the queues by one row
#pragma unroll
        for (int j = 0; j < Q - 1; ++j) {
            q[j] = q[j + 1];
            if (PML) qx[j] = qx[j + 1];
        }
        if (x + 1 < x1) {
            const int xn = x + 1 + R;
            q[Q - 1] = zin ? vld_ro(ucur + foff2(p, xn, zc)) : vzero<T>();
            if (PML) {
                const bool xpn = xn < p.pxl || xn >= p.nx - p.pxr;
                qx[Q - 1] = (zin && (zpad || xpn)) ? vld_ro(phx_in + foff2(p, xn, zc)) : vzero<T>();
            }
        }
        buf ^= 1;
    }
}

template <typename T, int R, int MODE>
__global__ void __launch_bounds__(256) wave2d_kernel(const WaveParams<T> p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* smem = reinterpret_cast<T*>(smem_raw);
    const int ntiles = p.ntz * p.ntx;
    const int b = blockIdx.x;
    if (b >= ntiles * p.nshot) {
        if (MODE == kFwd) record_block(p, b - ntiles * p.nshot);
        return;
    }
    const int shot = b / ntiles;
    const int tile = b - shot * ntiles;
    const int tzi = tile % p.ntz, txi = tile / p.ntz;
    const int TZ = blockDim.x * V16<T>::N;
    const int z0 = tzi * TZ;
    const int z1 = min(z0 + TZ, p.nz);
    const int x0 = txi * p.tx;
    const int x1 = min(x0 + p.tx, p.nx);
    const bool pml = (p.pxl > 0 && x0 - R < p.pxl) || (p.pxr > 0 && x1 + R > p.nx - p.pxr) ||
                     (p.pzl > 0 && z0 - R < p.pzl) || (p.pzr > 0 && z1 + R > p.nz - p.pzr);
    if (pml)
        sweep2d<T, R, MODE, true>(p, shot, x0, x1, z0, smem);
    else
        sweep2d<T, R, MODE, false>(p, shot, x0, x1, z0, smem);
}

}  // namespace

template <typename T, int R, int MODE>
void launch_wave2d(const WaveParams<T>& p, int bz, cudaStream_t s) {
    const int ntiles = p.ntz * p.ntx;
    int grid = ntiles * p.nshot + (MODE == kFwd ? p.rec.blocks : 0);
    const int srow = bz * V16<T>::N + 2 * kHalo;
    size_t smem = 4 * srow * sizeof(T);
    wave2d_kernel<T, R, MODE><<<grid, bz, smem, s>>>(p);
}

#define PGB_INST2D(T, R)                                                    \
    template void launch_wave2d<T, R, kFwd>(const WaveParams<T>&, int, cudaStream_t);    \
    template void launch_wave2d<T, R, kRecomp>(const WaveParams<T>&, int, cudaStream_t); \
    template void launch_wave2d<T, R, kAdj>(const WaveParams<T>&, int, cudaStream_t);
PGB_INST2D(float, 1)
PGB_INST2D(float, 2)
PGB_INST2D(float, 3)
PGB_INST2D(float, 4)
PGB_INST2D(double, 1)
PGB_INST2D(double, 2)
PGB_INST2D(double, 3)
PGB_INST2D(double, 4)

}  // namespace pgb
