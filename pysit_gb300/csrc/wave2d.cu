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
// Data movement (HBM-bound stencil, no tensor cores).  A block of 128 threads
// covers a z-tile of TZ = 128 * V cells (V = 16 bytes of T per thread) and
// sweeps `tx` rows along x.  Thread 0 streams every row the block needs into
// shared-memory rings with 1-D bulk copies (cp.async.bulk, "TMA"), D rows ahead
// of the computation, each stage completing on its own mbarrier:
//   u_k       ring of 2R + D rows with a 4-cell z-halo (x- and z-stencils)
//   Phi_x     ring of 2R + D rows, Phi_z one row per stage (PML tiles only, and
//             only the padding segments of interior rows)
//   u_{k-1}, C^2, [dWaveOp, ic]   one row per stage
// The 128 threads read their stencils from shared memory (16-byte vector reads)
// and write results straight to HBM with 16-byte stores.  One __syncthreads per
// row releases the ring slots.  Waits are bounded: on expiry the kernel sets the
// error word and finishes the sweep instead of hanging.
#include "tma.cuh"
#include "wave.cuh"

namespace pgb {
namespace {

constexpr int kNT = 128;          // threads per stencil block
constexpr int kD = 4;             // rows in flight ahead of the computation
constexpr uint32_t kWaitPolls = 1u << 22;

__host__ __device__ constexpr int round_up(int a, int b) { return (a + b - 1) / b * b; }

// shared-memory carve-up (elements of T after a 128-byte barrier area)
template <typename T, int R>
struct Smem2 {
    static constexpr int V = V16<T>::N;
    static constexpr int TZ = kNT * V;
    static constexpr int SROW = TZ + 2 * kHalo;
    static constexpr int NQ = 2 * R + kD;
    static constexpr int U = 0;
    static constexpr int PX = U + NQ * SROW;
    static constexpr int PZ = PX + NQ * SROW;
    static constexpr int UP = PZ + kD * SROW;
    static constexpr int CC = UP + kD * TZ;
    static constexpr int DW = CC + kD * TZ;
    static constexpr int IC = DW + kD * TZ;
    static constexpr int END = IC + kD * TZ;
    static constexpr size_t bytes = 128 + sizeof(T) * (size_t)END;
};

template <typename T, int R, int MODE>
__global__ void __launch_bounds__(kNT, 2) wave2d_kernel(const WaveParams<T> p) {
    using L = Smem2<T, R>;
    constexpr int V = L::V, H = kHalo, TZ = L::TZ, SROW = L::SROW, NQ = L::NQ;
    constexpr int NW = (V + 2 * H) / V;  // z-window vectors per thread
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    T* S = reinterpret_cast<T*>(smem_raw + 128);

    const int ntiles = p.ntz * p.ntx;
    const int b = blockIdx.x;
    if (b >= ntiles * p.nshot) {
        if (MODE != kAdj) record_block(p, b - ntiles * p.nshot);
        return;
    }
    const int shot = b / ntiles;
    const int tile = b - shot * ntiles;
    const int tzi = tile % p.ntz, txi = tile / p.ntz;
    const int z0 = tzi * TZ;
    const int zlen = min(TZ, p.nz - z0);
    const int x0 = txi * p.tx;
    const int x1 = min(x0 + p.tx, p.nx);
    const int niter = x1 - x0;
    const int t = threadIdx.x;
    const long long sh = (long long)shot * p.fstride;
    const bool pml = (p.pxl > 0 && x0 - R < p.pxl) || (p.pxr > 0 && x1 + R > p.nx - p.pxr) ||
                     (p.pzl > 0 && z0 - R < p.pzl) || (p.pzr > 0 && z0 + zlen + R > p.nz - p.pzr);
    const bool zpad_tile_l = p.pzl > 0 && z0 < p.pzl + H;
    const bool zpad_tile_r = p.pzr > 0 && z0 + zlen + H > p.nz - p.pzr;

    // ---- rings: zero once (copies never touch cells beyond the tile + halo) ----
    for (int i = t; i < L::END; i += kNT) S[i] = T(0);
    if (t == 0) {
        for (int s = 0; s < kD; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();

    auto xpad = [&](int x) { return x < p.pxl || x >= p.nx - p.pxr; };
    auto qslot = [&](int r) { return (r - x0 + R) % NQ; };
    const T* ucur = p.u_cur + sh;
    const T* uprev_g = p.u_prev + sh;
    const T* phx_g = p.phx_in + sh;
    const T* phz_g = p.phz_in + sh;
    const int nfull = round_up(zlen + 2 * H, V);   // halo rows
    const int nplain = round_up(zlen, V);          // rows without halo

    // copies of one PML-state row (halo layout): whole row in x-padding rows,
    // otherwise only the z-padding segments (the rest of the slot is never read)
    auto pml_row = [&](T* dst, const T* src_row_start, bool full, bool count_only, uint32_t& bytes,
                       uint64_t* br) {
        auto cp = [&](int j0, int j1) {
            if (j1 <= j0) return;
            uint32_t nb = (uint32_t)((j1 - j0) * sizeof(T));
            bytes += nb;
            if (!count_only) bulk_g2s(dst + j0, src_row_start + j0, nb, br);
        };
        if (full) {
            cp(0, nfull);
            return;
        }
        int l1 = zpad_tile_l ? min(nfull, round_up(p.pzl - z0 + 2 * H, V)) : 0;
        int r0 = zpad_tile_r ? max(0, ((p.nz - p.pzr - 2 * H) - (z0 - H)) / V * V) : nfull;
        if (l1 >= r0) {
            cp(0, nfull);
            return;
        }
        cp(0, l1);
        cp(r0, nfull);
    };

    // all copies of iteration i (row x0 + i); first pass counts bytes
    auto issue = [&](int i) {
        const int x = x0 + i;
        const int s = i % kD;
        uint64_t* br = &bar[s];
        for (int pass = 0; pass < 2; ++pass) {
            const bool count = pass == 0;
            uint32_t bytes = 0;
            auto cp = [&](T* dst, const T* src, int n) {
                uint32_t nb = (uint32_t)(n * sizeof(T));
                bytes += nb;
                if (!count) bulk_g2s(dst, src, nb, br);
            };
            const int rlo = (i == 0) ? x - R : x + R;
            for (int r = rlo; r <= x + R; ++r) {
                cp(S + L::U + qslot(r) * SROW, ucur + foff2(p, r, z0 - H), nfull);
                if (pml) pml_row(S + L::PX + qslot(r) * SROW, phx_g + foff2(p, r, z0 - H), xpad(r), count, bytes, br);
            }
            cp(S + L::UP + s * TZ, uprev_g + foff2(p, x, z0), nplain);
            cp(S + L::CC + s * TZ, p.c2 + foff2(p, x, z0), nplain);
            if (pml) pml_row(S + L::PZ + s * SROW, phz_g + foff2(p, x, z0 - H), xpad(x), count, bytes, br);
            if (MODE == kAdj && p.image) {
                cp(S + L::DW + s * TZ, p.dw_in + sh + foff2(p, x, z0), nplain);
                cp(S + L::IC + s * TZ, p.ic + sh + foff2(p, x, z0), nplain);
            }
            if (count) mbar_arrive_expect_tx(br, bytes);
        }
    };

    if (t == 0) {
        fence_proxy_async();
        for (int i = 0; i < min(kD, niter); ++i) issue(i);
    }

    // ---- per-thread constants ----
    const int zc = z0 + t * V;
    const bool zin = zc < p.nz;
    T sgz[V], mgz[V];
    bool zok[V], zpe[V];
#pragma unroll
    for (int v = 0; v < V; ++v) {
        const int z = zc + v;
        zok[v] = z > 0 && z < p.nz - 1;
        zpe[v] = z < p.pzl || z >= p.nz - p.pzr;
        sgz[v] = (z < p.nz) ? __ldg(p.sgz + z) : T(0);
        mgz[v] = (MODE == kRecomp && z < p.nz) ? __ldg(p.mgz + z) : T(0);
    }
    bool zpw[NW * V];  // z-padding test of each element of the z-window
#pragma unroll
    for (int j = 0; j < NW * V; ++j) {
        const int z = zc - H + j;
        zpw[j] = z < p.pzl || z >= p.nz - p.pzr;
    }
    bool zpad_vec = false;
#pragma unroll
    for (int v = 0; v < V; ++v) zpad_vec |= zpe[v];
    const int* bx = p.inj.box + shot * 6;
    const bool inj_blk = p.inj.on && bx[0] < x1 && bx[1] > x0 && bx[4] < z0 + zlen && bx[5] > z0;
    T* uprev_out = p.u_prev + sh;
    bool bad = false;

    for (int i = 0; i < niter; ++i) {
        const int x = x0 + i;
        const int s = i % kD;
        if (!mbar_wait_bounded(&bar[s], (uint32_t)((i / kD) & 1), kWaitPolls)) {
            if ((t & 31) == 0 && p.err) atomicOr(p.err, PGB_ERR_TIMEOUT);
        }
        const bool xp = xpad(x);
        const long long o = foff2(p, x, zc);
        const T* uc_row = S + L::U + qslot(x) * SROW;

        // z-window of u_k (and Phi_z) around this thread's V cells
        T w[NW * V];
#pragma unroll
        for (int j = 0; j < NW; ++j) {
            VReg<T> r = vld(uc_row + t * V + j * V);
#pragma unroll
            for (int v = 0; v < V; ++v) w[j * V + v] = r.v[v];
        }
        T xm[R][V], xpv[R][V];
#pragma unroll
        for (int m = 1; m <= R; ++m) {
            VReg<T> a = vld(S + L::U + qslot(x + m) * SROW + H + t * V);
            VReg<T> c = vld(S + L::U + qslot(x - m) * SROW + H + t * V);
#pragma unroll
            for (int v = 0; v < V; ++v) { xpv[m - 1][v] = a.v[v]; xm[m - 1][v] = c.v[v]; }
        }
        const VReg<T> um = vld(S + L::UP + s * TZ + t * V);
        const VReg<T> cc = vld(S + L::CC + s * TZ + t * V);
        VReg<T> dwi, ici;
        if (MODE == kAdj && p.image) {
            dwi = vld(S + L::DW + s * TZ + t * V);
            ici = vld(S + L::IC + s * TZ + t * V);
        }
        const T sgx = __ldg(p.sgx + x);
        const T mgx = (MODE == kRecomp) ? __ldg(p.mgx + x) : T(0);
        const bool xok = x > 0 && x < p.nx - 1;
        const bool inj_row = inj_blk && x >= bx[0] && x < bx[1];

        VReg<T> un, dwo, pxo, pzo;
        if (pml) {
            // PML state taps: rows / elements outside the padding are zero
            T px_c[V], pz_c[V], dpx[V], dpz[V];
            T wp[NW * V];
            const T* pz_row = S + L::PZ + s * SROW;
#pragma unroll
            for (int j = 0; j < NW; ++j) {
                VReg<T> r = vld(pz_row + t * V + j * V);
#pragma unroll
                for (int v = 0; v < V; ++v) wp[j * V + v] = (xp || zpw[j * V + v]) ? r.v[v] : T(0);
            }
            {
                VReg<T> r = vld(S + L::PX + qslot(x) * SROW + H + t * V);
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    px_c[v] = (xp || zpe[v]) ? r.v[v] : T(0);
                    pz_c[v] = wp[H + v];
                    dpx[v] = T(0);
                    dpz[v] = T(0);
                }
            }
#pragma unroll
            for (int m = 1; m <= R; ++m) {
                const bool xpp = xpad(x + m), xpm = xpad(x - m);
                VReg<T> a = vld(S + L::PX + qslot(x + m) * SROW + H + t * V);
                VReg<T> c = vld(S + L::PX + qslot(x - m) * SROW + H + t * V);
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    const T ap = (xpp || zpe[v]) ? a.v[v] : T(0);
                    const T am = (xpm || zpe[v]) ? c.v[v] : T(0);
                    dpx[v] += T(d1w(R, m)) * (ap - am);
                    dpz[v] += T(d1w(R, m)) * (wp[H + v + m] - wp[H + v - m]);
                }
            }
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const int z = zc + v;
                const T uc = w[H + v];
                T lz = T(0), lx = T(0), dz1 = T(0), dx1 = T(0);  // difference form (weights sum to 0)
#pragma unroll
                for (int m = 1; m <= R; ++m) {
                    lz += T(d2w(R, m)) * ((w[H + v + m] - uc) + (w[H + v - m] - uc));
                    lx += T(d2w(R, m)) * ((xpv[m - 1][v] - uc) + (xm[m - 1][v] - uc));
                    dz1 += T(d1w(R, m)) * (w[H + v + m] - w[H + v - m]);
                    dx1 += T(d1w(R, m)) * (xpv[m - 1][v] - xm[m - 1][v]);
                }
                T F = lx * p.idx2 + lz * p.idz2 + dpx[v] * p.idx + dpz[v] * p.idz;
                if (inj_row && z < p.nz) F += inject_rhs(p.inj, bx, shot, x, z);
                const T sx = sgx, sz = sgz[v];
                const T uo = um.v[v], c2 = cc.v[v];
                const bool ok = xok && zok[v];
                T unew, ph_x = T(0), ph_z = T(0);
                if (sx != T(0) || sz != T(0)) {
                    const T dudx = dx1 * p.idx, dudz = dz1 * p.idz;
                    ph_x = px_c[v] - p.dt * sx * px_c[v] + p.dt * (sz - sx) * dudx;
                    ph_z = pz_c[v] - p.dt * sz * pz_c[v] + p.dt * (sx - sz) * dudz;
                    const T fac1 = T(2) * p.dt2 / (T(2) + p.dt * (sx + sz));
                    const T fac2 = c2 * F - (uo - T(2) * uc) * p.idt2 + (sx + sz) * uo * p.i2dt - (sx * sz) * uc;
                    unew = fac1 * fac2;
                } else {
                    unew = p.dt2 * c2 * F - (uo - T(2) * uc);
                }
                if (!ok) { unew = T(0); ph_x = T(0); ph_z = T(0); }
                un.v[v] = unew;
                pxo.v[v] = ph_x;
                pzo.v[v] = ph_z;
                if (MODE == kRecomp) {
                    const T mz = mgz[v];
                    T d = c2 * F + ((mgx + mz) - (sx + sz)) * (unew - uo) * p.i2dt + (mgx * mz - sx * sz) * uc;
                    dwo.v[v] = ok ? d : T(0);
                }
            }
        } else {
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const int z = zc + v;
                const T uc = w[H + v];
                T lz = T(0), lx = T(0);  // difference form (weights sum to 0)
#pragma unroll
                for (int m = 1; m <= R; ++m) {
                    lz += T(d2w(R, m)) * ((w[H + v + m] - uc) + (w[H + v - m] - uc));
                    lx += T(d2w(R, m)) * ((xpv[m - 1][v] - uc) + (xm[m - 1][v] - uc));
                }
                T F = lx * p.idx2 + lz * p.idz2;
                if (inj_row && z < p.nz) F += inject_rhs(p.inj, bx, shot, x, z);
                const T c2 = cc.v[v];
                const bool ok = xok && zok[v];
                T unew = p.dt2 * c2 * F - (um.v[v] - T(2) * uc);
                un.v[v] = ok ? unew : T(0);
                if (MODE == kRecomp) dwo.v[v] = ok ? c2 * F : T(0);
            }
        }

        if (MODE == kFwd || (MODE == kRecomp && p.nan_check)) {
#pragma unroll
            for (int v = 0; v < V; ++v) bad |= !isfinite(un.v[v]);
        }
        if (zin) {
            vst(uprev_out + o, un);
            if (pml && (xp || zpad_vec)) {
                vst(p.phx_out + sh + o, pxo);
                vst(p.phz_out + sh + o, pzo);
            }
            if (MODE == kRecomp && p.dw_out) vst_stream(p.dw_out + sh + o, dwo);
            if (MODE == kAdj && p.image) {
                VReg<T> a;
#pragma unroll
                for (int v = 0; v < V; ++v) a.v[v] = ici.v[v] + w[H + v] * dwi.v[v];
                vst(p.ic + sh + o, a);
            }
        }
        __syncthreads();  // every thread is done with row x's slots
        if (t == 0 && i + kD < niter) {
            fence_proxy_async();
            issue(i + kD);
        }
    }
    if (MODE != kAdj && bad && p.err) atomicOr(p.err, PGB_ERR_NONFINITE);
}

}  // namespace

template <typename T, int R, int MODE>
void launch_wave2d(const WaveParams<T>& p, int bz, cudaStream_t s) {
    (void)bz;
    const int ntiles = p.ntz * p.ntx;
    int grid = ntiles * p.nshot + (MODE != kAdj ? p.rec.blocks : 0);
    wave2d_kernel<T, R, MODE><<<grid, kNT, Smem2<T, R>::bytes, s>>>(p);
}

template <typename T, int R>
static void prep_one() {
    cudaFuncSetAttribute(wave2d_kernel<T, R, kFwd>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)Smem2<T, R>::bytes);
    cudaFuncSetAttribute(wave2d_kernel<T, R, kRecomp>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)Smem2<T, R>::bytes);
    cudaFuncSetAttribute(wave2d_kernel<T, R, kAdj>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)Smem2<T, R>::bytes);
}

void wave2d_prepare() {
    prep_one<float, 1>(); prep_one<float, 2>(); prep_one<float, 3>(); prep_one<float, 4>();
    prep_one<double, 1>(); prep_one<double, 2>(); prep_one<double, 3>(); prep_one<double, 4>();
}

int wave2d_threads() { return kNT; }
int wave2d_tile_z(int dtype_bytes) { return kNT * (16 / dtype_bytes); }

#define PGB_INST2D(T, R)                                                                 \
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
