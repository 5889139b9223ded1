// Two-body contraction of the PNAMP energy on the Blackwell tensor cores (tcgen05).
//
// Replaces the sparse record loop of HFB_Energy_COMPLEX (Codes/PNAMP/PNAMP_Energy_OpenMP.f90:
// 31-90) for whole batches of kernel points. The exact regrouping of its 8-term sum,
//   E2 = sum_r V_r [rho_ki rho_lj - rho_li rho_kj + d_r (rho_ik rho_jl - rho_jk rho_il)]
//      + V_r/4 [K01_ij K10_kl + d_r K01_kl K10_ij],   K_xy = kappa_xy - kappa_yx,
// is two bilinear forms of the densities: a particle-hole form s^T Q s over the n^2
// entries s_e = rho_{r(e) c(e)} and a particle-particle form u^T C w over the antisymmetric
// pair vectors u = K01, w = K10 (i < j). Both are block-diagonal by conserved quantum
// numbers (ph: m_r - m_c, t_r - t_c, parity, closed under negation; pp: m_i + m_j,
// t_i + t_j, parity); the host packs the blocks into groups of <= 256 storage entries
// whose rows and columns are the same contiguous storage range (pnamp_capi.cu::build_tc),
// so every group is one dense square GEMM block G_g = M_g s_g.
//
// The point kernel writes, per kernel point p, the operand rows X[2p + ri][e] (ri = re, im)
// as S bf16 terms whose sum is the FP32 value (S = 2: hi + lo; S = 3: hi + mid + lo), the
// pp epilogue rows Y[2p + ri][e] (u) the same way, and the point's weight w_p = N_p / NFOM^2.
// This kernel computes, for tiles of 64 points (128 operand rows = one UMMA M):
//   D[m][n] = sum_k X[m][k] M_g[n][k]   (tcgen05.mma kind::f16, bf16 in, f32 accumulate)
// with the split products hi*hi + hi*lo + lo*hi (S = 2, "BF16x3") or the six products
// with i + j <= 2 (S = 3, "BF16x6"), then E2(p) = sum_g sum_n y_n(p) D_g[p][n] in the
// epilogue (y = s for ph groups, u for pp groups), complex from the re/im rows.
//
// Roles (192 threads, one CTA per SM, persistent over tiles):
//   warp 0  TMA producer: X tiles (128 x 64) and matrix tiles (NC x 64) per split into a
//           two-stage shared-memory ring, 128-byte swizzled, completion on mbarriers;
//   warp 1  tensor-core issuer: one thread issues the UMMAs of a stage into one of two TMEM
//           accumulators (NC fp32 columns each), commits to the stage's "empty" barrier
//           and, after the last K chunk of a group, to the accumulator's "full" barrier;
//   warps 2-5  epilogue: each reads its 32 TMEM lanes (32x32b loads), multiplies by the
//           epilogue vector read from global memory, and accumulates per-point sums; the
//           accumulator is released as soon as it has been read, so the MMAs of the next
//           group overlap the epilogue of this one.
// Every wait is bounded (kWaitNs); a role that times out sets the error word and all roles
// leave; in-flight copies and MMAs are drained (bounded) before TMEM is freed.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstring>

#include "pnamp_internal.h"
#include "tc_ptx.cuh"

namespace pnamp {

constexpr int kTcRows = 128;        // operand rows per tile: 64 points x (re, im)
constexpr int kTcK = 64;            // K elements per stage (one 128-byte swizzle atom)
constexpr int kTcStages = 2;
constexpr int kTcThreads = 192;
constexpr unsigned long long kWaitNs = 2000000000ull;   // 2 s per wait

template <int S>
struct TcShape {
    static constexpr int NC = (S == 2) ? 256 : 128;                  // UMMA N per group chunk
    static constexpr int XBytes = kTcRows * kTcK * 2;                // 16 KB
    static constexpr int MBytes = NC * kTcK * 2;
    static constexpr int StageBytes = S * (XBytes + MBytes);
    static constexpr int NProd = (S == 2) ? 3 : 6;
    static constexpr int TmemCols = 2 * NC;                          // two accumulators
    static constexpr int SmemBytes = kTcStages * StageBytes + 1024 /* alignment */ + 256 /* barriers */;
};

struct TcMaps {
    CUtensorMap x[3];   // X split arrays [2 npts][nk] bf16, box 64 x 128
    CUtensorMap m[3];   // group matrices [rows][kmax] bf16, box 64 x NC
};

// products (a, b): X term a times matrix term b
__device__ __forceinline__ void tc_product(int S, int i, int &a, int &b) {
    // S = 2: (0,0) (0,1) (1,0); S = 3 adds (0,2) (1,1) (2,0)
    const int pa[6] = {0, 0, 1, 0, 1, 2}, pb[6] = {0, 1, 0, 2, 1, 0};
    a = pa[i];
    b = pb[i];
    (void)S;
}

__device__ __forceinline__ float bf16_bits_to_float(unsigned short b) {
    return __uint_as_float(((unsigned int)b) << 16);
}

template <int S>
__global__ void __launch_bounds__(kTcThreads, 1)
contract_kernel(const __grid_constant__ TcMaps maps, TcArgs a) {
    using Sh = TcShape<S>;
    constexpr int NC = Sh::NC;
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    // 1024-byte aligned operand ring, then barriers
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
    unsigned char *ring = base;
    uint64_t *bars = reinterpret_cast<uint64_t *>(ring + kTcStages * Sh::StageBytes);
    uint64_t *full = bars, *empty = bars + kTcStages, *afull = bars + 2 * kTcStages,
             *aempty = bars + 2 * kTcStages + 2, *drain = bars + 2 * kTcStages + 4;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * kTcStages + 5);
    volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);
    auto xtile = [&](int s, int sp) { return ring + s * Sh::StageBytes + sp * Sh::XBytes; };
    auto mtile = [&](int s, int sp) { return ring + s * Sh::StageBytes + S * Sh::XBytes + sp * Sh::MBytes; };

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kTcStages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&afull[b], 1);
            tc::mbar_init(&aempty[b], 4);
        }
        tc::mbar_init(drain, 1);
        *abort = 0;
        tc::mbar_fence_init();
        for (int sp = 0; sp < S; ++sp) {
            tc::tma_prefetch_desc(&maps.x[sp]);
            tc::tma_prefetch_desc(&maps.m[sp]);
        }
    }
    if (warp == 1) {
        tc::tmem_alloc(tmem_slot, Sh::TmemCols);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tbase = *tmem_slot;
    const int ntiles = (a.npts + 63) / 64;
    auto fail = [&](int code) {
        *abort = 1;
        atomicOr(a.err, code);
    };

    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer
        int s = 0;
        uint32_t ph = 0;
        uint32_t issued_par[kTcStages];
        bool issued[kTcStages] = {};
        bool ok = true;
        for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x)
            for (int g = 0; g < a.ngroups && ok; ++g) {
                const TcGroup G = a.groups[g];
                for (int q = 0; q * NC < G.dpad && ok; ++q)
                    for (int c = 0; c * kTcK < G.dpad; ++c) {
                        if (!tc::mbar_wait(&empty[s], ph ^ 1u, abort, kWaitNs)) {
                            fail(1);
                            ok = false;
                            break;
                        }
                        tc::mbar_arrive_expect_tx(&full[s], Sh::StageBytes);
                        for (int sp = 0; sp < S; ++sp) {
                            tc::tma_load_2d(xtile(s, sp), &maps.x[sp], &full[s], G.off + c * kTcK, tile * kTcRows);
                            tc::tma_load_2d(mtile(s, sp), &maps.m[sp], &full[s], c * kTcK, G.rowbase + q * NC);
                        }
                        issued[s] = true;
                        issued_par[s] = ph;
                        if (++s == kTcStages) {
                            s = 0;
                            ph ^= 1u;
                        }
                    }
            }
        // the tensor core's last arrivals on the ring's empty barriers (one per stage in use)
        // must land before the CTA leaves: wait for each stage as if it were to be refilled
        for (int t = 0; t < kTcStages && ok; ++t) {
            if (!tc::mbar_wait(&empty[s], ph ^ 1u, abort, kWaitNs)) {
                fail(1);
                ok = false;
            }
            if (++s == kTcStages) {
                s = 0;
                ph ^= 1u;
            }
        }
        // and the ring's copies must land before the CTA can leave
        volatile int never = 0;
        for (int t = 0; t < kTcStages; ++t)
            if (issued[t] && !tc::mbar_wait(&full[t], issued_par[t], &never, kWaitNs)) atomicOr(a.err, 8);
    } else if (warp == 1 && lane == 0) {
        // ---------------- tensor-core issuer
        int s = 0;
        uint32_t ph = 0;
        long long u = 0;
        bool ok = true;
        bool any = false;
        for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x)
            for (int g = 0; g < a.ngroups && ok; ++g) {
                const TcGroup G = a.groups[g];
                for (int q = 0; q * NC < G.dpad && ok; ++q) {
                    const int buf = (int)(u & 1);
                    const uint32_t aph = (uint32_t)((u >> 1) & 1);
                    if (!tc::mbar_wait(&aempty[buf], aph ^ 1u, abort, kWaitNs)) {
                        fail(2);
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    const int nrows = min(NC, G.dpad - q * NC);
                    const uint32_t idesc = tc::idesc_bf16_f32(kTcRows, nrows);
                    const uint32_t d = tbase + (uint32_t)(buf * NC);
                    for (int c = 0; c * kTcK < G.dpad; ++c) {
                        if (!tc::mbar_wait(&full[s], ph, abort, kWaitNs)) {
                            fail(2);
                            ok = false;
                            break;
                        }
                        tc::tc_fence_after();
#pragma unroll
                        for (int k16 = 0; k16 < kTcK / 16; ++k16)
#pragma unroll
                            for (int pr = 0; pr < Sh::NProd; ++pr) {
                                int sa, sb;
                                tc_product(S, pr, sa, sb);
                                const uint64_t ad = tc::sdesc_sw128(tc::smem_u32(xtile(s, sa)) + 32u * k16);
                                const uint64_t bd = tc::sdesc_sw128(tc::smem_u32(mtile(s, sb)) + 32u * k16);
                                tc::mma_bf16(d, ad, bd, idesc, (c | k16 | pr) != 0 ? 1u : 0u);
                                any = true;
                            }
                        tc::mma_commit(&empty[s]);
                        if (++s == kTcStages) {
                            s = 0;
                            ph ^= 1u;
                        }
                    }
                    if (!ok) break;
                    tc::mma_commit(&afull[buf]);
                    ++u;
                }
            }
        if (!ok && any) {   // issued MMAs must finish before TMEM is freed
            volatile int never = 0;
            tc::mma_commit(drain);
            if (!tc::mbar_wait(drain, 0, &never, kWaitNs)) atomicOr(a.err, 8);
        }
    } else if (warp >= 2) {
        // ---------------- epilogue
        const int qd = warp & 3;                 // TMEM lane quadrant of this warp
        const int m = 32 * qd + lane;            // accumulator row
        const int ri = m & 1;
        long long u = 0;
        bool ok = true;
        for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
            const long long pt = (long long)tile * 64 + (m >> 1);
            const bool valid = pt < a.npts;
            double acc_a = 0.0, acc_b = 0.0;     // sum y_re D, sum y_im D over this row
            for (int g = 0; g < a.ngroups && ok; ++g) {
                const TcGroup G = a.groups[g];
                const unsigned short *ysrc[3];
                long long ystride;
                int ycol;
                if (G.kind == 0) {
                    for (int sp = 0; sp < 3; ++sp) ysrc[sp] = a.x[sp];
                    ystride = a.nk;
                    ycol = G.off;
                } else {
                    for (int sp = 0; sp < 3; ++sp) ysrc[sp] = a.y[sp];
                    ystride = a.npp;
                    ycol = G.yoff;
                }
                for (int q = 0; q * NC < G.dpad; ++q) {
                    const int buf = (int)(u & 1);
                    const uint32_t aph = (uint32_t)((u >> 1) & 1);
                    int got = 1;
                    if (lane == 0) got = tc::mbar_wait(&afull[buf], aph, abort, kWaitNs) ? 1 : 0;
                    got = __shfl_sync(0xffffffffu, got, 0);
                    if (!got) {
                        if (lane == 0) fail(4);
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    const int nrows = min(NC, G.dpad - q * NC);
                    for (int j = 0; j * 32 < nrows; ++j) {
                        float v[32];
                        tc::tmem_ld32(tbase + ((uint32_t)(32 * qd) << 16) + (uint32_t)(buf * NC + 32 * j), v);
                        if (valid) {
                            const long long col = (long long)ycol + q * NC + 32 * j;
                            float fa = 0.f, fb = 0.f;
#pragma unroll
                            for (int h = 0; h < 4; ++h) {       // 8 columns per 16-byte load
                                float yr[8] = {0, 0, 0, 0, 0, 0, 0, 0}, yi[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
                                for (int sp = 0; sp < S; ++sp) {
                                    const uint4 rr = *reinterpret_cast<const uint4 *>(
                                        ysrc[sp] + (2 * pt) * ystride + col + 8 * h);
                                    const uint4 ii = *reinterpret_cast<const uint4 *>(
                                        ysrc[sp] + (2 * pt + 1) * ystride + col + 8 * h);
                                    const unsigned int wr[4] = {rr.x, rr.y, rr.z, rr.w};
                                    const unsigned int wi[4] = {ii.x, ii.y, ii.z, ii.w};
#pragma unroll
                                    for (int k = 0; k < 4; ++k) {
                                        yr[2 * k] += bf16_bits_to_float((unsigned short)(wr[k] & 0xffffu));
                                        yr[2 * k + 1] += bf16_bits_to_float((unsigned short)(wr[k] >> 16));
                                        yi[2 * k] += bf16_bits_to_float((unsigned short)(wi[k] & 0xffffu));
                                        yi[2 * k + 1] += bf16_bits_to_float((unsigned short)(wi[k] >> 16));
                                    }
                                }
#pragma unroll
                                for (int k = 0; k < 8; ++k) {
                                    fa = fmaf(yr[k], v[8 * h + k], fa);
                                    fb = fmaf(yi[k], v[8 * h + k], fb);
                                }
                            }
                            acc_a += (double)fa;
                            acc_b += (double)fb;
                        }
                    }
                    tc::tc_fence_before();
                    __syncwarp();
                    if (lane == 0) tc::mbar_arrive(&aempty[buf]);
                    ++u;
                }
            }
            if (!ok) break;
            // rows 2p (G_re) and 2p + 1 (G_im): E_re = sum y_re G_re - y_im G_im, E_im = sum y_im G_re + y_re G_im
            const double oa = __shfl_xor_sync(0xffffffffu, acc_a, 1);
            const double ob = __shfl_xor_sync(0xffffffffu, acc_b, 1);
            if (valid && ri == 0) {
                a.e2[2 * pt] = acc_a - ob;
                a.e2[2 * pt + 1] = acc_b + oa;
            }
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tbase, Sh::TmemCols);
    }
}

// Per item (pair, Euler point) of a launch: ZRES(ie, 7) += sum_phi w_phi E2_phi, w = N / NFOM^2
// (0 where T22 was singular or the point was not evaluated), in a fixed order (one warp per
// item, lanes over the gauge points, a fixed shuffle tree): deterministic.
__global__ void contract_finish_kernel(int npairs, int n_euler, int n_gauge, long long nitems,
                                       const int2 *__restrict__ items,
                                       const double *__restrict__ w, const double *__restrict__ e2,
                                       double *__restrict__ zres, int *__restrict__ status,
                                       const int *__restrict__ err) {
    const long long item = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (item >= nitems) return;
    int pair, ie;
    if (items) {
        pair = items[item].x;
        ie = items[item].y;
        if (pair < 0 || pair >= npairs || ie < 0 || ie >= n_euler) return;  // skipped by the point kernel too
    } else {
        pair = (int)(item / n_euler);
        ie = (int)(item % n_euler);
    }
    double sr = 0.0, si = 0.0;
    for (int g = lane; g < n_gauge; g += 32) {
        const long long p = item * n_gauge + g;
        const double wr = w[2 * p], wi = w[2 * p + 1];
        if (wr == 0.0 && wi == 0.0) continue;
        const double er = e2[2 * p], ei = e2[2 * p + 1];
        sr += wr * er - wi * ei;
        si += wr * ei + wi * er;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
        si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    if (lane == 0) {
        double *z = zres + 2LL * ((long long)pair * kNobs * n_euler + 6LL * n_euler + ie);
        z[0] += sr;
        z[1] += si;
        int f = 0;
        if (!isfinite(z[0]) || !isfinite(z[1])) f |= 4;
        if (*err) f |= 16;   // a bounded wait of the contraction ran out: this energy is not valid
        if (f) status[(long long)pair * n_euler + ie] |= f;
    }
}

// ------------------------------------------------------------------ host side
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// 2-D bf16 tensor map: `rows` x `cols` (cols contiguous, a multiple of 8), box 64 x box_rows,
// 128-byte swizzle, out-of-range elements read as zero.
static bool encode_bf16(CUtensorMap *m, const void *base, unsigned long long cols, unsigned long long rows,
                        unsigned box_rows) {
    auto fn = encode_fn();
    if (!fn || (cols % 8) != 0 || (reinterpret_cast<uintptr_t>(base) & 15) != 0) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kTcK, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int tc_smem_bytes(int splits) { return splits == 3 ? TcShape<3>::SmemBytes : TcShape<2>::SmemBytes; }
int tc_chunk_rows(int splits) { return splits == 3 ? TcShape<3>::NC : TcShape<2>::NC; }

cudaError_t prepare_contract() {
    cudaError_t e = cudaFuncSetAttribute(contract_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         TcShape<2>::SmemBytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(contract_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 TcShape<3>::SmemBytes);
    return e;
}

cudaError_t launch_contract(const TcArgs &a, const void *const *mat, long long mat_rows, int kmax, int grid,
                            cudaStream_t st) {
    if (a.splits != 2 && a.splits != 3) return cudaErrorInvalidValue;
    TcMaps maps;
    memset(&maps, 0, sizeof(maps));
    const int nc = tc_chunk_rows(a.splits);
    for (int sp = 0; sp < a.splits; ++sp) {
        if (!encode_bf16(&maps.x[sp], a.x[sp], (unsigned long long)a.nk, 2ull * (unsigned long long)a.npts,
                         kTcRows) ||
            !encode_bf16(&maps.m[sp], mat[sp], (unsigned long long)kmax, (unsigned long long)mat_rows, nc))
            return cudaErrorInvalidValue;
    }
    const int ntiles = (int)((a.npts + 63) / 64);
    grid = grid < ntiles ? grid : ntiles;
    if (grid < 1) return cudaSuccess;
    if (a.splits == 2)
        contract_kernel<2><<<grid, kTcThreads, TcShape<2>::SmemBytes, st>>>(maps, a);
    else
        contract_kernel<3><<<grid, kTcThreads, TcShape<3>::SmemBytes, st>>>(maps, a);
    return cudaGetLastError();
}

cudaError_t launch_contract_finish(int npairs, int n_euler, int n_gauge, long long nitems, const int2 *items,
                                   const double *w, const double *e2, double *zres, int *status, const int *err,
                                   cudaStream_t st) {
    if (nitems <= 0) return cudaSuccess;
    const int per_block = 8;
    const long long blocks = (nitems + per_block - 1) / per_block;
    contract_finish_kernel<<<(unsigned)blocks, 32 * per_block, 0, st>>>(npairs, n_euler, n_gauge, nitems, items,
                                                                       w, e2, zres, status, err);
    return cudaGetLastError();
}

}  // namespace pnamp
