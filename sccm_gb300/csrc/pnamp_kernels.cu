// PNAMP kernels for GB300 (sm_103a): the per-point algebra in FP64 (zc) or double-float
// (zd, float pairs on the FP32 pipes), one template.
//
// Work decomposition (one CUDA launch per stage, batched over pairs):
//   setup_kernel   one CTA per (q,q') pair: W = V1 U1^-1, Z0 = V0 U0^-1, the
//                  bare-vacuum overlaps det(1 + Z^T Z)^(-1/4) (zbareover,
//                  Codes/PNAMP/PNAMP_Proj.f90:6-79), and the once-per-pair pieces of
//                  the reduced Pfaffian (Z0^-1, Pf(-c Z0)) and the species-split flag.
//   point_kernel   persistent; one CTA per (pair, Euler point) work item at a
//                  time. Per Euler point it builds the block-diagonal Wigner-D
//                  rotation R (ROTATION_MAT, PNAMP_Proj.f90:83-136) and the
//                  gauge-independent pieces X = R W R^T, R V1, R* U1 and the four
//                  species partials of T22; then for each of the NFOM^2 gauge points:
//                  the Pfaffian of the point's skew matrix (Pfaf_Over + ZPfaffianF +
//                  ZExch, PNAMP_Proj.f90:142-392; the n x n Schur complement c (D X D -
//                  Z0^-1) when V0 is well conditioned, two h x h species blocks for
//                  charge-conserving pairs, else the 2n x 2n matrix) beside the column
//                  Gauss-Jordan solve Y T22^-1 on other warps (named barriers), then
//                  rho, kappa10, kappa01 (ROKAPPAphiomega, :459-551) and the observables
//                  of Kernel3D.f90:296-358 (ZN_0, the energy of
//                  PNAMP_Energy_OpenMP.f90:31-90 or the split-bf16 rows for the tensor-
//                  core contraction in contract_tc.cu, ZJ2_0, ZQ2/ZQ2t), summed into
//                  ZRES(iang, io) (Kernel3D.f90:385-387). Species-split pairs run two
//                  gauge points at a time on the two halves of the CTA
//                  (split_pair_points) with compact species-block densities.
//   project_kernel J/K projection of ZRES (Kernel3D.f90:415-751, plain form of
//                  PNAMP_Kernel3D_v2.f90:477-498).
//
// Algebra used instead of the reference's per-point LU inverses (exact in
// exact arithmetic): with A = D_phi R, D_phi = diag(e^{i phi_p}, e^{i phi_n}),
//   conj(Vbar1) conj(Ubar1)^-1 = A V1 U1^-1 A^T = D (R W R^T) D,
//   T22 = V0^T A V1 + U0^T A* U1 = sum_s e^{+-i phi_s} (species partials),
//   rho = D (R V1 T22^-1) V0^T, kappa10 = D (R V1 T22^-1) U0^T,
//   kappa01 = -D* (R* U1 T22^-1) V0^T.
#include <cuda_bf16.h>

#include <type_traits>

#include "pnamp_df64.cuh"
#include "../../include/pnamp_gpu.h"
#include "pnamp_internal.h"

namespace pnamp {

// A value as S = 2 or 3 bf16 terms t0 + t1 (+ t2), each the bf16 rounding of what the
// previous terms leave (8 significant bits each: ~2^-17 relative left for S = 2, ~2^-25 for
// S = 3). v - t0 is exact in FP32 (t0 is v rounded to 8 bits); the double-float low word
// enters the first remainder.
__device__ __forceinline__ void bf16_terms(dd v, int S, unsigned short (&t)[3]) {
    const __nv_bfloat16 b0 = __float2bfloat16_rn(v.hi);
    const float r1 = __fadd_rn(__fsub_rn(v.hi, __bfloat162float(b0)), v.lo);
    const __nv_bfloat16 b1 = __float2bfloat16_rn(r1);
    const float r2 = __fsub_rn(r1, __bfloat162float(b1));
    t[0] = __bfloat16_as_ushort(b0);
    t[1] = __bfloat16_as_ushort(b1);
    t[2] = S > 2 ? __bfloat16_as_ushort(__float2bfloat16_rn(r2)) : (unsigned short)0;
}
__device__ __forceinline__ dd as_dd(double v) { return dd_from(v); }
__device__ __forceinline__ dd as_dd(dd v) { return v; }

// ------------------------------------------------------------------ scalars
__device__ __forceinline__ double sabs1(double a) { return fabs(a); }
__device__ __forceinline__ double sabs1(zc a) { return fabs(a.x) + fabs(a.y); }
__device__ __forceinline__ double srecip(double a) { return 1.0 / a; }
__device__ __forceinline__ zc srecip(zc a) { return zrecip(a); }
__device__ __forceinline__ double smul(double a, double b) { return a * b; }
__device__ __forceinline__ zc smul(zc a, zc b) { return a * b; }
__device__ __forceinline__ double sfms(double a, double b, double c) { return fma(-a, b, c); }
__device__ __forceinline__ zc sfms(zc a, zc b, zc c) { return zfms(a, b, c); }
template <typename T> __device__ __forceinline__ T szero();
template <> __device__ __forceinline__ double szero<double>() { return 0.0; }
template <> __device__ __forceinline__ zc szero<zc>() { return mk(0.0, 0.0); }
// pivot magnitude of a double-float value: the float sum of the high words, compared as a
// float (the FP64 pipe is narrow on this part, and a float compares the same as its double)
__device__ __forceinline__ float sabs1(zd a) { return fabsf(a.x.hi) + fabsf(a.y.hi); }
__device__ __forceinline__ zd srecip(zd a) { return zrecip(a); }
__device__ __forceinline__ zd smul(zd a, zd b) { return a * b; }
__device__ __forceinline__ zd sfms(zd a, zd b, zd c) { return zfms(a, b, c); }
template <> __device__ __forceinline__ zd szero<zd>() { return mkd(dd_make(0.0f, 0.0f), dd_make(0.0f, 0.0f)); }

// Arithmetic traits of the per-point algebra: zc = FP64 complex (plain form),
// zd = double-float complex (df64 form). R is the matching real type.
template <class Z> struct Ar;
template <> struct Ar<zc> {
    using R = double;
    static __device__ __forceinline__ zc from(zc a) { return a; }
    static __device__ __forceinline__ zc to(zc a) { return a; }
    static __device__ __forceinline__ R real(double v) { return v; }
    static __device__ __forceinline__ R rmul(R a, R b) { return a * b; }
    static __device__ __forceinline__ bool nz(R a) { return a != 0.0; }
    static __device__ __forceinline__ R pick(const double *d, const dd *, long long i) { return d[i]; }
    static __device__ __forceinline__ R rzero() { return 0.0; }
    static __device__ __forceinline__ R rconst(float v) { return (double)v; }   // exact
    static __device__ __forceinline__ R radd(R a, R b) { return a + b; }
    static __device__ __forceinline__ R rfma(R a, R b, R c) { return fma(a, b, c); }
    static __device__ __forceinline__ double dbl(R a) { return a; }
    static __device__ __forceinline__ R wsum(R v) {   // butterfly: the sum in every lane
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        return v;
    }
    // pivot key: max(|re|, |im|) as the bit pattern of a non-negative double
    static __device__ __forceinline__ unsigned long long key(zc z) {
        const unsigned long long kx = (unsigned long long)__double_as_longlong(z.x) & 0x7fffffffffffffffull;
        const unsigned long long ky = (unsigned long long)__double_as_longlong(z.y) & 0x7fffffffffffffffull;
        return kx > ky ? kx : ky;
    }
};
template <> struct Ar<zd> {
    using R = dd;
    static __device__ __forceinline__ zd from(zc a) { return zd_from(a); }
    static __device__ __forceinline__ zc to(zd a) { return zd_to(a); }
    static __device__ __forceinline__ R real(double v) { return dd_from(v); }
    static __device__ __forceinline__ R rmul(R a, R b) { return dd_mul(a, b); }
    static __device__ __forceinline__ bool nz(R a) { return a.hi != 0.0f; }
    static __device__ __forceinline__ R pick(const double *, const dd *f, long long i) { return f[i]; }
    static __device__ __forceinline__ R rzero() { return dd_make(0.0f, 0.0f); }
    static __device__ __forceinline__ R rconst(float v) { return dd_make(v, 0.0f); }   // exact
    static __device__ __forceinline__ R radd(R a, R b) { return dd_add(a, b); }
    static __device__ __forceinline__ R rfma(R a, R b, R c) { return dd_fma(a, b, c); }
    static __device__ __forceinline__ double dbl(R a) { return dd_to(a); }
    static __device__ __forceinline__ R wsum(R v) {   // in double-float on the FP32 pipes
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v = dd_add(v, dd_make(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)));
        return v;
    }
    static __device__ __forceinline__ unsigned long long key(zd z) {
        const unsigned int kx = __float_as_uint(z.x.hi) & 0x7fffffffu;
        const unsigned int ky = __float_as_uint(z.y.hi) & 0x7fffffffu;
        return kx > ky ? kx : ky;
    }
};


// Pivot row for column k (largest |re|+|im|, first on ties, as IZAMAX): warp 0
// searches, the result is broadcast through sh[0] (row) and sh[1] (zero column).
template <typename T>
__device__ __forceinline__ int pivot_search(const T *A, int lda, int k, int n, int *sh, T *invd, bool &zero) {
    using Mag = decltype(sabs1(A[0]));
    if (threadIdx.x < 32) {
        Mag v = -1;
        int idx = 0x7fffffff;
        for (int i = k + (int)threadIdx.x; i < n; i += 32) {
            const Mag a = sabs1(A[i * lda + k]);
            if (a > v) {
                v = a;
                idx = i;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const Mag ov = __shfl_down_sync(0xffffffffu, v, o);
            const int oi = __shfl_down_sync(0xffffffffu, idx, o);
            if (ov > v || (ov == v && oi < idx)) {
                v = ov;
                idx = oi;
            }
        }
        if (threadIdx.x == 0) {
            // no comparable entry (all NaN): report a zero column, keep row k
            const bool none = (idx == 0x7fffffff);
            const bool z = none || v == Mag(0);
            sh[0] = none ? k : idx;
            sh[1] = z ? 1 : 0;
            invd[k] = z ? szero<T>() : srecip(A[(none ? k : idx) * lda + k]);
        }
    }
    __syncthreads();
    zero = sh[1] != 0;
    return sh[0];
}

// In-place LU with partial pivoting, P A = L U (L unit lower). perm[k] is the
// row exchanged with row k at step k (LAPACK ipiv, 0-based); invd[k] = 1/U_kk.
// Returns true if an exactly zero pivot column was met.
template <typename T>
__device__ bool lu_factor(T *A, int n, int lda, int *perm, T *invd, int *sh) {
    bool sing = false;
    for (int k = 0; k < n; ++k) {
        bool zero;
        const int p = pivot_search(A, lda, k, n, sh, invd, zero);
        if (p != k)
            for (int j = threadIdx.x; j < n; j += blockDim.x) {
                const T t = A[k * lda + j];
                A[k * lda + j] = A[p * lda + j];
                A[p * lda + j] = t;
            }
        if (threadIdx.x == 0) perm[k] = p;
        __syncthreads();
        if (zero) {
            sing = true;
            continue;
        }
        const T inv = invd[k];
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) A[i * lda + k] = smul(A[i * lda + k], inv);
        __syncthreads();
        const int m = n - k - 1;
        if (m > 0) {
            const int dq = blockDim.x / m, dr = blockDim.x % m;
            int i = k + 1 + threadIdx.x / m, j = k + 1 + threadIdx.x % m;
            for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
                A[i * lda + j] = sfms(A[i * lda + k], A[k * lda + j], A[i * lda + j]);
                i += dq;
                j += dr;
                if (j >= k + 1 + m) {
                    j -= m;
                    ++i;
                }
            }
        }
        __syncthreads();
    }
    return sing;
}

// Warp argmax by one integer max-reduction (redux.sync): the key of candidate j (offset
// jrel = j - j0 < 64) is the magnitude's bit pattern (a non-negative float compares like its
// bits) with the low 6 bits replaced by 63 - jrel, so the largest magnitude wins and ties go
// to the first column, magnitudes being compared to 2^-17 relative. Lanes pass their best key
// (0 for no candidate). Returns the winning offset in bits 0..5 of the reduced key; the key's
// magnitude part is 0 when every candidate was zero (or not a number, which counts as zero).
__device__ __forceinline__ unsigned pack_key(float mag, int jrel) {
    return (mag >= 0.0f ? (__float_as_uint(mag) & ~63u) : 0u) | (unsigned)(63 - jrel);
}
__device__ __forceinline__ unsigned pack_key_bits(unsigned bits, int jrel) { return (bits & ~63u) | (unsigned)(63 - jrel); }
// the grouped eliminations search at most n <= PNAMP_MAX_NLEV candidates
static_assert(PNAMP_MAX_NLEV <= 64, "pivot offsets are packed into 6 bits (7 for the 2n x 2n Pfaffian)");

// A warp-aligned group of the CTA's threads with its own named barrier (bar.sync id,
// count; id 0 with the whole CTA is __syncthreads). Lets two independent latency-bound
// eliminations run at the same time on disjoint warps.
struct Grp {
    int tid, nthr, wid, bar;
};
__device__ __forceinline__ void gsync(const Grp &g) {
    asm volatile("bar.sync %0, %1;" ::"r"(g.bar), "r"(g.nthr) : "memory");
}

// Y <- Y A^-1 (Y: ny x n, A: n x n, both row-major with leading dimension n) by
// column-oriented Gauss-Jordan elimination: column operations E reduce A to the
// identity (A E = I, so E = A^-1), and the same operations applied to the rows of Y
// give Y A^-1. Step k takes the pivot in row k (largest |A_kc|, c >= k; partial
// pivoting on A^T), moves column c to k, scales it and removes row k from every other
// column. Rows < k of A are unit rows by then and are not touched again. Two barriers
// per step and (n - k - 1 + ny)(n - 1) independent updates per step, against the
// 2n + n sequential steps of an LU followed by two triangular column sweeps: the
// elimination is latency-bound at these sizes, so fewer, fuller steps win although
// the flop count is higher. A holds garbage on return; prow (n) and pinv (1) are
// shared scratch. Returns true if an exactly zero pivot row was met.
template <typename T>
__device__ bool gj_right_solve(T *A, int n, T *Y, int ny, T *prow, T *pinv, int *sh) {
    const int lane = threadIdx.x & 31;
    auto search = [&](int k) {  // warp 0: pivot column of row k -> sh[0], zero flag sh[1], pinv[0]
        if constexpr (std::is_same<T, zd>::value) {   // one redux.sync
            unsigned key = 0u;
            for (int j = k + lane; j < n; j += 32) {
                const unsigned kk = pack_key(sabs1(A[k * n + j]), j - k);
                key = key > kk ? key : kk;
            }
            const unsigned m = __reduce_max_sync(0xffffffffu, key);
            if (lane == 0) {
                const int idx = k + 63 - (int)(m & 63u);
                const bool z = (m >> 6) == 0u;
                sh[0] = idx;
                sh[1] = z ? 1 : 0;
                pinv[0] = z ? szero<T>() : srecip(A[k * n + idx]);
            }
        } else {
            using Mag = decltype(sabs1(A[0]));
            Mag v = -1;
            int idx = 0x7fffffff;
            for (int j = k + lane; j < n; j += 32) {
                const Mag a = sabs1(A[k * n + j]);
                if (a > v) {
                    v = a;
                    idx = j;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const Mag ov = __shfl_down_sync(0xffffffffu, v, o);
                const int oi = __shfl_down_sync(0xffffffffu, idx, o);
                if (ov > v || (ov == v && oi < idx)) {
                    v = ov;
                    idx = oi;
                }
            }
            if (lane == 0) {
                const bool none = (idx == 0x7fffffff);  // all NaN: keep column k, report zero
                const bool z = none || v == Mag(0);
                sh[0] = none ? k : idx;
                sh[1] = z ? 1 : 0;
                pinv[0] = z ? szero<T>() : srecip(A[k * n + (none ? k : idx)]);
            }
        }
    };
    bool sing = false;
    if (threadIdx.x < 32) search(0);
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        const int c = sh[0];
        if (sh[1]) sing = true;
        const T pv = pinv[0];
        // phase 1: each remaining row r gets m_r = M[r][c] / A[k][c] in column k and its old
        // column k in column c; the pivot row (columns k and c exchanged) goes to prow
        const int nrT = n - k - 1, nrows = nrT + ny;
        for (int t = threadIdx.x; t < nrows + n; t += blockDim.x) {
            if (t < nrows) {
                T *row = t < nrT ? A + (long long)(k + 1 + t) * n : Y + (long long)(t - nrT) * n;
                const T a = row[c], b = row[k];
                row[k] = smul(a, pv);
                if (c != k) row[c] = b;
            } else {
                const int j = t - nrows;
                prow[j] = (j == c) ? A[k * n + k] : A[k * n + j];
            }
        }
        __syncthreads();
        // phase 2: M[r][j] -= m_r prow[j] for j != k. Warp 0 takes row k + 1 of A and then
        // searches its pivot, so the next step needs no extra barrier.
        if (threadIdx.x < 32) {
            if (k + 1 < n) {
                T *row = A + (long long)(k + 1) * n;
                const T m = row[k];
                for (int j = lane; j < n; j += 32)
                    if (j != k) row[j] = sfms(m, prow[j], row[j]);
                __syncwarp();
                search(k + 1);
            }
        } else {
            const int nrA = n - k - 2 > 0 ? n - k - 2 : 0;
            const int total = (nrA + ny) * n, stride = blockDim.x - 32;
            const int dq = stride / n, dr = stride % n;
            int rr = (threadIdx.x - 32) / n, j = (threadIdx.x - 32) % n;
            for (int t = threadIdx.x - 32; t < total; t += stride) {
                if (j != k) {
                    T *row = rr < nrA ? A + (long long)(k + 2 + rr) * n : Y + (long long)(rr - nrA) * n;
                    row[j] = sfms(row[k], prow[j], row[j]);
                }
                rr += dq;
                j += dr;
                if (j >= n) {
                    j -= n;
                    ++rr;
                }
            }
        }
        __syncthreads();
    }
    return sing;
}

// gj_right_solve for NB = 1 or 2 independent systems at once, by the thread group g (at
// least NB warps plus h threads; warp b of the group searches the pivots of system b): A holds
// NB h x h matrices (compact, the second at A + h*h) and Y NB ny x h blocks (the second at
// Y + ny*h); Y_b <- Y_b A_b^-1 in h steps of two group barriers. prow holds NB*h scratch
// values, pinv NB, sh 2*NB ints. Returns true if an exactly zero pivot row was met in any
// system. NB = 2 serves the two species blocks of a species-split point, NB = 1 the whole
// n x n system of a general point while other warps eliminate its Pfaffian.
template <typename T, int NB = 2>
__device__ bool gj_right_solve_g(const Grp &g, T *A, int h, T *Y, int ny, T *prow, T *pinv, int *sh) {
    const int lane = g.tid & 31, wid = g.wid;
    const int hh = h * h, yh = ny * h;
    // The search of step k + 1 runs beside each step's updates, on its critical path, so in
    // the double-float form it is one redux.sync; the FP64 form keeps the shuffle search.
    constexpr bool kDF = std::is_same<T, zd>::value;
    auto search = [&](int b, int k) {  // warp b: pivot column of row k of A_b
        const T *Ab = A + b * hh;
        if constexpr (kDF) {
            unsigned key = 0u;
            for (int j = k + lane; j < h; j += 32) {
                const unsigned kk = pack_key(sabs1(Ab[k * h + j]), j - k);
                key = key > kk ? key : kk;
            }
            const unsigned m = __reduce_max_sync(0xffffffffu, key);
            if (lane == 0) {
                const int idx = k + 63 - (int)(m & 63u);
                const bool z = (m >> 6) == 0u;
                sh[2 * b] = idx;
                sh[2 * b + 1] = z ? 1 : 0;
                pinv[b] = z ? szero<T>() : srecip(Ab[k * h + idx]);
            }
        } else {
            using Mag = decltype(sabs1(A[0]));
            Mag v = -1;
            int idx = 0x7fffffff;
            for (int j = k + lane; j < h; j += 32) {
                const Mag a = sabs1(Ab[k * h + j]);
                if (a > v) {
                    v = a;
                    idx = j;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const Mag ov = __shfl_down_sync(0xffffffffu, v, o);
                const int oi = __shfl_down_sync(0xffffffffu, idx, o);
                if (ov > v || (ov == v && oi < idx)) {
                    v = ov;
                    idx = oi;
                }
            }
            if (lane == 0) {
                const bool none = (idx == 0x7fffffff);
                const bool z = none || v == Mag(0);
                sh[2 * b] = none ? k : idx;
                sh[2 * b + 1] = z ? 1 : 0;
                pinv[b] = z ? szero<T>() : srecip(Ab[k * h + (none ? k : idx)]);
            }
        }
    };
    bool sing = false;
    // phase-2 layout of warps NB..: rpi rows at a time, one column per thread
    constexpr int kRes = 32 * NB;
    const int rpi = (g.nthr - kRes) / h, jc = (g.tid - kRes) % h, r0 = (g.tid - kRes) / h;
    if (wid < NB) search(wid, 0);
    gsync(g);
    for (int k = 0; k < h; ++k) {
        const int c0 = sh[0], c1 = NB > 1 ? sh[2] : 0;
        if (sh[1] || (NB > 1 && sh[3])) sing = true;
        // phase 1 (all systems): m_r = M[r][c] / A[k][c] into column k, old column k into
        // column c, the exchanged pivot row into prow
        const int nrT = h - k - 1, nrows = nrT + ny, per1 = nrows + h;
        for (int t = g.tid; t < NB * per1; t += g.nthr) {
            const int b = t >= per1 ? 1 : 0, u = t - b * per1;
            const int c = b ? c1 : c0;
            T *Ab = A + b * hh;
            if (u < nrows) {
                T *row = u < nrT ? Ab + (k + 1 + u) * h : Y + b * yh + (u - nrT) * h;
                const T a = row[c], bb = row[k];
                row[k] = smul(a, pinv[b]);
                if (c != k) row[c] = bb;
            } else {
                const int j = u - nrows;
                prow[b * h + j] = (j == c) ? Ab[k * h + k] : Ab[k * h + j];
            }
        }
        gsync(g);
        // phase 2: M[r][j] -= m_r prow[j] for j != k; warp b takes row k + 1 of A_b, then its pivot
        if (wid < NB) {
            if (k + 1 < h) {
                T *row = A + wid * hh + (k + 1) * h;
                const T m = row[k];
                for (int j = lane; j < h; j += 32)
                    if (j != k) row[j] = sfms(m, prow[wid * h + j], row[j]);
                __syncwarp();
                search(wid, k + 1);
            }
        } else if (r0 < rpi && jc != k) {
            // thread (r0, jc): column jc of every rpi-th row of all systems; the pivot-row
            // values stay in registers and m_r = row[k] is a broadcast load
            const int nrA = h - k - 2 > 0 ? h - k - 2 : 0;
            const int rows_b = nrA + ny;
            const T pj0 = prow[jc], pj1 = NB > 1 ? prow[h + jc] : pj0;
            for (int R = r0; R < NB * rows_b; R += rpi) {
                const int b = R >= rows_b ? 1 : 0, rr = R - b * rows_b;
                T *row = rr < nrA ? A + b * hh + (k + 2 + rr) * h : Y + b * yh + (rr - nrA) * h;
                row[jc] = sfms(row[k], b ? pj1 : pj0, row[jc]);
            }
        }
        gsync(g);
    }
    return sing;
}

// Y <- Y A^-1 for nr rows of Y (leading dimension ldy), A = P^T L U from lu_factor.
template <typename T>
__device__ void row_solve(T *Y, int nr, int ldy, const T *A, int n, int lda, const int *perm,
                          const T *invd) {
    for (int j = 0; j < n; ++j) {  // Z U = B, column by column
        const T inv = invd[j];
        for (int r = threadIdx.x; r < nr; r += blockDim.x) Y[r * ldy + j] = smul(Y[r * ldy + j], inv);
        __syncthreads();
        const int m = n - j - 1;
        if (m > 0) {
            const int dq = blockDim.x / m, dr = blockDim.x % m;
            int r = threadIdx.x / m, c = j + 1 + threadIdx.x % m;
            for (int t = threadIdx.x; t < nr * m; t += blockDim.x) {
                Y[r * ldy + c] = sfms(Y[r * ldy + j], A[j * lda + c], Y[r * ldy + c]);
                r += dq;
                c += dr;
                if (c >= n) {
                    c -= m;
                    ++r;
                }
            }
            __syncthreads();
        }
    }
    for (int j = n - 1; j > 0; --j) {  // Y2 L = Z, last column first
        const int dq = blockDim.x / j, dr = blockDim.x % j;
        int r = threadIdx.x / j, c = threadIdx.x % j;
        for (int t = threadIdx.x; t < nr * j; t += blockDim.x) {
            Y[r * ldy + c] = sfms(Y[r * ldy + j], A[j * lda + c], Y[r * ldy + c]);
            r += dq;
            c += dr;
            if (c >= j) {
                c -= j;
                ++r;
            }
        }
        __syncthreads();
    }
    for (int r = threadIdx.x; r < nr; r += blockDim.x)  // Y = Y2 P: column swaps in reverse
        for (int k = n - 1; k >= 0; --k) {
            const int p = perm[k];
            if (p != k) {
                const T t = Y[r * ldy + k];
                Y[r * ldy + k] = Y[r * ldy + p];
                Y[r * ldy + p] = t;
            }
        }
    __syncthreads();
}

// ------------------------------------------------------------------ Pfaffian
// Exchange of indices p < q of a skew matrix held in its upper triangle, rows
// >= r only (ZExch, PNAMP_Proj.f90:356-392). Every thread touches distinct entries.
template <class Z>
__device__ __forceinline__ void exch_upper(Z *S, int N, int r, int p, int q) {
    for (int i = r + threadIdx.x; i < N; i += blockDim.x) {
        if (i < p) {
            const Z t = S[i * N + p];
            S[i * N + p] = S[i * N + q];
            S[i * N + q] = t;
        } else if (i > q) {
            const Z t = S[p * N + i];
            S[p * N + i] = S[q * N + i];
            S[q * N + i] = t;
        } else if (i > p && i < q) {
            const Z t = S[p * N + i];
            S[p * N + i] = -S[i * N + q];
            S[i * N + q] = -t;
        } else if (i == p) {
            S[p * N + q] = -S[p * N + q];
        }
    }
    __syncthreads();
}

// Running product of the Pfaffian's pivots. FP64 form: a complex double. Double-float
// form: a double-float mantissa renormalised to [1/2, 1) in its largest part after every
// factor, with the power of two kept as an integer, so that a product of many small or
// large pivots neither leaves the float range nor needs the (narrow) FP64 pipe; one
// conversion at the end.
template <class Z> struct PfProd;
template <> struct PfProd<zc> {
    zc v = {1.0, 0.0};
    __device__ __forceinline__ void mul(zc f, bool neg) { v = (neg ? -1.0 : 1.0) * (v * f); }
    __device__ __forceinline__ zc get() const { return v; }
};
template <> struct PfProd<zd> {
    zd m = {{1.0f, 0.0f}, {0.0f, 0.0f}};
    int e = 0;
    __device__ __forceinline__ void mul(zd f, bool neg) {
        m = m * f;
        if (neg) m = -m;
        const float a = fmaxf(fabsf(m.x.hi), fabsf(m.y.hi));
        if (a > 0.0f && a <= 3.0e38f) {
            int ex;
            frexpf(a, &ex);
            m.x.hi = ldexpf(m.x.hi, -ex);
            m.x.lo = ldexpf(m.x.lo, -ex);
            m.y.hi = ldexpf(m.y.hi, -ex);
            m.y.lo = ldexpf(m.y.lo, -ex);
            e += ex;
        }
    }
    __device__ __forceinline__ zc get() const {
        const zc z = zd_to(m);
        return mk(ldexp(z.x, e), ldexp(z.y, e));
    }
};
// Pivot test of the Pfaffians: 0 fine, 1 |pivot| <= 1e-13 (the reference's exit), 2 not finite.
__device__ __forceinline__ int pivot_flag(zc ss) { return !zfinite(ss) ? 2 : (!(abs2(ss) > 1.0e-26) ? 1 : 0); }
__device__ __forceinline__ int pivot_flag(zd ss) {
    if (!zfinite(ss)) return 2;
    const float a = fabsf(ss.x.hi), b = fabsf(ss.y.hi);
    // |ss|^2 > 1e-26 in float (the sum of squares underflows only far below the threshold)
    return (a > 1.0e-13f || b > 1.0e-13f || a * a + b * b > 1.0e-26f) ? 0 : 1;
}

// Pfaffian of the N x N skew matrix in the upper triangle of S (row-major), the
// 2x2-block elimination of ZPfaffianF (PNAMP_Proj.f90:218-350) with partial instead of
// global pivoting: at each step the largest entry of row r right of the diagonal (first
// maximum; magnitude max(|re|,|im|)) is moved to (r, r+1), the sign flips once per
// exchange, Pf = 0 when |pivot| <= 1e-13, and the Schur complement is updated in place.
// The running product is a PfProd. `vec` holds N scratch values; `flag` 2 ints.
template <class Z>
__device__ zc pfaffian_upper(Z *S, int N, Z *vec, double *red, int *flag, int &underflow) {
    // Parlett-Reid elimination with partial pivoting: step k takes the largest entry of
    // row r = 2k right of the diagonal as the 2x2 pivot (swapping its column with c = r + 1),
    // a one-warp search. (The reference's ZPfaffianF searches the whole remaining upper
    // triangle, PNAMP_Proj.f90:258-268; both are stable, results agree to rounding.)
    using A = Ar<Z>;
    PfProd<Z> pf;  // running product, meaningful in thread 0
    underflow = 0;
    const int NB = N / 2;
    for (int k = 0; k < NB - 1; ++k) {
        const int r = 2 * k, c = r + 1;
        if (std::is_same<Z, zd>::value && threadIdx.x < 32) {
            // one redux.sync over keys with 7 offset bits (N = 2n <= 128 candidates; the
            // high bits of the 31-bit magnitude key first, ties to the first column)
            unsigned key = 0u;
            for (int j = c + (int)threadIdx.x; j < N; j += 32) {
                const unsigned kk = ((unsigned)A::key(S[r * N + j]) & ~127u) | (unsigned)(127 - (j - c));
                key = key > kk ? key : kk;
            }
            const unsigned m = __reduce_max_sync(0xffffffffu, key);
            if (threadIdx.x == 0) flag[1] = c + 127 - (int)(m & 127u);
        } else if (threadIdx.x < 32) {
            unsigned long long best = 0ull;
            int bidx = 0x7fffffff;
            for (int j = c + (int)threadIdx.x; j < N; j += 32) {
                const unsigned long long key = A::key(S[r * N + j]);
                if (key > best || bidx == 0x7fffffff) {
                    best = key;
                    bidx = j;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long ob = __shfl_down_sync(0xffffffffu, best, o);
                const int oi = __shfl_down_sync(0xffffffffu, bidx, o);
                if (oi != 0x7fffffff && (bidx == 0x7fffffff || ob > best || (ob == best && oi < bidx))) {
                    best = ob;
                    bidx = oi;
                }
            }
            if (threadIdx.x == 0) flag[1] = bidx;
        }
        __syncthreads();
        const int i2 = flag[1];
        if (i2 == 0x7fffffff) {  // no candidate: cannot happen for N - c >= 1
            underflow = 2;
            return mk(0.0, 0.0);
        }
        // the global-pivot sign rule with i1 = r (PNAMP_Proj.f90:273-275): -1, +1 without exchange
        const bool neg = (i2 != c);
        if (i2 != c) exch_upper(S, N, r, c, i2);
        if (threadIdx.x == 0) {  // pivot test, reciprocal and running product by one thread
            const Z ssz = S[r * N + c];
            const int f = pivot_flag(ssz);
            flag[0] = f;
            if (f == 0) {
                vec[c] = zrecip(ssz);
                pf.mul(ssz, neg);
            }
        }
        __syncthreads();
        if (flag[0]) {
            underflow = flag[0];
            __syncthreads();
            return mk(0.0, 0.0);
        }
    const Z inv = vec[c];
        for (int i = c + 1 + threadIdx.x; i < N; i += blockDim.x) vec[i] = S[c * N + i] * inv;
        __syncthreads();
        const int mm = N - c - 1, TT = mm * (mm - 1) / 2;
        for (int t = threadIdx.x; t < TT; t += blockDim.x) {
            int i, j;
            tri_index(t, mm, i, j);
            i += c + 1;
            j += c + 1;
            Z s = S[i * N + j];
            s = zfma(vec[i], S[r * N + j], s);
            s = zfms(S[r * N + i], vec[j], s);
            S[i * N + j] = s;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) pf.mul(S[(N - 2) * N + N - 1], false);
    __syncthreads();
    return threadIdx.x == 0 ? pf.get() : mk(0.0, 0.0);
}

// Pfaffians of two independent skew h x h matrices stored compactly (upper triangles,
// row-major, ld h, the second at S + h*h), eliminated together by the thread group g:
// each step takes both 2x2 pivots (row pivoting as in pfaffian_upper; warp b of the group
// searches matrix b), so the species-split form of a point needs h/2 - 1 steps for both
// species. Two group barriers per step: (a) the exchange of column c with the pivot column
// and the scaled pivot row v = S[c][.] / S[r][c] in one pass, (b) the rank-2 update, in
// which warp b first updates the next pivot row of matrix b and searches it (pivot index,
// value and reciprocal for the next step), then joins the rest of the update. A small pivot
// (|S[r][c]|^2 <= 1e-26, PNAMP_Proj.f90:290,333) or a non-finite one is recorded and the
// elimination runs on (its values are discarded): the result is 0 with `underflow` set.
// Returns Pf(first) * Pf(second) and `underflow` in the group's thread 0. `vec` holds 2h
// scratch values, `pv` 4 (pivots and reciprocals), `flag` 4 ints.
// NB = 1 is the same elimination of one h x h matrix (a general point's n x n Schur
// complement, eliminated while the other warps run the Gauss-Jordan solve).
template <class Z, int NB = 2>
__device__ zc pfaffian_upper_g(const Grp &g, Z *S, int h, Z *vec, Z *pv, int *flag, int &underflow) {
    using A = Ar<Z>;
    const int lane = g.tid & 31, wid = g.wid;
    const int hh = h * h;
    const int nstep = h / 2 - 1;
    PfProd<Z> pf;
    int uf = 0;
    // warp b: pivot of row r of matrix b over columns c..h-1 -> flag[b] (index), flag[2 + b]
    // (0 fine, 1 small, 2 non-finite), pv[b] (value), pv[2 + b] (reciprocal)
    auto search = [&](int b, int r) {
        const Z *Sb = S + b * hh;
        if constexpr (std::is_same<Z, zd>::value) {   // one redux.sync; candidates r + 1 .. h - 1 exist
            unsigned key = 0u;
            for (int j = r + 1 + lane; j < h; j += 32) {
                const unsigned kk = pack_key_bits((unsigned)A::key(Sb[r * h + j]), j - r - 1);
                key = key > kk ? key : kk;
            }
            const unsigned m = __reduce_max_sync(0xffffffffu, key);
            if (lane == 0) {
                const int q = r + 1 + 63 - (int)(m & 63u);
                const Z ssz = Sb[r * h + q];
                const int f = pivot_flag(ssz);
                flag[b] = q;
                flag[2 + b] = f;
                pv[b] = ssz;
                pv[2 + b] = f ? ssz : zrecip(ssz);
            }
            return;
        }
        unsigned long long best = 0ull;
        int bidx = 0x7fffffff;
        for (int j = r + 1 + lane; j < h; j += 32) {
            const unsigned long long key = A::key(Sb[r * h + j]);
            if (key > best || bidx == 0x7fffffff) {
                best = key;
                bidx = j;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long ob = __shfl_down_sync(0xffffffffu, best, o);
            const int oi = __shfl_down_sync(0xffffffffu, bidx, o);
            if (oi != 0x7fffffff && (bidx == 0x7fffffff || ob > best || (ob == best && oi < bidx))) {
                best = ob;
                bidx = oi;
            }
        }
        if (lane == 0) {
            const int q = (bidx == 0x7fffffff) ? r + 1 : bidx;  // at least one candidate when r + 1 < h
            const Z ssz = Sb[r * h + q];
            const int f = (bidx == 0x7fffffff) ? 2 : pivot_flag(ssz);
            flag[b] = q;
            flag[2 + b] = f;
            pv[b] = ssz;
            pv[2 + b] = f ? ssz : zrecip(ssz);
        }
    };
    // warp w serves matrices w, w + nwg, ...: one warp per matrix, or one warp for both
    const int nwg = g.nthr >> 5;
    for (int b = wid; nstep > 0 && b < NB; b += nwg) search(b, 0);
    gsync(g);
    for (int k = 0; k < nstep; ++k) {
        const int r = 2 * k, c = r + 1;
        const int q0 = flag[0], q1 = NB > 1 ? flag[1] : 0;
        if (g.tid == 0) {
            const int fk = (NB > 1 && flag[3] > flag[2]) ? flag[3] : flag[2];
            if (uf == 0) uf = fk;  // the first failing step decides, as the early return did
            for (int b = 0; b < NB; ++b) pf.mul(pv[b], (b ? q1 : q0) != c);
        }
        // (a) exchange c <-> q (exch_upper on every matrix) and v_i = S'[c][i] / S'[r][c], i > c
        for (int t = g.tid; t < NB * (h - r); t += g.nthr) {
            const int b = t / (h - r), i = r + t % (h - r);
            const int q = b ? q1 : q0;
            const Z inv = pv[2 + b];
            Z *Sb = S + b * hh;
            Z *vb = vec + b * h;
            if (q == c) {
                if (i > c) vb[i] = Sb[c * h + i] * inv;
                continue;
            }
            if (i < c) {  // i == r: the pivot moves to column c
                const Z x = Sb[i * h + c];
                Sb[i * h + c] = Sb[i * h + q];
                Sb[i * h + q] = x;
            } else if (i > q) {
                const Z x = Sb[c * h + i];
                const Z y = Sb[q * h + i];
                Sb[c * h + i] = y;
                Sb[q * h + i] = x;
                vb[i] = y * inv;
            } else if (i > c && i < q) {
                const Z x = Sb[c * h + i];
                const Z y = -Sb[i * h + q];
                Sb[c * h + i] = y;
                Sb[i * h + q] = -x;
                vb[i] = y * inv;
            } else if (i == c) {  // S'[c][q] = -S[c][q]; its thread also sets v_q
                const Z y = -Sb[c * h + q];
                Sb[c * h + q] = y;
                vb[q] = y * inv;
            }
        }
        gsync(g);
        // (b) S_ij += v_i S_rj - S_ri v_j for c < i < j; row c + 1 (the next pivot row) first
        const bool more = k + 1 < nstep;
        for (int b = wid; b < NB; b += nwg) {
            Z *Sb = S + b * hh;
            const Z *vb = vec + b * h;
            const int i = c + 1;
            const Z vi = vb[i], sri = Sb[r * h + i];
            for (int j = i + 1 + lane; j < h; j += 32) {
                Z sv = Sb[i * h + j];
                sv = zfma(vi, Sb[r * h + j], sv);
                sv = zfms(sri, vb[j], sv);
                Sb[i * h + j] = sv;
            }
            __syncwarp();
            if (more) search(b, c + 1);
        }
        const int mm = h - c - 2, TT = mm * (mm - 1) / 2;
        for (int t = g.tid; t < NB * TT; t += g.nthr) {
            const int b = t / TT;
            int i, j;
            tri_index(t - b * TT, mm, i, j);
            i += c + 2;
            j += c + 2;
            Z *Sb = S + b * hh;
            const Z *vb = vec + b * h;
            Z sv = Sb[i * h + j];
            sv = zfma(vb[i], Sb[r * h + j], sv);
            sv = zfms(Sb[r * h + i], vb[j], sv);
            Sb[i * h + j] = sv;
        }
        gsync(g);
    }
    zc out = mk(0.0, 0.0);
    if (g.tid == 0) {
        pf.mul(S[(h - 2) * h + h - 1], false);
        if (NB > 1) pf.mul(S[hh + (h - 2) * h + h - 1], false);
        if (!uf) out = pf.get();
    }
    underflow = uf;
    return out;
}

// ------------------------------------------------------------------ setup
__global__ void __launch_bounds__(kSetupThreads)
setup_kernel(Params p, const double *__restrict__ uv, double *__restrict__ pairbuf) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = p.n;
    const long long nn = (long long)n * n;
    const double *in = uv + (long long)blockIdx.x * 4 * nn;
    double *out = pairbuf + (long long)blockIdx.x * p.pl.stride;
    double *A = reinterpret_cast<double *>(smem_raw);
    double *Yb = A + nn;
    double *invd = Yb + nn;
    double *red = invd + n;
    zc *vecz = reinterpret_cast<zc *>(red + 64);    // n complex: the Pfaffian's pivot row
    int *perm = reinterpret_cast<int *>(vecz + n);
    int *sh = perm + n;
    // column-major input -> row-major pair record (U0, V0, U1, V1)
    for (long long t = threadIdx.x; t < 4 * nn; t += blockDim.x) {
        const long long q = t / nn, e = t % nn;
        const int i = (int)(e / n), j = (int)(e % n);
        out[q * nn + e] = in[q * nn + i + (long long)j * n];
    }
    __syncthreads();
    int st = 0;
    for (int which = 0; which < 2; ++which) {
        const double *U = out + (which == 0 ? p.pl.u1 : p.pl.u0);
        const double *V = out + (which == 0 ? p.pl.v1 : p.pl.v0);
        double *Z = out + (which == 0 ? p.pl.w : p.pl.z0);
        for (long long t = threadIdx.x; t < nn; t += blockDim.x) {
            A[t] = U[t];
            Yb[t] = V[t];
        }
        __syncthreads();
        if (lu_factor<double>(A, n, n, perm, invd, sh)) st = 1;
        row_solve<double>(Yb, n, n, A, n, n, perm, invd);  // Z = V U^-1
        for (long long t = threadIdx.x; t < nn; t += blockDim.x) Z[t] = Yb[t];
        __syncthreads();
        // det(1 + Z^T Z)^(-1/4): the eigenvalue product of zbareover, via LU
        for (long long t = threadIdx.x; t < nn; t += blockDim.x) {
            const int i = (int)(t / n), j = (int)(t % n);
            double s = (i == j) ? 1.0 : 0.0;
            for (int k = 0; k < n; ++k) s = fma(Yb[k * n + i], Yb[k * n + j], s);
            A[t] = s;
        }
        __syncthreads();
        if (lu_factor<double>(A, n, n, perm, invd, sh)) st = 1;
        double v[1] = {0.0};
        for (int k = threadIdx.x; k < n; k += blockDim.x) v[0] += log(fabs(A[k * n + k]));
        block_sum<1>(v, red);
        if (threadIdx.x == 0) out[p.pl.dets + (which == 0 ? 1 : 0)] = exp(-0.25 * v[0]);
        __syncthreads();
    }
    // Reduced Pfaffian data: block elimination of the lower-right block of
    // S = c [[D X D, -I], [I, -Z0]] gives Pf(S) = Pf(c (D X D - Z0^-1)) Pf(-c Z0), so the point
    // kernel can eliminate an n x n matrix per point. Kept only when V0 is well conditioned
    // (Z0^-1 = U0 V0^-1 accurate); otherwise the flag stays 0 and the 2n x 2n form is used.
    {
        const double *U0 = out + p.pl.u0, *V0 = out + p.pl.v0, *Z0 = out + p.pl.z0;
        for (long long t = threadIdx.x; t < nn; t += blockDim.x) {
            A[t] = V0[t];
            Yb[t] = U0[t];
        }
        __syncthreads();
        const bool vsing = lu_factor<double>(A, n, n, perm, invd, sh);
        if (threadIdx.x == 0) {
            double mx = 0.0, mn = 1e300;
            for (int k = 0; k < n; ++k) {
                const double d = fabs(A[k * n + k]);
                mx = fmax(mx, d);
                mn = fmin(mn, d);
            }
            red[0] = (!vsing && mx > 0.0 && mn >= kReducedPivotRatio * mx) ? 1.0 : 0.0;
        }
        __syncthreads();
        const bool well = red[0] != 0.0;
        __syncthreads();
        double ok = 0.0;
        zc pf = mk(0.0, 0.0);
        if (well) {
            row_solve<double>(Yb, n, n, A, n, n, perm, invd);  // U0 V0^-1
            for (long long t = threadIdx.x; t < nn; t += blockDim.x) out[p.pl.zi + t] = Yb[t];
            __syncthreads();
            zc *Sz = reinterpret_cast<zc *>(A);  // n^2 complex over A and Yb
            for (long long t = threadIdx.x; t < nn; t += blockDim.x) {
                const int i = (int)(t / n), j = (int)(t % n);
                Sz[t] = mk(i < j ? -p.cscale * Z0[t] : 0.0, 0.0);
            }
            __syncthreads();
            int under = 0;
            pf = pfaffian_upper<zc>(Sz, n, vecz, red, sh, under);
            ok = (under == 0 && zfinite(pf)) ? 1.0 : 0.0;
        }
        // species split: U0, V0, U1, V1 without proton-neutron blocks (charge-conserving vacua)
        // make every per-point matrix block-diagonal by species (protons first, h = n/2 each)
        int cross = 0;
        for (long long t = threadIdx.x; t < 4 * nn; t += blockDim.x) {
            const long long e = t % nn;
            const int i = (int)(e / n), j = (int)(e % n);
            if ((i < p.h) != (j < p.h) && out[t] != 0.0) cross = 1;  // U0, V0, U1, V1 lead the record
        }
        cross = __syncthreads_or(cross);
        if (threadIdx.x == 0) {
            out[p.pl.dets + 2] = (double)st;
            out[p.pl.dets + 3] = ok;
            out[p.pl.pfz] = pf.x;
            out[p.pl.pfz + 1] = pf.y;
            out[p.pl.dets + 6] = (ok != 0.0 && !cross) ? 1.0 : 0.0;
        }
    }
}

int setup_smem_bytes(int n) { return (2 * n * n + n + 64 + 2 * n) * 8 + (n + 8) * 4; }

// The dynamic shared-memory limit of a kernel is a property of the function,
// shared by every context on the device: it is raised to the device maximum
// (never lowered to one context's need), so a context created later cannot
// invalidate the launches of an earlier one with a larger placement.
static cudaError_t raise_smem_limit(const void *f) {
    int dev = 0, optin = 0;
    cudaFuncAttributes fa;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, f);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
    return e;
}

cudaError_t prepare_setup(int n) {
    if (setup_smem_bytes(n) <= 48 * 1024) return cudaSuccess;
    return raise_smem_limit((const void *)setup_kernel);
}

// Enqueues only (no attribute calls): usable under stream capture once
// prepare_setup(n) ran at context creation.
cudaError_t launch_setup(const Params &p, int npairs, const double *uv, double *pairbuf, cudaStream_t st) {
    setup_kernel<<<npairs, kSetupThreads, setup_smem_bytes(p.n), st>>>(p, uv, pairbuf);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ points
static_assert(sizeof(dd) == sizeof(double), "per-warp double-float partials share the double slots of red");
constexpr int kNSlot = 36;  // observable sums: slots 0..37 final values, then per-warp partials
constexpr int kR1BSlot = 128;  // one-body density block sums: red[kR1BSlot + 2b], re and im
constexpr int kR2Norm = 260;   // the gauge point's norm, re and im, for the two-body density pass
constexpr int kPfScratch = 608;  // 4 point-arithmetic values (<= 64 B): species Pfaffian pivots
static_assert(kThreads >= 32 * (kNTrace + 1), "one warp per Q trace plus warp 0");

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---- species-split pairs, two gauge points in flight --------------------------------------
// The CTA's two halves (8 warps each) take alternate gauge points of the Euler point and run
// them independently: in each half warps 0-1 eliminate the two species' Schur-complement
// blocks while warps 2-7 solve the two T22 systems (named barriers 1 + 3 s and 2 + 3 s for
// half s), and one half-wide barrier (3 + 3 s) separates the densities, K and the
// observables; warp 0 of each half accumulates its gauge points. A step of one half that
// waits on a barrier leaves the SM to the other half, which the single-point path (one CTA
// of 16 warps per gauge point) cannot do. The densities are stored compactly, two h x (h + 1)
// species blocks per density (the proton-neutron blocks of a split pair vanish). Thread 0
// sums the halves' accumulators at the end.
template <class Z>
__device__ __forceinline__ void split_pair_points(const Params &p, unsigned char *smem, const Z *X, const Z *P,
                                                  const Z *B, const Z *CZ, const Z *ephz, zc pfz, double det0,
                                                  double det1, int pair, int ie, long long pt0, double *gout,
                                                  double *zout, int *status) {
    using A = Ar<Z>;
    using R = typename A::R;
    const int n = p.n, h = p.h, nn = n * n;
    const int half = threadIdx.x / kHalfThreads, lt = threadIdx.x % kHalfThreads;
    const int lane = lt & 31, lw = lt >> 5;
    const HalfLayout L = half_layout(h);
    unsigned char *hb = smem + p.place.off_half + half * L.bytes;
    const int hl = h + 1, bs = h * hl, ds = 2 * bs, hh = h * h;   // compact row stride, block, density
    Z *Dn = reinterpret_cast<Z *>(hb + L.dens);
    Z *rhoC = Dn, *k10C = Dn + ds, *k01C = Dn + 2 * ds, *KcC = Dn + 3 * ds;
    Z *S2 = Dn;
    Z *T2 = reinterpret_cast<Z *>(hb + L.t), *Y2 = reinterpret_cast<Z *>(hb + L.y);
    Z *inv2 = reinterpret_cast<Z *>(hb + L.invd), *vec2 = reinterpret_cast<Z *>(hb + L.vec);
    Z *pfs2 = reinterpret_cast<Z *>(hb + L.pfs);
    zc *acc2 = reinterpret_cast<zc *>(hb + L.acc);
    double *fin2 = reinterpret_cast<double *>(hb + L.fin);
    R *pw2 = reinterpret_cast<R *>(hb + L.pw);
    int *sh2 = reinterpret_cast<int *>(hb + L.sh);   // [0, 4) Pfaffian, [4, 8) solve, [8] flags
    // compact V0^T, U0^T: species b, [b][k][j] = V0(b h + j, b h + k)
    const R *V0c = reinterpret_cast<const R *>(smem + p.place.off_uvc), *U0c = V0c + 2 * hh;
    const int barH = 3 + 3 * half;
    // one warp eliminates both species' Pfaffians (it finished at half the solve's time on
    // two), so the Gauss-Jordan group, the critical path, has seven of the half's eight warps
    constexpr int kPfW2 = 1;
    auto hsync = [&]() { asm volatile("bar.sync %0, %1;" ::"r"(barH), "r"(kHalfThreads) : "memory"); };
    // compact index of (r, c), r and c of the same species
    auto cidx = [&](int r, int c) {
        const int b = r >= h ? 1 : 0;
        return b * bs + (r - b * h) * hl + (c - b * h);
    };
    const Z zero = A::from(mk(0.0, 0.0));
    const Z csz = A::from(mk(p.cscale, 0.0));
    for (int io = lt; io < kNobs; io += kHalfThreads) acc2[io] = mk(0.0, 0.0);
    if (lt == 0) sh2[8] = 0;
    hsync();
    for (int gi = half; gi < p.n_gauge; gi += 2) {
        const int lp = gi / p.nfom, ln = gi % p.nfom;
        const Z zep = ephz[lp], zepc = zconj(zep), zen = ephz[ln], zenc = zconj(zen);
        const Z dpp = csz * (zep * zep), dnn = csz * (zen * zen);
        int under = 0;
        zc pf = mk(0.0, 0.0);
        bool sing = false;
        if (lw < kPfW2) {   // the two species' Schur-complement blocks and their Pfaffians
            const Grp g{lt, 32 * kPfW2, lw, 1 + 3 * half};
            const int Th = h * (h - 1) / 2;
            for (int t = g.tid; t < 2 * Th; t += g.nthr) {
                const int b = t >= Th ? 1 : 0;
                int i, j;
                tri_index(t - b * Th, h, i, j);
                const int gi_ = b * h + i, gj_ = b * h + j;
                S2[b * hh + i * h + j] = X[gi_ * n + gj_] * (b ? dnn : dpp) + CZ[gi_ * n + gj_];
            }
            gsync(g);
            pf = pfaffian_upper_g<Z, 2>(g, S2, h, vec2, pfs2, sh2, under);
            pf = pf * pfz;   // meaningful in the half's thread 0
        } else if (!p.norm_only) {   // T22 blocks, right-hand sides, Y T22^-1
            const Grp g{lt - 32 * kPfW2, kHalfThreads - 32 * kPfW2, lw - kPfW2, 2 + 3 * half};
            for (int t = g.tid; t < 2 * hh; t += g.nthr) {
                const int b = t >= hh ? 1 : 0, e = t - b * hh, i = e / h, j = e % h;
                const int gg = (b * h + i) * n + b * h + j;
                Z sv = zep * P[gg];
                sv = zfma(zen, P[nn + gg], sv);
                sv = zfma(zepc, P[2 * nn + gg], sv);
                sv = zfma(zenc, P[3 * nn + gg], sv);
                T2[t] = sv;
            }
            for (int t = g.tid; t < 4 * hh; t += g.nthr) {
                const int b = t >= 2 * hh ? 1 : 0, e = t - 2 * b * hh, r = e / h, j = e % h;
                const int grow = r < h ? b * h + r : n + b * h + (r - h);
                Y2[t] = B[grow * n + b * h + j];
            }
            gsync(g);
            const bool sg = gj_right_solve_g<Z, 2>(g, T2, h, Y2, 2 * h, inv2, vec2 + 2 * h, sh2 + 4);
            if (g.tid == 0) sh2[4] = sg ? 1 : 0;
        }
        hsync();
        if (!p.norm_only) sing = sh2[4] != 0;
        if (!p.norm_only) {
            // ---- densities of each species block (rho, kappa10, kappa01 share the loads)
            for (int t = lt; t < 2 * hh; t += kHalfThreads) {
                const int b = t >= hh ? 1 : 0, e = t - b * hh, i = e / h, j = e % h;
                const Z *Yt = Y2 + 2 * b * hh + i * h;
                const Z *Yb = Yt + hh;
                const R *Mv = V0c + b * hh + j, *Mu = U0c + b * hh + j;
                Z sr = zero, s10 = zero, s01 = zero;
                for (int k = 0; k < h; ++k) {
                    const Z yt = Yt[k];
                    const R mv = Mv[k * h];
                    sr = rfma(mv, yt, sr);
                    s10 = rfma(Mu[k * h], yt, s10);
                    s01 = rfma(mv, Yb[k], s01);
                }
                const Z di = b ? zen : zep;
                const int o = b * bs + i * hl + j;
                rhoC[o] = di * sr;
                k10C[o] = di * s10;
                k01C[o] = -(zconj(di) * s01);
            }
            hsync();
            // ---- K01_ij (i < j) at K[i][j], K10_ij at K[j][i], within each block
            {
                const int Th = h * (h - 1) / 2;
                for (int t = lt; t < 2 * Th; t += kHalfThreads) {
                    const int b = t >= Th ? 1 : 0;
                    int i, j;
                    tri_index(t - b * Th, h, i, j);
                    const int oij = b * bs + i * hl + j, oji = b * bs + j * hl + i;
                    KcC[oij] = k01C[oij] - k01C[oji];
                    KcC[oji] = k10C[oij] - k10C[oji];
                }
            }
            hsync();
            // ---- observables: 13 trace jobs over the half's 8 warps (job = lw, lw + 8); then
            // the energy (records, or the bf16 rows of the tensor-core forms) and <J^2>
            for (int job = lw; job < kNTrace + 3; job += kHalfWarps) {
                if (job == 0 || job == kNTrace + 1 || job == kNTrace + 2) {
                    R v0 = A::rzero(), v1 = v0, v2 = v0, v3 = v0, v4 = v0, v5 = v0;
                    if (job == 0) {
                        for (int a = lane; a < n; a += 32) {
                            const Z d = rhoC[cidx(a, a)];
                            if (a < h) { v0 = A::radd(v0, d.x); v1 = A::radd(v1, d.y); }
                            else { v2 = A::radd(v2, d.x); v3 = A::radd(v3, d.y); }
                            const R jj = A::pick(p.obs.jj1, p.obs.jj1_d, a);
                            v4 = A::rfma(jj, d.x, v4);
                            v5 = A::rfma(jj, d.y, v5);
                        }
                    } else if (job == kNTrace + 1) {
                        for (int a = lane; a < n; a += 32) {
                            const R jpa = A::pick(p.obs.jp, p.obs.jp_d, a), jma = A::pick(p.obs.jm, p.obs.jm_d, a);
                            const R mza = A::pick(p.obs.mz, p.obs.mz_d, a);
                            if (A::nz(jpa)) {
                                const Z r = rhoC[cidx(a + 1, a)];
                                v0 = A::rfma(jpa, r.x, v0);
                                v1 = A::rfma(jpa, r.y, v1);
                            }
                            if (A::nz(jma)) {
                                const Z r = rhoC[cidx(a - 1, a)];
                                v2 = A::rfma(jma, r.x, v2);
                                v3 = A::rfma(jma, r.y, v3);
                            }
                            const Z d = rhoC[cidx(a, a)];
                            v4 = A::rfma(mza, d.x, v4);
                            v5 = A::rfma(mza, d.y, v5);
                        }
                    } else {
                        for (int e = lane; e < p.obs.n_t1b; e += 32) {
                            const int ix = p.obs.t1b_idx[e], r = ix >> 8, c = ix & 255;
                            if ((r >= h) != (c >= h)) continue;
                            const Z rv = rhoC[cidx(r, c)];
                            const R tv = A::pick(p.obs.t1b_val, p.obs.t1b_val_d, e);
                            v0 = A::rfma(tv, rv.x, v0);
                            v1 = A::rfma(tv, rv.y, v1);
                        }
                    }
                    const int s0 = job == 0 ? 0 : (job == kNTrace + 1 ? 10 : 4);
                    const int cnt = job == kNTrace + 2 ? 2 : 6;
                    const R vals[6] = {v0, v1, v2, v3, v4, v5};
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        if (q >= cnt) break;
                        const R v = A::wsum(vals[q]);
                        const int slot = (job == 0 && q >= 4) ? 12 + q : s0 + q;
                        if (lane == 0) fin2[slot] = A::dbl(v);
                    }
                } else if (p.iE2) {   // Q_{2mu} trace job - 1
                    const int q = job - 1;
                    R sr = A::rzero(), si = A::rzero();
                    for (int e = p.obs.q_off[q] + lane; e < p.obs.q_off[q + 1]; e += 32) {
                        const int ix = p.obs.q_idx[e], r = ix >> 8, c = ix & 255;
                        if ((r >= h) != (c >= h)) continue;
                        const Z rv = rhoC[cidx(r, c)];
                        const R qv = A::pick(p.obs.q_val, p.obs.q_val_d, e);
                        sr = A::rfma(qv, rv.x, sr);
                        si = A::rfma(qv, rv.y, si);
                    }
                    sr = A::wsum(sr);
                    si = A::wsum(si);
                    if (lane == 0) {
                        fin2[18 + 2 * q] = A::dbl(sr);
                        fin2[19 + 2 * q] = A::dbl(si);
                    }
                }
            }
            auto put = [&](int slot, R v) {   // slot 0..3: energy re/im, <J^2> re/im
                v = A::wsum(v);
                if (lane == 0) pw2[slot * kHalfWarps + lw] = v;
            };
            if (p.tc_splits) {   // the gauge point's split-bf16 rows for the tensor-core contraction
                const long long pt = pt0 + gi;
                const int S = p.tc_splits, nk = p.tc_nk, npp = p.tc_nk - p.tc_nph;
                for (int e = lt; e < nk; e += kHalfThreads) {
                    const int src = p.tc_src[e];
                    Z v = zero, y = zero;
                    if (src >= 0) {
                        const int r = src >> 8, c = src & 255;
                        if ((r >= h) == (c >= h)) {   // the proton-neutron entries vanish
                            if (e < p.tc_nph) {
                                v = rhoC[cidx(r, c)];
                            } else {
                                v = KcC[cidx(c, r)];   // K10_rc, r < c
                                y = KcC[cidx(r, c)];   // K01_rc
                            }
                        }
                    }
                    unsigned short tr[3], ti[3];
                    bf16_terms(as_dd(v.x), S, tr);
                    bf16_terms(as_dd(v.y), S, ti);
                    for (int sp = 0; sp < S; ++sp) {
                        p.tc_x[sp][(2 * pt) * nk + e] = tr[sp];
                        p.tc_x[sp][(2 * pt + 1) * nk + e] = ti[sp];
                    }
                    if (e >= p.tc_nph) {
                        bf16_terms(as_dd(y.x), S, tr);
                        bf16_terms(as_dd(y.y), S, ti);
                        const int ey = e - p.tc_nph;
                        for (int sp = 0; sp < S; ++sp) {
                            p.tc_y[sp][(2 * pt) * npp + ey] = tr[sp];
                            p.tc_y[sp][(2 * pt + 1) * npp + ey] = ti[sp];
                        }
                    }
                }
                if (lane == 0) {
                    pw2[lw] = A::rzero();
                    pw2[kHalfWarps + lw] = A::rzero();
                }
            } else {   // two-body energy: the point kernel's record loop on the compact blocks
                const R quarter = A::rconst(0.25f);
                Z e2 = zero;
                // same-species records: all four indices in species block b
                for (int e = lt; e < p.nrec_gen; e += kHalfThreads) {
                    const uint32_t pk = p.rec_idx[e];
                    const R v = A::pick(p.rec_v, p.rec_vd, e);
                    int i = pk & 0xff, j = (pk >> 8) & 0xff, k = (pk >> 16) & 0xff, l = pk >> 24;
                    const bool sym = i + j != k + l;
                    const int b = i >= h ? 1 : 0, o = b * bs;
                    i -= b * h;
                    j -= b * h;
                    k -= b * h;
                    l -= b * h;
                    Z t = rhoC[o + k * hl + i] * rhoC[o + l * hl + j];
                    t = zfms(rhoC[o + l * hl + i], rhoC[o + k * hl + j], t);
                    Z u = KcC[o + i * hl + j] * KcC[o + l * hl + k];
                    if (sym) {
                        t = zfma(rhoC[o + i * hl + k], rhoC[o + j * hl + l], t);
                        t = zfms(rhoC[o + j * hl + k], rhoC[o + i * hl + l], t);
                        u = zfma(KcC[o + k * hl + l], KcC[o + j * hl + i], u);
                    }
                    t = rfma(quarter, u, t);
                    e2 = rfma(v, t, e2);
                }
                // proton-neutron records: (i, k) protons, (j, l) neutrons; only the direct terms
                for (int e = p.nrec_gen + lt; e < p.nrec; e += kHalfThreads) {
                    const uint32_t pk = p.rec_idx[e];
                    const R v = A::pick(p.rec_v, p.rec_vd, e);
                    const int i = pk & 0xff, j = ((pk >> 8) & 0xff) - h, k = (pk >> 16) & 0xff, l = (pk >> 24) - h;
                    Z t = rhoC[k * hl + i] * rhoC[bs + l * hl + j];
                    if (i + j != k + l) t = zfma(rhoC[i * hl + k], rhoC[bs + j * hl + l], t);
                    e2 = rfma(v, t, e2);
                }
                put(0, e2.x);
                put(1, e2.y);
            }
            {   // <J^2>, the same terms as the single-point path, within the species blocks
                const R half_ = A::rconst(0.5f);
                Z rest = zero;
                for (int t = lt; t < 2 * hh; t += kHalfThreads) {
                    const int blk = t >= hh ? 1 : 0, e = t - blk * hh;
                    const int a = blk * h + e / h, c = blk * h + e % h;
                    const R jpa = A::pick(p.obs.jp, p.obs.jp_d, a), jma = A::pick(p.obs.jm, p.obs.jm_d, a);
                    const R jpc = A::pick(p.obs.jp, p.obs.jp_d, c), jmc = A::pick(p.obs.jm, p.obs.jm_d, c);
                    const R mzz = A::rmul(A::pick(p.obs.mz, p.obs.mz_d, a), A::pick(p.obs.mz, p.obs.mz_d, c));
                    const int ac = cidx(a, c);
                    Z q = mzz * (k10C[ac] * k01C[ac]);
                    q = zfms(mzz * rhoC[ac], rhoC[cidx(c, a)], q);
                    if (A::nz(jpa) && A::nz(jmc))
                        q = zfms(A::rmul(jpa, jmc) * rhoC[ac + hl], rhoC[cidx(c - 1, a)], q);
                    if (A::nz(jpa) && A::nz(jpc))
                        q = zfma(A::rmul(half_, A::rmul(jpa, jpc)) * k10C[ac + hl], k01C[ac + 1], q);
                    if (A::nz(jma) && A::nz(jmc))
                        q = zfma(A::rmul(half_, A::rmul(jma, jmc)) * k10C[ac - hl], k01C[ac - 1], q);
                    rest = rest + q;
                }
                put(2, rest.x);
                put(3, rest.y);
            }
        }
        hsync();
        if (lw == 0) {   // accumulation over this half's gauge points (single-lane FP64 values)
            const unsigned full = 0xffffffffu;
            R ws[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) ws[q] = A::wsum(lane < kHalfWarps ? pw2[q * kHalfWarps + lane] : A::rzero());
            const bool eval = !p.norm_only && !sing;
            zc norm = mk(0.0, 0.0);
            if (lane == 0) {
                const zc zph = mk(p.gphase[2 * gi], p.gphase[2 * gi + 1]);
                norm = (p.vacfac * det0 * det1) * (pf * zph);
            }
            norm.x = __shfl_sync(full, norm.x, 0);
            norm.y = __shfl_sync(full, norm.y, 0);
            zc o = mk(0.0, 0.0), hg = mk(0.0, 0.0);
            bool use = eval;
            if ((lane == 6 || (lane == 0 && gout)) && eval)
                hg = mk(fin2[4] + A::dbl(ws[0]) + p.e0, fin2[5] + A::dbl(ws[1]));
            if (lane == 1) o = mk(fin2[0], fin2[1]);
            else if (lane == 2) o = mk(fin2[2], fin2[3]);
            else if (lane == 3) o = mk(fin2[4], fin2[5]);
            else if (lane == 6) o = hg;
            else if (lane == 7) {
                const zc trp = mk(fin2[10], fin2[11]), trm = mk(fin2[12], fin2[13]), trz = mk(fin2[14], fin2[15]);
                o = mk(fin2[16] + A::dbl(ws[2]), fin2[17] + A::dbl(ws[3])) + trp * trm + trz * trz;
            } else if (lane >= 8 && lane < 18 && p.iE2) o = mk(fin2[2 * lane + 2], fin2[2 * lane + 3]);
            else use = false;
            if (p.tc_splits && lane == 0) {
                const long long pt = pt0 + gi;
                const double inv = 1.0 / ((double)p.nfom * p.nfom);
                p.tc_w[2 * pt] = eval ? inv * norm.x : 0.0;
                p.tc_w[2 * pt + 1] = eval ? inv * norm.y : 0.0;
            }
            if (lane == 0) {
                acc2[0] = acc2[0] + norm;
                if (gout) {
                    double *g = gout + 4LL * (((long long)pair * p.n_euler + ie) * p.n_gauge + gi);
                    g[0] = norm.x;
                    g[1] = norm.y;
                    g[2] = hg.x;
                    g[3] = hg.y;
                }
                int f = (under == 1) ? 1 : (under == 2 ? 4 : 0);
                if (!p.norm_only && sing) f |= 2;
                sh2[8] |= f;
            }
            if (use) acc2[lane] = zfma(norm, o, acc2[lane]);
            __syncwarp();
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {   // the two halves' sums
        const zc *a0 = reinterpret_cast<const zc *>(smem + p.place.off_half + L.acc);
        const zc *a1 = reinterpret_cast<const zc *>(smem + p.place.off_half + L.bytes + L.acc);
        const int f0 = reinterpret_cast<const int *>(smem + p.place.off_half + L.sh)[8];
        const int f1 = reinterpret_cast<const int *>(smem + p.place.off_half + L.bytes + L.sh)[8];
        const double inv = 1.0 / ((double)p.nfom * p.nfom);
        int f = f0 | f1;
        for (int io = 0; io < kNobs; ++io) {
            const zc v = io == kNobs - 1 ? mk(0.0, 0.0) : inv * (a0[io] + a1[io]);
            if (!zfinite(v)) f |= 4;
            zout[2LL * (io * p.n_euler + ie)] = v.x;
            zout[2LL * (io * p.n_euler + ie) + 1] = v.y;
        }
        status[(long long)pair * p.n_euler + ie] = f;
    }
    __syncthreads();
}

// One work item: Euler point `ie` of pair `pair`, all its gauge points, in the
// CTA's workspace `slot`. `reload` is set when the previous item of this CTA
// belonged to another pair (or context): V0^T, U0^T and the phase tables are
// then (re)loaded.
template <class Z>
__device__ __forceinline__ void point_item(const Params &p, const double *__restrict__ pairbuf, zc *slot,
                                           int pair, int ie, bool reload, double *__restrict__ zres,
                                           int *__restrict__ status, double *__restrict__ gout = nullptr,
                                           double *__restrict__ r1out = nullptr,
                                           double *__restrict__ r2out = nullptr, long long pt0 = 0) {
    using A = Ar<Z>;
    using R = typename A::R;
    extern __shared__ __align__(16) unsigned char smem[];
    const int n = p.n, h = p.h, N = p.N2;
    const int nn = n * n;
    const int ld = n + 1;  // density row stride: transposed reads stay bank-conflict free
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const Placement &pl = p.place;
    Z *X = reinterpret_cast<Z *>(slot + pl.g_x);    // R W R^T
    Z *B = reinterpret_cast<Z *>(slot + pl.g_b);    // rows 0..n-1: R V1, rows n..2n-1: conj(R) U1
    zc *Bz = slot + pl.g_b;                         // the same storage while it holds FP64 values
    Z *P = reinterpret_cast<Z *>(slot + pl.g_p);    // T22 partials: V0p, V0n, U0p, U0n
    zc *RW = slot + pl.g_rw;                        // R W
    // -Cscale Z0^-1 (reduced pairs) or -Cscale Z0: the constant block of the Pfaffian matrix,
    // converted once per pair so that building S takes no FP64 work per gauge point
    Z *CZ = reinterpret_cast<Z *>(slot + pl.g_zr);
    Z *S = reinterpret_cast<Z *>(pl.s_smem ? (void *)(smem + pl.off_s) : (void *)(slot + pl.g_s));
    Z *T = reinterpret_cast<Z *>(pl.t_smem ? (void *)(smem + pl.off_t) : (void *)(slot + pl.g_t));
    Z *Y = reinterpret_cast<Z *>(pl.y_smem ? (void *)(smem + pl.off_y) : (void *)(slot + pl.g_y));
    // V0^T and U0^T: V0t[k n + j] = V0(j, k)
    R *V0t = reinterpret_cast<R *>(pl.uv_smem ? (void *)(smem + pl.off_uv) : (void *)(slot + pl.g_uv));
    R *U0t = V0t + nn;
    int *perm = reinterpret_cast<int *>(smem + pl.off_piv);
    int *sh = perm + n;
    Z *invd = reinterpret_cast<Z *>(smem + pl.off_inv);
    double *red = reinterpret_cast<double *>(smem + pl.off_red);
    zc *rot = reinterpret_cast<zc *>(smem + pl.off_rot);
    Z *vec = reinterpret_cast<Z *>(smem + pl.off_vec);
    zc *acc = reinterpret_cast<zc *>(vec + N);      // kNobs accumulators (thread 0)
    zc *eph = acc + kNobs;                          // e^{i phi_l}, l < NFOM
    Z *ephz = reinterpret_cast<Z *>(eph + p.nfom);  // the same in the point arithmetic
    zc *acc_r1b = reinterpret_cast<zc *>(ephz + p.nfom);  // one-body density blocks (thread 0)
    Z *rho = S, *k10 = S + n * ld, *k01 = S + 2 * n * ld;
    Z *Kc = S + 3 * n * ld;  // antisymmetrised pairing tensors

    const double twopi = 6.283185307179586476925287;
    {
        const double *pr = pairbuf + (long long)pair * p.pl.stride;
        const double *gU1 = pr + p.pl.u1, *gV1 = pr + p.pl.v1, *gU0 = pr + p.pl.u0, *gV0 = pr + p.pl.v0;
        const double *gW = pr + p.pl.w, *gZ0 = pr + p.pl.z0;
        const double det0 = pr[p.pl.dets], det1 = pr[p.pl.dets + 1];
        const int pst = (int)pr[p.pl.dets + 2];
        // reduced Pfaffian (set-up kernel): eliminate c (D X D - Z0^-1), n x n, times Pf(-c Z0)
        const bool reduced = pr[p.pl.dets + 3] != 0.0;
        const double *gZi = pr + p.pl.zi;
        const zc pfz = mk(pr[p.pl.pfz], pr[p.pl.pfz + 1]);
        const int NP = reduced ? n : N;  // order of the eliminated skew matrix
        // species split (set-up kernel): no proton-neutron blocks, so the Schur complement, T22,
        // the solve and the densities are block-diagonal; both species are eliminated together
        // on compact h x h blocks
        const bool split = reduced && pr[p.pl.dets + 6] != 0.0;
        // two gauge points in flight (split_pair_points) when the halves' storage fits
        const bool use2 = pl.sp2 && split && p.nfom > 1 && !r2out && !r1out && blockDim.x == kThreads;
        double *zout = zres + 2LL * (long long)pair * kNobs * p.n_euler;
        if (pst) {
            for (int io = threadIdx.x; io < kNobs; io += blockDim.x) {
                zout[2LL * (io * p.n_euler + ie)] = 0.0;
                zout[2LL * (io * p.n_euler + ie) + 1] = 0.0;
            }
            if (threadIdx.x == 0) status[(long long)pair * p.n_euler + ie] = 8;
            for (int g = threadIdx.x; g < (p.tc_splits ? p.n_gauge : 0); g += blockDim.x) {
                p.tc_w[2 * (pt0 + g)] = 0.0;
                p.tc_w[2 * (pt0 + g) + 1] = 0.0;
            }
            return;
        }
        if (reload) {
            __syncthreads();
            for (int t = threadIdx.x; t < nn; t += blockDim.x) {
                const int k = t / n, j = t % n;
                if (!use2) {
                    V0t[t] = A::real(gV0[j * n + k]);
                    U0t[t] = A::real(gU0[j * n + k]);
                }
                CZ[t] = A::from(mk(-p.cscale * (reduced ? gZi[t] : gZ0[t]), 0.0));
            }
            if (use2) {   // the diagonal species blocks only: [b][k][j] = V0(b h + j, b h + k)
                R *V0c = reinterpret_cast<R *>(smem + pl.off_uvc), *U0c = V0c + 2 * h * h;
                for (int t = threadIdx.x; t < 2 * h * h; t += blockDim.x) {
                    const int b = t / (h * h), e = t % (h * h), k = e / h, j = e % h;
                    V0c[t] = A::real(gV0[(b * h + j) * n + b * h + k]);
                    U0c[t] = A::real(gU0[(b * h + j) * n + b * h + k]);
                }
            }
            for (int l = threadIdx.x; l < p.nfom; l += blockDim.x) {
                const zc e = expi(p.nfom == 1 ? 0.0 : twopi * l / p.nfom);
                eph[l] = e;
                ephz[l] = A::from(e);
            }
        }
        // ---- rotation blocks R_b(i,k) = e^{-i alp m_i} d^j_{m_i m_k}(bet) e^{-i gam m_k}  (FP64)
        const double alp = p.euler[4 * ie], bet = p.euler[4 * ie + 1], gam = p.euler[4 * ie + 2];
        double cb, sb;
        sincos(0.5 * bet, &sb, &cb);
        for (int b = 0; b < p.nblk; ++b) {
            const int d = p.blk_size[b], tj = p.blk_tj[b], ro = p.blk_roff[b];
            for (int e = threadIdx.x; e < d * d; e += blockDim.x) {
                const int i = e / d, k = e % d;
                const int mi = tj - 2 * i, mkk = tj - 2 * k;
                const double dv = wigner_d(tj, mi, mkk, cb, sb, p.fact);
                rot[ro + e] = dv * expi(-0.5 * (alp * mi + gam * mkk));
            }
        }
        if (threadIdx.x == 0) {
            for (int io = 0; io < kNobs; ++io) acc[io] = mk(0.0, 0.0);
            for (int b = 0; b < (r1out ? p.obs.n_r1b : 0); ++b) acc_r1b[b] = mk(0.0, 0.0);
        }
        // two-body density sums of this Euler point: thread t owns quadruples t, t + blockDim, ...
        // (zeroed, accumulated and flushed by the same thread, so no barrier between the steps)
        double *r2acc = r2out ? p.r2acc + 2LL * p.n_r2q * blockIdx.x : nullptr;
        for (int q = threadIdx.x; q < (r2out ? p.n_r2q : 0); q += blockDim.x) {
            r2acc[2 * q] = 0.0;
            r2acc[2 * q + 1] = 0.0;
        }
        __syncthreads();
        // ---- R W (or, for the Onishi norm, R U1 and conj(R) V1), R V1, conj(R) U1 (FP64)
        const bool onishi = (p.nfom == 1);
        zc *Xz = reinterpret_cast<zc *>(X);
        for (int t = threadIdx.x; t < nn; t += blockDim.x) {
            const int a = t / n, j = t % n;
            const int b = p.row_blk[a], s0 = p.blk_start[b], d = p.blk_size[b];
            const zc *Rr = rot + p.blk_roff[b] + (a - s0) * d;
            zc rw = mk(0, 0), b1 = mk(0, 0), b2 = mk(0, 0), cv = mk(0, 0);
            for (int k = 0; k < d; ++k) {
                const zc r = Rr[k];
                rw = rfma(onishi ? gU1[(s0 + k) * n + j] : gW[(s0 + k) * n + j], r, rw);
                b1 = rfma(gV1[(s0 + k) * n + j], r, b1);
                b2 = rfma(gU1[(s0 + k) * n + j], zconj(r), b2);
                cv = rfma(gV1[(s0 + k) * n + j], zconj(r), cv);
            }
            RW[t] = rw;
            Bz[t] = b1;
            Bz[nn + t] = b2;
            if (onishi) Xz[t] = cv;
        }
        __syncthreads();
        // ---- X = (R W) R^T and the T22 partials (FP64), stored in the point arithmetic
        for (int t = threadIdx.x; t < (onishi ? 0 : nn); t += blockDim.x) {
            const int a = t / n, c = t % n;
            const int b = p.row_blk[c], s0 = p.blk_start[b], d = p.blk_size[b];
            const zc *Rr = rot + p.blk_roff[b] + (c - s0) * d;
            zc x = mk(0, 0);
            for (int k = 0; k < d; ++k) x = zfma(RW[a * n + s0 + k], Rr[k], x);
            X[t] = A::from(x);
        }
        for (int t = threadIdx.x; t < (p.norm_only ? 0 : 4 * nn); t += blockDim.x) {
            const int q = t / nn, e = t % nn, i = e / n, j = e % n;
            const double *M = (q < 2) ? gV0 : gU0;
            const zc *Bq = (q < 2) ? Bz : Bz + nn;
            const int k0 = (q & 1) ? h : 0;
            zc s = mk(0, 0);
            for (int k = k0; k < k0 + h; ++k) s = rfma(M[k * n + i], Bq[k * n + j], s);
            P[t] = A::from(s);
        }
        __syncthreads();
        for (int t = threadIdx.x; t < (p.norm_only ? 0 : 2 * nn); t += blockDim.x) {  // in place
            const zc v = Bz[t];
            B[t] = A::from(v);
        }
        __syncthreads();
        if (use2) {
            split_pair_points<Z>(p, smem, X, P, B, CZ, ephz, pfz, det0, det1, pair, ie, pt0, gout, zout, status);
            return;
        }

        int flags = 0;
        const Z zero = A::from(mk(0.0, 0.0));
        const Z csz = A::from(mk(p.cscale, 0.0)), mcs = A::from(mk(-p.cscale, 0.0));
        for (int lp = 0; lp < p.nfom; ++lp) {
            const Z zep = ephz[lp], zepc = zconj(zep);
            for (int ln = 0; ln < p.nfom; ++ln) {
                const Z zen = ephz[ln], zenc = zconj(zen);
                // ---- S = Cscale [[D X D, -I], [I, -Z0]] (upper triangle), or for a reduced
                // pair its Schur complement Cscale (D X D - Z0^-1) (n x n, row stride n)
                const Z dpp = csz * (zep * zep), dpn = csz * (zep * zen), dnn = csz * (zen * zen);
                // species split: warps 0-1 build and eliminate the two Schur-complement blocks
                // while warps 2-15 build T22 and Y and run the Gauss-Jordan solve (named barriers
                // 1 and 2); both are latency-bound, so running them side by side hides the
                // Pfaffians behind the solve, which is the longer of the two (per-group clock
                // marks: the Pfaffian group of 4 warps finished at 60-76 % of the solve; with the
                // two-barrier Pfaffian 2, 3 and 4 Pfaffian warps time within 0.4 % of each other,
                // so the solve keeps 14). One CTA barrier joins them before the densities.
                const bool conc = split && !onishi;
                // general reduced points (vacua that mix protons and neutrons): the same overlap of
                // the n x n Schur complement's elimination (warps 0 .. kPfWarpsG-1, named barrier 1)
                // with the n x n Gauss-Jordan solve on the other warps (named barrier 2)
                const bool concg = !split && reduced && !onishi;
                int under = 0;
                zc pf = mk(0.0, 0.0);
                bool sing = false;
                if (concg) {
                    constexpr int kPfWarpsG = 3;
                    if (wid < kPfWarpsG) {
                        const Grp g{(int)threadIdx.x, kPfWarpsG * 32, wid, 1};
                        for (int t = g.tid; t < n * (n - 1) / 2; t += g.nthr) {
                            int i, j;
                            tri_index(t, n, i, j);
                            const Z dd_ = (j < h) ? dpp : ((i < h) ? dpn : dnn);
                            S[i * n + j] = X[i * n + j] * dd_ + CZ[i * n + j];
                        }
                        gsync(g);
                        pf = pfaffian_upper_g<Z, 1>(g, S, n, vec, reinterpret_cast<Z *>(red + kPfScratch), sh, under);
                        pf = pf * pfz;  // meaningful in thread 0
                    } else if (!p.norm_only) {
                        const Grp g{(int)threadIdx.x - kPfWarpsG * 32, (int)blockDim.x - kPfWarpsG * 32,
                                    wid - kPfWarpsG, 2};
                        for (int t = g.tid; t < nn; t += g.nthr) {
                            Z sv = zep * P[t];
                            sv = zfma(zen, P[nn + t], sv);
                            sv = zfma(zepc, P[2 * nn + t], sv);
                            sv = zfma(zenc, P[3 * nn + t], sv);
                            T[t] = sv;
                        }
                        for (int t = g.tid; t < 2 * nn; t += g.nthr) Y[t] = B[t];
                        gsync(g);
                        const bool sg = gj_right_solve_g<Z, 1>(g, T, n, Y, 2 * n, invd, vec + n, sh + 4);
                        if (g.tid == 0) sh[4] = sg ? 1 : 0;
                    }
                    __syncthreads();
                    if (!p.norm_only) sing = sh[4] != 0;
                }
                if (conc) {
                    constexpr int kPfWarps = 2;  // the two pivot searches need one warp each
                    if (wid < kPfWarps) {
                        const Grp g{(int)threadIdx.x, kPfWarps * 32, wid, 1};
                        const int Th = h * (h - 1) / 2;
                        for (int t = g.tid; t < 2 * Th; t += g.nthr) {
                            const int b = t >= Th ? 1 : 0;
                            int i, j;
                            tri_index(t - b * Th, h, i, j);
                            const int gi = b * h + i, gj = b * h + j;
                            Z v = X[gi * n + gj] * (b ? dnn : dpp);
                            v = v + CZ[gi * n + gj];
                            S[b * h * h + i * h + j] = v;
                        }
                        gsync(g);
                        pf = pfaffian_upper_g<Z, 2>(g, S, h, vec, reinterpret_cast<Z *>(red + kPfScratch), sh, under);
                        pf = pf * pfz;  // meaningful in thread 0
                    } else if (!p.norm_only) {
                        const Grp g{(int)threadIdx.x - kPfWarps * 32, (int)blockDim.x - kPfWarps * 32,
                                    wid - kPfWarps, 2};
                        for (int t = g.tid; t < 2 * h * h; t += g.nthr) {
                            const int b = t >= h * h ? 1 : 0, e = t - b * h * h, i = e / h, j = e % h;
                            const int gg = (b * h + i) * n + b * h + j;
                            Z sv = zep * P[gg];
                            sv = zfma(zen, P[nn + gg], sv);
                            sv = zfma(zepc, P[2 * nn + gg], sv);
                            sv = zfma(zenc, P[3 * nn + gg], sv);
                            T[t] = sv;
                        }
                        for (int t = g.tid; t < 4 * h * h; t += g.nthr) {
                            const int b = t >= 2 * h * h ? 1 : 0, e = t - 2 * b * h * h, r = e / h, j = e % h;
                            const int grow = r < h ? b * h + r : n + b * h + (r - h);
                            Y[t] = B[grow * n + b * h + j];
                        }
                        gsync(g);
                        const bool sg = gj_right_solve_g<Z, 2>(g, T, h, Y, 2 * h, invd, vec + 2 * h, sh + 4);
                        if (g.tid == 0) sh[4] = sg ? 1 : 0;
                    }
                    __syncthreads();
                    if (!p.norm_only) sing = sh[4] != 0;
                }
                for (int t = threadIdx.x; t < (onishi || split || concg ? 0 : NP * (NP - 1) / 2); t += blockDim.x) {
                    int i, j;
                    tri_index(t, NP, i, j);
                    Z v;
                    if (j < n) {
                        const Z dd_ = (j < h) ? dpp : ((i < h) ? dpn : dnn);
                        v = X[i * n + j] * dd_;
                        if (reduced) v = v + CZ[i * n + j];
                    } else if (i < n) {
                        v = (j - n == i) ? mcs : zero;
                    } else {
                        v = CZ[(i - n) * n + (j - n)];
                    }
                    S[i * NP + j] = v;
                }
                if (!conc && !concg) __syncthreads();
                if (conc || concg) {
                } else if (onishi) {
                    // Onishi (PNAMP_Onishi.f90:21-37): sqrt(det(Ubar^T U0 + Vbar^T V0)),
                    // Ubar = R U1, Vbar = conj(R) V1 at phi = 0; LU determinant, principal root
                    zc *Bm = reinterpret_cast<zc *>(S);
                    for (int t = threadIdx.x; t < nn; t += blockDim.x) {
                        const int i = t / n, j = t % n;
                        zc acc2 = mk(0, 0);
                        for (int k = 0; k < n; ++k) {
                            acc2 = rfma(gU0[k * n + j], RW[k * n + i], acc2);
                            acc2 = rfma(gV0[k * n + j], Xz[k * n + i], acc2);
                        }
                        Bm[t] = acc2;
                    }
                    __syncthreads();
                    zc *invz = reinterpret_cast<zc *>(invd);
                    const bool bsing = lu_factor<zc>(Bm, n, n, perm, invz, sh);
                    if (threadIdx.x == 0) {
                        zc det = mk(1.0, 0.0);
                        for (int k = 0; k < n; ++k) {
                            det = det * Bm[k * n + k];
                            if (perm[k] != k) det = -det;
                        }
                        if (bsing) det = mk(0.0, 0.0);
                        const double r = sqrt(det.x * det.x + det.y * det.y);
                        const double re = sqrt(0.5 * (r + det.x)), im = copysign(sqrt(0.5 * fmax(r - det.x, 0.0)), det.y);
                        acc[kNobs - 1] = mk(re, im);  // scratch slot: observable 19 is never set
                    }
                    __syncthreads();
                    pf = acc[kNobs - 1];
                    __syncthreads();
                } else {
                    pf = pfaffian_upper<Z>(S, NP, vec, red, sh + 2, under);
                    if (reduced) pf = pf * pfz;  // meaningful in thread 0, like pf
                }
                // fin: final sums (double); pwR: per-warp energy and <J^2> partials in R (8 bytes,
                // like a double, in both forms)
                double *fin = red;
                R *pwR = reinterpret_cast<R *>(red + kNSlot + 2);
                if (!p.norm_only) {  // uniform over the block: norm-only launches skip the densities
                // ---- T22(phi) and right-hand sides
                if (split) {  // compact species blocks: T_b (h x h), Y_b = [R V1; R* U1] rows and columns of b
                    for (int t = threadIdx.x; t < (conc ? 0 : 2 * h * h); t += blockDim.x) {
                        const int b = t >= h * h ? 1 : 0, e = t - b * h * h, i = e / h, j = e % h;
                        const int g = (b * h + i) * n + b * h + j;
                        Z s = zep * P[g];
                        s = zfma(zen, P[nn + g], s);
                        s = zfma(zepc, P[2 * nn + g], s);
                        s = zfma(zenc, P[3 * nn + g], s);
                        T[t] = s;
                    }
                    for (int t = threadIdx.x; t < (conc ? 0 : 4 * h * h); t += blockDim.x) {
                        const int b = t >= 2 * h * h ? 1 : 0, e = t - 2 * b * h * h, r = e / h, j = e % h;
                        const int grow = r < h ? b * h + r : n + b * h + (r - h);
                        Y[t] = B[grow * n + b * h + j];
                    }
                    if (!conc) {  // (Onishi norm) the whole CTA solves after the norm
                        __syncthreads();
                        const Grp gall{(int)threadIdx.x, (int)blockDim.x, wid, 0};
                        sing = gj_right_solve_g<Z, 2>(gall, T, h, Y, 2 * h, invd, vec, sh);
                    }
                    // densities of each species block in one pass (rho, kappa10 and kappa01 of an
                    // entry share the loads of Y and V0^T), and zeros across the species
                    for (int t = threadIdx.x; t < 2 * h * h; t += blockDim.x) {
                        const int b = t >= h * h ? 1 : 0, e = t - b * h * h, i = e / h, j = e % h;
                        const Z *Yt = Y + 2 * b * h * h + i * h;   // R V1 T22^-1 rows of species b
                        const Z *Yb = Yt + h * h;                  // R* U1 T22^-1 rows
                        const R *Mv = V0t + (b * h) * n + b * h + j, *Mu = U0t + (b * h) * n + b * h + j;
                        Z sr = zero, s10 = zero, s01 = zero;
                        for (int k = 0; k < h; ++k) {
                            const Z yt = Yt[k];
                            const R mv = Mv[k * n];
                            sr = rfma(mv, yt, sr);
                            s10 = rfma(Mu[k * n], yt, s10);
                            s01 = rfma(mv, Yb[k], s01);
                        }
                        const Z di = b ? zen : zep;
                        const int o = (b * h + i) * ld + b * h + j;
                        S[o] = di * sr;
                        S[n * ld + o] = di * s10;
                        S[2 * n * ld + o] = -(zconj(di) * s01);
                    }
                    for (int t = threadIdx.x; t < 6 * h * h; t += blockDim.x) {  // cross-species zeros
                        const int q = t / (2 * h * h), e = t % (2 * h * h), b = e >= h * h ? 1 : 0;
                        const int i = (e - b * h * h) / h, j = (e - b * h * h) % h;
                        S[q * n * ld + (b * h + i) * ld + (1 - b) * h + j] = zero;
                    }
                } else {
                if (!concg) {  // (2n x 2n Pfaffian or Onishi norm) the whole CTA solves after the norm
                    for (int t = threadIdx.x; t < nn; t += blockDim.x) {
                        Z s = zep * P[t];
                        s = zfma(zen, P[nn + t], s);
                        s = zfma(zepc, P[2 * nn + t], s);
                        s = zfma(zenc, P[3 * nn + t], s);
                        T[t] = s;
                    }
                    for (int t = threadIdx.x; t < 2 * nn; t += blockDim.x) Y[t] = B[t];
                    __syncthreads();
                    sing = gj_right_solve<Z>(T, n, Y, 2 * n, invd, vec, sh);
                }
                // ---- densities into the Pfaffian's storage, row stride ld
                {
                    const int dq = blockDim.x / n, dr = blockDim.x % n;
                    for (int q = 0; q < 3; ++q) {
                        const R *Mq = (q == 1) ? U0t : V0t;
                        const Z *Yq = (q == 2) ? Y + nn : Y;
                        Z *Sq = S + q * n * ld;
                        int i = threadIdx.x / n, j = threadIdx.x % n;
                        for (int t = threadIdx.x; t < nn; t += blockDim.x) {
                            const Z *Yr = Yq + i * n;
                            const R *M = Mq + j;
                            Z s = zero;
                            for (int k = 0; k < n; ++k) s = rfma(M[k * n], Yr[k], s);
                            const Z di = (i < h) ? zep : zen;
                            Sq[i * ld + j] = (q == 2) ? -(zconj(di) * s) : di * s;
                            i += dq;
                            j += dr;
                            if (j >= n) {
                                j -= n;
                                ++i;
                            }
                        }
                    }
                }
                }  // split
                __syncthreads();
                // K01_ij (i < j) at Kc[i ld + j], K10_ij at Kc[j ld + i]
                for (int t = threadIdx.x; t < n * (n - 1) / 2; t += blockDim.x) {
                    int i, j;
                    tri_index(t, n, i, j);
                    Kc[i * ld + j] = k01[i * ld + j] - k01[j * ld + i];
                    Kc[j * ld + i] = k10[i * ld + j] - k10[j * ld + i];
                }
                __syncthreads();
                // ---- observables. Final sums land in red[0..kNSlot); the energy and <J^2>
                // sums, spread over all warps, leave per-warp partials in red[kNSlot + ..].
                // traces of rho, spread over warps 0 (species traces, sum j(j+1) rho_aa), 11 (J+, J-,
                // Jz) and 12 (one-body energy) so that no warp starts the energy loop much later
                // The sums run in the point arithmetic's real type R (double-float on the FP32
                // pipes in that form) and leave it once per warp, in lane 0.
                if (wid == 0 || wid == kNTrace + 1 || wid == kNTrace + 2) {
                    R v0 = A::rzero(), v1 = v0, v2 = v0, v3 = v0, v4 = v0, v5 = v0;
                    if (wid == 0) {
                        for (int a = lane; a < n; a += 32) {
                            const Z d = rho[a * ld + a];
                            if (a < h) { v0 = A::radd(v0, d.x); v1 = A::radd(v1, d.y); }
                            else { v2 = A::radd(v2, d.x); v3 = A::radd(v3, d.y); }
                            const R jj = A::pick(p.obs.jj1, p.obs.jj1_d, a);
                            v4 = A::rfma(jj, d.x, v4);
                            v5 = A::rfma(jj, d.y, v5);
                        }
                    } else if (wid == kNTrace + 1) {
                        for (int a = lane; a < n; a += 32) {
                            const R jpa = A::pick(p.obs.jp, p.obs.jp_d, a), jma = A::pick(p.obs.jm, p.obs.jm_d, a);
                            const R mza = A::pick(p.obs.mz, p.obs.mz_d, a);
                            if (A::nz(jpa)) {
                                const Z r = rho[(a + 1) * ld + a];
                                v0 = A::rfma(jpa, r.x, v0);
                                v1 = A::rfma(jpa, r.y, v1);
                            }
                            if (A::nz(jma)) {
                                const Z r = rho[(a - 1) * ld + a];
                                v2 = A::rfma(jma, r.x, v2);
                                v3 = A::rfma(jma, r.y, v3);
                            }
                            const Z d = rho[a * ld + a];
                            v4 = A::rfma(mza, d.x, v4);
                            v5 = A::rfma(mza, d.y, v5);
                        }
                    } else {
                        for (int e = lane; e < p.obs.n_t1b; e += 32) {
                            const int ix = p.obs.t1b_idx[e];
                            const Z r = rho[(ix >> 8) * ld + (ix & 255)];
                            const R tv = A::pick(p.obs.t1b_val, p.obs.t1b_val_d, e);
                            v0 = A::rfma(tv, r.x, v0);
                            v1 = A::rfma(tv, r.y, v1);
                        }
                    }
                    // result slots: z 0,1  n 2,3  t1b 4,5  J+ 10,11  J- 12,13  Jz 14,15  j(j+1) 16,17
                    const int s0 = wid == 0 ? 0 : (wid == kNTrace + 1 ? 10 : 4);
                    const int cnt = wid == kNTrace + 2 ? 2 : 6;
                    const R vals[6] = {v0, v1, v2, v3, v4, v5};
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        if (q >= cnt) break;
                        const R v = A::wsum(vals[q]);
                        const int slot = (wid == 0 && q >= 4) ? 12 + q : s0 + q;
                        if (lane == 0) fin[slot] = A::dbl(v);
                    }
                } else if (p.iE2 && wid <= kNTrace) {  // Q_{2mu} traces: one warp per trace
                    const int q = wid - 1;
                    R sr = A::rzero(), si = A::rzero();
                    for (int e = p.obs.q_off[q] + lane; e < p.obs.q_off[q + 1]; e += 32) {
                        const int ix = p.obs.q_idx[e];
                        const Z r = rho[(ix >> 8) * ld + (ix & 255)];
                        const R qv = A::pick(p.obs.q_val, p.obs.q_val_d, e);
                        sr = A::rfma(qv, r.x, sr);
                        si = A::rfma(qv, r.y, si);
                    }
                    sr = A::wsum(sr);
                    si = A::wsum(si);
                    if (lane == 0) {
                        fin[18 + 2 * q] = A::dbl(sr);
                        fin[19 + 2 * q] = A::dbl(si);
                    }
                }
                if (r1out && wid > kNTrace) {  // one-body density blocks (ZRho1B_Angles): the idle warps
                    for (int b = wid - kNTrace - 1; b < p.obs.n_r1b; b += nw - kNTrace - 1) {
                        R sr = A::rzero(), si = A::rzero();
                        for (int e = p.obs.r1b_off[b] + lane; e < p.obs.r1b_off[b + 1]; e += 32) {
                            const int ix = p.obs.r1b_idx[e];
                            const Z r = rho[(ix >> 8) * ld + (ix & 255)];
                            const R bv = A::pick(p.obs.r1b_val, p.obs.r1b_val_d, e);
                            sr = A::rfma(bv, r.x, sr);
                            si = A::rfma(bv, r.y, si);
                        }
                        sr = A::wsum(sr);
                        si = A::wsum(si);
                        if (lane == 0) {
                            red[kR1BSlot + 2 * b] = A::dbl(sr);
                            red[kR1BSlot + 2 * b + 1] = A::dbl(si);
                        }
                    }
                }
                auto put = [&](int slot, R v) {  // slot 0..3: energy re/im, <J^2> re/im
                    v = A::wsum(v);
                    if (lane == 0) pwR[slot * nw + wid] = v;
                };
                if (p.tc_splits) {
                    // tensor-core contraction: this gauge point's operand rows X[2 pt + ri] (rho
                    // entries, then K10 pairs) and epilogue rows Y[2 pt + ri] (K01 pairs) as bf16
                    // terms; contract_tc.cu forms the two bilinear forms for the whole launch
                    const long long pt = pt0 + lp * p.nfom + ln;
                    const int S = p.tc_splits, nk = p.tc_nk, npp = p.tc_nk - p.tc_nph;
                    for (int e = threadIdx.x; e < nk; e += blockDim.x) {
                        const int src = p.tc_src[e];
                        Z v = zero, y = zero;
                        if (src >= 0) {
                            const int r = src >> 8, c = src & 255;
                            if (e < p.tc_nph) {
                                v = rho[r * ld + c];
                            } else {
                                v = Kc[c * ld + r];   // K10_rc, r < c
                                y = Kc[r * ld + c];   // K01_rc
                            }
                        }
                        unsigned short tr[3], ti[3];
                        bf16_terms(as_dd(v.x), S, tr);
                        bf16_terms(as_dd(v.y), S, ti);
                        for (int sp = 0; sp < S; ++sp) {
                            p.tc_x[sp][(2 * pt) * nk + e] = tr[sp];
                            p.tc_x[sp][(2 * pt + 1) * nk + e] = ti[sp];
                        }
                        if (e >= p.tc_nph) {
                            bf16_terms(as_dd(y.x), S, tr);
                            bf16_terms(as_dd(y.y), S, ti);
                            const int ey = e - p.tc_nph;
                            for (int sp = 0; sp < S; ++sp) {
                                p.tc_y[sp][(2 * pt) * npp + ey] = tr[sp];
                                p.tc_y[sp][(2 * pt + 1) * npp + ey] = ti[sp];
                            }
                        }
                    }
                    if (lane == 0) {   // no energy sum in this form
                        pwR[wid] = A::rzero();
                        pwR[nw + wid] = A::rzero();
                    }
                } else {   // two-body energy, exact regrouping of the 8-term sum of
                    // PNAMP_Energy_OpenMP.f90:40-78:
                    // V[rho_ki rho_lj - rho_li rho_kj + d(rho_ik rho_jl - rho_jk rho_il)]
                    // + V/4 [K01_ij K10_kl + d K01_kl K10_ij],  K_xy = kappa_xy - kappa_yx
                    const R quarter = A::rconst(0.25f);
                    Z e2 = zero;
                    auto rec = [&](uint32_t pk, R v) {
                        const int i = pk & 0xff, j = (pk >> 8) & 0xff, k = (pk >> 16) & 0xff, l = pk >> 24;
                        Z t = rho[k * ld + i] * rho[l * ld + j];
                        t = zfms(rho[l * ld + i], rho[k * ld + j], t);
                        Z u = Kc[i * ld + j] * Kc[l * ld + k];
                        if (i + j != k + l) {
                            t = zfma(rho[i * ld + k], rho[j * ld + l], t);
                            t = zfms(rho[j * ld + k], rho[i * ld + l], t);
                            u = zfma(Kc[k * ld + l], Kc[j * ld + i], u);
                        }
                        t = rfma(quarter, u, t);
                        e2 = rfma(v, t, e2);
                    };
                    // proton-neutron records of a species-split pair: rho_li, rho_kj, rho_jk, rho_il
                    // and both pairing tensors cross the species and vanish
                    auto rec_pn = [&](uint32_t pk, R v) {
                        const int i = pk & 0xff, j = (pk >> 8) & 0xff, k = (pk >> 16) & 0xff, l = pk >> 24;
                        Z t = rho[k * ld + i] * rho[l * ld + j];
                        if (i + j != k + l) t = zfma(rho[i * ld + k], rho[j * ld + l], t);
                        e2 = rfma(v, t, e2);
                    };
                    const int stride = blockDim.x;
                    const int ngen = split ? p.nrec_gen : p.nrec;
                    for (int e = threadIdx.x; e < ngen; e += 2 * stride) {
                        const int e1 = e + stride;
                        const uint32_t pk0 = p.rec_idx[e];
                        const R v0 = A::pick(p.rec_v, p.rec_vd, e);
                        const bool two = e1 < ngen;
                        const uint32_t pk1 = two ? p.rec_idx[e1] : 0u;
                        const R v1 = two ? A::pick(p.rec_v, p.rec_vd, e1) : A::rzero();
                        rec(pk0, v0);
                        if (two) rec(pk1, v1);
                    }
                    for (int e = ngen + threadIdx.x; e < p.nrec; e += 2 * stride) {
                        const int e1 = e + stride;
                        const uint32_t pk0 = p.rec_idx[e];
                        const R v0 = A::pick(p.rec_v, p.rec_vd, e);
                        const bool two = e1 < p.nrec;
                        const uint32_t pk1 = two ? p.rec_idx[e1] : 0u;
                        const R v1 = two ? A::pick(p.rec_v, p.rec_vd, e1) : A::rzero();
                        rec_pn(pk0, v0);
                        if (two) rec_pn(pk1, v1);
                    }
                    put(0, e2.x);
                    put(1, e2.y);
                }
                {   // <J^2> (ZJ2_0, PNAMP_ME2B.f90:45-147) summed over x, y, z with
                    // Jx, Jy = (J+ +- J-)/(2, 2i):  sum_a j(j+1) rho_aa [above]
                    // + Tr(J+ rho) Tr(J- rho) + Tr(Jz rho)^2 - Tr(J+ rho J- rho) - Tr(Jz rho Jz rho)
                    // + [Tr(J+ k10 J+ k01^T) + Tr(J- k10 J- k01^T)]/2 + Tr(Jz k10 Jz k01^T)
                    const R half = A::rconst(0.5f);
                    Z rest = zero;
                    // a species-split pair has no proton-neutron densities and J+-, Jz keep the
                    // species, so every term with a and c of different species vanishes: only the
                    // two diagonal h x h blocks are summed (index t -> block, row, column)
                    const int cnt = split ? 2 * h * h : nn, w = split ? h : n;
                    for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
                        const int blk = split ? t / (h * h) : 0, e = t - blk * h * h;
                        const int a = blk * h + e / w, c = blk * h + e % w;
                        const R jpa = A::pick(p.obs.jp, p.obs.jp_d, a), jma = A::pick(p.obs.jm, p.obs.jm_d, a);
                        const R jpc = A::pick(p.obs.jp, p.obs.jp_d, c), jmc = A::pick(p.obs.jm, p.obs.jm_d, c);
                        const R mzz = A::rmul(A::pick(p.obs.mz, p.obs.mz_d, a), A::pick(p.obs.mz, p.obs.mz_d, c));
                        const int ac = a * ld + c;
                        Z q = mzz * (k10[ac] * k01[ac]);
                        q = zfms(mzz * rho[ac], rho[c * ld + a], q);
                        if (A::nz(jpa) && A::nz(jmc))
                            q = zfms(A::rmul(jpa, jmc) * rho[ac + ld], rho[(c - 1) * ld + a], q);
                        if (A::nz(jpa) && A::nz(jpc))
                            q = zfma(A::rmul(half, A::rmul(jpa, jpc)) * k10[ac + ld], k01[ac + 1], q);
                        if (A::nz(jma) && A::nz(jmc))
                            q = zfma(A::rmul(half, A::rmul(jma, jmc)) * k10[ac - ld], k01[ac - 1], q);
                        rest = rest + q;
                    }
                    put(2, rest.x);
                    put(3, rest.y);
                }
                }  // !norm_only
                __syncthreads();
                if (wid == 0) {  // accumulation over the gauge points: warp 0, one observable per lane
                    // The FP64 pipe is narrow on this part and its cost grows with the active lanes,
                    // so each FP64 value is formed by the one lane that needs it: the norm by lane
                    // 0 (then broadcast), H/N by lane 6 (and 0 for the per-gauge output), <J^2> by
                    // lane 7; the per-warp energy and <J^2> partials are summed in the point
                    // arithmetic first.
                    const unsigned full = 0xffffffffu;
                    R ws[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) ws[q] = A::wsum(lane < nw ? pwR[q * nw + lane] : A::rzero());
                    const bool eval = !p.norm_only && !sing;
                    zc norm = mk(0.0, 0.0);
                    if (lane == 0) {
                        const zc zph = mk(p.gphase[2 * (lp * p.nfom + ln)], p.gphase[2 * (lp * p.nfom + ln) + 1]);
                        norm = onishi ? pf : (p.vacfac * det0 * det1) * (pf * zph);
                    }
                    norm.x = __shfl_sync(full, norm.x, 0);
                    norm.y = __shfl_sync(full, norm.y, 0);
                    zc o = mk(0.0, 0.0), hg = mk(0.0, 0.0);   // hg: H/N at this gauge point (0 if not computed)
                    bool use = eval;
                    if ((lane == 6 || (lane == 0 && gout)) && eval)
                        hg = mk(fin[4] + A::dbl(ws[0]) + p.e0, fin[5] + A::dbl(ws[1]));
                    if (lane == 1) o = mk(fin[0], fin[1]);
                    else if (lane == 2) o = mk(fin[2], fin[3]);
                    else if (lane == 3) o = mk(fin[4], fin[5]);      // one-body energy
                    else if (lane == 6) o = hg;
                    else if (lane == 7) {
                        const zc trp = mk(fin[10], fin[11]), trm = mk(fin[12], fin[13]), trz = mk(fin[14], fin[15]);
                        o = mk(fin[16] + A::dbl(ws[2]), fin[17] + A::dbl(ws[3])) + trp * trm + trz * trz;
                    } else if (lane >= 8 && lane < 18 && p.iE2) o = mk(fin[2 * lane + 2], fin[2 * lane + 3]);  // Q slots 18..37
                    else use = false;
                    if (p.tc_splits && lane == 0) {   // w = N / NFOM^2 of this gauge point, 0 if not evaluated
                        const long long pt = pt0 + lp * p.nfom + ln;
                        const double inv = 1.0 / ((double)p.nfom * p.nfom);
                        p.tc_w[2 * pt] = eval ? inv * norm.x : 0.0;
                        p.tc_w[2 * pt + 1] = eval ? inv * norm.y : 0.0;
                    }
                    if (lane == 0) {
                        acc[0] = acc[0] + norm;
                        if (r2out) {
                            red[kR2Norm] = norm.x;
                            red[kR2Norm + 1] = norm.y;
                        }
                        if (gout) {  // per gauge point: N (with the gauge phase) and H/N
                            double *g = gout + 4LL * (((long long)pair * p.n_euler + ie) * p.n_gauge + lp * p.nfom + ln);
                            g[0] = norm.x;
                            g[1] = norm.y;
                            g[2] = hg.x;
                            g[3] = hg.y;
                        }
                        int f = (under == 1) ? 1 : (under == 2 ? 4 : 0);
                        if (!p.norm_only && sing) f |= 2;
                        flags |= f;
                    }
                    if (use) acc[lane] = zfma(norm, o, acc[lane]);
                    if (eval)
                        for (int b = lane; b < (r1out ? p.obs.n_r1b : 0); b += 32)
                            acc_r1b[b] = zfma(norm, mk(red[kR1BSlot + 2 * b], red[kR1BSlot + 2 * b + 1]), acc_r1b[b]);
                    __syncwarp();   // thread 0 reads every lane's accumulator after the last gauge point
                }
                // No CTA barrier here: the other warps go on to the next gauge point while warp 0
                // accumulates this one. What warp 0 reads (the sums in red, pf, sing) is written
                // again only after the next point's first CTA-wide barrier, which waits for warp 0;
                // the two-body density pass reads the densities, so it keeps the barrier.
                if (r2out) __syncthreads();
                if (r2out && !p.norm_only && !sing) {
                    // ZRho2B_Angles (PNAMP_Rho2B.f90:105-112) before its Clebsch-Gordan sums:
                    // N [ZRO(k,i) ZRO(l,j) - ZRO(l,i) ZRO(k,j) + ZKAPA01(i,j) ZKAPA10(k,l)] per quadruple,
                    // summed over the gauge points in FP64; the densities are still in S here
                    const zc nrm = mk(red[kR2Norm], red[kR2Norm + 1]);
                    for (int q = threadIdx.x; q < p.n_r2q; q += blockDim.x) {
                        const uint32_t pk = p.r2q[q];
                        const int i = pk & 0xff, j = (pk >> 8) & 0xff, k = (pk >> 16) & 0xff, l = pk >> 24;
                        Z t = rho[k * ld + i] * rho[l * ld + j];
                        t = zfms(rho[l * ld + i], rho[k * ld + j], t);
                        t = zfma(k01[i * ld + j], k10[k * ld + l], t);
                        const zc a = zfma(nrm, A::to(t), mk(r2acc[2 * q], r2acc[2 * q + 1]));
                        r2acc[2 * q] = a.x;
                        r2acc[2 * q + 1] = a.y;
                    }
                    __syncthreads();  // the next gauge point overwrites the densities
                }
            }
        }
        if (threadIdx.x == 0) {
            const double inv = 1.0 / ((double)p.nfom * p.nfom);
            int f = flags;
            acc[kNobs - 1] = mk(0.0, 0.0);
            for (int io = 0; io < kNobs; ++io) {
                const zc v = inv * acc[io];
                if (!zfinite(v)) f |= 4;
                zout[2LL * (io * p.n_euler + ie)] = v.x;
                zout[2LL * (io * p.n_euler + ie) + 1] = v.y;
            }
            status[(long long)pair * p.n_euler + ie] = f;
            for (int b = 0; b < (r1out ? p.obs.n_r1b : 0); ++b) {
                const zc v = inv * acc_r1b[b];
                r1out[2LL * (((long long)pair * p.obs.n_r1b + b) * p.n_euler + ie)] = v.x;
                r1out[2LL * (((long long)pair * p.obs.n_r1b + b) * p.n_euler + ie) + 1] = v.y;
            }
        }
        if (r2out) {  // Euler weight x gauge mean, added into the pair's sums (ZRho2B_Integral at J = 0)
            const double wgt = p.euler[4 * ie + 3] / ((double)p.nfom * p.nfom);
            double *o = r2out + 2LL * p.n_r2q * pair;
            for (int q = threadIdx.x; q < p.n_r2q; q += blockDim.x) {
                atomicAdd(o + 2 * q, wgt * r2acc[2 * q]);
                atomicAdd(o + 2 * q + 1, wgt * r2acc[2 * q + 1]);
            }
        }
        __syncthreads();
    }
}

template <class Z>
__global__ void __launch_bounds__(kThreads, 1)
point_kernel(Params p, int npairs, const double *__restrict__ pairbuf, zc *scratch,
             double *__restrict__ zres, int *__restrict__ status, const int2 *__restrict__ items,
             long long nitems, double *__restrict__ gout, double *__restrict__ r1out,
             double *__restrict__ r2out) {
    // items == nullptr: every (pair, Euler point) of the batch; else the listed (pair, ie)
    zc *slot = scratch + (long long)blockIdx.x * p.place.slot_elems;
    const long long total = items ? nitems : (long long)npairs * p.n_euler;
    int cur_pair = -1;
    for (long long item = blockIdx.x; item < total; item += gridDim.x) {
        int pair, ie;
        if (items) {
            const int2 it = items[item];
            pair = it.x;
            ie = it.y;
            if (pair < 0 || pair >= npairs || ie < 0 || ie >= p.n_euler) continue;  // out of range: skipped
        } else {
            pair = (int)(item / p.n_euler);
            ie = (int)(item % p.n_euler);
        }
        point_item<Z>(p, pairbuf, slot, pair, ie, pair != cur_pair, zres, status, gout, r1out, r2out,
                      item * p.n_gauge);
        cur_pair = pair;
    }
}

// Persistent kernel over an uneven batch: work items (context, pair, Euler point)
// of up to kMultiCtx contexts (model spaces, meshes, placements), taken `grab`
// at a time from a global counter in the order of `items` (set by the schedule).
// Every context's parameters travel by value in the launch's parameter space and
// each context has its own inlined copy of the point body, so the per-point code
// reads its sizes and table pointers as constant-bank operands exactly as the
// single-context kernel does (an indexed parameter array would become a load per
// use inside the hot loops).
template <class Z>
__device__ __forceinline__ void multi_item(const MultiArgs &a, int4 m, zc *slot, bool reload) {
    switch (m.x) {
    case 0: point_item<Z>(a.p[0], a.pairbuf[0], slot, m.y, m.z, reload, a.zres[0], a.status[0]); break;
    case 1: point_item<Z>(a.p[1], a.pairbuf[1], slot, m.y, m.z, reload, a.zres[1], a.status[1]); break;
    case 2: point_item<Z>(a.p[2], a.pairbuf[2], slot, m.y, m.z, reload, a.zres[2], a.status[2]); break;
    default: point_item<Z>(a.p[3], a.pairbuf[3], slot, m.y, m.z, reload, a.zres[3], a.status[3]); break;
    }
}
static_assert(kMultiCtx == 4, "multi_item dispatches four contexts");

template <class Z>
__global__ void __launch_bounds__(kThreads, 1)
multi_point_kernel(const __grid_constant__ MultiArgs a, const int4 *__restrict__ items, int nitems, int grab,
                   zc *scratch, int *counter, int smem_tail) {
    // the work counter's broadcast lives past every context's placement (no static
    // shared memory, so the dynamic limit can be the device maximum)
    extern __shared__ __align__(16) unsigned char smem_all[];
    int &s_next = *reinterpret_cast<int *>(smem_all + smem_tail);
    zc *slot = scratch + (long long)blockIdx.x * a.slot_stride;
    int cur_ctx = -1, cur_pair = -1;
    for (;;) {
        if (threadIdx.x == 0) s_next = atomicAdd(counter, grab);
        __syncthreads();
        const int base = s_next;
        __syncthreads();
        if (base >= nitems) break;
        const int end = min(base + grab, nitems);
        for (int it = base; it < end; ++it) {
            const int4 m = items[it];  // (context, pair, Euler point, unused)
            multi_item<Z>(a, m, slot, m.x != cur_ctx || m.y != cur_pair);
            cur_ctx = m.x;
            cur_pair = m.y;
        }
    }
}

template <class Z>
static const void *point_fn() {
    return reinterpret_cast<const void *>(point_kernel<Z>);
}

template <class Z>
static const void *multi_fn() {
    return reinterpret_cast<const void *>(multi_point_kernel<Z>);
}

cudaError_t multi_blocks_per_sm(int form, int smem_bytes, int *per_sm) {
    const void *f = form == 1 ? multi_fn<zd>() : multi_fn<zc>();
    cudaError_t e = raise_smem_limit(f);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, f, kThreads, smem_bytes);
}

cudaError_t launch_multi(int form, const MultiArgs &a, const int4 *items, int nitems, int grab, int *counter,
                         zc *scratch, int grid, int smem, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    if (form == 1)
        multi_point_kernel<zd><<<grid, kThreads, smem, st>>>(a, items, nitems, grab, scratch, counter,
                                                            smem - kMultiSmemTail);
    else
        multi_point_kernel<zc><<<grid, kThreads, smem, st>>>(a, items, nitems, grab, scratch, counter,
                                                            smem - kMultiSmemTail);
    return cudaGetLastError();
}

cudaError_t point_blocks_per_sm(int form, int smem_bytes, int *per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        per_sm, form == 1 ? point_fn<zd>() : point_fn<zc>(), kThreads, smem_bytes);
}

cudaError_t set_point_smem(int form, int bytes) {
    (void)bytes;  // checked against the device maximum by the placement planner
    return raise_smem_limit(form == 1 ? point_fn<zd>() : point_fn<zc>());
}

cudaError_t launch_points(const Params &p, int npairs, const double *pairbuf, zc *scratch, int grid,
                          double *zres, int *status, cudaStream_t st, const int2 *items, long long nitems,
                          double *gout, double *r1out, double *r2out) {
    if (r2out && (p.n_r2q <= 0 || !p.r2q || !p.r2acc)) return cudaErrorInvalidValue;
    if (p.form == 1)
        point_kernel<zd><<<grid, kThreads, p.place.smem_bytes, st>>>(p, npairs, pairbuf, scratch, zres, status,
                                                                    items, nitems, gout, r1out, r2out);
    else
        point_kernel<zc><<<grid, kThreads, p.place.smem_bytes, st>>>(p, npairs, pairbuf, scratch, zres, status,
                                                                    items, nitems, gout, r1out, r2out);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ projection
// Weights W[ie][jkk] = wJ * w_ie * e^{i K1 alp} d^J_{K1K2}(bet) e^{i K2 gam}, jkk over
// (J = 0,2,4,6; K1 = -J..J; K2 = -J..J), wJ = (2J+1)/(8 pi^2) or (2J+1)/2 for an
// N_alp N_gam = 1 mesh (Kernel3D.f90:78-81).
__global__ void proj_weights_kernel(Params p, int axial, zc *w) {
    const int ie = blockIdx.x;
    const double alp = p.euler[4 * ie], bet = p.euler[4 * ie + 1], gam = p.euler[4 * ie + 2],
                 wt = p.euler[4 * ie + 3];
    double cb, sb;
    sincos(0.5 * bet, &sb, &cb);
    for (int jkk = threadIdx.x; jkk < kNJKK; jkk += blockDim.x) {
        int J = 0, rem = jkk;
        while (rem >= (2 * J + 1) * (2 * J + 1)) {
            rem -= (2 * J + 1) * (2 * J + 1);
            J += 2;
        }
        const int K1 = rem / (2 * J + 1) - J, K2 = rem % (2 * J + 1) - J;
        const double wj = axial ? (2.0 * J + 1.0) / 2.0 : (2.0 * J + 1.0) / (8.0 * M_PI * M_PI);
        const double d = wigner_d(2 * J, 2 * K1, 2 * K2, cb, sb, p.fact);
        w[(long long)ie * kNJKK + jkk] = (wj * wt * d) * expi(K1 * alp + K2 * gam);
    }
}

__global__ void project_kernel(Params p, const zc *__restrict__ w, const double *__restrict__ zres,
                               int core_prot, int core_neut, int chop, double *__restrict__ out) {
    const int pair = blockIdx.x;
    const int jkk = blockIdx.y * blockDim.x + threadIdx.x;
    if (jkk >= kNJKK) return;
    const double *z = zres + 2LL * pair * kNobs * p.n_euler;
    zc s[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) s[q] = mk(0, 0);
    for (int ie = 0; ie < p.n_euler; ++ie) {
        const zc wv = w[(long long)ie * kNJKK + jkk];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const zc zv = mk(z[2LL * (q * p.n_euler + ie)], z[2LL * (q * p.n_euler + ie) + 1]);
            s[q] = zfma(wv, zv, s[q]);
        }
    }
    int J = 0, rem = jkk;
    while (rem >= (2 * J + 1) * (2 * J + 1)) {
        rem -= (2 * J + 1) * (2 * J + 1);
        J += 2;
    }
    const int K1 = rem / (2 * J + 1) - J, K2 = rem % (2 * J + 1) - J;
    const long long fs = (long long)(kJJMax + 1) * kNK * kNK;
    const long long o = ((long long)J * kNK + (K1 + kJJMax)) * kNK + (K2 + kJJMax);
    double *op = out + 2LL * pair * kProjFields * fs;
    if (chop && !(sqrt(abs2(s[0])) >= 1.0e-8)) return;  // fields stay 0 (Kernel3D.f90:732)
    const zc inv0 = zrecip(s[0]);
    const zc f[kProjFields] = {s[0], s[6], s[2] * inv0 + mk(core_neut, 0), s[1] * inv0 + mk(core_prot, 0),
                               s[7] * inv0};
#pragma unroll
    for (int q = 0; q < kProjFields; ++q) {
        op[2 * (q * fs + o)] = f[q].x;
        op[2 * (q * fs + o) + 1] = f[q].y;
    }
}

cudaError_t launch_project(const Params &p, int npairs, const zc *w, const double *zres, int core_prot,
                           int core_neut, int chop, double *out, cudaStream_t st) {
    dim3 grid(npairs, (kNJKK + 127) / 128);
    project_kernel<<<grid, 128, 0, st>>>(p, w, zres, core_prot, core_neut, chop, out);
    return cudaGetLastError();
}

// Quadrupole reduced elements <J1 K1||Q2||J2 K2>, J1 = J2 + dJ, dJ = 0, 1, 2
// (PNAMP_Kernel3D_v2.f90:515-600): one thread per (J2, dJ, K1, K2) output,
// direct and, when `exchange`, the q1 <-> q2 exchanged element from the Q^dagger
// traces. `tj` holds the 3j symbols (J1 2 J2; -K1 mu K2p) per output and mu.
// Output [pair][2][7][3][17][13] complex (direct, exchanged), zeroed beforehand.
__global__ void project_q_kernel(Params p, int axial, const double *__restrict__ zres, const double *__restrict__ tj,
                                 int exchange, double *__restrict__ out) {
    const int pair = blockIdx.x;
    const int o = blockIdx.y * blockDim.x + threadIdx.x;  // index into the (J2, dJ, K1, K2) list
    int J2 = 0, dJ = 0, rem = o, found = 0;
    for (J2 = 0; J2 <= kJJMax && !found; J2 += 2)
        for (dJ = 0; dJ < 3; ++dJ) {
            const int cnt = (2 * (J2 + dJ) + 1) * (2 * J2 + 1);
            if (rem < cnt) {
                found = 1;
                break;
            }
            rem -= cnt;
        }
    if (!found) return;
    J2 -= 2;  // undo the outer loop's final increment
    const int J1 = J2 + dJ;
    const int K1 = rem / (2 * J2 + 1) - J1, K2 = rem % (2 * J2 + 1) - J2;
    const double *z = zres + 2LL * pair * kNobs * p.n_euler;
    zc sd = mk(0, 0), sx = mk(0, 0);
    for (int ie = 0; ie < p.n_euler; ++ie) {
        const double alp = p.euler[4 * ie], bet = p.euler[4 * ie + 1], gam = p.euler[4 * ie + 2],
                     w = p.euler[4 * ie + 3];
        double cb, sb;
        sincos(0.5 * bet, &sb, &cb);
        for (int mu = -2; mu <= 2; ++mu) {
            const int K2p = K1 - mu;
            const double t3 = tj[5 * o + mu + 2];
            if (K2p > J2 || -K2p > J2 || t3 == 0.0) continue;
            const double ph = ((J1 - K1) & 1) ? -1.0 : 1.0;
            const zc zq = mk(z[2LL * ((10 + mu) * p.n_euler + ie)], z[2LL * ((10 + mu) * p.n_euler + ie) + 1]);
            const double d1 = wigner_d(2 * J2, 2 * K2p, 2 * K2, cb, sb, p.fact);
            sd = zfma((w * ph * t3 * d1) * expi(K2p * alp + K2 * gam), zq, sd);
            if (exchange) {
                const double d2 = wigner_d(2 * J2, 2 * K2, 2 * K2p, cb, sb, p.fact);
                const zc e2 = expi(-(K2 * alp + K2p * gam));
                for (int nu = -2; nu <= 2; ++nu) {
                    const int ix = 15 + nu;
                    const zc zt = mk(z[2LL * (ix * p.n_euler + ie)], -z[2LL * (ix * p.n_euler + ie) + 1]);
                    const double sg = ((mu - nu) & 1) ? -1.0 : 1.0;
                    const double dq = wigner_d(4, -2 * nu, -2 * mu, cb, sb, p.fact);
                    sx = zfma((w * ph * sg * dq * t3 * d2) * (expi(-(nu * alp + mu * gam)) * e2), zt, sx);
                }
            }
        }
    }
    const double wj = axial ? (2.0 * J2 + 1.0) / 2.0 : (2.0 * J2 + 1.0) / (8.0 * M_PI * M_PI);
    const double f = wj * (2 * J1 + 1);
    const long long blk = 7LL * 3 * 17 * 13;
    const long long idx = (((long long)J2 * 3 + dJ) * 17 + (K1 + 8)) * 13 + (K2 + 6);
    double *op = out + 2LL * pair * 2 * blk;
    op[2 * idx] = f * sd.x;
    op[2 * idx + 1] = f * sd.y;
    op[2 * (blk + idx)] = f * sx.x;
    op[2 * (blk + idx) + 1] = f * sx.y;
}

int n_q_outputs() {
    int c = 0;
    for (int J2 = 0; J2 <= kJJMax; J2 += 2)
        for (int dJ = 0; dJ < 3; ++dJ) c += (2 * (J2 + dJ) + 1) * (2 * J2 + 1);
    return c;
}

cudaError_t launch_project_q(const Params &p, int axial, int npairs, const double *zres, const double *tj,
                             int exchange, double *out, cudaStream_t st) {
    dim3 grid(npairs, (n_q_outputs() + 127) / 128);
    project_q_kernel<<<grid, 128, 0, st>>>(p, axial, zres, tj, exchange, out);
    return cudaGetLastError();
}

cudaError_t launch_proj_weights(const Params &p, int axial, zc *w, cudaStream_t st) {
    proj_weights_kernel<<<p.n_euler, 128, 0, st>>>(p, axial, w);
    return cudaGetLastError();
}

}  // namespace pnamp
