// Internal interface between the C ABI (pnamp_capi.cu) and the kernels
// (pnamp_kernels.cu). Not part of the public header.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pnamp_df64.cuh"

namespace pnamp {

constexpr int kNobs = 19;
constexpr int kJJMax = 6;
constexpr int kNK = 2 * kJJMax + 1;
constexpr int kMaxN = 64;
constexpr int kMaxBlocks = 64;           // rotation blocks (t, n, l, j) of a model space
constexpr int kThreads = 512;            // threads per CTA of the point kernel (<= 128 registers)
constexpr int kNTrace = 10;              // proton traces of Q_{2mu} rho and Q_{2mu}^dagger rho
constexpr int kNJKK = 1 + 25 + 81 + 169; // (J, K1, K2) with even J <= 6
constexpr int kProjFields = 5;           // njkk, hjkk, nn, zz, j2
constexpr int kSetupThreads = 256;
constexpr int kMultiSmemTail = 16;       // dynamic shared bytes after the placement: multi kernel's counter

// One pair record (doubles), all matrices row-major n x n:
// U0 V0 U1 V1 W Z0 ZI then [det0, det1, status-as-double, reduced flag, Pf(-c Z0) re, im, pad, pad].
// ZI = Z0^-1 = U0 V0^-1; with the reduced flag set the point kernel eliminates the n x n
// matrix c (D X D - ZI) and multiplies by Pf(-c Z0) instead of eliminating the 2n x 2n one.
struct PairLayout {
    long long u0, v0, u1, v1, w, z0, zi, dets, pfz, stride;
    __host__ __device__ void make(int n) {
        long long nn = (long long)n * n;
        u0 = 0; v0 = nn; u1 = 2 * nn; v1 = 3 * nn; w = 4 * nn; z0 = 5 * nn; zi = 6 * nn; dets = 7 * nn;
        pfz = dets + 4;
        stride = 7 * nn + 8;
    }
};
// min/max |LU pivot| of V0 for the reduced Pfaffian. A bra with nearly empty levels (small
// singular values of V0) makes Z0^-1 dominate the Schur complement c (D X D - Z0^-1), whose
// Pfaffian then carries the point's dependence in its low-order bits: on the shipped Ti48
// vacua a ratio of 2e-6 cost 2e-9 relative and 8e-5 cost 3e-7, while every bra at >= 3e-2
// stayed within 6e-13 of the 2n x 2n elimination. Below the bound the pair keeps the
// 2n x 2n form.
constexpr double kReducedPivotRatio = 1e-2;

// Where the per-point work arrays live: shared memory or the CTA's global slot.
// Offsets are in bytes (shared) or complex elements (global slot).
struct Placement {
    int s_smem, t_smem, y_smem, uv_smem;
    int off_s, off_t, off_y, off_uv;     // shared byte offsets (when *_smem)
    int off_piv, off_inv, off_red, off_rot, off_vec;
    // species-split pairs, two gauge points in flight (when sp2): compact V0^T, U0^T
    // diagonal blocks at off_uvc, then the two halves' regions (half_layout) from off_half
    int sp2, off_uvc, off_half;
    int smem_bytes;
    long long g_x, g_b, g_p, g_rw, g_zr, g_s, g_t, g_y, g_uv;
    long long slot_elems;
};

// One half's shared region for the species-split path with two gauge points in flight:
// byte offsets of the compact densities (rho, kappa10, kappa01, K; each two h x (h + 1)
// species blocks; the Pfaffian's two h x h blocks come first in the same storage), T22's
// two blocks, the right-hand sides, the solve's pivot row, the Pfaffian vector and pivots,
// the accumulators, the final sums, the per-warp partials and the flags.
constexpr int kHalfThreads = kThreads / 2, kHalfWarps = kHalfThreads / 32;
struct HalfLayout {
    int dens, t, y, invd, vec, pfs, acc, fin, pw, sh, bytes;
};
__host__ __device__ inline HalfLayout half_layout(int h) {
    constexpr int zs = 16;   // complex element, both arithmetics
    HalfLayout L;
    int o = 0;
    auto take = [&](int bytes) { const int at = o; o += (bytes + 15) & ~15; return at; };
    L.dens = take(8 * h * (h + 1) * zs);
    L.t = take(2 * h * h * zs);
    L.y = take(4 * h * h * zs);
    L.invd = take(2 * h * zs);
    L.vec = take((2 * h + 4) * zs);
    L.pfs = take(4 * zs);
    L.acc = take(kNobs * 16);
    L.fin = take(40 * 8);
    L.pw = take(4 * kHalfWarps * 8);
    L.sh = take(16 * 4);
    L.bytes = o;
    return L;
}

// Sparse one-body data used by the observables, built on the host once.
struct ObsTables {
    int n_t1b;                 // entries of the single-particle matrix
    const int *t1b_idx;        // index into rho (c*n + a) for t(a,c) rho(c,a)
    const double *t1b_val;
    int q_off[kNTrace + 1];    // entry ranges per trace
    const int *q_idx;          // index into rho
    const double *q_val;
    const double *jp;          // [n] J+_{a,a+1} (0 at the last state of a block)
    const double *jm;          // [n] J-_{a,a-1} (0 at the first state of a block)
    const double *mz;          // [n] m_a
    const double *jj1;         // [n] j(j+1)
    const dd *jp_d, *jm_d, *mz_d;   // the same coefficients as double-float
    const dd *jj1_d, *t1b_val_d, *q_val_d;
    // one-body density blocks (t, lj, n1, n2) of ZRho1B_Angles: block b sums
    // r1b_val[e] rho(row, col) over e in [r1b_off[b], r1b_off[b + 1]), packed row*256+col
    int n_r1b;
    const int *r1b_off, *r1b_idx;
    const double *r1b_val;
    const dd *r1b_val_d;
};
constexpr int kMaxR1B = 64;               // one-body density blocks per model space

struct Params {
    int n, h, N2;              // n, n/2, 2n
    int nprot, nneut;
    int n_euler, nfom, n_gauge;
    double cscale;
    double e0;                 // H%E0, added to every energy (Kernel3D.f90:324)
    double vacfac;             // (-1)^{n(n+1)/2} * 10^(-2*(n*iscale/2))
    int iE2;
    int form;                  // 0: FP64 (plain), 1: double-float per-point algebra
    int norm_only;             // 1: only the norm kernel N(Omega) (observable 0); the others are 0
    // rotation blocks
    int nblk, rot_elems;
    const int *blk_start, *blk_size, *blk_tj, *blk_roff, *row_blk, *twom;
    const double *euler;       // [n_euler][4] alpha, beta, gamma, weight
    const double *gphase;      // [nfom][nfom] complex e^{-i (phi_lp Z + phi_ln N)}, the projection phase
    const double *fact;        // k!, k = 0..23
    // Hamiltonian two-body list
    int nrec;
    int nrec_gen;              // records [0, nrec_gen): general; [nrec_gen, nrec): a, c protons and b, d neutrons
    const uint32_t *rec_idx;   // packed 8-bit a,b,c,d (0-based)
    const double *rec_v;
    const dd *rec_vd;          // rec_v as double-float (df64 form)
    ObsTables obs;
    PairLayout pl;
    Placement place;
    // two-body density quadruples (ZRho2B_Angles): packed 8-bit k_i, k_j, k_k, k_l, and the
    // per-CTA FP64 accumulators [grid][n_r2q] complex; n_r2q = 0 outside Rho2B launches
    int n_r2q;
    const uint32_t *r2q;
    double *r2acc;
    // tensor-core contraction (contract_tc.cu): tc_splits = 0 runs the record loop here;
    // 2 or 3 makes the point kernel write each gauge point's density rows as that many bf16
    // terms instead (X: tc_nk entries, ph part first, pp part from tc_nph; Y: the pp
    // epilogue vector, tc_nk - tc_nph entries) and its weight N / NFOM^2 (0 when T22 was
    // singular); point p of a launch is item * n_gauge + gauge index
    int tc_splits, tc_nk, tc_nph;
    const int *tc_src;         // [tc_nk]: r << 8 | c (ph entries), i << 8 | j (pp, i < j), -1 padding
    unsigned short *tc_x[3], *tc_y[3];
    double *tc_w;
};

// One group of the contraction: a contiguous range [off, off + dpad) of the X row (and, for
// a pp group, [yoff, yoff + dpad) of the Y row), whose square matrix occupies rows
// [rowbase, rowbase + dpad) of the stacked bf16 matrices (columns 0..dpad-1).
struct TcGroup {
    int kind;      // 0 particle-hole (epilogue vector = X), 1 particle-particle (epilogue vector = Y)
    int off, dpad, rowbase, yoff;
};
struct TcArgs {
    int splits;
    int ngroups;
    long long npts;
    int nk, npp;
    const TcGroup *groups;
    const unsigned short *x[3], *y[3];
    double *e2;        // [npts][2]
    int *err;
};

// Contexts of one multi-context launch, passed by value (kernel parameter space).
constexpr int kMultiCtx = 4;
struct MultiArgs {
    Params p[kMultiCtx];
    const double *pairbuf[kMultiCtx];
    double *zres[kMultiCtx];
    int *status[kMultiCtx];
    long long slot_stride;     // complex elements of one CTA's global slot
};

// launchers (pnamp_kernels.cu)
cudaError_t launch_setup(const Params &p, int npairs, const double *uv, double *pairbuf,
                         cudaStream_t st);
cudaError_t launch_points(const Params &p, int npairs, const double *pairbuf, zc *scratch,
                          int grid, double *zres, int *status, cudaStream_t st,
                          const int2 *items = nullptr, long long nitems = 0, double *gout = nullptr,
                          double *r1out = nullptr, double *r2out = nullptr);
cudaError_t launch_proj_weights(const Params &p, int axial, zc *w, cudaStream_t st);
cudaError_t launch_project(const Params &p, int npairs, const zc *w, const double *zres,
                           int core_prot, int core_neut, int chop, double *out, cudaStream_t st);
cudaError_t launch_project_q(const Params &p, int axial, int npairs, const double *zres, const double *tj,
                             int exchange, double *out, cudaStream_t st);
int n_q_outputs();
cudaError_t multi_blocks_per_sm(int form, int smem_bytes, int *per_sm);
cudaError_t launch_multi(int form, const MultiArgs &a, const int4 *items, int nitems, int grab, int *counter,
                         zc *scratch, int grid, int smem, cudaStream_t st);
cudaError_t set_point_smem(int form, int bytes);
cudaError_t point_blocks_per_sm(int form, int smem_bytes, int *per_sm);
int setup_smem_bytes(int n);
cudaError_t prepare_setup(int n);
// tensor-core contraction (contract_tc.cu)
cudaError_t prepare_contract();
int tc_smem_bytes(int splits);
int tc_chunk_rows(int splits);
cudaError_t launch_contract(const TcArgs &a, const void *const *mat, long long mat_rows, int kmax, int grid,
                            cudaStream_t st);
cudaError_t launch_contract_finish(int npairs, int n_euler, int n_gauge, long long nitems, const int2 *items,
                                   const double *w, const double *e2, double *zres, int *status, const int *err,
                                   cudaStream_t st);

}  // namespace pnamp
