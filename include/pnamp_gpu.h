/*
 * pnamp_gpu.h -- C ABI of the GB300 (sm_103a) PNAMP kernel library.
 *
 * Replaces the hot path of SCCM's PNAMP stage: the per-pair subroutine
 *   subroutine Kernel4Triaxial(lpr, Nphi1, Nphi2, NLEV)
 *     (Codes/PNAMP/PNAMP_Kernel3D.f90:1, called once per (q,q') pair from
 *      Codes/PNAMP/PNAMP_Main.f90:113)
 * and its per-point callees ROTATION_MAT, UVphiomega, Pfaf_Over/ZPfaffianF,
 * ROKAPPAphiomega (Codes/PNAMP/PNAMP_Proj.f90:83-551), ZN_0/ZQ2/ZQ2t
 * (PNAMP_ME1B.f90), ZJ2_0 (PNAMP_ME2B.f90) and HFB_Energy_COMPLEX
 * (PNAMP_Energy_OpenMP.f90:5-100), followed by the J/K projection
 * (PNAMP_Kernel3D.f90:415-751) whose result `post_general`/`post_axial`
 * write to the kernel file (PNAMP_IO.f90:2-96).
 *
 * Conventions
 *  - Plain C types only. Matrices are column-major like the Fortran arrays they
 *    replace: element (i,j) of an n x n matrix is at [i + j*n].
 *  - Complex numbers are interleaved (re, im) doubles, i.e. Fortran complex*16 /
 *    C `double _Complex` layout.
 *  - Every entry point returns a status code (0 = success) where the reference
 *    `stop`s; `pnamp_strerror` gives the text. The library keeps no global
 *    state: all state lives in a context, used by one host thread at a time.
 *  - The caller owns every buffer passed in. The context owns its device memory.
 *  - There is no CPU fallback: without a usable CUDA device `pnamp_init`
 *    returns PNAMP_ERR_CUDA.
 */
#ifndef PNAMP_GPU_H
#define PNAMP_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define PNAMP_NOBS 19   /* observables per Euler point, NOBS (VAPHFB_Par.f90:168) */
#define PNAMP_JJMAX 6   /* largest projected J, JJmax (VAPHFB_Par.f90:278) */
#define PNAMP_NK (2 * PNAMP_JJMAX + 1)
#define PNAMP_MAX_NLEV 64

/* return codes */
#define PNAMP_OK 0
#define PNAMP_ERR_ARG 1          /* invalid argument (sizes, NULL pointers, model space) */
#define PNAMP_ERR_CUDA 2         /* CUDA runtime error or no device */
#define PNAMP_ERR_NOMEM 3        /* device allocation failed */
#define PNAMP_ERR_SINGULAR_U 4   /* U of a vacuum is singular: zbareover/Pfaf_Over ZGETRF info != 0 */
#define PNAMP_ERR_UNSUPPORTED 5  /* a size beyond what this build supports */
#define PNAMP_ERR_STATE 6        /* call order violated */
#define PNAMP_ERR_SCRATCH_LIMIT 7 /* request does not fit the fixed scratch of pnamp_batch_device_noalloc */
#define PNAMP_ERR_SMALL_NORM 8   /* |N^0| <= CHOP: Write_ME1B prints a warning and writes nothing
                                    (PNAMP_Rho1B.f90:74-77) */

/* Size of the fixed device scratch array used by pnamp_batch_device_noalloc. */
#define PNAMP_NOALLOC_SCRATCH_BYTES (32u << 20)

/* arithmetic forms of the per-point algebra (pnamp_set_form) */
#define PNAMP_FORM_FP64 0   /* FP64 throughout: the reference's arithmetic (default) */
#define PNAMP_FORM_DF64 1   /* Pfaffian, LU, solves, densities and contractions in double-float
                               (pairs of FP32, ~48-bit significand) on the FP32 pipes; per-Euler
                               preparation, the Pfaffian product and all reductions stay FP64 */
#define PNAMP_FORM_TC3 2    /* PNAMP_FORM_DF64 with the two-body contraction of HFB_Energy_COMPLEX
                               (PNAMP_Energy_OpenMP.f90:31-90) recast as dense block GEMMs on the
                               tensor cores (tcgen05, bf16 inputs, FP32 accumulation): each value
                               as two bf16 terms, three products ("BF16x3", ~1e-5 relative) */
#define PNAMP_FORM_TC6 3    /* the same with three bf16 terms and six products ("BF16x6", ~1e-7).
                               Both tensor-core forms apply to pnamp_pair, pnamp_batch(_device) and
                               pnamp_batch_items_device (without gauge output; norm-only outputs give
                               PNAMP_ERR_STATE) and stage the densities of up to min(24 GiB, half the
                               free device memory) of points per launch; the other entry points
                               compute in the PNAMP_FORM_DF64 arithmetic under these forms */

/* per-Euler-point status bits (OR over the gauge points of that Euler point) */
#define PNAMP_ST_PIVOT_UNDERFLOW 1  /* Pfaffian pivot |ss| <= 1e-13: norm set to 0 (PNAMP_Proj.f90:290,333) */
#define PNAMP_ST_SINGULAR_T22 2     /* exact zero pivot in the LU of T22 */
#define PNAMP_ST_NONFINITE 4        /* a non-finite value reached ZRES */
#define PNAMP_ST_SINGULAR_U 8       /* the pair's U0 or U1 is singular */
#define PNAMP_ST_CONTRACTION 16     /* tensor-core forms: the contraction kernel gave up (a bounded wait
                                       ran out); the energy ZRES(:, 7) of this point is not valid */

/* Model space: the m-scheme `tnljm` arrays (VAPHFB_Par.f90:39-43), ordered
 * protons (t = -1) first, then neutrons (t = +1); within a species orbits in
 * .val order, m = j, j-1, ..., -j (Codes/GCM/HFBA_Hamiltonian.f90:43-68). */
typedef struct {
    int nlev;                     /* n = HO%NLEV, even, <= PNAMP_MAX_NLEV */
    int nprot, nneut;             /* valence Z and N (Input%nprot, Input%nneut) */
    int core_prot, core_neut;     /* Nucl%ncore(1), Nucl%ncore(0) */
    const int *t, *n, *l, *twoj, *twom;   /* length nlev each */
} pnamp_space;

/* Hamiltonian and one-body operators (module H and cME1B, VAPHFB_Par.f90:45-81). */
typedef struct {
    double e0;                    /* H%E0 */
    const double *t1b;            /* n x n single-particle matrix H%ME1BM */
    int nrec;                     /* H%iabcd_max */
    const int *ka, *kb, *kc, *kd; /* 1-based m-scheme indices, ka < kb, kc < kd, ka+kb <= kc+kd */
    const double *vbar;           /* H%ME2BM, antisymmetrised m-scheme V */
    const double *q2;             /* 5 blocks of n x n: Q_{2mu}, mu = -2..2 (cME1B%Q2_2t..Q22t);
                                     NULL skips observables 9..18 (Input%iE2 = 0) */
} pnamp_hamiltonian;

/* Euler and gauge mesh (module AMP/PNP, VAPHFB_Par.f90:131-151; Codes/GCM/PNAMP_Gaus.f90). */
typedef struct {
    int nalp, nbet, ngam;         /* AMP%NLEG_ALP, NLEG_BET, NLEG_GAM */
    int nfom;                     /* PNP%NFOM gauge points per species */
    int ncosbet;                  /* 1, or 2 to use only the first nbet/2 beta nodes with doubled weight */
    const double *alpha, *walp;   /* length nalp */
    const double *beta, *wbet;    /* length nbet (beta = acos of the Gauss node) */
    const double *gamma, *wgam;   /* length ngam */
    double cscale;                /* Input%Cscale: Pfaffian matrix scale (PNAMP_Proj.f90:204-208) */
    int iscale;                   /* Input%iscale: vacuum factor 10^(-NLEV*iscale/2) (Kernel3D.f90:149) */
} pnamp_mesh;

/* Projected kernels, the `Kernel%` fields consumed by post_general/post_axial
 * (VAPHFB_Par.f90:281-290). Each array is complex [J][K1+JJMAX][K2+JJMAX],
 * J = 0..JJMAX, with only even J filled (Kernel3D.f90:415); entries whose
 * |N^J_{K1K2}| < CHOP = 1e-8 are 0 unless `chop` is 0. */
typedef struct {
    double *njkk, *hjkk, *nn, *zz, *j2;   /* each (JJMAX+1)*NK*NK complex */
} pnamp_kernels;

typedef struct pnamp_ctx pnamp_ctx;

/* Set up a context: uploads the model space, Hamiltonian and mesh, builds the
 * projection weights. Replaces the one-off part of PNAMP_Main.f90:27-50. */
int pnamp_init(const pnamp_space *sp, const pnamp_hamiltonian *h,
               const pnamp_mesh *m, pnamp_ctx **out);

/* Select the arithmetic form of later pnamp_pair/batch calls (PNAMP_FORM_*).
 * No counterpart in the reference, which computes in FP64 only. */
int pnamp_set_form(pnamp_ctx *ctx, int form);

/* Outputs of later pair/batch calls: PNAMP_OUT_ALL (default) computes the 19
 * observables of ZRES; PNAMP_OUT_NORM only the norm kernel N(Omega) (column
 * io = 0; the other columns are written as 0), skipping T22, the densities
 * and the energy. No counterpart in the reference, which always evaluates
 * everything at every point; the learned mode needs the exact norm on the
 * whole fine mesh and the rest only where it computes points exactly. */
#define PNAMP_OUT_ALL 0
#define PNAMP_OUT_NORM 1
int pnamp_set_outputs(pnamp_ctx *ctx, int outputs);

/* Number of Euler points P_E of the context's mesh (rows of ZRES). */
int pnamp_n_euler(const pnamp_ctx *ctx);

/* One (q, q') pair, host buffers: the mesh loop of Kernel4Triaxial
 * (PNAMP_Kernel3D.f90:70-407). U0,V0 (bra q) and U1,V1 (ket q') are the real
 * n x n HFB%U0.. arrays read from the .wf files. zres receives ZRES(P_E, NOBS)
 * (column-major complex, ZRES(iang, io) at [iang + io*P_E]). point_status
 * (length P_E) may be NULL. */
int pnamp_pair(pnamp_ctx *ctx, const double *U0, const double *V0,
               const double *U1, const double *V1, double *zres, int *point_status);

/* A batch of pairs, host buffers. uv is [npairs][4][n*n]: U0, V0, U1, V1 of
 * each pair, column-major; zres is [npairs][NOBS*P_E]; point_status is
 * [npairs][P_E] or NULL. The per-pair MPI round robin of PNAMP_Main.f90:79-84
 * feeds this batched entry. */
int pnamp_batch(pnamp_ctx *ctx, int npairs, const double *uv, double *zres, int *point_status);

/* Same as pnamp_batch with DEVICE buffers, enqueued on `stream` (a
 * cudaStream_t, NULL = legacy default stream); returns after the launch. */
int pnamp_batch_device(pnamp_ctx *ctx, int npairs, const double *d_uv,
                       double *d_zres, int *d_point_status, void *stream);

/* pnamp_batch_device restricted to listed Euler points: d_items holds nitems
 * (pair, Euler point) int pairs (0-based); only those entries of d_zres and
 * d_point_status ([npairs][NOBS][P_E] complex, [npairs][P_E]) are written.
 * d_gauge_out, when not NULL, receives per gauge point (phi_p outer, phi_n
 * inner) [npairs][P_E][NFOM*NFOM][4] doubles: the norm N(Omega, phi) with its
 * gauge phase (complex) and H/N at that point (complex; 0 when only the norm
 * was computed or T22 was singular), so that ZRES(ie, 1) is the mean of the
 * first and ZRES(ie, 7) the mean of their products. Items with a pair index
 * outside [0, npairs) or an Euler index outside [0, P_E) are skipped (nothing
 * written). No reference counterpart (the reference always sweeps the whole
 * mesh). */
int pnamp_batch_items_device(pnamp_ctx *ctx, int npairs, const double *d_uv,
                             long long nitems, const int *d_items, double *d_zres,
                             int *d_point_status, double *d_gauge_out, void *stream);

/* ---- One-body density of the projected ground state (Rho1B) --------------
 * Replaces ZRho1B_Angles / ZRho1B_Integral / Write_ME1B (PNAMP_Rho1B.f90:2-91,
 * called from PNAMP_Kernel3D.f90:367,377,719): the J = 0 projected one-body
 * density <q| rho_{(t lj n1), (t lj n2)} P^{J=0} P^N P^Z |q'> / <q| P |q'>,
 * summed over m and divided by (2j + 1), per block (it, lj, n1, n2): it = 1
 * protons, 0 neutrons; lj = l + j - 1/2; n1, n2 radial quantum numbers from 0.
 *
 * pnamp_rho1b_blocks returns the number of blocks and fills the arrays (each
 * may be NULL) in Write_ME1B's order; a negative value is an error code. */
int pnamp_rho1b_blocks(const pnamp_ctx *ctx, int *it, int *lj, int *n1, int *n2, int *twoj);

/* pnamp_batch_device that also writes, per pair, block and Euler point, the
 * gauge mean of N(Omega, phi) x sum_m rho / sqrt(2j + 1) (ZOBDJ0) into
 * d_rho1b [npairs][nblocks][P_E] complex. PNAMP_ERR_STATE in norm-only mode. */
int pnamp_batch_rho1b_device(pnamp_ctx *ctx, int npairs, const double *d_uv, double *d_zres,
                             int *d_point_status, double *d_rho1b, void *stream);

/* The same with host buffers (uv, zres, point_status as pnamp_batch; rho1b
 * [npairs][nblocks][P_E] complex). */
int pnamp_batch_rho1b(pnamp_ctx *ctx, int npairs, const double *uv, double *zres,
                      int *point_status, double *rho1b);

/* One pair's Write_ME1B values out[nblocks] = Re(sum_e w_e rho1b(e) / sum_e
 * w_e N(e)) / sqrt(2j + 1) from its zres (ZRES(P_E, NOBS) column-major) and
 * rho1b ([nblocks][P_E] complex). PNAMP_ERR_SMALL_NORM when |N^0| <= 1e-8. */
int pnamp_project_rho1b(const pnamp_ctx *ctx, const double *zres, const double *rho1b, double *out);

/* ---- Two-body transition density of the projected ground state (Rho2B) ---
 * Replaces ZRho2B_Angles / ZRho2B_Integral and the valence entries of Write_ME2B
 * (PNAMP_Rho2B.f90:6-296, called from PNAMP_Kernel3D.f90:369,379,722 when
 * Input%idens != 0), over the two-particle blocks of ME2B_Base_Full
 * (PNAMP_ME2B_Base.f90:112-205) built on the model space's orbits:
 *   Rho2BN(bm, a_ij, a_kl) = sum_{m} <j_i m_i j_j m_j|J M> <j_k m_k j_l m_l|J M> / (2J + 1)
 *       x <q| c+_i c+_j c_l c_k P^{J=0} P^N P^Z |q'> / <q| P^{J=0} P^N P^Z |q'>.
 * Orbits are numbered in order of first appearance of (n, l, 2j) in the model
 * space (protons first); tt = 0 nn, 1 np, 2 pp; PP = 0 positive parity.
 *
 * pnamp_rho2b_layout needs no device: sizes[5] = {blocks, states, elements
 * (sum over blocks of states^2), quadruples, terms}. pnamp_rho2b_tables fills
 * (each may be NULL) blocks [nblocks][4] = (tt, PP, J, states), states
 * [nstates][2] = (o1, o2), quads [nquads] = levels k_i | k_j << 8 | k_k << 16 |
 * k_l << 24 (0-based, the tnljm order), elem_ptr [nelements + 1] and, per term,
 * term_q (quadruple) and term_c (cg1 cg2 / (2J + 1)). PNAMP_ERR_UNSUPPORTED when
 * an orbit exists for one species only. */
int pnamp_rho2b_layout(const pnamp_space *sp, int *sizes);
int pnamp_rho2b_tables(const pnamp_space *sp, int *blocks, int *states, unsigned int *quads, int *elem_ptr,
                       int *term_q, double *term_c);

/* pnamp_batch_device that also writes, per pair and quadruple (k_i, k_j, k_k, k_l),
 * sum_e w_e (1/N_FOM^2) sum_phi N(Omega_e, phi) [rho_ki rho_lj - rho_li rho_kj +
 * kappa01_ij kappa10_kl] into d_rho2b [npairs][nquads] complex (overwritten). Each
 * CTA keeps its sums in FP64 in device memory the context owns ([grid][nquads]
 * complex) and adds them into d_rho2b once per Euler point. PNAMP_ERR_STATE in
 * norm-only mode. */
int pnamp_batch_rho2b_device(pnamp_ctx *ctx, int npairs, const double *d_uv, double *d_zres,
                             int *d_point_status, double *d_rho2b, void *stream);

/* The same with host buffers (uv, zres, point_status as pnamp_batch; rho2b
 * [npairs][nquads] complex). */
int pnamp_batch_rho2b(pnamp_ctx *ctx, int npairs, const double *uv, double *zres,
                      int *point_status, double *rho2b);

/* Both densities from one pass over the mesh: pnamp_batch_rho1b_device and
 * pnamp_batch_rho2b_device in one launch (either output may be NULL, not both). */
int pnamp_batch_densities_device(pnamp_ctx *ctx, int npairs, const double *d_uv, double *d_zres,
                                 int *d_point_status, double *d_rho1b, double *d_rho2b, void *stream);

/* The same with host buffers (layouts as pnamp_batch_rho1b and pnamp_batch_rho2b). */
int pnamp_batch_densities(pnamp_ctx *ctx, int npairs, const double *uv, double *zres,
                          int *point_status, double *rho1b, double *rho2b);

/* One pair's Rho2BN per element (bm, a_ij, a_kl) in block order, out[nelements]
 * complex, from its zres (ZRES(P_E, NOBS) column-major) and rho2b ([nquads]
 * complex); Write_ME2B prints the real parts. PNAMP_ERR_SMALL_NORM when
 * |N^0| <= 1e-8. */
int pnamp_project_rho2b(pnamp_ctx *ctx, const double *zres, const double *rho2b, double *out);

/* Same computation as pnamp_batch_device, for callers that must not allocate
 * device memory per call: code running under a runtime that owns the device
 * memory budget (a caching allocator or an MPS client with a hard memory cap),
 * or code that must not risk the implicit device synchronisation of
 * cudaMalloc/cudaFree between stream-ordered steps. It calls no cudaMalloc,
 * cudaFree or allocating library routine: the per-pair records and the per-CTA
 * workspace live in one file-scope device array of PNAMP_NOALLOC_SCRATCH_BYTES
 * (32 MiB), which every GPU that loads the library holds until exit. The context
 * itself is still created once by pnamp_init. A request whose pair records plus
 * one CTA workspace exceed the array is rejected with PNAMP_ERR_SCRATCH_LIMIT;
 * otherwise the grid shrinks to the CTA workspaces that fit. The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) and caches
 * it; make that first call before any stream capture. The cached address
 * assumes the device's context lives for the rest of the process (no
 * cudaDeviceReset after the first call). All calls share the array
 * and it keeps the last call's contents; the kernels write every scratch byte
 * before reading it, so nothing is cleared. Calls whose work overlaps on the GPU
 * (different streams, or different host threads) race on the array: serialise
 * them. This entry point has no counterpart in the reference. */
int pnamp_batch_device_noalloc(pnamp_ctx *ctx, int npairs, const double *d_uv,
                               double *d_zres, int *d_point_status, void *stream);

/* J/K projection of one pair's ZRES into kernel-file fields (Kernel3D.f90:415-751,
 * plain D-function form of PNAMP_Kernel3D_v2.f90:477-498; for an N_alp*N_gam = 1
 * mesh the weight is (2J+1)/2 as in Kernel3D.f90:80). Host buffers. */
int pnamp_project(pnamp_ctx *ctx, const double *zres, int chop, pnamp_kernels *out);

/* Batched projection with DEVICE buffers: d_zres as from pnamp_batch_device,
 * d_out is [npairs][5][(JJMAX+1)*NK*NK] complex (njkk, hjkk, nn, zz, j2). */
int pnamp_project_device(pnamp_ctx *ctx, int npairs, const double *d_zres, int chop,
                         double *d_out, void *stream);

/* Quadrupole reduced elements of one pair's ZRES (PNAMP_Kernel3D_v2.f90:515-600; the
 * Kernel%qpred/qcpred blocks post_general writes, PNAMP_IO.f90:202-217):
 * qpred[J2][dJ][K1+8][K2+6] = <J2+dJ, K1, q1 || Q2 || J2, K2, q2>, dJ = 0 (spectroscopic),
 * 1, 2; qcpred the q1 <-> q2 exchanged element from the Q^dagger traces, computed
 * when `exchange` is non-zero (the reference does so when q1 != q2). Each output
 * holds (JJMAX+1)*3*17*13 complex; only even J2 are filled. Host buffers. */
int pnamp_project_q(pnamp_ctx *ctx, const double *zres, int exchange, double *qpred, double *qcpred);

/* Batched form with DEVICE buffers: d_out is [npairs][2][(JJMAX+1)*3*17*13] complex
 * (qpred, then qcpred). */
int pnamp_project_q_device(pnamp_ctx *ctx, int npairs, const double *d_zres, int exchange,
                           double *d_out, void *stream);

/* Synchronise the context's work; returns the first CUDA error seen. */
int pnamp_sync(pnamp_ctx *ctx);

/* Stage timing (no counterpart in the reference, whose timers are commented out,
 * PNAMP_Kernel3D.f90:189-192,241-242): with `on` set, each later pnamp_batch_device /
 * pnamp_batch_items_device call records CUDA events around its launches on the launching
 * stream (no host synchronisation); pnamp_stage_times waits for those events and writes the
 * milliseconds of the calls since pnamp_set_timing or the previous pnamp_stage_times, summed
 * per stage, to ms[4] = {setup, point kernel, tensor-core contraction, contraction sum into
 * ZRES}, returning 4 (or an error code). */
int pnamp_set_timing(pnamp_ctx *ctx, int on);
int pnamp_stage_times(pnamp_ctx *ctx, double *ms);

/* Free the context and its device memory. */
void pnamp_free(pnamp_ctx *ctx);

/* ---- Uneven batches: several contexts in one persistent launch ----------
 * No reference counterpart: the reference runs one (q, q') pair at a time per
 * MPI rank (Codes/PNAMP/PNAMP_Main.f90:79-115), each pair looping over its own
 * Euler mesh. Here pairs of different model spaces and meshes (all contexts
 * in the same form) are cut into (context, pair, Euler point) items that the
 * CTAs of ONE persistent launch take from a device counter in the order of a
 * schedule. Results land in each context's own d_zres / d_status exactly as
 * pnamp_batch_device would write them.
 *
 * pnamp_multi_create allocates everything (pair records, per-CTA scratch,
 * work list) and copies each context's parameters: the contexts and the
 * device buffers d_uv[c] ([npairs[c]][4][n][n] column-major), d_zres[c] and
 * d_status[c] stay owned by the caller and must outlive the plan, and a later
 * pnamp_set_form on a context does not change a plan made before it. pnamp_multi_launch enqueues only kernels and a memset on `stream`
 * (NULL: legacy default stream), so it may be captured into a CUDA graph and
 * replayed; a plan must not be launched on two streams at once. */
typedef struct pnamp_multi pnamp_multi;

/* nctx = 1..4 (PNAMP_ERR_UNSUPPORTED above: every context's parameters travel
 * by value in the launch). */
int pnamp_multi_create(int nctx, pnamp_ctx *const *ctxs, const int *npairs,
                       const double *const *d_uv, double *const *d_zres,
                       int *const *d_status, pnamp_multi **out);

/* Work order: order 0 = contexts as given, 1 = heaviest per-item cost first
 * (gauge points x n^3), 2 = round robin over contexts item by item; grab =
 * items a CTA takes per counter increment (1..64); grid = CTAs (0: one per
 * resident slot on the device). The default after create is (1, 1, 0). */
int pnamp_multi_schedule(pnamp_multi *plan, int order, int grab, int grid);

/* Shared-memory budget per CTA (bytes; 0 = the device maximum, the default):
 * each context's per-point arrays are re-placed (shared memory vs the CTA's
 * global slot) under the budget and the launch holds the largest result,
 * written to *smem_bytes when that is not NULL. What a CTA does not take as
 * shared memory serves as L1, so a smaller budget can be faster when one
 * context's arrays do not fit anyway. Not while a launch of the plan runs. */
int pnamp_multi_placement(pnamp_multi *plan, int smem_budget, int *smem_bytes);

int pnamp_multi_launch(pnamp_multi *plan, void *stream);

/* Number of (context, pair, Euler point) items; -1 for a NULL plan. */
int pnamp_multi_items(const pnamp_multi *plan);

void pnamp_multi_free(pnamp_multi *plan);

/* Static text for a return code. */
const char *pnamp_strerror(int code);

/* Library version string. */
const char *pnamp_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PNAMP_GPU_H */
