/*
 * pnamp_mlp.h -- FP32 kernels of the learned mode (GB300, sm_103a).
 *
 * No reference counterpart: the reference evaluates every Euler x gauge point
 * of the PNAMP mesh exactly (Codes/PNAMP/PNAMP_Kernel3D.f90:178-260). The
 * learned mode predicts the normalised energy kernel H/N on a fine mesh with a
 * small MLP and computes exactly only the points it flags; these entry points
 * are its hand-written training and inference kernels. All pointers are
 * DEVICE pointers, matrices row-major, `stream` a cudaStream_t (NULL = legacy
 * default stream). Return codes: 0 ok, 1 invalid argument, 2 CUDA error.
 */
#ifndef PNAMP_MLP_H
#define PNAMP_MLP_H

#ifdef __cplusplus
extern "C" {
#endif

/* Y[r][o] = act(sum_i X[r][i] W[o][i] + b[o]), X [rows][in], W [out][in],
 * b [out] (NULL: no bias); act 0 = identity, 1 = tanh. */
int pnamp_mlp_linear_forward(const float *X, const float *W, const float *b, float *Y,
                             int rows, int in, int out, int act, void *stream);

/* Floats of workspace pnamp_mlp_linear_backward needs for these sizes. */
long long pnamp_mlp_work_floats(int rows, int in, int out);

/* Backward of that layer. dY [rows][out] (gradient of the loss w.r.t. Y) is
 * overwritten with dZ = dY (act 0) or dY (1 - Y^2) (act 1, Y = the layer's
 * output); then dW = dZ^T X [out][in], db = column sums of dZ [out] and, if
 * dX is not NULL, dX = dZ W [rows][in]. The weight and bias gradients are
 * summed over row chunks in chunk order (deterministic). */
int pnamp_mlp_linear_backward(const float *X, const float *W, const float *Y, float *dY,
                              float *dW, float *db, float *dX, int rows, int in, int out,
                              int act, float *work, void *stream);

/* Blocks of pnamp_mlp_gauss_loss = length of its loss_part output. */
int pnamp_mlp_loss_blocks(int rows);

/* Heteroscedastic Gaussian loss of outputs out [rows][3] = (mu_re, mu_im,
 * s = log sigma, clamped to [-12, 6]) against targets y [rows][2] with row
 * weights w [rows] (NULL: 1):  mean_r w_r [|y - mu|^2 e^{-2s}/2 + 2s].
 * mode 0: gradients to mu and s; 1: s taken as 0 and left alone (weighted
 * least squares on mu); 2: gradient to s only (the uncertainty fitted to the
 * current errors). Writes dout [rows][3] = d loss / d out and per-block
 * partial losses (sum them for the loss). */
int pnamp_mlp_gauss_loss(const float *out, const float *y, const float *w, int rows, int mode,
                         float *dout, float *loss_part, void *stream);

/* Adam step (bias-corrected, step >= 1) on n parameters. */
int pnamp_mlp_adam(float *p, const float *g, float *m, float *v, long long n, float lr,
                   float beta1, float beta2, float eps, int step, void *stream);

/* ---- learned mode around the network ------------------------------------
 * Fine-mesh arrays are indexed (pair, Euler point ie, gauge point ig), gauge
 * points phi_p outer and phi_n inner (ig = lp * NFOM + ln, phi = 2 pi l / NFOM),
 * Euler points in the reference's order (beta outer, alpha, gamma inner). */
#define PNAMP_LEARNED_FEATURES 25
#define PNAMP_LEARNED_NOBS 19

/* Network inputs x [rows][25] (standardised: (f - mean) * inv_std) from
 * deform [npairs][4] (beta2 and gamma in degrees of q, then q'), euler
 * [n_euler][4] (alpha, beta, gamma, weight), the exact per-gauge norms
 * gout [pairs][ie][ig][4] (as pnamp_batch_items_device writes them),
 * h_interp and n_interp [pairs][ie][ig][2] (coarse-mesh H/N and N
 * interpolated to the fine mesh) and nscale [npairs] (the pair's norm scale).
 * Inputs: beta2, gamma/60 of q and q'; cos, sin of alpha, beta, gamma, 2 alpha,
 * 2 gamma, phi_n, phi_p; interpolated H/N; N / nscale; log10|N / nscale| / 12;
 * (N - interpolated N) / nscale. sel == NULL: rows for every (pair, ie, ig);
 * else rows only for the nsel (pair, ie) int pairs in sel, all gauge points,
 * in sel's order (the other arrays keep their full layout; an out-of-range
 * entry gives zero rows). */
int pnamp_learned_features(int npairs, int n_euler, int nfom, const int *sel, long long nsel,
                           const double *deform, const double *euler, const double *gout,
                           const double *h_interp, const double *n_interp, const double *nscale,
                           const float *mean, const float *inv_std, float *x, void *stream);

/* From the network outputs out [rows][3] (mu re, mu im, s): the predicted
 * H/N = h_interp + scale * mu into h_pred [rows][2]; ZRES column 6 (H, gauge
 * mean of N H/N, complex) of every (pair, ie) into zres [npairs][19][n_euler];
 * and importance [npairs][n_euler] = wts[ie] / (8 pi^2) / P_G *
 * sqrt(sum_g |N|^2 (scale e^s)^2), the predicted error of that Euler point's
 * contribution to the J = 0 energy kernel. */
int pnamp_learned_assemble(int npairs, int n_euler, int n_gauge, const double *gout,
                           const double *h_interp, const float *out, double scale,
                           const double *wts, double *zres, double *importance,
                           double *h_pred, void *stream);

/* Coarse -> fine interpolation of per-gauge kernels, separable in the Euler angles.
 * gc [npairs][cb][ca][cg][n_gauge][4] holds the coarse mesh's per-gauge output
 * (N re, im, H/N re, im; Euler points beta outer, alpha, gamma inner, as
 * pnamp_batch_items_device writes them); wb [fb][cb], wa [fa][ca], wg [fg][cg]
 * are the 1-D interpolation weights (fine node x coarse node). Writes
 * n_interp and h_interp [npairs][fb][fa][fg][n_gauge][2]:
 * value(fb, fa, fg) = sum wb(fb, kb) wa(fa, ka) wg(fg, kg) value(kb, ka, kg).
 * Needs ca cg n_gauge 32 bytes of shared memory (at most 227 KB). */
int pnamp_learned_interp(int npairs, int cb, int ca, int cg, int fb, int fa, int fg, int n_gauge,
                         const double *wb, const double *wa, const double *wg, const double *gc,
                         double *h_interp, double *n_interp, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* PNAMP_MLP_H */
