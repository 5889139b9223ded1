// Hand-written kernels of the learned mode around the network: the network's
// inputs for fine-mesh (pair, Euler point, gauge point) rows, and the
// assembly of the predicted energy kernel into ZRES with the per-Euler-point
// error importance that decides which points are computed exactly.
//
// Layouts (row-major, fine mesh): gout [pair][ie][ig][4] = exact N (with the
// gauge phase, complex) then H/N (complex, unused here) as written by the
// point kernel's per-gauge output; h_interp and n_interp [pair][ie][ig][2]
// (complex, interpolated from the coarse mesh); network rows in the same
// (pair, ie, ig) order.
#include <cuda_runtime.h>

#include "../../include/pnamp_mlp.h"

namespace {

__global__ void features_kernel(int npairs, int n_euler, int n_gauge, int nfom, const int *__restrict__ sel,
                                long long nsel, const double *__restrict__ deform, const double *__restrict__ euler,
                                const double *__restrict__ gout, const double *__restrict__ h_interp,
                                const double *__restrict__ n_interp, const double *__restrict__ nscale,
                                const float *__restrict__ mean, const float *__restrict__ inv_std,
                                float *__restrict__ x) {
    // rows: every (pair, ie, ig), or with sel the (sel[2k], sel[2k + 1], ig) of k < nsel
    const long long rows = (sel ? nsel : (long long)npairs * n_euler) * n_gauge;
    const double twopi = 6.283185307179586476925287;
    for (long long row = blockIdx.x * (long long)blockDim.x + threadIdx.x; row < rows;
         row += (long long)gridDim.x * blockDim.x) {
        const int ig = (int)(row % n_gauge);
        long long pe = row / n_gauge;
        if (sel) {
            const int sp = sel[2 * pe], se = sel[2 * pe + 1];
            if (sp < 0 || sp >= npairs || se < 0 || se >= n_euler) {  // out of range: a zero row
                for (int k = 0; k < PNAMP_LEARNED_FEATURES; ++k) x[row * PNAMP_LEARNED_FEATURES + k] = 0.f;
                continue;
            }
            pe = (long long)sp * n_euler + se;
        }
        const int ie = (int)(pe % n_euler), pr = (int)(pe / n_euler);
        const long long r = pe * n_gauge + ig;   // index into the full arrays
        const double *dfm = deform + 4 * pr;
        const double al = euler[4 * ie], be = euler[4 * ie + 1], ga = euler[4 * ie + 2];
        const double php = twopi * (ig / nfom) / nfom, phn = twopi * (ig % nfom) / nfom;
        const double ns = nscale[pr] > 0.0 ? 1.0 / nscale[pr] : 0.0;
        const double nr = gout[4 * r] * ns, ni = gout[4 * r + 1] * ns;
        const double mag = sqrt(nr * nr + ni * ni);
        float f[PNAMP_LEARNED_FEATURES];
        f[0] = (float)dfm[0];
        f[1] = (float)(dfm[1] / 60.0);
        f[2] = (float)dfm[2];
        f[3] = (float)(dfm[3] / 60.0);
        f[4] = (float)cos(al);
        f[5] = (float)sin(al);
        f[6] = (float)cos(be);
        f[7] = (float)sin(be);
        f[8] = (float)cos(ga);
        f[9] = (float)sin(ga);
        f[10] = (float)cos(2.0 * al);
        f[11] = (float)sin(2.0 * al);
        f[12] = (float)cos(2.0 * ga);
        f[13] = (float)sin(2.0 * ga);
        f[14] = (float)cos(phn);
        f[15] = (float)sin(phn);
        f[16] = (float)cos(php);
        f[17] = (float)sin(php);
        f[18] = (float)h_interp[2 * r];
        f[19] = (float)h_interp[2 * r + 1];
        f[20] = (float)nr;
        f[21] = (float)ni;
        f[22] = (float)(log10(mag + 1e-12) / 12.0);
        f[23] = (float)(nr - n_interp[2 * r] * ns);
        f[24] = (float)(ni - n_interp[2 * r + 1] * ns);
        float *xr = x + row * PNAMP_LEARNED_FEATURES;
#pragma unroll
        for (int k = 0; k < PNAMP_LEARNED_FEATURES; ++k) xr[k] = (f[k] - mean[k]) * inv_std[k];
    }
}

// One block (128 threads) per (pair, Euler point): h = h_interp + scale mu over the
// gauge points, ZRES_H(ie) = mean_g N h (column 6), importance = w_e / (8 pi^2) /
// P_G * sqrt(sum_g |N|^2 (scale e^s)^2), and h_pred per gauge point.
__global__ void assemble_kernel(int npairs, int n_euler, int n_gauge, const double *__restrict__ gout,
                                const double *__restrict__ h_interp, const float *__restrict__ out, double scale,
                                const double *__restrict__ wts, double *__restrict__ zres,
                                double *__restrict__ importance, double *__restrict__ h_pred) {
    __shared__ double red[3][128];
    const long long pe = blockIdx.x;
    const int ie = (int)(pe % n_euler), pr = (int)(pe / n_euler);
    double hr = 0.0, hi = 0.0, v = 0.0;
    for (int ig = threadIdx.x; ig < n_gauge; ig += blockDim.x) {
        const long long r = pe * n_gauge + ig;
        const double nr = gout[4 * r], ni = gout[4 * r + 1];
        const double pr_ = h_interp[2 * r] + scale * (double)out[3 * r];
        const double pi_ = h_interp[2 * r + 1] + scale * (double)out[3 * r + 1];
        const double s = fmin(fmax((double)out[3 * r + 2], -12.0), 6.0);
        const double sig = scale * exp(s);
        h_pred[2 * r] = pr_;
        h_pred[2 * r + 1] = pi_;
        hr += nr * pr_ - ni * pi_;
        hi += nr * pi_ + ni * pr_;
        v += (nr * nr + ni * ni) * sig * sig;
    }
    red[0][threadIdx.x] = hr;
    red[1][threadIdx.x] = hi;
    red[2][threadIdx.x] = v;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k)
            for (int q = 0; q < 3; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double inv = 1.0 / n_gauge;
        double *z = zres + 2LL * (long long)pr * PNAMP_LEARNED_NOBS * n_euler;
        z[2LL * (6 * n_euler + ie)] = red[0][0] * inv;
        z[2LL * (6 * n_euler + ie) + 1] = red[1][0] * inv;
        const double eight_pi2 = 78.95683520871486;
        importance[pe] = wts[ie] / eight_pi2 * inv * sqrt(red[2][0]);
    }
}

// Coarse -> fine interpolation of the per-gauge coarse kernels, separable in the
// three Euler angles: one block per (fine beta node, pair). The block first folds the
// beta weights into T[ca][cg][g][4] (shared), then each output (fine alpha, fine gamma,
// gauge point) takes sum_ca wa sum_cg wg T, gauge points innermost so the writes
// are contiguous. Per output 4 x (cb + ca cg) multiply-adds instead of the cb ca cg of
// the dense [P_fine x P_coarse] matrix product.
__global__ void interp_kernel(int cb, int ca, int cg, int fb, int fa, int fg, int n_gauge,
                              const double *__restrict__ wb, const double *__restrict__ wa,
                              const double *__restrict__ wg, const double *__restrict__ gc,
                              double *__restrict__ h_interp, double *__restrict__ n_interp) {
    extern __shared__ double tsh[];          // [ca][cg][n_gauge][4]
    const int ib = blockIdx.x, pr = blockIdx.y;
    const long long pc = (long long)cb * ca * cg, pf = (long long)fb * fa * fg;
    const double *src = gc + (long long)pr * pc * n_gauge * 4;
    const int nt = ca * cg * n_gauge * 4;
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
        const int q = t & 3, g = (t >> 2) % n_gauge, ac = (t >> 2) / n_gauge;   // ac = ka cg + kg
        double v = 0.0;
        for (int kb = 0; kb < cb; ++kb)
            v = fma(wb[ib * cb + kb], src[(((long long)kb * ca * cg + ac) * n_gauge + g) * 4 + q], v);
        tsh[t] = v;
    }
    __syncthreads();
    const int no = fa * fg * n_gauge;
    double *ho = h_interp + ((long long)pr * pf + (long long)ib * fa * fg) * n_gauge * 2;
    double *nout = n_interp + ((long long)pr * pf + (long long)ib * fa * fg) * n_gauge * 2;
    for (int t = threadIdx.x; t < no; t += blockDim.x) {
        const int g = t % n_gauge, ag = t / n_gauge, ja = ag / fg, jg = ag % fg;
        double v0 = 0.0, v1 = 0.0, v2 = 0.0, v3 = 0.0;
        for (int ka = 0; ka < ca; ++ka) {
            double u0 = 0.0, u1 = 0.0, u2 = 0.0, u3 = 0.0;
            for (int kg = 0; kg < cg; ++kg) {
                const double w = wg[jg * cg + kg];
                const double *tv = tsh + (((ka * cg + kg) * n_gauge + g) << 2);
                u0 = fma(w, tv[0], u0);
                u1 = fma(w, tv[1], u1);
                u2 = fma(w, tv[2], u2);
                u3 = fma(w, tv[3], u3);
            }
            const double w = wa[ja * ca + ka];
            v0 = fma(w, u0, v0);
            v1 = fma(w, u1, v1);
            v2 = fma(w, u2, v2);
            v3 = fma(w, u3, v3);
        }
        nout[2LL * t] = v0;
        nout[2LL * t + 1] = v1;
        ho[2LL * t] = v2;
        ho[2LL * t + 1] = v3;
    }
}

}  // namespace

extern "C" {

int pnamp_learned_features(int npairs, int n_euler, int nfom, const int *sel, long long nsel, const double *deform,
                           const double *euler, const double *gout, const double *h_interp, const double *n_interp,
                           const double *nscale, const float *mean, const float *inv_std, float *x, void *stream) {
    if (npairs < 0 || n_euler < 1 || nfom < 1 || nsel < 0 || !deform || !euler || !gout || !h_interp || !n_interp ||
        !nscale || !mean || !inv_std || !x)
        return 1;
    const long long rows = (sel ? nsel : (long long)npairs * n_euler) * nfom * nfom;
    if (rows == 0) return 0;
    const int grid = (int)((rows + 255) / 256 < 8192 ? (rows + 255) / 256 : 8192);
    features_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(npairs, n_euler, nfom * nfom, nfom, sel, nsel, deform,
                                                            euler, gout, h_interp, n_interp, nscale, mean, inv_std, x);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int pnamp_learned_assemble(int npairs, int n_euler, int n_gauge, const double *gout, const double *h_interp,
                           const float *out, double scale, const double *wts, double *zres, double *importance,
                           double *h_pred, void *stream) {
    if (npairs < 0 || n_euler < 1 || n_gauge < 1 || !gout || !h_interp || !out || !wts || !zres || !importance ||
        !h_pred)
        return 1;
    if (npairs == 0) return 0;
    assemble_kernel<<<npairs * n_euler, 128, 0, (cudaStream_t)stream>>>(npairs, n_euler, n_gauge, gout, h_interp, out,
                                                                       scale, wts, zres, importance, h_pred);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int pnamp_learned_interp(int npairs, int cb, int ca, int cg, int fb, int fa, int fg, int n_gauge, const double *wb,
                         const double *wa, const double *wg, const double *gc, double *h_interp, double *n_interp,
                         void *stream) {
    if (npairs < 0 || cb < 1 || ca < 1 || cg < 1 || fb < 1 || fa < 1 || fg < 1 || n_gauge < 1 || !wb || !wa ||
        !wg || !gc || !h_interp || !n_interp || fb > 65535 || npairs > 65535)
        return 1;
    const long long smem = (long long)ca * cg * n_gauge * 4 * sizeof(double);
    if (smem > 227 * 1024) return 1;
    if (npairs == 0) return 0;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(interp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return 2;
    interp_kernel<<<dim3(fb, npairs), 256, (size_t)smem, (cudaStream_t)stream>>>(cb, ca, cg, fb, fa, fg, n_gauge, wb,
                                                                                 wa, wg, gc, h_interp, n_interp);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // extern "C"
