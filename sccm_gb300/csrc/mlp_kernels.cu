// Hand-written FP32 kernels of the learned mode's network: dense layers
// (forward with fused bias + tanh, backward with deterministic split-K weight
// gradients), the heteroscedastic Gaussian loss and the Adam update.
//
// The network predicts the normalised energy kernel H/N at fine-mesh points
// from cheap inputs; it has no counterpart in the reference, which evaluates
// every mesh point exactly. All layers are small (width 256) and the batch is
// large (10^4 - 10^6 rows), so a 64 x 64 register-tiled SIMT GEMM on the FP32
// pipes is used for every product; the weight gradient (K = rows) is split
// over row chunks into a workspace and summed in chunk order, so results do
// not depend on scheduling.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pnamp_mlp.h"

namespace {

constexpr int BM = 64, BN = 64, BK = 16, TH = 256;  // tile, 16 x 16 threads x (4 x 4) outputs

// C[m][n] = sum_k A(m, k) B(k, n) over k in [k0, k1) of this split
//   A(m, k) = TA ? A[k * lda + m] : A[m * lda + k]
//   B(k, n) = TB ? B[n * ldb + k] : B[k * ldb + n]
// Epilogue: + bias[n] (if bias), tanh (if act == 1). Split z writes C + z * c_split_stride.
template <bool TA, bool TB>
__global__ void __launch_bounds__(TH) gemm_kernel(const float *__restrict__ A, int lda, const float *__restrict__ B,
                                                  int ldb, float *__restrict__ C, int ldc, int M, int N, int K,
                                                  int kchunk, long long c_split_stride, const float *__restrict__ bias,
                                                  int act) {
    __shared__ float As[BK][BM + 4];
    __shared__ float Bs[BK][BN + 4];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int k0 = blockIdx.z * kchunk, k1 = min(K, k0 + kchunk);
    float acc[4][4] = {};
    for (int kt = k0; kt < k1; kt += BK) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {  // A tile: BM x BK, 4 values per thread
            const int e = threadIdx.x + r * TH;
            int mm, kk;
            if (TA) {  // contiguous along m
                kk = e / BM;
                mm = e % BM;
            } else {   // contiguous along k
                mm = e / BK;
                kk = e % BK;
            }
            const int gm = m0 + mm, gk = kt + kk;
            float v = 0.f;
            if (gm < M && gk < k1) v = TA ? A[(long long)gk * lda + gm] : A[(long long)gm * lda + gk];
            As[kk][mm] = v;
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {  // B tile: BK x BN
            const int e = threadIdx.x + r * TH;
            int nn, kk;
            if (TB) {  // contiguous along k
                nn = e / BK;
                kk = e % BK;
            } else {   // contiguous along n
                kk = e / BN;
                nn = e % BN;
            }
            const int gn = n0 + nn, gk = kt + kk;
            float v = 0.f;
            if (gn < N && gk < k1) v = TB ? B[(long long)gn * ldb + gk] : B[(long long)gk * ldb + gn];
            Bs[kk][nn] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
    float *Cs = C + blockIdx.z * c_split_stride;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int gm = m0 + ty + 16 * i;
        if (gm >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int gn = n0 + tx + 16 * j;
            if (gn >= N) continue;
            float v = acc[i][j];
            if (bias) v += bias[gn];
            if (act == 1) v = tanhf(v);
            Cs[(long long)gm * ldc + gn] = v;
        }
    }
}

// out[i] = sum_s part[s * n + i], s in order
__global__ void sum_splits(const float *__restrict__ part, int splits, long long n, float *__restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int k = 0; k < splits; ++k) s += part[k * n + i];
        out[i] = s;
    }
}

// dZ = dY * (1 - Y^2) (tanh) in place
__global__ void tanh_grad(float *__restrict__ dy, const float *__restrict__ y, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dy[i] *= 1.f - y[i] * y[i];
}

// partial column sums of dZ [rows][out] over row chunks: part[s][o]
__global__ void colsum_partial(const float *__restrict__ dz, int rows, int out, int chunk, float *__restrict__ part) {
    const int s = blockIdx.x;
    const int r0 = s * chunk, r1 = min(rows, r0 + chunk);
    for (int o = threadIdx.x; o < out; o += blockDim.x) {
        float acc = 0.f;
        for (int r = r0; r < r1; ++r) acc += dz[(long long)r * out + o];
        part[(long long)s * out + o] = acc;
    }
}

// mode 0: loss_r = w_r [ |y - mu|^2 e^{-2s} / 2 + 2 s ],  s = clamp(out[2], -12, 6)
//         dout = w_r / rows * [ -(y - mu) e^{-2s},  -|y - mu|^2 e^{-2s} + 2 ]
// mode 1: the same with s = 0 and no gradient to s (weighted least squares on mu)
// mode 2: the same with no gradient to mu (fits s to the current errors)
__global__ void gauss_loss(const float *__restrict__ out, const float *__restrict__ y, const float *__restrict__ w,
                           int rows, int mode, float *__restrict__ dout, float *__restrict__ loss_part) {
    __shared__ float red[256];
    float acc = 0.f;
    const float inv_rows = 1.f / (float)rows;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
        const float mr = out[3 * r], mi = out[3 * r + 1], s_raw = out[3 * r + 2];
        const float s = mode == 1 ? 0.f : fminf(fmaxf(s_raw, -12.f), 6.f);
        const float er = y[2 * r] - mr, ei = y[2 * r + 1] - mi;
        const float iv = expf(-2.f * s);
        const float e2 = er * er + ei * ei;
        const float wr = w ? w[r] : 1.f;
        acc += wr * (0.5f * e2 * iv + 2.f * s);
        const float g = wr * inv_rows;
        dout[3 * r] = mode == 2 ? 0.f : -g * er * iv;
        dout[3 * r + 1] = mode == 2 ? 0.f : -g * ei * iv;
        dout[3 * r + 2] = (mode != 1 && s_raw > -12.f && s_raw < 6.f) ? g * (2.f - e2 * iv) : 0.f;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss_part[blockIdx.x] = red[0] * inv_rows;
}

__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, long long n, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

int grid_1d(long long n) { return (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096); }

constexpr int kSplitRows = 512;  // rows per weight-gradient chunk
constexpr int kMaxSplits = 128;

}  // namespace

extern "C" {

long long pnamp_mlp_work_floats(int rows, int in, int out) {
    const int splits = rows <= 0 ? 1 : (rows + kSplitRows - 1) / kSplitRows;
    const int s = splits < kMaxSplits ? splits : kMaxSplits;
    return (long long)s * in * out + (long long)s * out;
}

int pnamp_mlp_linear_forward(const float *X, const float *W, const float *b, float *Y, int rows, int in, int out,
                             int act, void *stream) {
    if (!X || !W || !Y || rows < 0 || in < 1 || out < 1 || (act != 0 && act != 1)) return 1;
    if (rows == 0) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    dim3 grid((out + BN - 1) / BN, (rows + BM - 1) / BM, 1);
    gemm_kernel<false, true><<<grid, TH, 0, st>>>(X, in, W, in, Y, out, rows, out, in, in, 0, b, act);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int pnamp_mlp_linear_backward(const float *X, const float *W, const float *Y, float *dY, float *dW, float *db,
                              float *dX, int rows, int in, int out, int act, float *work, void *stream) {
    if (!X || !W || !dY || !dW || !db || !work || rows < 1 || in < 1 || out < 1 || (act != 0 && act != 1) ||
        (act == 1 && !Y))
        return 1;
    cudaStream_t st = (cudaStream_t)stream;
    const long long nzy = (long long)rows * out;
    if (act == 1) tanh_grad<<<grid_1d(nzy), 256, 0, st>>>(dY, Y, nzy);
    // split-K over row chunks: chunk a multiple of BK, at most kMaxSplits chunks
    int splits = (rows + kSplitRows - 1) / kSplitRows;
    if (splits > kMaxSplits) splits = kMaxSplits;
    int chunk = (rows + splits - 1) / splits;
    chunk = (chunk + BK - 1) / BK * BK;
    splits = (rows + chunk - 1) / chunk;
    float *partW = work, *partB = work + (long long)splits * in * out;
    // dW[o][i] = sum_r dZ[r][o] X[r][i]: A = dZ^T (TA, lda = out), B = X (ldb = in)
    dim3 gw((in + BN - 1) / BN, (out + BM - 1) / BM, splits);
    gemm_kernel<true, false><<<gw, TH, 0, st>>>(dY, out, X, in, partW, in, out, in, rows, chunk,
                                                (long long)out * in, nullptr, 0);
    sum_splits<<<grid_1d((long long)out * in), 256, 0, st>>>(partW, splits, (long long)out * in, dW);
    colsum_partial<<<splits, 256, 0, st>>>(dY, rows, out, chunk, partB);
    sum_splits<<<grid_1d(out), 256, 0, st>>>(partB, splits, out, db);
    if (dX) {  // dX[r][i] = sum_o dZ[r][o] W[o][i]
        dim3 gx((in + BN - 1) / BN, (rows + BM - 1) / BM, 1);
        gemm_kernel<false, false><<<gx, TH, 0, st>>>(dY, out, W, in, dX, in, rows, in, out, out, 0, nullptr, 0);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int pnamp_mlp_loss_blocks(int rows) { return rows < 1 ? 1 : (grid_1d(rows) < 1024 ? grid_1d(rows) : 1024); }

int pnamp_mlp_gauss_loss(const float *out, const float *y, const float *w, int rows, int mode, float *dout,
                         float *loss_part, void *stream) {
    if (!out || !y || !dout || !loss_part || rows < 1 || mode < 0 || mode > 2) return 1;
    gauss_loss<<<pnamp_mlp_loss_blocks(rows), 256, 0, (cudaStream_t)stream>>>(out, y, w, rows, mode, dout,
                                                                             loss_part);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int pnamp_mlp_adam(float *p, const float *g, float *m, float *v, long long n, float lr, float beta1, float beta2,
                   float eps, int step, void *stream) {
    if (!p || !g || !m || !v || n < 0 || step < 1) return 1;
    if (n == 0) return 0;
    const float c1 = 1.f / (1.f - powf(beta1, (float)step)), c2 = 1.f / (1.f - powf(beta2, (float)step));
    adam_kernel<<<grid_1d(n), 256, 0, (cudaStream_t)stream>>>(p, g, m, v, n, lr, beta1, beta2, eps, c1, c2);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // extern "C"
