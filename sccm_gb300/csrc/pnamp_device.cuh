// Device-side helpers for the PNAMP kernels: complex FP64 arithmetic, block
// reductions, the Wigner small-d function and the strict-upper-triangle index
// map used to spread triangular updates evenly over a CTA.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace pnamp {

struct zc {
    double x, y;
};

__host__ __device__ __forceinline__ zc mk(double a, double b) {
    zc r;
    r.x = a;
    r.y = b;
    return r;
}
__device__ __forceinline__ zc operator+(zc a, zc b) { return mk(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ zc operator-(zc a, zc b) { return mk(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ zc operator-(zc a) { return mk(-a.x, -a.y); }
__device__ __forceinline__ zc operator*(zc a, zc b) {
    return mk(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ zc operator*(double s, zc a) { return mk(s * a.x, s * a.y); }
__device__ __forceinline__ zc zconj(zc a) { return mk(a.x, -a.y); }
__device__ __forceinline__ double abs2(zc a) { return fma(a.x, a.x, a.y * a.y); }
// c + a*b
__device__ __forceinline__ zc zfma(zc a, zc b, zc c) {
    return mk(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
// c - a*b
__device__ __forceinline__ zc zfms(zc a, zc b, zc c) {
    return mk(fma(-a.x, b.x, fma(a.y, b.y, c.x)), fma(-a.x, b.y, fma(-a.y, b.x, c.y)));
}
// c + r*a, r real
__device__ __forceinline__ zc rfma(double r, zc a, zc c) { return mk(fma(r, a.x, c.x), fma(r, a.y, c.y)); }
__device__ __forceinline__ zc zrecip(zc b) {
    double d = 1.0 / abs2(b);
    return mk(b.x * d, -b.y * d);
}
__device__ __forceinline__ zc expi(double phi) {
    double s, c;
    sincos(phi, &s, &c);
    return mk(c, s);
}
__device__ __forceinline__ bool zfinite(zc a) { return isfinite(a.x) && isfinite(a.y); }

// ---------------------------------------------------------------------------
// Strict upper triangle of an m x m matrix, enumerated row by row:
// t = 0 -> (0,1), (0,2), ..., (0,m-1), (1,2), ...  Inverts the triangular
// numbers counted from the last element; FP32 sqrt is exact enough to land
// within one of the answer and the two integer loops fix it.
__device__ __forceinline__ void tri_index(int t, int m, int &i, int &j) {
    const int T = m * (m - 1) / 2;
    const int u = T - 1 - t;
    int k = (int)((sqrtf((float)(8 * u + 1)) - 1.0f) * 0.5f);
    while ((k + 1) * (k + 2) / 2 <= u) ++k;
    while (k * (k + 1) / 2 > u) --k;
    i = m - 2 - k;
    j = m - 1 - (u - k * (k + 1) / 2);
}

// ---------------------------------------------------------------------------
// Block-wide reductions. `buf` must hold at least 2 * (blockDim.x / 32) doubles
// (argmax) or nval * (blockDim.x / 32) doubles (sums).

// max of v; ties broken towards the smallest idx. Result broadcast to all threads.
__device__ __forceinline__ void block_argmax(double &v, int &idx, double *buf) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        double ov = __shfl_down_sync(0xffffffffu, v, o);
        int oi = __shfl_down_sync(0xffffffffu, idx, o);
        if (ov > v || (ov == v && oi < idx)) {
            v = ov;
            idx = oi;
        }
    }
    int *ibuf = reinterpret_cast<int *>(buf + nw);
    if (lane == 0) {
        buf[wid] = v;
        ibuf[wid] = idx;
    }
    __syncthreads();
    if (wid == 0) {
        v = lane < nw ? buf[lane] : -2.0;
        idx = lane < nw ? ibuf[lane] : 0x7fffffff;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double ov = __shfl_down_sync(0xffffffffu, v, o);
            int oi = __shfl_down_sync(0xffffffffu, idx, o);
            if (ov > v || (ov == v && oi < idx)) {
                v = ov;
                idx = oi;
            }
        }
        if (lane == 0) {
            buf[0] = v;
            ibuf[0] = idx;
        }
    }
    __syncthreads();
    v = buf[0];
    idx = ibuf[0];
    __syncthreads();
}

// Max of a 64-bit key; ties broken towards the smallest idx. Broadcast to all.
__device__ __forceinline__ void block_argmax_u64(unsigned long long &v, int &idx, double *buf) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    auto better = [](unsigned long long ov, int oi, unsigned long long v0, int i0) {
        return oi != 0x7fffffff && (i0 == 0x7fffffff || ov > v0 || (ov == v0 && oi < i0));
    };
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ov = __shfl_down_sync(0xffffffffu, v, o);
        const int oi = __shfl_down_sync(0xffffffffu, idx, o);
        if (better(ov, oi, v, idx)) {
            v = ov;
            idx = oi;
        }
    }
    unsigned long long *kbuf = reinterpret_cast<unsigned long long *>(buf);
    int *ibuf = reinterpret_cast<int *>(buf + nw);
    if (lane == 0) {
        kbuf[wid] = v;
        ibuf[wid] = idx;
    }
    __syncthreads();
    if (wid == 0) {
        v = lane < nw ? kbuf[lane] : 0ull;
        idx = lane < nw ? ibuf[lane] : 0x7fffffff;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long ov = __shfl_down_sync(0xffffffffu, v, o);
            const int oi = __shfl_down_sync(0xffffffffu, idx, o);
            if (better(ov, oi, v, idx)) {
                v = ov;
                idx = oi;
            }
        }
        if (lane == 0) {
            kbuf[0] = v;
            ibuf[0] = idx;
        }
    }
    __syncthreads();
    v = kbuf[0];
    idx = ibuf[0];
    __syncthreads();
}

// Sum NV doubles across the block; result valid in all threads.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *buf) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double a = v[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        v[q] = a;
    }
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) buf[q * nw + wid] = v[q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double a = 0.0;
        for (int w = 0; w < nw; ++w) a += buf[q * nw + w];
        v[q] = a;
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Wigner small-d in Edmonds' convention, d^j_{m1 m2}(beta) =
// <j m1| exp(-i beta J_y) |j m2>, arguments doubled, from Wigner's explicit
// sum; c = cos(beta/2), s = sin(beta/2). `fact` holds k! for k = 0..23.
__device__ __forceinline__ double wigner_d(int tj, int tm1, int tm2, double c, double s,
                                           const double *fact) {
    if (tm1 > tj || -tm1 > tj || tm2 > tj || -tm2 > tj) return 0.0;
    const int jpm1 = (tj + tm1) / 2, jmm1 = (tj - tm1) / 2;
    const int jpm2 = (tj + tm2) / 2, jmm2 = (tj - tm2) / 2;
    const double pre = sqrt(fact[jpm1] * fact[jmm1] * fact[jpm2] * fact[jmm2]);
    const int dm = (tm1 - tm2) / 2;
    double d = 0.0;
    for (int k = 0; k <= tj; ++k) {
        const int a = jpm2 - k, e = jmm1 - k, f = k + dm;
        if (a < 0 || e < 0 || f < 0) continue;
        const int ec = tj - 2 * k - dm, es = 2 * k + dm;
        double t = 1.0 / (fact[a] * fact[k] * fact[e] * fact[f]);
        if (f & 1) t = -t;
        double pc = 1.0, ps = 1.0;
        for (int q = 0; q < ec; ++q) pc *= c;
        for (int q = 0; q < es; ++q) ps *= s;
        d = fma(t * pc, ps, d);
    }
    return pre * d;
}

}  // namespace pnamp
