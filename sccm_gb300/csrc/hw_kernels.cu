// Batched Hill-Wheeler solves (HNDIAG, Codes/GCM/GCM_HNDiag.f90:2-103) on the GPU: one
// CTA per problem. Both Hermitian eigenproblems (the norm matrix, then N^-1/2 H N^-1/2 in
// the kept natural states) are solved by cyclic complex Jacobi rotations in FP64: each
// round applies M/2 disjoint rotations at once (round-robin pairing of the M indices, M
// = m rounded up to even, an odd m's extra index idle), a column pass over A and V and
// a row pass over A, three CTA barriers per round, M - 1 rounds per sweep, until the
// off-diagonal norm is below 1e-15 of the matrix norm (or, below 1e-12 of it, stops
// falling: the rounding floor of a large matrix). The problems of a GCM basis are
// small (m = vacua x (2J + 1) <= a few hundred) and few; the work lives in L2.
#include <cuda_runtime.h>

#include "../../include/pnamp_gcm.h"
#include "pnamp_device.cuh"

namespace {
using pnamp::abs2;
using pnamp::mk;
using pnamp::zc;
using pnamp::zconj;
using pnamp::zfma;

constexpr int kThreads = 512;
constexpr int kMaxSweeps = 40;

struct Prob {
    int m;
    long long off;    // complex elements into H, N, F; doubles into E
    long long woff;   // bytes into the work space
};

__device__ __forceinline__ zc cmul(zc a, zc b) { return a * b; }

// Block sum of one double; every thread gets the result. red: >= kThreads / 32 doubles.
__device__ double block_sum(double v, double *red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < nw; ++w) t += red[w];
    return t;
}

// Round r of the round-robin schedule over M (even) indices: pair i = (p, q).
__device__ __forceinline__ void rr_pair(int M, int r, int i, int &p, int &q) {
    p = (i == 0) ? 0 : 1 + (r + i - 1) % (M - 1);
    q = 1 + (r + M - 2 - i) % (M - 1);
}

// Jacobi eigen-decomposition of the Hermitian m x m matrix A (row-major, ld) in place:
// on return A is diagonal to rounding (eigenvalues on the diagonal) and V (ld, set to the
// identity by the caller) holds the eigenvectors in its columns: A_in = V diag V^+.
__device__ void jacobi(zc *A, zc *V, int m, int ld, double *red, double *rc, double *rs, zc *rph, int *rp,
                       int *rq) {
    if (m < 2) return;
    const int M = m + (m & 1), half = M / 2;
    double prev = -1.0;
    for (int sweep = 0; sweep < kMaxSweeps; ++sweep) {
        double off = 0.0, dia = 0.0;
        for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
            const int i = t / m, j = t % m;
            const double a = abs2(A[i * ld + j]);
            if (i == j) dia += a;
            else off += a;
        }
        off = block_sum(off, red);
        dia = block_sum(dia, red);
        // converged: off-diagonal norm below 1e-15 of the matrix norm, or no longer falling
        // (the rounding floor of a large matrix; convergence is quadratic before it)
        if (off <= 1e-30 * (off + dia) || off == 0.0) break;
        if (prev >= 0.0 && off > 0.25 * prev && off <= 1e-24 * (off + dia)) break;
        prev = off;
        for (int r = 0; r < M - 1; ++r) {
            // rotation parameters of the round's pairs
            for (int i = threadIdx.x; i < half; i += blockDim.x) {
                int p, q;
                rr_pair(M, r, i, p, q);
                if (p > q) {
                    const int t = p;
                    p = q;
                    q = t;
                }
                rp[i] = p;
                rq[i] = q;
                double c = 1.0, s = 0.0;
                zc ph = mk(1.0, 0.0);
                if (q < m) {
                    const zc apq = A[p * ld + q];
                    const double rr = sqrt(abs2(apq));
                    const double a = A[p * ld + p].x, b = A[q * ld + q].x;
                    if (rr > 1e-300 && rr > 1e-18 * (fabs(a) + fabs(b))) {
                        const double tau = (b - a) / (2.0 * rr);
                        const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                        c = 1.0 / sqrt(1.0 + t * t);
                        s = t * c;
                        ph = mk(apq.x / rr, -apq.y / rr);   // e^{-i phi}, a_pq = |a_pq| e^{i phi}
                    }
                }
                rc[i] = c;
                rs[i] = s;
                rph[i] = ph;
            }
            __syncthreads();
            // column pass: A <- A U, V <- V U;  U = [[c, s], [-s ph, c ph]] on columns (p, q)
            for (int t = threadIdx.x; t < 2 * m * half; t += blockDim.x) {
                const int w = t / (m * half), u = t % (m * half);
                const int x = u / half, i = u % half;
                const int p = rp[i], q = rq[i];
                if (q >= m || rs[i] == 0.0) continue;
                zc *R = (w ? V : A) + (long long)x * ld;
                const double c = rc[i], s = rs[i];
                const zc ph = rph[i];
                const zc ap = R[p], aq = cmul(ph, R[q]);
                R[p] = mk(c * ap.x - s * aq.x, c * ap.y - s * aq.y);
                R[q] = mk(s * ap.x + c * aq.x, s * ap.y + c * aq.y);
            }
            __syncthreads();
            // row pass: A <- U^+ A on rows (p, q); the pair's off-diagonal entries are then 0
            for (int t = threadIdx.x; t < m * half; t += blockDim.x) {
                const int i = t / m, y = t % m;
                const int p = rp[i], q = rq[i];
                if (q >= m || rs[i] == 0.0) continue;
                const double c = rc[i], s = rs[i];
                const zc phc = zconj(rph[i]);
                const zc ap = A[p * ld + y], aq = cmul(phc, A[q * ld + y]);
                zc np = mk(c * ap.x - s * aq.x, c * ap.y - s * aq.y);
                zc nq = mk(s * ap.x + c * aq.x, s * ap.y + c * aq.y);
                if (y == q) np = mk(0.0, 0.0);
                if (y == p) nq = mk(0.0, 0.0);
                if (y == p) np.y = 0.0;
                if (y == q) nq.y = 0.0;
                A[p * ld + y] = np;
                A[q * ld + y] = nq;
            }
            __syncthreads();
        }
    }
}

// order[k] = index of the k-th largest (desc) or smallest (asc) of v[0..m), ties by index.
__device__ void rank_sort(const double *v, int m, bool desc, int *order) {
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const double vi = v[i];
        int rank = 0;
        for (int j = 0; j < m; ++j) {
            const double vj = v[j];
            const bool before = desc ? (vj > vi) : (vj < vi);
            if (before || (vj == vi && j < i)) ++rank;
        }
        order[rank] = i;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kThreads)
hw_kernel(const Prob *probs, const double *__restrict__ Hd, const double *__restrict__ Nd, double eps, double *E,
          int *kept, double *F, unsigned char *work) {
    __shared__ double red[kThreads / 32];
    __shared__ int s_k;
    extern __shared__ __align__(16) unsigned char dyn[];
    const Prob pb = probs[blockIdx.x];
    const int m = pb.m, ld = m + (m & 1), half = ld / 2;
    double *rc = reinterpret_cast<double *>(dyn);
    double *rs = rc + half;
    zc *rph = reinterpret_cast<zc *>(rs + half);
    int *rp = reinterpret_cast<int *>(rph + half);
    int *rq = rp + half;
    const zc *H = reinterpret_cast<const zc *>(Hd) + pb.off;
    const zc *N = reinterpret_cast<const zc *>(Nd) + pb.off;
    zc *A = reinterpret_cast<zc *>(work + pb.woff);
    zc *V = A + (long long)ld * ld;
    zc *RR = V + (long long)ld * ld;   // m x m: the kept natural states / sqrt(eigenvalue)
    zc *T = RR + (long long)m * m;     // m x m: H RR
    double *lam = reinterpret_cast<double *>(T + (long long)m * m);
    int *order = reinterpret_cast<int *>(lam + ld);
    double *Eo = E + pb.off;
    zc *Fo = F ? reinterpret_cast<zc *>(F) + pb.off : nullptr;

    // ---- the norm matrix (its Hermitian part) and its eigenvectors
    for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
        const int i = t / m, j = t % m;
        const zc a = N[i * m + j], b = zconj(N[j * m + i]);
        A[i * ld + j] = mk(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));
        V[i * ld + j] = mk(i == j ? 1.0 : 0.0, 0.0);
    }
    __syncthreads();
    jacobi(A, V, m, ld, red, rc, rs, rph, rp, rq);
    for (int i = threadIdx.x; i < m; i += blockDim.x) lam[i] = A[i * ld + i].x;
    __syncthreads();
    rank_sort(lam, m, true, order);
    if (threadIdx.x == 0) {
        const double top = lam[order[0]];
        int k = 0;
        if (top > 0.0)
            while (k < m && lam[order[k]] / top >= eps) ++k;
        s_k = k;
        kept[blockIdx.x] = k;
    }
    __syncthreads();
    const int k = s_k;
    // ---- RR = V_kept / sqrt(lambda), T = H RR, G = RR^+ T (k x k, into A), V = I
    for (int t = threadIdx.x; t < m * k; t += blockDim.x) {
        const int x = t / k, j = t % k;
        const int c = order[j];
        RR[x * m + j] = (1.0 / sqrt(lam[c])) * V[x * ld + c];
    }
    __syncthreads();
    for (int t = threadIdx.x; t < m * k; t += blockDim.x) {
        const int x = t / k, j = t % k;
        zc s = mk(0.0, 0.0);
        for (int y = 0; y < m; ++y) {
            const zc h = H[x * m + y], hc = zconj(H[y * m + x]);
            s = zfma(mk(0.5 * (h.x + hc.x), 0.5 * (h.y + hc.y)), RR[y * m + j], s);
        }
        T[x * m + j] = s;
    }
    __syncthreads();
    const int ldg = k + (k & 1);
    for (int t = threadIdx.x; t < k * k; t += blockDim.x) {
        const int i = t / k, j = t % k;
        zc s = mk(0.0, 0.0);
        for (int x = 0; x < m; ++x) s = zfma(zconj(RR[x * m + i]), T[x * m + j], s);
        A[i * ldg + j] = s;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < k * k; t += blockDim.x) {   // Hermitian part; V = I
        const int i = t / k, j = t % k;
        if (i <= j) {
            const zc a = A[i * ldg + j], b = zconj(A[j * ldg + i]);
            const zc hgt = mk(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));
            A[i * ldg + j] = hgt;
            A[j * ldg + i] = zconj(hgt);
        }
        V[i * ldg + j] = mk(i == j ? 1.0 : 0.0, 0.0);
    }
    __syncthreads();
    jacobi(A, V, k, ldg, red, rc, rs, rph, rp, rq);
    for (int i = threadIdx.x; i < k; i += blockDim.x) lam[i] = A[i * ldg + i].x;
    __syncthreads();
    rank_sort(lam, k, false, order);
    for (int j = threadIdx.x; j < m; j += blockDim.x) Eo[j] = j < k ? lam[order[j]] : 0.0;
    if (Fo) {   // f_j = RR v_order[j]
        for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
            const int x = t / m, j = t % m;
            zc s = mk(0.0, 0.0);
            if (j < k) {
                const int c = order[j];
                for (int i = 0; i < k; ++i) s = zfma(RR[x * m + i], V[i * ldg + c], s);
            }
            Fo[x * m + j] = s;
        }
    }
}

long long prob_bytes(int m) {
    const long long ld = m + (m & 1);
    return (2 * ld * ld + 2LL * m * m) * (long long)sizeof(zc) + ld * (long long)(sizeof(double) + sizeof(int)) + 256;
}

}  // namespace

extern "C" {

long long pnamp_hw_work_bytes(int nprob, const int *dim) {
    if (nprob < 0 || (nprob > 0 && !dim)) return -1;
    long long b = ((long long)nprob * sizeof(Prob) + 255) / 256 * 256;
    for (int i = 0; i < nprob; ++i) {
        if (dim[i] < 1 || dim[i] > PNAMP_HW_MAX_DIM) return -1;
        b += (prob_bytes(dim[i]) + 255) / 256 * 256;
    }
    return b;
}

int pnamp_hw_solve(int nprob, const int *dim, const long long *off, const double *H, const double *N, double eps,
                   double *E, int *kept, double *F, void *work, void *stream) {
    if (nprob < 0 || (nprob > 0 && (!dim || !off || !H || !N || !E || !kept || !work)) || !(eps >= 0.0))
        return 1;
    if (nprob == 0) return 0;
    const long long head = ((long long)nprob * sizeof(Prob) + 255) / 256 * 256;
    Prob *hp = new Prob[nprob];
    long long w = head;
    int maxm = 1;
    for (int i = 0; i < nprob; ++i) {
        if (dim[i] < 1 || dim[i] > PNAMP_HW_MAX_DIM || off[i] < 0) {
            delete[] hp;
            return 1;
        }
        hp[i].m = dim[i];
        hp[i].off = off[i];
        hp[i].woff = w;
        w += (prob_bytes(dim[i]) + 255) / 256 * 256;
        maxm = dim[i] > maxm ? dim[i] : maxm;
    }
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char *wk = (unsigned char *)work;
    const cudaError_t e1 = cudaMemcpyAsync(wk, hp, nprob * sizeof(Prob), cudaMemcpyHostToDevice, st);
    const cudaError_t e2 = cudaStreamSynchronize(st);   // the host table goes out of scope here
    delete[] hp;
    if (e1 != cudaSuccess || e2 != cudaSuccess) return 2;
    const int half = (maxm + 1) / 2;
    const size_t smem = (size_t)half * (2 * sizeof(double) + sizeof(zc) + 2 * sizeof(int));
    hw_kernel<<<nprob, kThreads, smem, st>>>(reinterpret_cast<const Prob *>(wk), H, N, eps, E, kept, F, wk);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // extern "C"
