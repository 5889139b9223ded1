// ORACLE / CPU BASELINE -- test infrastructure only; the product path never links or calls it.
//
// A C++ restatement of SCCM's PNAMP mesh loop (Kernel4Triaxial, Codes/PNAMP/PNAMP_Kernel3D.f90:
// 70-407) for the CPU baseline that the GPU library is timed against, on the same inputs
// (include/pnamp_gpu.h structs, column-major U, V) and with the same ZRES(P_E, NOBS) output.
// OpenMP over Euler points, one thread's work arrays per Euler point.
//
// Two forms:
//   form 0 "as implemented": the reference's per-point call sequence -- UVphiomega
//     (2 ZGEMM, PNAMP_Proj.f90:396-455), Pfaf_Over (LU inverse of conj(Ubar), ZGEMM, the
//     2n x 2n ZPfaffianF with global pivoting, :142-392), ROKAPPAphiomega (T22 by 4 ZGEMM,
//     LU inverse, 7 ZGEMM, :459-551), ZN_0, the 8-term energy loop of HFB_Energy_COMPLEX
//     (PNAMP_Energy_OpenMP.f90:31-90), ZJ2_0 (18 ZGEMM, PNAMP_ME2B.f90) and ZQ2/ZQ2t
//     (10 ZGEMM, PNAMP_ME1B.f90:52-136): about 379 n^3 flops plus the record loop;
//   form 1 "minimal": the same mathematics with the GPU library's algebra -- per Euler point
//     R W R^T, R V1, R* U1 and the four T22 species partials; per gauge point the reduced
//     n x n Pfaffian c (D X D - Z0^-1) times Pf(-c Z0) (when V0's LU pivots span < 1e2),
//     Y T22^-1 by LU, complex-by-real density products, O(n^2) traces and J products.
// Dense kernels are plain loops over contiguous columns (the compiler vectorises them); no
// BLAS is linked, so the baseline builds the same on x86-64 and aarch64.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <tuple>
#include <vector>

#include "pnamp_gpu.h"

namespace {

using cd = std::complex<double>;
constexpr int kNobs = PNAMP_NOBS;

// ---------------------------------------------------------------- dense helpers (column-major)
struct M {
    int r = 0, c = 0;
    std::vector<cd> a;
    M() = default;
    M(int r_, int c_) : r(r_), c(c_), a((size_t)r_ * c_) {}
    cd &operator()(int i, int j) { return a[i + (size_t)j * r]; }
    const cd &operator()(int i, int j) const { return a[i + (size_t)j * r]; }
    void zero() { std::fill(a.begin(), a.end(), cd(0)); }
};

// C = op(A) op(B), op = N (as is), T (transpose), C (conjugate, no transpose). op(A) is
// formed first, so the inner loop always runs down a contiguous column.
void gemm(char ta, char tb, const M &A0, const M &B, M &C) {
    M At;
    const M *Ap = &A0;
    if (ta != 'N') {
        At = (ta == 'T') ? M(A0.c, A0.r) : M(A0.r, A0.c);
        for (int j = 0; j < A0.c; ++j)
            for (int i = 0; i < A0.r; ++i) {
                if (ta == 'T') At(j, i) = A0(i, j);
                else At(i, j) = std::conj(A0(i, j));
            }
        Ap = &At;
    }
    const M &A = *Ap;
    const int m = A.r, k = A.c;
    const int n = (tb == 'T') ? B.r : B.c;
    C = M(m, n);
    for (int j = 0; j < n; ++j) {
        cd *cj = &C.a[(size_t)j * m];
        for (int kk = 0; kk < k; ++kk) {
            cd b = (tb == 'T') ? B(j, kk) : B(kk, j);
            if (tb == 'C') b = std::conj(b);
            if (b == cd(0)) continue;
            const cd *ak = &A.a[(size_t)kk * m];
            for (int i = 0; i < m; ++i) cj[i] += ak[i] * b;
        }
    }
}

// LU with partial pivoting (ZGETRF); returns false on an exactly zero pivot
bool lu(M &A, std::vector<int> &piv) {
    const int n = A.r;
    piv.assign(n, 0);
    for (int k = 0; k < n; ++k) {
        int p = k;
        double best = std::abs(A(k, k).real()) + std::abs(A(k, k).imag());
        for (int i = k + 1; i < n; ++i) {
            const double v = std::abs(A(i, k).real()) + std::abs(A(i, k).imag());
            if (v > best) {
                best = v;
                p = i;
            }
        }
        piv[k] = p;
        if (best == 0.0) return false;
        if (p != k)
            for (int j = 0; j < n; ++j) std::swap(A(k, j), A(p, j));
        const cd inv = 1.0 / A(k, k);
        for (int i = k + 1; i < n; ++i) A(i, k) *= inv;
        for (int j = k + 1; j < n; ++j) {
            const cd akj = A(k, j);
            if (akj == cd(0)) continue;
            for (int i = k + 1; i < n; ++i) A(i, j) -= A(i, k) * akj;
        }
    }
    return true;
}

// A^-1 from its LU (ZGETRI): solve A X = I column by column
M lu_inverse(const M &LU, const std::vector<int> &piv) {
    const int n = LU.r;
    M X(n, n);
    for (int j = 0; j < n; ++j) {
        std::vector<cd> b(n, cd(0));
        b[j] = 1.0;
        for (int k = 0; k < n; ++k) std::swap(b[k], b[piv[k]]);
        for (int k = 0; k < n; ++k)
            for (int i = k + 1; i < n; ++i) b[i] -= LU(i, k) * b[k];
        for (int k = n - 1; k >= 0; --k) {
            b[k] /= LU(k, k);
            for (int i = 0; i < k; ++i) b[i] -= LU(i, k) * b[k];
        }
        for (int i = 0; i < n; ++i) X(i, j) = b[i];
    }
    return X;
}

bool inverse(const M &A, M &X) {
    M LU = A;
    std::vector<int> piv;
    if (!lu(LU, piv)) return false;
    X = lu_inverse(LU, piv);
    return true;
}

// Pfaffian of the skew matrix that the strict upper triangle of S defines, by 2x2-block
// elimination. global = true: the largest remaining upper entry as pivot (ZPfaffianF,
// PNAMP_Proj.f90:218-350); false: the largest entry of the pivot row (partial pivoting).
// Pf = 0 when |pivot| <= 1e-13 (PNAMP_Proj.f90:290,333).
cd pfaffian(const M &S0, bool global) {
    const int N = S0.r;
    M A(N, N);
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < j; ++i) {
            A(i, j) = S0(i, j);
            A(j, i) = -S0(i, j);
        }
    cd pf = 1.0;
    auto swap_rc = [&](int p, int q) {
        for (int j = 0; j < N; ++j) std::swap(A(p, j), A(q, j));
        for (int i = 0; i < N; ++i) std::swap(A(i, p), A(i, q));
    };
    for (int k = 0; k < N / 2 - 1; ++k) {
        const int r = 2 * k, c = r + 1;
        int i1 = r, i2 = c;
        double big = -1.0;
        if (global) {
            for (int i = r; i < N - 1; ++i)
                for (int j = i + 1; j < N; ++j)
                    if (std::abs(A(i, j)) > big) {
                        big = std::abs(A(i, j));
                        i1 = i;
                        i2 = j;
                    }
        } else {
            for (int j = c; j < N; ++j) {
                const double v = std::max(std::abs(A(r, j).real()), std::abs(A(r, j).imag()));
                if (v > big) {
                    big = v;
                    i2 = j;
                }
            }
        }
        double phas = 1.0;
        if (i1 == r) phas = -phas;
        if (i2 == c) phas = -phas;
        if (i1 != r) swap_rc(r, i1);
        if (i2 != c) swap_rc(c, i2);
        const cd ss = A(r, c);
        if (!(std::abs(ss) > 1.0e-13)) return 0.0;
        for (int i = c + 1; i < N; ++i)
            for (int j = i + 1; j < N; ++j) {
                A(i, j) += (A(c, i) * A(r, j) - A(r, i) * A(c, j)) / ss;
                A(j, i) = -A(i, j);
            }
        pf *= ss * phas;
    }
    return pf * A(N - 2, N - 1);
}

double wigner_d(int tj, int tm1, int tm2, double beta) {
    if (std::abs(tm1) > tj || std::abs(tm2) > tj) return 0.0;
    auto f = [](int k) { return std::tgamma(k + 1.0); };
    const int jp1 = (tj + tm1) / 2, jm1 = (tj - tm1) / 2, jp2 = (tj + tm2) / 2, jm2 = (tj - tm2) / 2;
    const double pre = std::sqrt(f(jp1) * f(jm1) * f(jp2) * f(jm2));
    const double c = std::cos(0.5 * beta), s = std::sin(0.5 * beta);
    const int dm = (tm1 - tm2) / 2;
    double d = 0.0;
    for (int k = 0; k <= tj; ++k) {
        const int a = jp2 - k, e = jm1 - k, g = k + dm;
        if (a < 0 || e < 0 || g < 0) continue;
        const double t = ((g & 1) ? -1.0 : 1.0) / (f(a) * f(k) * f(e) * f(g));
        d += t * std::pow(c, tj - 2 * k - dm) * std::pow(s, 2 * k + dm);
    }
    return pre * d;
}

struct Problem {
    int n, h, nprot, nneut, nfom, P;
    double cscale, vacfac;
    std::vector<int> t, nn, l, tj, tm;
    std::vector<double> euler;   // [P][4]
    std::vector<int> ka, kb, kc, kd;
    std::vector<double> vbar;
    M t1b;                       // t(a, c)
    std::vector<M> q2;           // mu = -2..2
    bool iE2;
    M J[3], J2[3];               // Jx, Jy, Jz and their squares
    std::vector<std::tuple<int, int, cd>> jnz[3], j2nz[3];   // their non-zeros (row, column, value)
    double e0;
};

void j_ops(Problem &p) {
    const int n = p.n;
    for (int q = 0; q < 3; ++q) {
        p.J[q] = M(n, n);
        p.J2[q] = M(n, n);
    }
    for (int a = 0; a < n; ++a)
        for (int b = 0; b < n; ++b) {
            if (p.nn[a] != p.nn[b] || p.l[a] != p.l[b] || p.tj[a] != p.tj[b] || p.t[a] != p.t[b]) continue;
            const double jb = p.tj[b] / 2.0, mb = p.tm[b] / 2.0;
            const int ma2 = p.tm[a], mb2 = p.tm[b];
            const double fp1 = jb * (jb + 1) - mb * (mb + 1), fm1 = jb * (jb + 1) - mb * (mb - 1);
            const double fp1p2 = jb * (jb + 1) - (mb + 1) * (mb + 2), fm1m2 = jb * (jb + 1) - (mb - 1) * (mb - 2);
            const double f02 = jb * (jb + 1) - mb * mb;
            const double dp1 = ma2 == mb2 + 2, dm1 = ma2 == mb2 - 2, dp2 = ma2 == mb2 + 4, dm2 = ma2 == mb2 - 4,
                         d0 = ma2 == mb2;
            const double sp1 = std::sqrt(std::max(fp1, 0.0)), sm1 = std::sqrt(std::max(fm1, 0.0));
            p.J[0](a, b) = 0.5 * (sp1 * dp1 + sm1 * dm1);
            p.J[1](a, b) = cd(0, -0.5) * (sp1 * dp1 - sm1 * dm1);
            p.J[2](a, b) = mb * d0;
            const double s1 = std::sqrt(std::max(fp1 * fp1p2, 0.0)), s2 = std::sqrt(std::max(fm1 * fm1m2, 0.0));
            p.J2[0](a, b) = 0.25 * (s1 * dp2 + s2 * dm2 + 2 * f02 * d0);
            p.J2[1](a, b) = -0.25 * (s1 * dp2 + s2 * dm2 - 2 * f02 * d0);
            p.J2[2](a, b) = (mb * d0) * (mb * d0);
        }
    for (int q = 0; q < 3; ++q)
        for (int b = 0; b < n; ++b)
            for (int a = 0; a < n; ++a) {
                if (p.J[q](a, b) != cd(0)) p.jnz[q].emplace_back(a, b, p.J[q](a, b));
                if (p.J2[q](a, b) != cd(0)) p.j2nz[q].emplace_back(a, b, p.J2[q](a, b));
            }
}

M rotation(const Problem &p, double alp, double bet, double gam) {
    M R(p.n, p.n);
    for (int a = 0; a < p.n; ++a)
        for (int b = 0; b < p.n; ++b)
            if (p.t[a] == p.t[b] && p.nn[a] == p.nn[b] && p.l[a] == p.l[b] && p.tj[a] == p.tj[b])
                R(a, b) = std::polar(1.0, -0.5 * (alp * p.tm[a] + gam * p.tm[b])) *
                          wigner_d(p.tj[a], p.tm[a], p.tm[b], bet);
    return R;
}

// zbareover (PNAMP_Proj.f90:6-79): Z = V U^-1 and det(1 + Z^T Z)^(-1/4)
bool bare(const M &U, const M &V, M &Z, double &det) {
    M Ui;
    if (!inverse(U, Ui)) return false;
    gemm('N', 'N', V, Ui, Z);
    M T;
    gemm('T', 'N', Z, Z, T);
    for (int i = 0; i < T.r; ++i) T(i, i) += 1.0;
    std::vector<int> piv;
    if (!lu(T, piv)) return false;
    double s = 0.0;
    for (int i = 0; i < T.r; ++i) s += std::log(std::abs(T(i, i)));
    det = std::exp(-0.25 * s);
    return true;
}

// observables of one gauge point from the densities, weighted by the norm (Kernel3D.f90:296-358)
void observables(const Problem &p, const M &rho, const M &k10, const M &k01, bool as_implemented, cd norm,
                 cd *out) {
    const int n = p.n, h = p.h;
    cd zp = 0, zn = 0;
    for (int a = 0; a < h; ++a) zp += rho(a, a);
    for (int a = h; a < n; ++a) zn += rho(a, a);
    cd e2 = 0;
    for (size_t r = 0; r < p.vbar.size(); ++r) {
        const int i = p.ka[r], j = p.kb[r], k = p.kc[r], l = p.kd[r];
        const double d = (i + j == k + l) ? 0.0 : 1.0;
        const cd z_ijkl = rho(k, i) * rho(l, j) - rho(l, i) * rho(k, j) + k01(i, j) * k10(k, l);
        const cd z_jikl = rho(k, j) * rho(l, i) - rho(l, j) * rho(k, i) + k01(j, i) * k10(k, l);
        const cd z_jilk = rho(l, j) * rho(k, i) - rho(k, j) * rho(l, i) + k01(j, i) * k10(l, k);
        const cd z_ijlk = rho(l, i) * rho(k, j) - rho(k, i) * rho(l, j) + k01(i, j) * k10(l, k);
        const cd z_klij = rho(i, k) * rho(j, l) - rho(j, k) * rho(i, l) + k01(k, l) * k10(i, j);
        const cd z_klji = rho(j, k) * rho(i, l) - rho(i, k) * rho(j, l) + k01(k, l) * k10(j, i);
        const cd z_lkij = rho(i, l) * rho(j, k) - rho(j, l) * rho(i, k) + k01(l, k) * k10(i, j);
        const cd z_lkji = rho(j, l) * rho(i, k) - rho(i, l) * rho(j, k) + k01(l, k) * k10(j, i);
        e2 += 0.25 * p.vbar[r] *
              (z_ijkl + d * z_klij - z_jikl - d * z_klji - z_ijlk - d * z_lkij + z_jilk + d * z_lkji);
    }
    cd ekin = 0;
    for (int a = 0; a < n; ++a)
        for (int c = 0; c < n; ++c) ekin += rho(c, a) * p.t1b(a, c);
    cd j2 = 0;
    if (as_implemented) {   // ZJ2_0: 18 ZGEMM
        for (int q = 0; q < 3; ++q) {
            M a1, a2, a3, a4, a22, a34;
            gemm('N', 'N', p.J2[q], rho, a1);
            gemm('N', 'N', p.J[q], rho, a2);
            gemm('N', 'N', p.J[q], k10, a3);
            M k01t(n, n);
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) k01t(i, j) = k01(j, i);
            gemm('T', 'N', p.J[q], k01t, a4);
            gemm('N', 'N', a2, a2, a22);
            gemm('N', 'N', a3, a4, a34);
            cd t1 = 0, t2 = 0, t22 = 0, t34 = 0;
            for (int i = 0; i < n; ++i) {
                t1 += a1(i, i);
                t2 += a2(i, i);
                t22 += a22(i, i);
                t34 += a34(i, i);
            }
            j2 += t1 + t2 * t2 - t22 + t34;
        }
    } else {   // J has <= 2 non-zeros per row: products with it are O(n^2)
        for (int q = 0; q < 3; ++q) {
            M a2(n, n), a3(n, n), a4(n, n);
            cd t1 = 0;
            for (const auto &e : p.jnz[q]) {   // (a, b, J_ab)
                const int a = std::get<0>(e), b = std::get<1>(e);
                const cd v = std::get<2>(e);
                for (int c = 0; c < n; ++c) {
                    a2(a, c) += v * rho(b, c);     // J rho
                    a3(a, c) += v * k10(b, c);     // J kappa10
                    a4(b, c) += v * k01(c, a);     // (J^T kappa01^T)(b, c) = sum_a J_ab kappa01(c, a)
                }
            }
            for (const auto &e : p.j2nz[q]) t1 += std::get<2>(e) * rho(std::get<1>(e), std::get<0>(e));
            cd t2 = 0, t22 = 0, t34 = 0;
            for (int a = 0; a < n; ++a) {
                t2 += a2(a, a);
                for (int c = 0; c < n; ++c) {
                    t22 += a2(a, c) * a2(c, a);
                    t34 += a3(a, c) * a4(c, a);
                }
            }
            j2 += t1 + t2 * t2 - t22 + t34;
        }
    }
    out[0] += norm;
    out[1] += norm * zp;
    out[2] += norm * zn;
    out[3] += norm * ekin;
    out[6] += norm * (e2 + ekin + p.e0);
    out[7] += norm * j2;
    if (p.iE2) {
        for (int mu = 0; mu < 5; ++mu) {
            cd tq = 0, tqt = 0;
            if (as_implemented) {
                M aq, aqt;
                gemm('N', 'N', p.q2[mu], rho, aq);
                M qh(n, n);
                for (int i = 0; i < n; ++i)
                    for (int j = 0; j < n; ++j) qh(i, j) = std::conj(p.q2[mu](j, i));
                gemm('N', 'N', qh, rho, aqt);
                for (int a = 0; a < h; ++a) {
                    tq += aq(a, a);
                    tqt += aqt(a, a);
                }
            } else {
                for (int a = 0; a < h; ++a)
                    for (int b = 0; b < n; ++b) {
                        tq += p.q2[mu](a, b) * rho(b, a);
                        tqt += std::conj(p.q2[mu](b, a)) * rho(b, a);
                    }
            }
            out[8 + mu] += norm * tq;
            out[13 + mu] += norm * tqt;
        }
    }
}

struct Pair {
    M U0, V0, U1, V1, Z0, W, Z0inv;
    double det0 = 0, det1 = 0;
    bool reduced = false;
    cd pfz = 0;
    int err = 0;
};

// one Euler point, all gauge points; acc receives the gauge sums (not yet divided by NFOM^2)
void euler_point(const Problem &p, const Pair &q, int ie, int form, cd *acc) {
    const int n = p.n, h = p.h, nf = p.nfom;
    const double alp = p.euler[4 * ie], bet = p.euler[4 * ie + 1], gam = p.euler[4 * ie + 2];
    const M R = rotation(p, alp, bet, gam);
    const double twopi = 6.283185307179586476925287;
    // minimal form: per-Euler pieces
    M X, B1, B2, Pt[4];
    if (form == 1) {
        M RW;
        gemm('N', 'N', R, q.W, RW);
        gemm('N', 'T', RW, R, X);
        gemm('N', 'N', R, q.V1, B1);
        gemm('C', 'N', R, q.U1, B2);
        for (int s = 0; s < 4; ++s) {   // V0p^T B1p, V0n^T B1n, U0p^T B2p, U0n^T B2n
            const M &Mq = s < 2 ? q.V0 : q.U0;
            const M &Bq = s < 2 ? B1 : B2;
            const int k0 = (s & 1) ? h : 0;
            Pt[s] = M(n, n);
            for (int j = 0; j < n; ++j)
                for (int k = k0; k < k0 + h; ++k) {
                    const cd b = Bq(k, j);
                    for (int i = 0; i < n; ++i) Pt[s](i, j) += Mq(k, i) * b;
                }
        }
    }
    for (int lp = 0; lp < nf; ++lp)
        for (int ln = 0; ln < nf; ++ln) {
            const double php = nf == 1 ? 0.0 : twopi * lp / nf, phn = nf == 1 ? 0.0 : twopi * ln / nf;
            const cd ep = std::polar(1.0, php), en = std::polar(1.0, phn);
            M rho, k10, k01;
            cd pf;
            bool sing = false;
            if (form == 0) {
                M A = R;
                for (int j = 0; j < n; ++j)
                    for (int i = 0; i < n; ++i) A(i, j) *= (i < h ? ep : en);
                M ub, vb;
                gemm('N', 'N', A, q.U1, ub);
                gemm('C', 'N', A, q.V1, vb);
                M ubc = ub, ubi;
                for (auto &v : ubc.a) v = std::conj(v);
                if (!inverse(ubc, ubi)) sing = true;
                M m1;
                gemm('C', 'N', vb, ubi, m1);
                M S(2 * n, 2 * n);
                for (int j = 0; j < n; ++j)
                    for (int i = 0; i < n; ++i) {
                        S(i, j) = p.cscale * m1(i, j);
                        S(n + i, n + j) = -p.cscale * q.Z0(i, j);
                    }
                for (int i = 0; i < n; ++i) {
                    S(i, n + i) = -p.cscale;
                    S(n + i, i) = p.cscale;
                }
                pf = pfaffian(S, true);
                // ROKAPPAphiomega
                M av1, acu1, t22a, t22b, t22, ti;
                gemm('N', 'N', A, q.V1, av1);
                gemm('C', 'N', A, q.U1, acu1);
                gemm('T', 'N', q.V0, av1, t22a);
                gemm('T', 'N', q.U0, acu1, t22b);
                t22 = t22a;
                for (size_t e = 0; e < t22.a.size(); ++e) t22.a[e] += t22b.a[e];
                if (!inverse(t22, ti)) sing = true;
                M aux3, aux4, aux2 = acu1;
                for (auto &v : aux2.a) v = -v;
                gemm('N', 'T', ti, q.V0, aux3);
                gemm('N', 'T', ti, q.U0, aux4);
                gemm('N', 'N', av1, aux3, rho);
                gemm('N', 'N', av1, aux4, k10);
                gemm('N', 'N', aux2, aux3, k01);
            } else {
                const cd dpp = p.cscale * ep * ep, dpn = p.cscale * ep * en, dnn = p.cscale * en * en;
                if (q.reduced) {
                    M S(n, n);
                    for (int j = 0; j < n; ++j)
                        for (int i = 0; i < j; ++i)
                            S(i, j) = X(i, j) * (j < h ? dpp : (i < h ? dpn : dnn)) - p.cscale * q.Z0inv(i, j);
                    pf = pfaffian(S, false) * q.pfz;
                } else {
                    M S(2 * n, 2 * n);
                    for (int j = 0; j < n; ++j)
                        for (int i = 0; i < n; ++i) {
                            S(i, j) = X(i, j) * (j < h ? (i < h ? dpp : dpn) : (i < h ? dpn : dnn));
                            S(n + i, n + j) = -p.cscale * q.Z0(i, j);
                        }
                    for (int i = 0; i < n; ++i) S(i, n + i) = -p.cscale;
                    pf = pfaffian(S, false);
                }
                M T(n, n);
                for (size_t e = 0; e < T.a.size(); ++e)
                    T.a[e] = ep * Pt[0].a[e] + en * Pt[1].a[e] + std::conj(ep) * Pt[2].a[e] +
                             std::conj(en) * Pt[3].a[e];
                std::vector<int> piv;
                M LU = T;
                if (!lu(LU, piv)) sing = true;
                // Y T22^-1 for Y = B1 and B2 via (T^T)^-1 applied to Y^T
                M Ti = sing ? M(n, n) : lu_inverse(LU, piv);
                M Y1, Y2;
                gemm('N', 'N', B1, Ti, Y1);
                gemm('N', 'N', B2, Ti, Y2);
                rho = M(n, n);
                k10 = M(n, n);
                k01 = M(n, n);
                for (int j = 0; j < n; ++j)
                    for (int k = 0; k < n; ++k) {
                        const cd v0 = q.V0(j, k), u0 = q.U0(j, k);   // V0^T(k, j), U0^T(k, j)
                        for (int i = 0; i < n; ++i) {
                            rho(i, j) += Y1(i, k) * v0;
                            k10(i, j) += Y1(i, k) * u0;
                            k01(i, j) += Y2(i, k) * v0;
                        }
                    }
                for (int j = 0; j < n; ++j)
                    for (int i = 0; i < n; ++i) {
                        const cd di = i < h ? ep : en;
                        rho(i, j) *= di;
                        k10(i, j) *= di;
                        k01(i, j) *= -std::conj(di);
                    }
            }
            const cd zph = std::polar(1.0, -(php * p.nprot + phn * p.nneut));
            const cd norm = p.vacfac * q.det0 * q.det1 * pf * zph;
            if (sing) {
                acc[0] += norm;
                continue;
            }
            observables(p, rho, k10, k01, form == 0, norm, acc);
        }
}

}  // namespace

extern "C" {

// ZRES(P_E, NOBS) of one pair (column-major complex, zres[2 * (ie + io * P_E)]); `euler` lists
// the Euler points to evaluate (NULL: all; the other rows are left as passed). Returns 0, or
// PNAMP_ERR_ARG / PNAMP_ERR_SINGULAR_U.
int cpu_pnamp_pair(const pnamp_space *sp, const pnamp_hamiltonian *hm, const pnamp_mesh *m, const double *U0,
                   const double *V0, const double *U1, const double *V1, const int *euler, int neuler, int form,
                   int nthreads, double *zres) {
    if (!sp || !hm || !m || !U0 || !V0 || !U1 || !V1 || !zres || (form != 0 && form != 1)) return PNAMP_ERR_ARG;
    Problem p;
    p.n = sp->nlev;
    p.h = p.n / 2;
    p.nprot = sp->nprot;
    p.nneut = sp->nneut;
    p.nfom = m->nfom;
    p.cscale = m->cscale;
    p.e0 = hm->e0;
    const int n = p.n;
    p.t.assign(sp->t, sp->t + n);
    p.nn.assign(sp->n, sp->n + n);
    p.l.assign(sp->l, sp->l + n);
    p.tj.assign(sp->twoj, sp->twoj + n);
    p.tm.assign(sp->twom, sp->twom + n);
    const int nbu = std::max(m->nbet / std::max(m->ncosbet, 1), 1);
    for (int k = 0; k < nbu; ++k)
        for (int a = 0; a < m->nalp; ++a)
            for (int g = 0; g < m->ngam; ++g) {
                p.euler.push_back(m->alpha[a]);
                p.euler.push_back(m->beta[k]);
                p.euler.push_back(m->gamma[g]);
                p.euler.push_back(m->walp[a] * m->wbet[k] * m->wgam[g] * m->ncosbet);
            }
    p.P = (int)p.euler.size() / 4;
    for (int r = 0; r < hm->nrec; ++r) {
        p.ka.push_back(hm->ka[r] - 1);
        p.kb.push_back(hm->kb[r] - 1);
        p.kc.push_back(hm->kc[r] - 1);
        p.kd.push_back(hm->kd[r] - 1);
        p.vbar.push_back(hm->vbar[r]);
    }
    p.t1b = M(n, n);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) p.t1b(i, j) = hm->t1b[i + (size_t)j * n];
    p.iE2 = hm->q2 != nullptr;
    if (p.iE2)
        for (int mu = 0; mu < 5; ++mu) {
            M q(n, n);
            for (int j = 0; j < n; ++j)
                for (int i = 0; i < n; ++i) q(i, j) = hm->q2[(size_t)mu * n * n + i + (size_t)j * n];
            p.q2.push_back(q);
        }
    j_ops(p);
    const long long aaa = (long long)n * (n + 1) / 2;
    p.vacfac = ((aaa & 1) ? -1.0 : 1.0) * std::pow(10.0, -2.0 * (n * m->iscale / 2));

    Pair q;
    auto load = [&](const double *src) {
        M X(n, n);
        for (size_t e = 0; e < X.a.size(); ++e) X.a[e] = src[e];
        return X;
    };
    q.U0 = load(U0);
    q.V0 = load(V0);
    q.U1 = load(U1);
    q.V1 = load(V1);
    if (!bare(q.U0, q.V0, q.Z0, q.det0) || !bare(q.U1, q.V1, q.W, q.det1)) return PNAMP_ERR_SINGULAR_U;
    if (form == 1) {   // reduced Pfaffian when V0 is well conditioned
        M LU = q.V0;
        std::vector<int> piv;
        if (lu(LU, piv)) {
            double mx = 0, mn = 1e300;
            for (int i = 0; i < n; ++i) {
                mx = std::max(mx, std::abs(LU(i, i)));
                mn = std::min(mn, std::abs(LU(i, i)));
            }
            if (mn >= 1e-2 * mx) {
                M Vi = lu_inverse(LU, piv);
                gemm('N', 'N', q.U0, Vi, q.Z0inv);
                M S(n, n);
                for (size_t e = 0; e < S.a.size(); ++e) S.a[e] = -p.cscale * q.Z0.a[e];
                q.pfz = pfaffian(S, false);
                q.reduced = std::abs(q.pfz) > 0.0;
            }
        }
    }
    std::vector<int> list;
    if (euler) list.assign(euler, euler + neuler);
    else
        for (int e = 0; e < p.P; ++e) list.push_back(e);
    for (int e : list)
        if (e < 0 || e >= p.P) return PNAMP_ERR_ARG;
    const double inv = 1.0 / ((double)p.nfom * p.nfom);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : omp_get_max_threads())
    for (int k = 0; k < (int)list.size(); ++k) {
        cd acc[kNobs];
        for (auto &v : acc) v = 0;
        euler_point(p, q, list[k], form, acc);
        for (int io = 0; io < kNobs; ++io) {
            zres[2 * (list[k] + (size_t)io * p.P)] = (acc[io] * inv).real();
            zres[2 * (list[k] + (size_t)io * p.P) + 1] = (acc[io] * inv).imag();
        }
    }
    return PNAMP_OK;
}

int cpu_pnamp_max_threads(void) { return omp_get_max_threads(); }

}  // extern "C"
