// C ABI of the PNAMP kernel library (declared in include/pnamp_gpu.h).
//
// Host side of Kernel4Triaxial: validates the caller's model space, Hamiltonian
// and mesh, builds the small constant tables the kernels read (rotation block
// map, Euler point list, sparse one-body operators, packed two-body list,
// projection weights), plans where the per-point work arrays live (shared
// memory when they fit a CTA, otherwise an L2-resident global slot per CTA),
// and enqueues setup -> points -> projection on one stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "pnamp_gpu.h"
#include "pnamp_internal.h"

using namespace pnamp;

struct pnamp_ctx {
    Params p;
    int core_prot, core_neut;
    int axial;
    int grid;
    int grid_form[2];
    std::vector<void *> allocs;
    double *d_pairbuf = nullptr;
    long long pair_cap = 0;
    zc *d_scratch = nullptr;
    zc *d_projw = nullptr;
    const double *d_tj = nullptr;   // 3j symbols of the Q2 projection
    double *d_projq = nullptr;
    double *d_uv = nullptr, *d_zres = nullptr, *d_proj = nullptr;
    int *d_status = nullptr;
    long long batch_cap = 0;
    cudaStream_t stream = nullptr;
    int sticky = 0;
    // one-body density blocks (host copies) and the Euler quadrature weights
    std::vector<int> r1b_it, r1b_lj, r1b_n1, r1b_n2, r1b_twoj;
    std::vector<double> euler_w;
    double *d_r1b = nullptr;
    long long r1b_cap = 0;
    // two-body density tables (built on first use) and device buffers
    std::vector<int> sp_t, sp_n, sp_l, sp_tj, sp_tm;
    bool r2_built = false;
    std::vector<int> r2_blocks, r2_states, r2_ptr, r2_tq;
    std::vector<uint32_t> r2_quads;
    std::vector<double> r2_tc;
    uint32_t *d_r2q = nullptr;
    double *d_r2acc = nullptr, *d_r2out = nullptr;
    long long r2acc_cap = 0, r2out_cap = 0;
    // tensor-core contraction of the two-body energy (contract_tc.cu): bf16 terms per value
    // (0 = the record loop in the point kernel), tables built on first use, staging buffers
    int tc_splits = 0;
    std::vector<uint32_t> h_rec_idx;
    std::vector<double> h_rec_v;
    bool tc_built = false;
    int tc_nk = 0, tc_nph = 0, tc_kmax = 0;
    long long tc_rows = 0;
    std::vector<TcGroup> tc_groups;
    std::vector<int> tc_src;
    TcGroup *d_tc_groups = nullptr;
    int *d_tc_src = nullptr;
    unsigned short *d_tc_mat[3] = {nullptr, nullptr, nullptr};
    unsigned short *d_tc_x[3] = {nullptr, nullptr, nullptr}, *d_tc_y[3] = {nullptr, nullptr, nullptr};
    double *d_tc_w = nullptr, *d_tc_e2 = nullptr;
    int *d_tc_err = nullptr;
    long long tc_cap_pts = 0;
    int tc_cap_splits = 0;                       // bf16 terms the staging was allocated for
    int nsm = 0;
    // per-stage CUDA-event timing of the last pnamp_batch_device / items call (pnamp_set_timing)
    int timing = 0;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::array<int, 3>> ev_marks;   // (stage, start event, end event)
};

namespace {

#define CK(call)                                                                  \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) {                                                  \
            if (getenv("PNAMP_DEBUG"))                                            \
                fprintf(stderr, "pnamp: %s:%d %s\n", __FILE__, __LINE__,          \
                        cudaGetErrorString(e_));                                  \
            return (e_ == cudaErrorMemoryAllocation) ? PNAMP_ERR_NOMEM : PNAMP_ERR_CUDA; \
        }                                                                         \
    } while (0)

template <typename T>
int dev_upload(pnamp_ctx *c, const std::vector<T> &h, const T **out) {
    T *d = nullptr;
    const size_t bytes = std::max<size_t>(h.size(), 1) * sizeof(T);
    CK(cudaMalloc(&d, bytes));
    c->allocs.push_back(d);
    if (!h.empty()) CK(cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    *out = d;
    return PNAMP_OK;
}

double fact_h(int k) {
    double f = 1.0;
    for (int i = 2; i <= k; ++i) f *= i;
    return f;
}

// <j1 m1 j2 m2 | J M>, doubled arguments, Racah's formula
double cg_h(int tj1, int tj2, int tJ, int tm1, int tm2, int tM) {
    if (tm1 + tm2 != tM) return 0.0;
    if (tJ < std::abs(tj1 - tj2) || tJ > tj1 + tj2 || (tj1 + tj2 + tJ) % 2) return 0.0;
    if (std::abs(tm1) > tj1 || std::abs(tm2) > tj2 || std::abs(tM) > tJ) return 0.0;
    if ((tj1 + tm1) % 2 || (tj2 + tm2) % 2 || (tJ + tM) % 2) return 0.0;
    const double tri = fact_h((tj1 + tj2 - tJ) / 2) * fact_h((tj1 - tj2 + tJ) / 2) *
                       fact_h((-tj1 + tj2 + tJ) / 2) / fact_h((tj1 + tj2 + tJ) / 2 + 1);
    const double pre = std::sqrt((tJ + 1) * tri * fact_h((tj1 + tm1) / 2) * fact_h((tj1 - tm1) / 2) *
                                 fact_h((tj2 + tm2) / 2) * fact_h((tj2 - tm2) / 2) * fact_h((tJ + tM) / 2) *
                                 fact_h((tJ - tM) / 2));
    double sum = 0.0;
    for (int k = 0; k < 100; ++k) {
        const int a1 = (tj1 + tj2 - tJ) / 2 - k, a2 = (tj1 - tm1) / 2 - k, a3 = (tj2 + tm2) / 2 - k;
        const int a4 = (tJ - tj2 + tm1) / 2 + k, a5 = (tJ - tj1 - tm2) / 2 + k;
        if (a1 < 0 || a2 < 0 || a3 < 0) break;
        if (a4 < 0 || a5 < 0) continue;
        sum += ((k & 1) ? -1.0 : 1.0) /
               (fact_h(k) * fact_h(a1) * fact_h(a2) * fact_h(a3) * fact_h(a4) * fact_h(a5));
    }
    return pre * sum;
}

// Wigner 3j (j1 j2 j3; m1 m2 m3), doubled arguments
double threej_h(int tj1, int tj2, int tj3, int tm1, int tm2, int tm3) {
    if (tm1 + tm2 + tm3 != 0) return 0.0;
    const double ph = (((tj1 - tj2 - tm3) / 2) % 2) ? -1.0 : 1.0;
    return ph * cg_h(tj1, tj2, tj3, tm1, tm2, -tm3) / std::sqrt(tj3 + 1.0);
}

dd host_dd(double x) {
    dd r;
    r.hi = (float)x;
    r.lo = (float)(x - (double)r.hi);
    return r;
}

std::vector<dd> to_dd(const std::vector<double> &v) {
    std::vector<dd> out(v.size());
    for (size_t i = 0; i < v.size(); ++i) out[i] = host_dd(v[i]);
    return out;
}

int plan_placement(Params &p, int smem_max) {
    const int n = p.n, N = p.N2;
    const long long nn = (long long)n * n;
    Placement &pl = p.place;
    auto align = [](int x) { return (x + 15) & ~15; };
    // fixed shared pieces
    int fixed = 0, fixed2 = 0;
    pl.off_piv = fixed; fixed += align((n + 8) * 4);
    pl.off_inv = fixed; fixed += align(n * 16);
    pl.off_red = fixed; fixed += align(40 * (kThreads / 32) * 8);  // 36 observable slots per warp
    pl.off_rot = fixed; fixed += align(p.rot_elems * 16);
    pl.off_vec = fixed; fixed += align((N + kNobs + 2 * p.nfom + p.obs.n_r1b) * 16);  // + phase tables
    // the Pfaffian matrix (N^2) shares storage with rho, kappa10, kappa01, K (4 n (n+1))
    const long long s_elems = std::max<long long>((long long)N * N, 4LL * n * (n + 1));
    const int bs = (int)(s_elems * 16), bt = (int)(nn * 16), by = (int)(2 * nn * 16), buv = (int)(2 * nn * 8);
    // Greedy: spill UV first, then Y, T and last S (the Pfaffian matrix, the most
    // reused). Measured at n = 64, where S alone exceeds 227 KB: everything in the
    // global slot with the freed shared memory serving as L1 beats keeping T + Y
    // in shared memory, so the greedy order (which ends with all four spilled)
    // is kept rather than a fullest-fit choice.
    int flags[4] = {1, 1, 1, 1};  // s, t, y, uv
    const int order[4] = {3, 2, 1, 0};
    auto total = [&]() { return fixed + flags[0] * bs + flags[1] * bt + flags[2] * by + flags[3] * buv; };
    for (int k = 0; k < 4 && total() > smem_max; ++k) flags[order[k]] = 0;
    if (total() > smem_max) return PNAMP_ERR_UNSUPPORTED;
    // species-split pairs with two gauge points in flight: after the fixed pieces, the compact
    // V0^T / U0^T diagonal blocks and two half regions, when they fit (pf: 213 KB)
    {
        const int h = n / 2;
        const int uvc = align(4 * h * h * 8);
        const long long need = (long long)align(fixed) + uvc + 2LL * half_layout(h).bytes;
        pl.sp2 = need <= smem_max ? 1 : 0;
        pl.off_uvc = align(fixed);
        pl.off_half = pl.off_uvc + uvc;
        if (pl.sp2) fixed2 = (int)need;
    }
    int off = fixed;
    pl.s_smem = flags[0]; pl.t_smem = flags[1]; pl.y_smem = flags[2]; pl.uv_smem = flags[3];
    if (pl.s_smem) { pl.off_s = off; off += bs; }
    if (pl.t_smem) { pl.off_t = off; off += bt; }
    if (pl.y_smem) { pl.off_y = off; off += by; }
    if (pl.uv_smem) { pl.off_uv = off; off += buv; }
    pl.smem_bytes = std::max(off, fixed2);
    long long g = 0;
    pl.g_x = g; g += nn;
    pl.g_b = g; g += 2 * nn;
    pl.g_p = g; g += 4 * nn;
    pl.g_rw = g; g += nn;
    pl.g_zr = g; g += nn;   // -Cscale Z0^-1 (reduced) or -Cscale Z0, in the point arithmetic
    pl.g_s = g; if (!pl.s_smem) g += s_elems;
    pl.g_t = g; if (!pl.t_smem) g += nn;
    pl.g_y = g; if (!pl.y_smem) g += 2 * nn;
    pl.g_uv = g; if (!pl.uv_smem) g += nn;  // 2 n^2 doubles = n^2 complex slots
    pl.slot_elems = (g + 15) & ~15LL;
    return PNAMP_OK;
}

int ensure_pairs(pnamp_ctx *c, int npairs) {
    if (npairs <= c->pair_cap) return PNAMP_OK;
    if (c->d_pairbuf) cudaFree(c->d_pairbuf);
    c->d_pairbuf = nullptr;
    c->pair_cap = 0;
    CK(cudaMalloc(&c->d_pairbuf, (size_t)npairs * c->p.pl.stride * sizeof(double)));
    c->pair_cap = npairs;
    return PNAMP_OK;
}

int ensure_batch(pnamp_ctx *c, int npairs) {
    if (npairs <= c->batch_cap) return PNAMP_OK;
    for (void *q : {(void *)c->d_uv, (void *)c->d_zres, (void *)c->d_status, (void *)c->d_proj})
        if (q) cudaFree(q);
    c->d_uv = c->d_zres = c->d_proj = nullptr;
    c->d_status = nullptr;
    c->batch_cap = 0;
    const long long nn = (long long)c->p.n * c->p.n;
    const long long fs = (long long)(kJJMax + 1) * kNK * kNK;
    CK(cudaMalloc(&c->d_uv, (size_t)npairs * 4 * nn * sizeof(double)));
    CK(cudaMalloc(&c->d_zres, (size_t)npairs * 2 * kNobs * c->p.n_euler * sizeof(double)));
    CK(cudaMalloc(&c->d_status, (size_t)npairs * c->p.n_euler * sizeof(int)));
    CK(cudaMalloc(&c->d_proj, (size_t)npairs * 2 * kProjFields * fs * sizeof(double)));
    c->batch_cap = npairs;
    return PNAMP_OK;
}


// Two-body density tables: the blocks of ME2B_Base_Full (PNAMP_ME2B_Base.f90:112-205)
// over the model space's orbits and the m sums of ZRho2B_Angles (PNAMP_Rho2B.f90:31-118).
struct R2Tables {
    std::vector<int> blocks;        // [nblocks][4]: tt (0 nn, 1 np, 2 pp), PP, J, number of states
    std::vector<int> states;        // [nstates][2]: orbits o1, o2 (first-appearance order of (n, l, j))
    std::vector<uint32_t> quads;    // packed k_i | k_j << 8 | k_k << 16 | k_l << 24, first-use order
    std::vector<int> ptr, tq;       // per element (bm, a_ij, a_kl): terms [ptr[e], ptr[e+1])
    std::vector<double> tc;         // cg1 cg2 / (2J + 1) of each term
};

int build_r2(int n, const int *t, const int *nn1, const int *l, const int *tj, const int *tm, R2Tables &r) {
    // orbits (n, l, 2j) in order of first appearance (protons first, .val order)
    std::vector<std::array<int, 3>> orb;
    std::vector<int> lev_orb(n);
    for (int k = 0; k < n; ++k) {
        const std::array<int, 3> key{nn1[k], l[k], tj[k]};
        int o = (int)(std::find(orb.begin(), orb.end(), key) - orb.begin());
        if (o == (int)orb.size()) orb.push_back(key);
        lev_orb[k] = o;
    }
    const int no = (int)orb.size();
    // level of (reference t: 1 proton / 0 neutron, orbit, 2m)
    std::vector<int> lev((size_t)2 * no * 16, -1);
    for (int k = 0; k < n; ++k) {
        if (tj[k] > 15 || std::abs(tm[k]) > tj[k]) return PNAMP_ERR_ARG;
        const int tr = (t[k] == -1) ? 1 : 0;
        lev[((size_t)tr * no + lev_orb[k]) * 16 + (tm[k] + tj[k]) / 2] = k;
    }
    auto level = [&](int tr, int o, int m2) { return lev[((size_t)tr * no + o) * 16 + (m2 + orb[o][2]) / 2]; };
    for (int o = 0; o < no; ++o)
        for (int tr = 0; tr < 2; ++tr)
            for (int m2 = -orb[o][2]; m2 <= orb[o][2]; m2 += 2)
                if (level(tr, o, m2) < 0) return PNAMP_ERR_UNSUPPORTED;  // orbit of one species only
    int nmax = 0;
    for (const auto &q : orb) nmax = std::max(nmax, q[0]);
    auto lj = [&](int o) { return (2 * orb[o][1] + orb[o][2] - 1) / 2; };
    auto ident = [&](int o) { return orb[o][0] + nmax * lj(o); };
    std::vector<int> sorted(no);
    for (int o = 0; o < no; ++o) sorted[o] = o;
    std::stable_sort(sorted.begin(), sorted.end(), [&](int a, int b) {
        return lj(a) != lj(b) ? lj(a) < lj(b) : orb[a][0] < orb[b][0];
    });
    std::vector<int> ljs;
    for (int o : sorted)
        if (ljs.empty() || ljs.back() != lj(o)) ljs.push_back(lj(o));
    // enumeration of PNAMP_ME2B_Base.f90:128-171 grouped by block (tt, PP, J)
    std::map<std::array<int, 3>, std::vector<std::array<int, 2>>> blk;
    for (int tt = 0; tt < 3; ++tt)
        for (int lj1 : ljs)
            for (int lj2 : ljs) {
                std::vector<int> o1s, o2s;
                for (int o : sorted) {
                    if (lj(o) == lj1) o1s.push_back(o);
                    if (lj(o) == lj2) o2s.push_back(o);
                }
                const int l1 = orb[o1s[0]][1], tj1 = orb[o1s[0]][2], l2 = orb[o2s[0]][1], tj2 = orb[o2s[0]][2];
                const int pp = (l1 + l2) % 2;
                for (int J = std::abs(tj1 - tj2) / 2; J <= (tj1 + tj2) / 2; ++J)
                    for (int o1 : o1s)
                        for (int o2 : o2s) {
                            if (tt != 1 && ident(o1) > ident(o2)) continue;
                            if (J % 2 == 1 && o1 == o2 && tt != 1) continue;
                            blk[{tt, pp, J}].push_back({o1, o2});
                        }
            }
    std::map<uint32_t, int> qidx;
    r.ptr.assign(1, 0);
    for (const auto &kv : blk) {
        const int tt = kv.first[0], J = kv.first[2];
        const int t1 = tt / 2, t2 = (tt + 1) / 2;
        const auto &st = kv.second;
        r.blocks.insert(r.blocks.end(), {tt, kv.first[1], J, (int)st.size()});
        for (const auto &a : st) r.states.insert(r.states.end(), {a[0], a[1]});
        for (const auto &ij : st)
            for (const auto &kl : st) {
                const int tji = orb[ij[0]][2], tjj = orb[ij[1]][2], tjk = orb[kl[0]][2], tjl = orb[kl[1]][2];
                for (int mi = -tji; mi <= tji; mi += 2)
                    for (int mj = -tjj; mj <= tjj; mj += 2) {
                        const double c1 = cg_h(tji, tjj, 2 * J, mi, mj, mi + mj);
                        for (int mk = -tjk; mk <= tjk; mk += 2) {
                            const int ml = mi + mj - mk;
                            if (std::abs(ml) > tjl) continue;
                            const double c2 = cg_h(tjk, tjl, 2 * J, mk, ml, mi + mj);
                            if (c1 * c2 == 0.0) continue;
                            const uint32_t key = (uint32_t)level(t1, ij[0], mi) | ((uint32_t)level(t2, ij[1], mj) << 8) |
                                                 ((uint32_t)level(t1, kl[0], mk) << 16) |
                                                 ((uint32_t)level(t2, kl[1], ml) << 24);
                            auto it = qidx.find(key);
                            int q;
                            if (it == qidx.end()) {
                                q = (int)r.quads.size();
                                qidx.emplace(key, q);
                                r.quads.push_back(key);
                            } else {
                                q = it->second;
                            }
                            r.tq.push_back(q);
                            r.tc.push_back(c1 * c2 / (2 * J + 1));
                        }
                    }
                r.ptr.push_back((int)r.tq.size());
            }
    }
    return PNAMP_OK;
}

// ---------------------------------------------------------------- stage timing
// Events around each launch of a batch call, on the launching stream, when timing is on.
enum { kStageSetup = 0, kStagePoints = 1, kStageContract = 2, kStageFinish = 3, kStages = 4 };
int stage_begin(pnamp_ctx *c, cudaStream_t st) {
    if (!c->timing) return -1;
    const int k = (int)c->ev_marks.size();
    while ((int)c->ev_pool.size() < 2 * (k + 1)) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return -1;
        c->ev_pool.push_back(e);
    }
    if (cudaEventRecord(c->ev_pool[2 * k], st) != cudaSuccess) return -1;
    return k;
}
void stage_end(pnamp_ctx *c, cudaStream_t st, int k, int stage) {
    if (k < 0) return;
    if (cudaEventRecord(c->ev_pool[2 * k + 1], st) == cudaSuccess) c->ev_marks.push_back({stage, 2 * k, 2 * k + 1});
}

// ---------------------------------------------------------------- tensor-core contraction
// Tables of the two bilinear forms the two-body energy regroups into (contract_tc.cu):
// particle-hole entries s_e = rho(r, c), labelled (m_r - m_c, t_r - t_c, parity) and packed
// with their negated labels into groups of <= kTcGroupCap storage entries; particle-particle
// pair entries (i < j) labelled (m_i + m_j, t_i + t_j, parity) and packed the same way. Each
// group's storage range is padded to 64 entries (one TMA/UMMA K chunk); its square matrix
// (rows = output entries, columns = operand entries) is stacked into one [rows][kmax]
// array and kept as three bf16 terms t0 + t1 + t2 of each FP64 value.
constexpr int kTcGroupCap = 256;

uint16_t bf16_rn_host(float f) {
    uint32_t b;
    memcpy(&b, &f, 4);
    if ((b & 0x7fffffffu) > 0x7f800000u) return 0x7fc0;       // NaN
    b += 0x7fffu + ((b >> 16) & 1u);                          // round to nearest, ties to even
    return (uint16_t)(b >> 16);
}
double bf16_value(uint16_t h) {
    const uint32_t b = (uint32_t)h << 16;
    float f;
    memcpy(&f, &b, 4);
    return (double)f;
}

template <class Key>
std::vector<std::vector<Key>> pack_groups(const std::vector<std::vector<Key>> &units,
                                          const std::map<Key, std::vector<int>> &members) {
    // first fit, largest units first (ties keep label order)
    std::vector<int> order(units.size());
    for (size_t i = 0; i < units.size(); ++i) order[i] = (int)i;
    auto size_of = [&](int u) {
        int sz = 0;
        for (const Key &k : units[u]) sz += (int)members.at(k).size();
        return sz;
    };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return size_of(a) > size_of(b); });
    std::vector<std::vector<Key>> groups;
    std::vector<int> fill;
    for (int u : order) {
        const int sz = size_of(u);
        size_t g = 0;
        for (; g < groups.size(); ++g)
            if (fill[g] + sz <= kTcGroupCap) break;
        if (g == groups.size()) {
            groups.emplace_back();
            fill.push_back(0);
        }
        groups[g].insert(groups[g].end(), units[u].begin(), units[u].end());
        fill[g] += sz;
    }
    return groups;
}

int build_tc(pnamp_ctx *c) {
    const int n = c->p.n;
    using L3 = std::array<int, 3>;
    std::map<L3, std::vector<int>> ph, pp;   // label -> entries (r << 8 | c), row-major order
    for (int r = 0; r < n; ++r)
        for (int q = 0; q < n; ++q)
            ph[{c->sp_tm[r] - c->sp_tm[q], c->sp_t[r] - c->sp_t[q], (c->sp_l[r] + c->sp_l[q]) & 1}].push_back(
                (r << 8) | q);
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j)
            pp[{c->sp_tm[i] + c->sp_tm[j], c->sp_t[i] + c->sp_t[j], (c->sp_l[i] + c->sp_l[j]) & 1}].push_back(
                (i << 8) | j);
    std::vector<std::vector<L3>> ph_units, pp_units;
    for (const auto &kv : ph) {
        const L3 L = kv.first, N = {-L[0], -L[1], L[2]};
        if (N < L && ph.count(N)) continue;          // the pair (N, L) was made at N
        ph_units.push_back(N == L || !ph.count(N) ? std::vector<L3>{L} : std::vector<L3>{L, N});
    }
    for (const auto &kv : pp) pp_units.push_back({kv.first});
    const auto ph_groups = pack_groups(ph_units, ph), pp_groups = pack_groups(pp_units, pp);

    std::vector<int> pos_ph((size_t)n * n, -1), pos_pp((size_t)n * n, -1);
    c->tc_groups.clear();
    c->tc_src.clear();
    int off = 0, rowbase = 0, kmax = 0;
    auto place = [&](const std::vector<std::vector<L3>> &groups, const std::map<L3, std::vector<int>> &mem,
                     std::vector<int> &pos, int kind, int yoff0) {
        for (const auto &g : groups) {
            TcGroup G;
            G.kind = kind;
            G.off = off;
            int d = 0;
            for (const L3 &k : g)
                for (int e : mem.at(k)) {
                    pos[(size_t)(e >> 8) * n + (e & 255)] = off + d++;
                    c->tc_src.push_back(e);
                }
            G.dpad = (d + 63) / 64 * 64;
            for (int k = d; k < G.dpad; ++k) c->tc_src.push_back(-1);
            G.rowbase = rowbase;
            G.yoff = kind ? off - yoff0 : 0;
            off += G.dpad;
            rowbase += G.dpad;
            kmax = std::max(kmax, G.dpad);
            c->tc_groups.push_back(G);
        }
    };
    place(ph_groups, ph, pos_ph, 0, 0);
    c->tc_nph = off;
    place(pp_groups, pp, pos_pp, 1, c->tc_nph);
    c->tc_nk = off;
    c->tc_kmax = kmax;
    c->tc_rows = rowbase;
    // group of each storage position
    std::vector<int> grp_of(off, -1);
    for (size_t g = 0; g < c->tc_groups.size(); ++g)
        for (int k = 0; k < c->tc_groups[g].dpad; ++k) grp_of[c->tc_groups[g].off + k] = (int)g;
    std::vector<double> mat((size_t)rowbase * kmax, 0.0);
    auto add = [&](int e1, int e2, double v) {  // storage positions (row, column) of one group
        const TcGroup &G = c->tc_groups[grp_of[e1]];
        mat[(size_t)(G.rowbase + e1 - G.off) * kmax + (e2 - G.off)] += v;
    };
    auto ph_at = [&](int r, int q) { return pos_ph[(size_t)r * n + q]; };
    auto pp_at = [&](int i, int j) { return pos_pp[(size_t)i * n + j]; };
    for (size_t e = 0; e < c->h_rec_idx.size(); ++e) {
        const uint32_t pk = c->h_rec_idx[e];
        const int i = pk & 0xff, j = (pk >> 8) & 0xff, k = (pk >> 16) & 0xff, l = pk >> 24;
        const double V = c->h_rec_v[e];
        const bool d = (i + j) != (k + l);
        // particle hole: V rho_ki rho_lj - V rho_li rho_kj + d (V rho_ik rho_jl - V rho_jk rho_il)
        // as s_e1 M s_e2 with the second factor read transposed
        add(ph_at(k, i), ph_at(l, j), V);
        add(ph_at(l, i), ph_at(k, j), -V);
        if (d) {
            add(ph_at(i, k), ph_at(j, l), V);
            add(ph_at(j, k), ph_at(i, l), -V);
        }
        // particle particle: V/4 (K01_ij K10_kl + d K01_kl K10_ij)
        if (i >= j || k >= l) return PNAMP_ERR_ARG;
        add(pp_at(i, j), pp_at(k, l), 0.25 * V);
        if (d) add(pp_at(k, l), pp_at(i, j), 0.25 * V);
    }
    std::vector<uint16_t> terms[3];
    for (auto &t : terms) t.resize(mat.size());
    for (size_t q = 0; q < mat.size(); ++q) {
        double r = mat[q];
        for (int sp = 0; sp < 3; ++sp) {
            terms[sp][q] = bf16_rn_host((float)r);
            r -= bf16_value(terms[sp][q]);
        }
    }
    CK(cudaMalloc(&c->d_tc_groups, c->tc_groups.size() * sizeof(TcGroup)));
    CK(cudaMemcpy(c->d_tc_groups, c->tc_groups.data(), c->tc_groups.size() * sizeof(TcGroup),
                  cudaMemcpyHostToDevice));
    CK(cudaMalloc(&c->d_tc_src, c->tc_src.size() * sizeof(int)));
    CK(cudaMemcpy(c->d_tc_src, c->tc_src.data(), c->tc_src.size() * sizeof(int), cudaMemcpyHostToDevice));
    for (int sp = 0; sp < 3; ++sp) {
        CK(cudaMalloc(&c->d_tc_mat[sp], mat.size() * sizeof(uint16_t)));
        CK(cudaMemcpy(c->d_tc_mat[sp], terms[sp].data(), mat.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
    }
    CK(cudaMalloc(&c->d_tc_err, sizeof(int)));
    CK(prepare_contract());
    c->tc_built = true;
    return PNAMP_OK;
}

// Staging for `pts` kernel points: X and Y rows per bf16 term, weights, E2.
int ensure_tc_staging(pnamp_ctx *c, long long pts) {
    // a form switch from BF16x3 to BF16x6 needs the third term's arrays too
    if (pts <= c->tc_cap_pts && c->tc_splits <= c->tc_cap_splits) return PNAMP_OK;
    pts = std::max(pts, c->tc_cap_pts);
    for (int sp = 0; sp < 3; ++sp) {
        if (c->d_tc_x[sp]) cudaFree(c->d_tc_x[sp]);
        if (c->d_tc_y[sp]) cudaFree(c->d_tc_y[sp]);
        c->d_tc_x[sp] = c->d_tc_y[sp] = nullptr;
    }
    if (c->d_tc_w) cudaFree(c->d_tc_w);
    if (c->d_tc_e2) cudaFree(c->d_tc_e2);
    c->d_tc_w = c->d_tc_e2 = nullptr;
    c->tc_cap_pts = 0;
    c->tc_cap_splits = 0;
    const int npp = c->tc_nk - c->tc_nph;
    for (int sp = 0; sp < c->tc_splits; ++sp) {
        CK(cudaMalloc(&c->d_tc_x[sp], (size_t)pts * 2 * c->tc_nk * sizeof(uint16_t)));
        CK(cudaMalloc(&c->d_tc_y[sp], (size_t)pts * 2 * npp * sizeof(uint16_t)));
    }
    CK(cudaMalloc(&c->d_tc_w, (size_t)pts * 2 * sizeof(double)));
    CK(cudaMalloc(&c->d_tc_e2, (size_t)pts * 2 * sizeof(double)));
    c->tc_cap_pts = pts;
    c->tc_cap_splits = c->tc_splits;
    return PNAMP_OK;
}

// Points per launch of the tensor-core forms: the staging of one chunk stays under
// min(24 GiB, half the free device memory), and at least one pair (or item) fits.
long long tc_chunk_points(pnamp_ctx *c, long long unit_pts) {
    const long long per_pt = (long long)c->tc_splits * 2 * (2LL * c->tc_nk - c->tc_nph) * 2 + 32;
    size_t fr = 0, tot = 0;
    long long budget = 24LL << 30;
    if (cudaMemGetInfo(&fr, &tot) == cudaSuccess) budget = std::min<long long>(budget, (long long)(fr / 2));
    const long long units = std::max<long long>(1, budget / per_pt / unit_pts);
    return units * unit_pts;
}

// The tensor-core forms: setup, then per chunk the point kernel (double-float algebra, densities
// staged), the contraction and the per-item sum into ZRES(:, 7). `items` selects (pair, Euler
// point) entries as pnamp_batch_items_device does; NULL means every Euler point of every pair.
int tc_run(pnamp_ctx *c, int npairs, const double *d_uv, double *d_zres, int *d_status, cudaStream_t st,
           const int *items, long long nitems) {
    if (c->p.norm_only) return PNAMP_ERR_STATE;
    int rc;
    if (!c->tc_built && (rc = build_tc(c)) != PNAMP_OK) return rc;
    int mk = stage_begin(c, st);
    CK(launch_setup(c->p, npairs, d_uv, c->d_pairbuf, st));
    stage_end(c, st, mk, kStageSetup);
    const int P = c->p.n_euler, G = c->p.n_gauge;
    const long long total_items = items ? nitems : (long long)npairs * P;
    const long long chunk_pts =
        std::min<long long>(tc_chunk_points(c, items ? (long long)G : (long long)P * G), total_items * G);
    if ((rc = ensure_tc_staging(c, chunk_pts)) != PNAMP_OK) return rc;
    for (int sp = 0; sp < c->tc_splits; ++sp)   // every term the kernels write and read must exist
        if (!c->d_tc_x[sp] || !c->d_tc_y[sp] || !c->d_tc_mat[sp]) return PNAMP_ERR_STATE;
    if (!c->d_tc_w || !c->d_tc_e2 || chunk_pts > c->tc_cap_pts) return PNAMP_ERR_STATE;
    const long long chunk_items = chunk_pts / G;
    Params q = c->p;
    q.tc_splits = c->tc_splits;
    q.tc_nk = c->tc_nk;
    q.tc_nph = c->tc_nph;
    q.tc_src = c->d_tc_src;
    for (int sp = 0; sp < 3; ++sp) {
        q.tc_x[sp] = c->d_tc_x[sp];
        q.tc_y[sp] = c->d_tc_y[sp];
    }
    q.tc_w = c->d_tc_w;
    TcArgs a;
    memset(&a, 0, sizeof(a));
    a.splits = c->tc_splits;
    a.ngroups = (int)c->tc_groups.size();
    a.nk = c->tc_nk;
    a.npp = c->tc_nk - c->tc_nph;
    a.groups = c->d_tc_groups;
    for (int sp = 0; sp < 3; ++sp) {
        a.x[sp] = c->d_tc_x[sp];
        a.y[sp] = c->d_tc_y[sp];
    }
    a.e2 = c->d_tc_e2;
    a.err = c->d_tc_err;
    const void *mat[3] = {c->d_tc_mat[0], c->d_tc_mat[1], c->d_tc_mat[2]};
    const long long zstride = 2LL * kNobs * P;
    for (long long i0 = 0; i0 < total_items; i0 += chunk_items) {
        const long long cnt = std::min<long long>(chunk_items, total_items - i0);
        CK(cudaMemsetAsync(c->d_tc_err, 0, sizeof(int), st));
        a.npts = cnt * G;
        if (items) {
            const int2 *it = reinterpret_cast<const int2 *>(items) + i0;
            const int grid = (int)std::min<long long>(c->grid_form[1], cnt);
            mk = stage_begin(c, st);
            CK(launch_points(q, npairs, c->d_pairbuf, c->d_scratch, grid, d_zres, d_status, st, it, cnt));
            stage_end(c, st, mk, kStagePoints);
            mk = stage_begin(c, st);
            CK(launch_contract(a, mat, c->tc_rows, c->tc_kmax, c->nsm, st));
            stage_end(c, st, mk, kStageContract);
            mk = stage_begin(c, st);
            CK(launch_contract_finish(npairs, P, G, cnt, it, c->d_tc_w, c->d_tc_e2, d_zres, d_status, c->d_tc_err,
                                      st));
            stage_end(c, st, mk, kStageFinish);
        } else {
            const int pair0 = (int)(i0 / P), np = (int)(cnt / P);
            mk = stage_begin(c, st);
            CK(launch_points(q, np, c->d_pairbuf + (long long)pair0 * c->p.pl.stride, c->d_scratch,
                             c->grid_form[1], d_zres + pair0 * zstride, d_status + (long long)pair0 * P, st));
            stage_end(c, st, mk, kStagePoints);
            mk = stage_begin(c, st);
            CK(launch_contract(a, mat, c->tc_rows, c->tc_kmax, c->nsm, st));
            stage_end(c, st, mk, kStageContract);
            mk = stage_begin(c, st);
            CK(launch_contract_finish(np, P, G, cnt, nullptr, c->d_tc_w, c->d_tc_e2, d_zres + pair0 * zstride,
                                      d_status + (long long)pair0 * P, c->d_tc_err, st));
            stage_end(c, st, mk, kStageFinish);
        }
    }
    return PNAMP_OK;
}

}  // namespace

extern "C" {

const char *pnamp_strerror(int code) {
    switch (code) {
        case PNAMP_OK: return "ok";
        case PNAMP_ERR_ARG: return "invalid argument";
        case PNAMP_ERR_CUDA: return "CUDA runtime error or no CUDA device";
        case PNAMP_ERR_NOMEM: return "device allocation failed";
        case PNAMP_ERR_SINGULAR_U: return "U of a vacuum is singular (zbareover/Pfaf_Over LU failure)";
        case PNAMP_ERR_UNSUPPORTED: return "size not supported by this build";
        case PNAMP_ERR_STATE: return "call order violated";
        case PNAMP_ERR_SCRATCH_LIMIT:
            return "request exceeds the fixed no-allocation scratch (PNAMP_NOALLOC_SCRATCH_BYTES)";
        case PNAMP_ERR_SMALL_NORM: return "projected norm too small (|N^0| <= 1e-8) to normalise the density";
        default: return "unknown error";
    }
}

const char *pnamp_version(void) { return "sccm_gb300 pnamp 0.1 (sm_103a, fp64)"; }

int pnamp_n_euler(const pnamp_ctx *ctx) { return ctx ? ctx->p.n_euler : -1; }

int pnamp_set_form(pnamp_ctx *ctx, int form) {
    if (!ctx) return PNAMP_ERR_ARG;
    switch (form) {
        case PNAMP_FORM_FP64:
        case PNAMP_FORM_DF64:
            ctx->p.form = form;
            ctx->tc_splits = 0;
            return PNAMP_OK;
        case PNAMP_FORM_TC3:
        case PNAMP_FORM_TC6:
            ctx->p.form = PNAMP_FORM_DF64;   // the per-point algebra of the mixed form
            ctx->tc_splits = form == PNAMP_FORM_TC3 ? 2 : 3;
            return PNAMP_OK;
        default:
            return PNAMP_ERR_ARG;
    }
}

int pnamp_set_outputs(pnamp_ctx *ctx, int outputs) {
    if (!ctx || (outputs != PNAMP_OUT_ALL && outputs != PNAMP_OUT_NORM)) return PNAMP_ERR_ARG;
    ctx->p.norm_only = outputs == PNAMP_OUT_NORM ? 1 : 0;
    return PNAMP_OK;
}

void pnamp_free(pnamp_ctx *ctx) {
    if (!ctx) return;
    for (void *q : ctx->allocs) cudaFree(q);
    if (ctx->d_r1b) cudaFree(ctx->d_r1b);
    for (void *q : {(void *)ctx->d_r2q, (void *)ctx->d_r2acc, (void *)ctx->d_r2out})
        if (q) cudaFree(q);
    for (void *q : {(void *)ctx->d_pairbuf, (void *)ctx->d_scratch, (void *)ctx->d_uv, (void *)ctx->d_zres,
                    (void *)ctx->d_status, (void *)ctx->d_proj, (void *)ctx->d_projq})
        if (q) cudaFree(q);
    for (int sp = 0; sp < 3; ++sp)
        for (void *q : {(void *)ctx->d_tc_mat[sp], (void *)ctx->d_tc_x[sp], (void *)ctx->d_tc_y[sp]})
            if (q) cudaFree(q);
    for (void *q : {(void *)ctx->d_tc_groups, (void *)ctx->d_tc_src, (void *)ctx->d_tc_w, (void *)ctx->d_tc_e2,
                    (void *)ctx->d_tc_err})
        if (q) cudaFree(q);
    for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

int pnamp_init(const pnamp_space *sp, const pnamp_hamiltonian *h, const pnamp_mesh *m, pnamp_ctx **out) {
    if (!out) return PNAMP_ERR_ARG;
    *out = nullptr;
    if (!sp || !h || !m) return PNAMP_ERR_ARG;
    const int n = sp->nlev;
    if (n < 2 || n % 2 || !sp->t || !sp->n || !sp->l || !sp->twoj || !sp->twom) return PNAMP_ERR_ARG;
    if (n > PNAMP_MAX_NLEV) return PNAMP_ERR_UNSUPPORTED;
    if (sp->nprot < 0 || sp->nneut < 0) return PNAMP_ERR_ARG;
    const int hh = n / 2;
    // species halves and rotation blocks: runs of 2j+1 states of one (t,n,l,j), m = j..-j
    std::vector<int> blk_start, blk_size, blk_tj, blk_roff, row_blk(n), twom(sp->twom, sp->twom + n);
    int rot = 0;
    for (int a = 0; a < n;) {
        const int tj = sp->twoj[a];
        if (tj < 1 || tj % 2 == 0 || tj > 15) return PNAMP_ERR_ARG;
        if ((a < hh) != (sp->t[a] == -1)) return PNAMP_ERR_ARG;
        const int d = tj + 1;
        if (a + d > n) return PNAMP_ERR_ARG;
        for (int i = 0; i < d; ++i) {
            const int b = a + i;
            if (sp->t[b] != sp->t[a] || sp->n[b] != sp->n[a] || sp->l[b] != sp->l[a] || sp->twoj[b] != tj ||
                sp->twom[b] != tj - 2 * i)
                return PNAMP_ERR_ARG;
            row_blk[b] = (int)blk_start.size();
        }
        if ((int)blk_start.size() >= kMaxBlocks) return PNAMP_ERR_UNSUPPORTED;
        blk_start.push_back(a);
        blk_size.push_back(d);
        blk_tj.push_back(tj);
        blk_roff.push_back(rot);
        rot += d * d;
        a += d;
    }
    // mesh
    if (m->nalp < 1 || m->nbet < 1 || m->ngam < 1 || m->nfom < 1) return PNAMP_ERR_ARG;
    if (m->nfom > 64) return PNAMP_ERR_UNSUPPORTED;
    if (m->ncosbet != 1 && m->ncosbet != 2) return PNAMP_ERR_ARG;
    if (!m->alpha || !m->beta || !m->gamma || !m->walp || !m->wbet || !m->wgam) return PNAMP_ERR_ARG;
    const int nbu = std::max(m->nbet / m->ncosbet, 1);
    std::vector<double> euler;
    for (int k = 0; k < nbu; ++k)  // beta outer, alpha, gamma inner (Kernel3D.f90:200-217)
        for (int ka = 0; ka < m->nalp; ++ka)
            for (int kg = 0; kg < m->ngam; ++kg) {
                euler.push_back(m->alpha[ka]);
                euler.push_back(m->beta[k]);
                euler.push_back(m->gamma[kg]);
                euler.push_back(m->walp[ka] * m->wbet[k] * m->wgam[kg] * m->ncosbet);
            }
    // two-body list
    if (h->nrec < 0 || (h->nrec > 0 && (!h->ka || !h->kb || !h->kc || !h->kd || !h->vbar))) return PNAMP_ERR_ARG;
    if (!h->t1b) return PNAMP_ERR_ARG;
    std::vector<uint32_t> rec_idx(h->nrec);
    std::vector<double> rec_v(h->vbar, h->vbar + h->nrec);
    for (int e = 0; e < h->nrec; ++e) {
        const int a = h->ka[e] - 1, b = h->kb[e] - 1, c = h->kc[e] - 1, d = h->kd[e] - 1;
        if (a < 0 || b < 0 || c < 0 || d < 0 || a >= n || b >= n || c >= n || d >= n) return PNAMP_ERR_ARG;
        rec_idx[e] = (uint32_t)a | ((uint32_t)b << 8) | ((uint32_t)c << 16) | ((uint32_t)d << 24);
    }
    // proton-neutron records (a, c protons; b, d neutrons) last: for species-split pairs half
    // of their terms vanish and the point kernel takes a shorter path over that range
    int nrec_gen = 0;
    {
        std::vector<uint32_t> gi, pi;
        std::vector<double> gv, pv;
        for (int e = 0; e < h->nrec; ++e) {
            const int a = rec_idx[e] & 0xff, b = (rec_idx[e] >> 8) & 0xff, c = (rec_idx[e] >> 16) & 0xff,
                      d = rec_idx[e] >> 24;
            const bool pn = a < hh && b >= hh && c < hh && d >= hh;
            (pn ? pi : gi).push_back(rec_idx[e]);
            (pn ? pv : gv).push_back(rec_v[e]);
        }
        nrec_gen = (int)gi.size();
        gi.insert(gi.end(), pi.begin(), pi.end());
        gv.insert(gv.end(), pv.begin(), pv.end());
        rec_idx.swap(gi);
        rec_v.swap(gv);
    }
    std::vector<uint32_t> h_rec_idx = rec_idx;
    std::vector<double> h_rec_v = rec_v;
    // one-body tables
    std::vector<int> t1b_idx;
    std::vector<double> t1b_val;
    for (int a = 0; a < n; ++a)
        for (int c = 0; c < n; ++c) {  // sum_{a,c} rho(c,a) t(a,c)
            const double v = h->t1b[a + (size_t)c * n];
            if (v != 0.0) {
                t1b_idx.push_back(c * 256 + a);  // row c, column a of rho
                t1b_val.push_back(v);
            }
        }
    std::vector<int> q_idx;
    std::vector<double> q_val;
    ObsTables ot{};
    ot.q_off[0] = 0;
    for (int q = 0; q < kNTrace; ++q) {
        if (h->q2) {
            const double *Q = h->q2 + (size_t)(q % 5) * n * n;
            for (int a = 0; a < hh; ++a)
                for (int b = 0; b < n; ++b) {
                    // ZQ2: Q(a,b) rho(b,a); ZQ2t: Q(b,a) rho(b,a), proton rows a
                    const double v = (q < 5) ? Q[a + (size_t)b * n] : Q[b + (size_t)a * n];
                    if (v != 0.0) {
                        q_idx.push_back(b * 256 + a);  // row b, column a of rho
                        q_val.push_back(v);
                    }
                }
        }
        ot.q_off[q + 1] = (int)q_idx.size();
    }
    // J operators (zJiME, PNAMP_ME1B.f90:332-422) as ladder coefficients: within a
    // block m decreases by 1 from one state to the next, so J+ (m -> m+1) links
    // a+1 -> a and J- links a-1 -> a.
    std::vector<double> jpv(n, 0.0), jmv(n, 0.0), mzv(n), jj1(n);
    for (int a = 0; a < n; ++a) {
        const double j = sp->twoj[a] / 2.0, mm = sp->twom[a] / 2.0;
        jj1[a] = j * (j + 1.0);
        mzv[a] = mm;
        if (a + 1 < n && row_blk[a + 1] == row_blk[a]) jpv[a] = std::sqrt(j * (j + 1.0) - (mm - 1.0) * mm);
        if (a >= 1 && row_blk[a - 1] == row_blk[a]) jmv[a] = std::sqrt(j * (j + 1.0) - (mm + 1.0) * mm);
    }

    pnamp_ctx *c = new pnamp_ctx();
    int dev = 0, rc = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        delete c;
        return PNAMP_ERR_CUDA;
    }
    Params &p = c->p;
    p.n = n;
    p.h = hh;
    p.N2 = 2 * n;
    p.nprot = sp->nprot;
    p.nneut = sp->nneut;
    p.n_euler = (int)(euler.size() / 4);
    p.nfom = m->nfom;
    p.n_gauge = m->nfom * m->nfom;
    p.cscale = m->cscale;
    p.e0 = h->e0;
    {
        const long long aaa = (long long)n * (n + 1) / 2;
        const double snpfaf = (aaa % 2) ? -1.0 : 1.0;
        const int ex = n * m->iscale / 2;
        p.vacfac = snpfaf * std::pow(10.0, -2.0 * ex);
    }
    p.iE2 = h->q2 ? 1 : 0;
    p.nblk = (int)blk_start.size();
    p.rot_elems = rot;
    p.nrec = h->nrec;
    p.nrec_gen = nrec_gen;
    p.pl.make(n);
    c->core_prot = sp->core_prot;
    c->core_neut = sp->core_neut;
    c->axial = (m->nalp * m->ngam == 1) ? 1 : 0;
    std::vector<double> fact(24);
    fact[0] = 1.0;
    for (int k = 1; k < 24; ++k) fact[k] = fact[k - 1] * k;
#define UP(vec, dst)                                   \
    if ((rc = dev_upload(c, vec, &(dst))) != PNAMP_OK) { \
        pnamp_free(c);                                 \
        return rc;                                     \
    }
    UP(blk_start, p.blk_start);
    UP(blk_size, p.blk_size);
    UP(blk_tj, p.blk_tj);
    UP(blk_roff, p.blk_roff);
    UP(row_blk, p.row_blk);
    UP(twom, p.twom);
    UP(euler, p.euler);
    {
        std::vector<double> gph(2 * (size_t)m->nfom * m->nfom);
        const double twopi = 6.283185307179586476925287;
        for (int lp = 0; lp < m->nfom; ++lp)
            for (int ln = 0; ln < m->nfom; ++ln) {
                const double a = -(twopi * lp / m->nfom * sp->nprot + twopi * ln / m->nfom * sp->nneut);
                gph[2 * (lp * m->nfom + ln)] = std::cos(a);
                gph[2 * (lp * m->nfom + ln) + 1] = std::sin(a);
            }
        UP(gph, p.gphase);
    }
    UP(fact, p.fact);
    UP(rec_idx, p.rec_idx);
    UP(rec_v, p.rec_v);
    const std::vector<dd> rec_vd = to_dd(rec_v), jp_d = to_dd(jpv), jm_d = to_dd(jmv), mz_d = to_dd(mzv);
    UP(rec_vd, p.rec_vd);
    ot.n_t1b = (int)t1b_idx.size();
    UP(t1b_idx, ot.t1b_idx);
    UP(t1b_val, ot.t1b_val);
    UP(q_idx, ot.q_idx);
    UP(q_val, ot.q_val);
    UP(jpv, ot.jp);
    UP(jmv, ot.jm);
    UP(mzv, ot.mz);
    UP(jj1, ot.jj1);
    UP(jp_d, ot.jp_d);
    UP(jm_d, ot.jm_d);
    UP(mz_d, ot.mz_d);
    {
        const std::vector<dd> jj1_d = to_dd(jj1), t1b_d = to_dd(t1b_val), q_d = to_dd(q_val);
        UP(jj1_d, ot.jj1_d);
        UP(t1b_d, ot.t1b_val_d);
        UP(q_d, ot.q_val_d);
    }
    {   // one-body density blocks of ZRho1B_Angles (PNAMP_Rho1B.f90:14-29): states k1, k2 of the
        // same isospin, lj and m; it = 1 for protons (t = -1), 0 for neutrons; ordered it, lj, n1, n2
        // as Write_ME1B loops (PNAMP_Rho1B.f90:80-88)
        std::map<std::vector<int>, std::vector<int>> blocks;
        for (int k1 = 0; k1 < n; ++k1)
            for (int k2 = 0; k2 < n; ++k2) {
                const int lj1 = (2 * sp->l[k1] + sp->twoj[k1] - 1) / 2, lj2 = (2 * sp->l[k2] + sp->twoj[k2] - 1) / 2;
                if (sp->t[k1] != sp->t[k2] || lj1 != lj2 || sp->twom[k1] != sp->twom[k2]) continue;
                const int it = sp->t[k1] == -1 ? 1 : 0;
                blocks[{it, lj1, sp->n[k1] - 1, sp->n[k2] - 1, sp->twoj[k1]}].push_back(k1 * 256 + k2);
            }
        std::vector<int> off{0}, idx;
        std::vector<double> val;
        if ((int)blocks.size() <= kMaxR1B) {
            for (const auto &kv : blocks) {
                c->r1b_it.push_back(kv.first[0]);
                c->r1b_lj.push_back(kv.first[1]);
                c->r1b_n1.push_back(kv.first[2]);
                c->r1b_n2.push_back(kv.first[3]);
                c->r1b_twoj.push_back(kv.first[4]);
                for (int e : kv.second) {
                    idx.push_back(e);
                    val.push_back(1.0 / std::sqrt(kv.first[4] + 1.0));
                }
                off.push_back((int)idx.size());
            }
        }
        ot.n_r1b = (int)c->r1b_it.size();
        UP(off, ot.r1b_off);
        if (!idx.empty()) {
            UP(idx, ot.r1b_idx);
            UP(val, ot.r1b_val);
            const std::vector<dd> val_d = to_dd(val);
            UP(val_d, ot.r1b_val_d);
        }
        for (size_t e = 3; e < euler.size(); e += 4) c->euler_w.push_back(euler[e]);
        c->h_rec_idx.swap(h_rec_idx);
        c->h_rec_v.swap(h_rec_v);
        c->sp_t.assign(sp->t, sp->t + n);
        c->sp_n.assign(sp->n, sp->n + n);
        c->sp_l.assign(sp->l, sp->l + n);
        c->sp_tj.assign(sp->twoj, sp->twoj + n);
        c->sp_tm.assign(sp->twom, sp->twom + n);
    }
#undef UP
    p.obs = ot;
    int smem_optin = 0, nsm = 0;
    if (cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        pnamp_free(c);
        return PNAMP_ERR_CUDA;
    }
    if (prepare_setup(n) != cudaSuccess) {
        pnamp_free(c);
        return PNAMP_ERR_CUDA;
    }
    // kMultiSmemTail bytes stay free at the end for the multi-context kernel's work counter
    if ((rc = plan_placement(p, smem_optin - kMultiSmemTail)) != PNAMP_OK) {
        pnamp_free(c);
        return rc;
    }
    for (int form = 0; form < 2; ++form) {
        int per_sm = 0;
        if (set_point_smem(form, p.place.smem_bytes) != cudaSuccess ||
            point_blocks_per_sm(form, p.place.smem_bytes, &per_sm) != cudaSuccess || per_sm < 1) {
            pnamp_free(c);
            return PNAMP_ERR_CUDA;
        }
        c->grid_form[form] = nsm * per_sm;
    }
    c->nsm = nsm;
    p.form = 0;
    p.norm_only = 0;
    p.n_r2q = 0;  // two-body density launches set their own copy
    p.r2q = nullptr;
    p.r2acc = nullptr;
    c->grid = std::max(c->grid_form[0], c->grid_form[1]);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        pnamp_free(c);
        return PNAMP_ERR_CUDA;
    }
    if (cudaMalloc(&c->d_scratch, (size_t)c->grid * p.place.slot_elems * sizeof(zc)) != cudaSuccess) {
        pnamp_free(c);
        return PNAMP_ERR_NOMEM;
    }
    if (cudaMalloc(&c->d_projw, (size_t)p.n_euler * kNJKK * sizeof(zc)) != cudaSuccess) {
        pnamp_free(c);
        return PNAMP_ERR_NOMEM;
    }
    {   // 3j symbols (J1 2 J2; -K1 mu K1-mu) in the order of project_q_kernel's outputs
        std::vector<double> tj;
        for (int J2 = 0; J2 <= kJJMax; J2 += 2)
            for (int dJ = 0; dJ < 3; ++dJ) {
                const int J1 = J2 + dJ;
                for (int r = 0; r < (2 * J1 + 1) * (2 * J2 + 1); ++r) {
                    const int K1 = r / (2 * J2 + 1) - J1;
                    for (int mu = -2; mu <= 2; ++mu)
                        tj.push_back(threej_h(2 * J1, 4, 2 * J2, -2 * K1, 2 * mu, 2 * (K1 - mu)));
                }
            }
        if ((int)tj.size() != 5 * n_q_outputs() || (rc = dev_upload(c, tj, &c->d_tj)) != PNAMP_OK) {
            pnamp_free(c);
            return rc ? rc : PNAMP_ERR_STATE;
        }
    }
    if (launch_proj_weights(p, c->axial, c->d_projw, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) {
        pnamp_free(c);
        return PNAMP_ERR_CUDA;
    }
    *out = c;
    return PNAMP_OK;
}

int pnamp_batch_device(pnamp_ctx *c, int npairs, const double *d_uv, double *d_zres, int *d_status, void *stream) {
    if (!c || npairs < 0 || (npairs > 0 && (!d_uv || !d_zres || !d_status))) return PNAMP_ERR_ARG;
    if (npairs == 0) return PNAMP_OK;
    int rc = ensure_pairs(c, npairs);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;  // NULL: legacy default stream
    if (c->tc_splits) return tc_run(c, npairs, d_uv, d_zres, d_status, st, nullptr, 0);
    int mk = stage_begin(c, st);
    CK(launch_setup(c->p, npairs, d_uv, c->d_pairbuf, st));
    stage_end(c, st, mk, kStageSetup);
    mk = stage_begin(c, st);
    CK(launch_points(c->p, npairs, c->d_pairbuf, c->d_scratch, c->grid_form[c->p.form], d_zres, d_status, st));
    stage_end(c, st, mk, kStagePoints);
    return PNAMP_OK;
}

int pnamp_batch_items_device(pnamp_ctx *c, int npairs, const double *d_uv, long long nitems, const int *d_items,
                             double *d_zres, int *d_status, double *d_gauge_out, void *stream) {
    if (!c || npairs < 0 || nitems < 0 || (nitems > 0 && (npairs == 0 || !d_uv || !d_items || !d_zres || !d_status)))
        return PNAMP_ERR_ARG;
    if (nitems == 0) return PNAMP_OK;
    int rc = ensure_pairs(c, npairs);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;  // NULL: legacy default stream
    if (c->tc_splits) {
        if (d_gauge_out) return PNAMP_ERR_STATE;  // per-gauge H/N would lack the contracted energy
        return tc_run(c, npairs, d_uv, d_zres, d_status, st, d_items, nitems);
    }
    CK(launch_setup(c->p, npairs, d_uv, c->d_pairbuf, st));
    const int grid = (int)std::min<long long>(c->grid_form[c->p.form], nitems);
    CK(launch_points(c->p, npairs, c->d_pairbuf, c->d_scratch, grid, d_zres, d_status, st,
                     reinterpret_cast<const int2 *>(d_items), nitems, d_gauge_out));
    return PNAMP_OK;
}

int pnamp_rho1b_blocks(const pnamp_ctx *c, int *it, int *lj, int *n1, int *n2, int *twoj) {
    if (!c) return -PNAMP_ERR_ARG;
    const int nb = (int)c->r1b_it.size();
    for (int b = 0; b < nb; ++b) {
        if (it) it[b] = c->r1b_it[b];
        if (lj) lj[b] = c->r1b_lj[b];
        if (n1) n1[b] = c->r1b_n1[b];
        if (n2) n2[b] = c->r1b_n2[b];
        if (twoj) twoj[b] = c->r1b_twoj[b];
    }
    return nb;
}

int pnamp_batch_rho1b_device(pnamp_ctx *c, int npairs, const double *d_uv, double *d_zres, int *d_status,
                             double *d_rho1b, void *stream) {
    if (!c || npairs < 0 || (npairs > 0 && (!d_uv || !d_zres || !d_status || !d_rho1b))) return PNAMP_ERR_ARG;
    if (c->p.obs.n_r1b == 0) return PNAMP_ERR_UNSUPPORTED;
    if (c->p.norm_only) return PNAMP_ERR_STATE;
    if (npairs == 0) return PNAMP_OK;
    int rc = ensure_pairs(c, npairs);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;  // NULL: legacy default stream
    CK(launch_setup(c->p, npairs, d_uv, c->d_pairbuf, st));
    CK(launch_points(c->p, npairs, c->d_pairbuf, c->d_scratch, c->grid_form[c->p.form], d_zres, d_status, st,
                     nullptr, 0, nullptr, d_rho1b));
    return PNAMP_OK;
}

int pnamp_batch_rho1b(pnamp_ctx *c, int npairs, const double *uv, double *zres, int *point_status,
                      double *rho1b) {
    if (!c || npairs < 0 || (npairs > 0 && (!uv || !zres || !rho1b))) return PNAMP_ERR_ARG;
    if (npairs == 0) return PNAMP_OK;
    int rc = ensure_batch(c, npairs);
    if (rc) return rc;
    const long long rb = (long long)npairs * c->p.obs.n_r1b * c->p.n_euler * 2;
    if (rb > c->r1b_cap) {
        if (c->d_r1b) cudaFree(c->d_r1b);
        c->d_r1b = nullptr;
        c->r1b_cap = 0;
        CK(cudaMalloc(&c->d_r1b, (size_t)rb * sizeof(double)));
        c->r1b_cap = rb;
    }
    const long long nn = (long long)c->p.n * c->p.n;
    const size_t zbytes = (size_t)npairs * 2 * kNobs * c->p.n_euler * sizeof(double);
    const size_t sbytes = (size_t)npairs * c->p.n_euler * sizeof(int);
    CK(cudaMemcpyAsync(c->d_uv, uv, (size_t)npairs * 4 * nn * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    rc = pnamp_batch_rho1b_device(c, npairs, c->d_uv, c->d_zres, c->d_status, c->d_r1b, c->stream);
    if (rc) return rc;
    CK(cudaMemcpyAsync(zres, c->d_zres, zbytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(rho1b, c->d_r1b, (size_t)rb * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    std::vector<int> st((size_t)npairs * c->p.n_euler);
    CK(cudaMemcpyAsync(st.data(), c->d_status, sbytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (point_status) memcpy(point_status, st.data(), sbytes);
    for (int v : st)
        if (v & PNAMP_ST_SINGULAR_U) return PNAMP_ERR_SINGULAR_U;
    return PNAMP_OK;
}

int pnamp_project_rho1b(const pnamp_ctx *c, const double *zres, const double *rho1b, double *out) {
    if (!c || !zres || !rho1b || !out) return PNAMP_ERR_ARG;
    const int P = c->p.n_euler, nb = (int)c->r1b_it.size();
    // J = 0 projection (ZRho1B_Integral, PNAMP_Rho1B.f90:36-60) over the Euler weights; the J = 0
    // weight and, for K = 0, the D-function are common to numerator and norm and cancel in the ratio
    double nr = 0.0, ni = 0.0;
    for (int e = 0; e < P; ++e) {
        nr += c->euler_w[e] * zres[2 * e];
        ni += c->euler_w[e] * zres[2 * e + 1];
    }
    if (std::sqrt(nr * nr + ni * ni) <= 1e-8) return PNAMP_ERR_SMALL_NORM;  // Write_ME1B: CHOP
    const double d = nr * nr + ni * ni;
    for (int b = 0; b < nb; ++b) {
        double sr = 0.0, si = 0.0;
        for (int e = 0; e < P; ++e) {
            sr += c->euler_w[e] * rho1b[2 * ((long long)b * P + e)];
            si += c->euler_w[e] * rho1b[2 * ((long long)b * P + e) + 1];
        }
        // AE = Re(sum / N), written divided by sqrt(2j + 1) (PNAMP_Rho1B.f90:82-84)
        out[b] = (sr * nr + si * ni) / d / std::sqrt(c->r1b_twoj[b] + 1.0);
    }
    return PNAMP_OK;
}

int pnamp_rho2b_layout(const pnamp_space *sp, int *sizes) {
    if (!sp || !sizes || !sp->t || !sp->n || !sp->l || !sp->twoj || !sp->twom) return PNAMP_ERR_ARG;
    if (sp->nlev < 2 || sp->nlev > PNAMP_MAX_NLEV) return PNAMP_ERR_ARG;
    R2Tables r;
    const int rc = build_r2(sp->nlev, sp->t, sp->n, sp->l, sp->twoj, sp->twom, r);
    if (rc) return rc;
    sizes[0] = (int)r.blocks.size() / 4;
    sizes[1] = (int)r.states.size() / 2;
    sizes[2] = (int)r.ptr.size() - 1;
    sizes[3] = (int)r.quads.size();
    sizes[4] = (int)r.tq.size();
    return PNAMP_OK;
}

int pnamp_rho2b_tables(const pnamp_space *sp, int *blocks, int *states, unsigned int *quads, int *elem_ptr,
                       int *term_q, double *term_c) {
    if (!sp || !sp->t || !sp->n || !sp->l || !sp->twoj || !sp->twom) return PNAMP_ERR_ARG;
    if (sp->nlev < 2 || sp->nlev > PNAMP_MAX_NLEV) return PNAMP_ERR_ARG;
    R2Tables r;
    const int rc = build_r2(sp->nlev, sp->t, sp->n, sp->l, sp->twoj, sp->twom, r);
    if (rc) return rc;
    if (blocks) std::copy(r.blocks.begin(), r.blocks.end(), blocks);
    if (states) std::copy(r.states.begin(), r.states.end(), states);
    if (quads) std::copy(r.quads.begin(), r.quads.end(), quads);
    if (elem_ptr) std::copy(r.ptr.begin(), r.ptr.end(), elem_ptr);
    if (term_q) std::copy(r.tq.begin(), r.tq.end(), term_q);
    if (term_c) std::copy(r.tc.begin(), r.tc.end(), term_c);
    return PNAMP_OK;
}

namespace {
int ensure_r2(pnamp_ctx *c) {
    if (!c->r2_built) {
        R2Tables r;
        const int n = c->p.n;
        const int rc = build_r2(n, c->sp_t.data(), c->sp_n.data(), c->sp_l.data(), c->sp_tj.data(),
                                c->sp_tm.data(), r);
        if (rc) return rc;
        if (r.quads.empty()) return PNAMP_ERR_UNSUPPORTED;
        CK(cudaMalloc(&c->d_r2q, r.quads.size() * sizeof(uint32_t)));
        CK(cudaMemcpy(c->d_r2q, r.quads.data(), r.quads.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
        c->r2_blocks.swap(r.blocks);
        c->r2_states.swap(r.states);
        c->r2_quads.swap(r.quads);
        c->r2_ptr.swap(r.ptr);
        c->r2_tq.swap(r.tq);
        c->r2_tc.swap(r.tc);
        c->r2_built = true;
    }
    const long long need = 2LL * (long long)c->r2_quads.size() * c->grid_form[c->p.form];
    if (need > c->r2acc_cap) {
        if (c->d_r2acc) cudaFree(c->d_r2acc);
        c->d_r2acc = nullptr;
        c->r2acc_cap = 0;
        CK(cudaMalloc(&c->d_r2acc, (size_t)need * sizeof(double)));
        c->r2acc_cap = need;
    }
    return PNAMP_OK;
}
}  // namespace

int pnamp_batch_rho2b_device(pnamp_ctx *c, int npairs, const double *d_uv, double *d_zres, int *d_status,
                             double *d_rho2b, void *stream) {
    if (!c || npairs < 0 || (npairs > 0 && (!d_uv || !d_zres || !d_status || !d_rho2b))) return PNAMP_ERR_ARG;
    if (c->p.norm_only) return PNAMP_ERR_STATE;
    int rc = ensure_r2(c);
    if (rc) return rc;
    if (npairs == 0) return PNAMP_OK;
    rc = ensure_pairs(c, npairs);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;  // NULL: legacy default stream
    Params q = c->p;
    q.n_r2q = (int)c->r2_quads.size();
    q.r2q = c->d_r2q;
    q.r2acc = c->d_r2acc;
    CK(cudaMemsetAsync(d_rho2b, 0, (size_t)npairs * q.n_r2q * 2 * sizeof(double), st));
    CK(launch_setup(q, npairs, d_uv, c->d_pairbuf, st));
    CK(launch_points(q, npairs, c->d_pairbuf, c->d_scratch, c->grid_form[q.form], d_zres, d_status, st, nullptr, 0,
                     nullptr, nullptr, d_rho2b));
    return PNAMP_OK;
}

int pnamp_batch_rho2b(pnamp_ctx *c, int npairs, const double *uv, double *zres, int *point_status,
                      double *rho2b) {
    if (!c || npairs < 0 || (npairs > 0 && (!uv || !zres || !rho2b))) return PNAMP_ERR_ARG;
    if (npairs == 0) return PNAMP_OK;
    int rc = ensure_batch(c, npairs);
    if (rc) return rc;
    rc = ensure_r2(c);
    if (rc) return rc;
    const long long rb = 2LL * npairs * (long long)c->r2_quads.size();
    if (rb > c->r2out_cap) {
        if (c->d_r2out) cudaFree(c->d_r2out);
        c->d_r2out = nullptr;
        c->r2out_cap = 0;
        CK(cudaMalloc(&c->d_r2out, (size_t)rb * sizeof(double)));
        c->r2out_cap = rb;
    }
    const long long nn = (long long)c->p.n * c->p.n;
    const size_t zbytes = (size_t)npairs * 2 * kNobs * c->p.n_euler * sizeof(double);
    const size_t sbytes = (size_t)npairs * c->p.n_euler * sizeof(int);
    CK(cudaMemcpyAsync(c->d_uv, uv, (size_t)npairs * 4 * nn * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    rc = pnamp_batch_rho2b_device(c, npairs, c->d_uv, c->d_zres, c->d_status, c->d_r2out, c->stream);
    if (rc) return rc;
    CK(cudaMemcpyAsync(zres, c->d_zres, zbytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(rho2b, c->d_r2out, (size_t)rb * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    std::vector<int> st((size_t)npairs * c->p.n_euler);
    CK(cudaMemcpyAsync(st.data(), c->d_status, sbytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (point_status) memcpy(point_status, st.data(), sbytes);
    for (int v : st)
        if (v & PNAMP_ST_SINGULAR_U) return PNAMP_ERR_SINGULAR_U;
    return PNAMP_OK;
}

int pnamp_batch_densities_device(pnamp_ctx *c, int npairs, const double *d_uv, double *d_zres, int *d_status,
                                 double *d_rho1b, double *d_rho2b, void *stream) {
    if (!c || npairs < 0 || (!d_rho1b && !d_rho2b)) return PNAMP_ERR_ARG;
    if (npairs > 0 && (!d_uv || !d_zres || !d_status)) return PNAMP_ERR_ARG;
    if (d_rho1b && c->p.obs.n_r1b == 0) return PNAMP_ERR_UNSUPPORTED;
    if (c->p.norm_only) return PNAMP_ERR_STATE;
    int rc = d_rho2b ? ensure_r2(c) : PNAMP_OK;
    if (rc) return rc;
    if (npairs == 0) return PNAMP_OK;
    rc = ensure_pairs(c, npairs);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;  // NULL: legacy default stream
    Params q = c->p;
    if (d_rho2b) {
        q.n_r2q = (int)c->r2_quads.size();
        q.r2q = c->d_r2q;
        q.r2acc = c->d_r2acc;
        CK(cudaMemsetAsync(d_rho2b, 0, (size_t)npairs * q.n_r2q * 2 * sizeof(double), st));
    }
    CK(launch_setup(q, npairs, d_uv, c->d_pairbuf, st));
    CK(launch_points(q, npairs, c->d_pairbuf, c->d_scratch, c->grid_form[q.form], d_zres, d_status, st, nullptr, 0,
                     nullptr, d_rho1b, d_rho2b));
    return PNAMP_OK;
}

int pnamp_batch_densities(pnamp_ctx *c, int npairs, const double *uv, double *zres, int *point_status,
                          double *rho1b, double *rho2b) {
    if (!c || npairs < 0 || (!rho1b && !rho2b) || (npairs > 0 && (!uv || !zres))) return PNAMP_ERR_ARG;
    if (rho1b && c->p.obs.n_r1b == 0) return PNAMP_ERR_UNSUPPORTED;
    if (npairs == 0) return PNAMP_OK;
    int rc = ensure_batch(c, npairs);
    if (rc) return rc;
    const long long r1 = rho1b ? (long long)npairs * c->p.obs.n_r1b * c->p.n_euler * 2 : 0;
    if (r1 > c->r1b_cap) {
        if (c->d_r1b) cudaFree(c->d_r1b);
        c->d_r1b = nullptr;
        c->r1b_cap = 0;
        CK(cudaMalloc(&c->d_r1b, (size_t)r1 * sizeof(double)));
        c->r1b_cap = r1;
    }
    long long r2 = 0;
    if (rho2b) {
        rc = ensure_r2(c);
        if (rc) return rc;
        r2 = 2LL * npairs * (long long)c->r2_quads.size();
        if (r2 > c->r2out_cap) {
            if (c->d_r2out) cudaFree(c->d_r2out);
            c->d_r2out = nullptr;
            c->r2out_cap = 0;
            CK(cudaMalloc(&c->d_r2out, (size_t)r2 * sizeof(double)));
            c->r2out_cap = r2;
        }
    }
    const long long nn = (long long)c->p.n * c->p.n;
    const size_t zbytes = (size_t)npairs * 2 * kNobs * c->p.n_euler * sizeof(double);
    const size_t sbytes = (size_t)npairs * c->p.n_euler * sizeof(int);
    CK(cudaMemcpyAsync(c->d_uv, uv, (size_t)npairs * 4 * nn * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    rc = pnamp_batch_densities_device(c, npairs, c->d_uv, c->d_zres, c->d_status, rho1b ? c->d_r1b : nullptr,
                                      rho2b ? c->d_r2out : nullptr, c->stream);
    if (rc) return rc;
    CK(cudaMemcpyAsync(zres, c->d_zres, zbytes, cudaMemcpyDeviceToHost, c->stream));
    if (rho1b) CK(cudaMemcpyAsync(rho1b, c->d_r1b, (size_t)r1 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (rho2b) CK(cudaMemcpyAsync(rho2b, c->d_r2out, (size_t)r2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    std::vector<int> stv((size_t)npairs * c->p.n_euler);
    CK(cudaMemcpyAsync(stv.data(), c->d_status, sbytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (point_status) memcpy(point_status, stv.data(), sbytes);
    for (int v : stv)
        if (v & PNAMP_ST_SINGULAR_U) return PNAMP_ERR_SINGULAR_U;
    return PNAMP_OK;
}

int pnamp_project_rho2b(pnamp_ctx *c, const double *zres, const double *rho2b, double *out) {
    if (!c || !zres || !rho2b || !out) return PNAMP_ERR_ARG;
    const int rc = ensure_r2(c);
    if (rc) return rc;
    const int P = c->p.n_euler;
    // N^0 over the Euler weights (the J = 0 weight cancels against ZRho2B_Integral's)
    double nr = 0.0, ni = 0.0;
    for (int e = 0; e < P; ++e) {
        nr += c->euler_w[e] * zres[2 * e];
        ni += c->euler_w[e] * zres[2 * e + 1];
    }
    if (std::sqrt(nr * nr + ni * ni) <= 1e-8) return PNAMP_ERR_SMALL_NORM;  // Rho2BN = 0 in Write_ME2B
    const double d = nr * nr + ni * ni;
    const int ne = (int)c->r2_ptr.size() - 1;
    for (int e = 0; e < ne; ++e) {
        double sr = 0.0, si = 0.0;
        for (int t = c->r2_ptr[e]; t < c->r2_ptr[e + 1]; ++t) {
            sr += c->r2_tc[t] * rho2b[2 * c->r2_tq[t]];
            si += c->r2_tc[t] * rho2b[2 * c->r2_tq[t] + 1];
        }
        out[2 * e] = (sr * nr + si * ni) / d;       // (sr + i si) / (nr + i ni)
        out[2 * e + 1] = (si * nr - sr * ni) / d;
    }
    return PNAMP_OK;
}

int pnamp_batch(pnamp_ctx *c, int npairs, const double *uv, double *zres, int *point_status) {
    if (!c || npairs < 0 || (npairs > 0 && (!uv || !zres))) return PNAMP_ERR_ARG;
    if (npairs == 0) return PNAMP_OK;
    int rc = ensure_batch(c, npairs);
    if (rc) return rc;
    const long long nn = (long long)c->p.n * c->p.n;
    const size_t zbytes = (size_t)npairs * 2 * kNobs * c->p.n_euler * sizeof(double);
    const size_t sbytes = (size_t)npairs * c->p.n_euler * sizeof(int);
    CK(cudaMemcpyAsync(c->d_uv, uv, (size_t)npairs * 4 * nn * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    rc = pnamp_batch_device(c, npairs, c->d_uv, c->d_zres, c->d_status, c->stream);
    if (rc) return rc;
    CK(cudaMemcpyAsync(zres, c->d_zres, zbytes, cudaMemcpyDeviceToHost, c->stream));
    std::vector<int> st((size_t)npairs * c->p.n_euler);
    CK(cudaMemcpyAsync(st.data(), c->d_status, sbytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (point_status) memcpy(point_status, st.data(), sbytes);
    for (int v : st)
        if (v & PNAMP_ST_SINGULAR_U) return PNAMP_ERR_SINGULAR_U;
    return PNAMP_OK;
}

int pnamp_pair(pnamp_ctx *c, const double *U0, const double *V0, const double *U1, const double *V1, double *zres,
               int *point_status) {
    if (!c || !U0 || !V0 || !U1 || !V1 || !zres) return PNAMP_ERR_ARG;
    const size_t nn = (size_t)c->p.n * c->p.n;
    std::vector<double> uv(4 * nn);
    memcpy(uv.data(), U0, nn * sizeof(double));
    memcpy(uv.data() + nn, V0, nn * sizeof(double));
    memcpy(uv.data() + 2 * nn, U1, nn * sizeof(double));
    memcpy(uv.data() + 3 * nn, V1, nn * sizeof(double));
    return pnamp_batch(c, 1, uv.data(), zres, point_status);
}

int pnamp_project_device(pnamp_ctx *c, int npairs, const double *d_zres, int chop, double *d_out, void *stream) {
    if (!c || npairs < 0 || (npairs > 0 && (!d_zres || !d_out))) return PNAMP_ERR_ARG;
    if (npairs == 0) return PNAMP_OK;
    cudaStream_t st = (cudaStream_t)stream;  // NULL: legacy default stream
    const long long fs = (long long)(kJJMax + 1) * kNK * kNK;
    CK(cudaMemsetAsync(d_out, 0, (size_t)npairs * 2 * kProjFields * fs * sizeof(double), st));
    CK(launch_project(c->p, npairs, c->d_projw, d_zres, c->core_prot, c->core_neut, chop, d_out, st));
    return PNAMP_OK;
}

int pnamp_project(pnamp_ctx *c, const double *zres, int chop, pnamp_kernels *out) {
    if (!c || !zres || !out || !out->njkk || !out->hjkk || !out->nn || !out->zz || !out->j2) return PNAMP_ERR_ARG;
    int rc = ensure_batch(c, 1);
    if (rc) return rc;
    const size_t zbytes = (size_t)2 * kNobs * c->p.n_euler * sizeof(double);
    const size_t fs = (size_t)(kJJMax + 1) * kNK * kNK;
    CK(cudaMemcpyAsync(c->d_zres, zres, zbytes, cudaMemcpyHostToDevice, c->stream));
    rc = pnamp_project_device(c, 1, c->d_zres, chop, c->d_proj, c->stream);
    if (rc) return rc;
    std::vector<double> h(2 * kProjFields * fs);
    CK(cudaMemcpyAsync(h.data(), c->d_proj, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    double *dst[kProjFields] = {out->njkk, out->hjkk, out->nn, out->zz, out->j2};
    for (int q = 0; q < kProjFields; ++q) memcpy(dst[q], h.data() + 2 * q * fs, 2 * fs * sizeof(double));
    return PNAMP_OK;
}

int pnamp_project_q_device(pnamp_ctx *c, int npairs, const double *d_zres, int exchange, double *d_out,
                           void *stream) {
    if (!c || npairs < 0 || (npairs > 0 && (!d_zres || !d_out))) return PNAMP_ERR_ARG;
    if (npairs == 0) return PNAMP_OK;
    cudaStream_t st = (cudaStream_t)stream;  // NULL: legacy default stream
    const size_t blk = (size_t)(kJJMax + 1) * 3 * 17 * 13;
    CK(cudaMemsetAsync(d_out, 0, (size_t)npairs * 2 * 2 * blk * sizeof(double), st));
    CK(launch_project_q(c->p, c->axial, npairs, d_zres, c->d_tj, exchange ? 1 : 0, d_out, st));
    return PNAMP_OK;
}

int pnamp_project_q(pnamp_ctx *c, const double *zres, int exchange, double *qpred, double *qcpred) {
    if (!c || !zres || !qpred || !qcpred) return PNAMP_ERR_ARG;
    int rc = ensure_batch(c, 1);
    if (rc) return rc;
    const size_t blk = (size_t)(kJJMax + 1) * 3 * 17 * 13;
    if (!c->d_projq) CK(cudaMalloc(&c->d_projq, 2 * 2 * blk * sizeof(double)));
    const size_t zbytes = (size_t)2 * kNobs * c->p.n_euler * sizeof(double);
    CK(cudaMemcpyAsync(c->d_zres, zres, zbytes, cudaMemcpyHostToDevice, c->stream));
    rc = pnamp_project_q_device(c, 1, c->d_zres, exchange, c->d_projq, c->stream);
    if (rc) return rc;
    CK(cudaMemcpyAsync(qpred, c->d_projq, 2 * blk * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(qcpred, c->d_projq + 2 * blk, 2 * blk * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return PNAMP_OK;
}

int pnamp_sync(pnamp_ctx *c) {
    if (!c) return PNAMP_ERR_ARG;
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaGetLastError());
    return PNAMP_OK;
}

int pnamp_set_timing(pnamp_ctx *c, int on) {
    if (!c) return PNAMP_ERR_ARG;
    c->timing = on ? 1 : 0;
    c->ev_marks.clear();
    return PNAMP_OK;
}

int pnamp_stage_times(pnamp_ctx *c, double *ms) {
    if (!c || !ms) return PNAMP_ERR_ARG;
    for (int k = 0; k < kStages; ++k) ms[k] = 0.0;
    for (const auto &m : c->ev_marks) {
        float t = 0.f;
        CK(cudaEventSynchronize(c->ev_pool[m[2]]));
        CK(cudaEventElapsedTime(&t, c->ev_pool[m[1]], c->ev_pool[m[2]]));
        ms[m[0]] += t;
    }
    c->ev_marks.clear();
    return kStages;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// No-allocation variant of pnamp_batch_device. The scratch it needs (pair
// records from setup_kernel, per-CTA workspace slots of point_kernel) lives in
// this file-scope array instead of context buffers from cudaMalloc. In host
// code `g_noalloc_scratch` names a host-side stand-in, not a device address, so
// the device address is looked up once per device with cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[PNAMP_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (first call per
// device resolves and caches it).
int noalloc_scratch(void **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return PNAMP_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return PNAMP_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return PNAMP_ERR_CUDA;
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return PNAMP_OK;
}
}  // namespace

extern "C" int pnamp_batch_device_noalloc(pnamp_ctx *c, int npairs, const double *d_uv, double *d_zres,
                                          int *d_status, void *stream) {
    if (!c || npairs < 0 || (npairs > 0 && (!d_uv || !d_zres || !d_status))) return PNAMP_ERR_ARG;
    if (npairs == 0) return PNAMP_OK;
    const unsigned long long cap = PNAMP_NOALLOC_SCRATCH_BYTES;
    const unsigned long long pair_bytes =
        ((unsigned long long)npairs * (unsigned long long)c->p.pl.stride * sizeof(double) + 255ull) & ~255ull;
    const unsigned long long slot_bytes = (unsigned long long)c->p.place.slot_elems * sizeof(zc);
    if (pair_bytes + slot_bytes > cap) return PNAMP_ERR_SCRATCH_LIMIT;
    const unsigned long long fit = (cap - pair_bytes) / slot_bytes;
    const int grid = (int)std::min<unsigned long long>((unsigned long long)c->grid_form[c->p.form], fit);
    void *base = nullptr;
    const int rc = noalloc_scratch(&base);
    if (rc) return rc;
    double *pairbuf = reinterpret_cast<double *>(base);
    zc *slots = reinterpret_cast<zc *>(reinterpret_cast<unsigned char *>(base) + pair_bytes);
    cudaStream_t st = (cudaStream_t)stream;  // NULL: legacy default stream
    CK(launch_setup(c->p, npairs, d_uv, pairbuf, st));
    CK(launch_points(c->p, npairs, pairbuf, slots, grid, d_zres, d_status, st));
    return PNAMP_OK;
}

// ---------------------------------------------------------------------------
// Uneven batches in one persistent launch (several contexts: model spaces,
// meshes, placements). The plan owns its per-context pair records, scratch,
// work list and device copies of the contexts' parameters; launching only
// enqueues kernels and a memset, so it can be captured in a CUDA graph.
struct pnamp_multi {
    int nctx = 0, form = 0, nitems = 0, grab = 1, grid = 0, grid_max = 0, smem = 0, order = 1;
    int nsm = 0, optin = 0, grid_req = 0;
    long long stride = 0, scratch_elems = 0;
    std::vector<pnamp_ctx *> ctxs;
    std::vector<int> npairs;
    std::vector<const double *> uv;
    std::vector<double *> pairbuf;
    MultiArgs args{};
    int4 *d_items = nullptr;
    zc *scratch = nullptr;
    int *counter = nullptr;
};

extern "C" {

void pnamp_multi_free(pnamp_multi *m) {
    if (!m) return;
    for (double *q : m->pairbuf) if (q) cudaFree(q);
    for (void *q : {(void *)m->d_items, (void *)m->scratch, (void *)m->counter})
        if (q) cudaFree(q);
    delete m;
}

int pnamp_multi_schedule(pnamp_multi *m, int order, int grab, int grid) {
    if (!m || order < 0 || order > 2 || grab < 1 || grab > 64 || grid < 0) return PNAMP_ERR_ARG;
    std::vector<int4> items;
    std::vector<int> cidx(m->nctx);
    for (int c = 0; c < m->nctx; ++c) cidx[c] = c;
    auto cost = [&](int c) {  // per item: gauge points x n^3
        const Params &p = m->ctxs[c]->p;
        return (double)p.n_gauge * p.n * p.n * p.n;
    };
    if (order == 1) std::stable_sort(cidx.begin(), cidx.end(), [&](int a, int b) { return cost(a) > cost(b); });
    if (order == 2) {  // round robin over contexts, item by item
        std::vector<long long> pos(m->nctx, 0);
        bool more = true;
        while (more) {
            more = false;
            for (int c = 0; c < m->nctx; ++c) {
                const long long tot = (long long)m->npairs[c] * m->ctxs[c]->p.n_euler;
                if (pos[c] < tot) {
                    const long long k = pos[c]++;
                    items.push_back(make_int4(c, (int)(k / m->ctxs[c]->p.n_euler), (int)(k % m->ctxs[c]->p.n_euler), 0));
                    more = true;
                }
            }
        }
    } else {
        for (int c : cidx)
            for (int q = 0; q < m->npairs[c]; ++q)
                for (int e = 0; e < m->ctxs[c]->p.n_euler; ++e) items.push_back(make_int4(c, q, e, 0));
    }
    if ((int)items.size() != m->nitems) return PNAMP_ERR_STATE;
    CK(cudaMemcpy(m->d_items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice));
    m->order = order;
    m->grab = grab;
    m->grid_req = grid;
    m->grid = grid == 0 ? m->grid_max : std::min(grid, m->grid_max);
    return PNAMP_OK;
}

int pnamp_multi_placement(pnamp_multi *m, int smem_budget, int *smem_out) {
    if (!m || smem_budget < 0) return PNAMP_ERR_ARG;
    const int cap = m->optin - kMultiSmemTail;
    const int budget = smem_budget == 0 ? cap : std::min(smem_budget, cap);
    // each context's arrays under the same budget; the launch holds the largest
    MultiArgs a = m->args;
    int smem = 0;
    long long stride = 0;
    for (int c = 0; c < m->nctx; ++c) {
        Params q = m->ctxs[c]->p;
        if (plan_placement(q, budget) != PNAMP_OK) return PNAMP_ERR_UNSUPPORTED;
        a.p[c] = q;
        smem = std::max(smem, (q.place.smem_bytes + 15) & ~15);
        stride = std::max(stride, q.place.slot_elems);
    }
    for (int c = m->nctx; c < kMultiCtx; ++c) a.p[c] = a.p[0];
    a.slot_stride = stride;
    smem += kMultiSmemTail;
    int per_sm = 0;
    if (multi_blocks_per_sm(m->form, smem, &per_sm) != cudaSuccess || per_sm < 1) return PNAMP_ERR_CUDA;
    const int grid_max = m->nsm * per_sm;
    if ((long long)grid_max * stride > m->scratch_elems) {
        if (m->scratch) cudaFree(m->scratch);
        m->scratch = nullptr;
        m->scratch_elems = 0;
        if (cudaMalloc(&m->scratch, (size_t)grid_max * stride * sizeof(zc)) != cudaSuccess) return PNAMP_ERR_NOMEM;
        m->scratch_elems = (long long)grid_max * stride;
    }
    m->args = a;
    m->smem = smem;
    m->stride = stride;
    m->grid_max = grid_max;
    m->grid = m->grid_req == 0 ? grid_max : std::min(m->grid_req, grid_max);
    if (smem_out) *smem_out = smem;
    return PNAMP_OK;
}

int pnamp_multi_create(int nctx, pnamp_ctx *const *ctxs, const int *npairs, const double *const *d_uv,
                       double *const *d_zres, int *const *d_status, pnamp_multi **out) {
    if (!out || nctx < 1 || !ctxs || !npairs || !d_uv || !d_zres || !d_status) return PNAMP_ERR_ARG;
    *out = nullptr;
    if (nctx > kMultiCtx) return PNAMP_ERR_UNSUPPORTED;
    pnamp_multi *m = new pnamp_multi();
    m->nctx = nctx;
    m->form = ctxs[0] ? ctxs[0]->p.form : 0;
    long long nitems = 0;
    for (int c = 0; c < nctx; ++c) {
        if (!ctxs[c] || npairs[c] < 1 || !d_uv[c] || !d_zres[c] || !d_status[c] || ctxs[c]->p.form != m->form) {
            pnamp_multi_free(m);
            return PNAMP_ERR_ARG;
        }
        m->ctxs.push_back(ctxs[c]);
        m->npairs.push_back(npairs[c]);
        m->uv.push_back(d_uv[c]);
        m->args.p[c] = ctxs[c]->p;
        m->args.zres[c] = d_zres[c];
        m->args.status[c] = d_status[c];
        nitems += (long long)npairs[c] * ctxs[c]->p.n_euler;
        double *pb = nullptr;
        if (cudaMalloc(&pb, (size_t)npairs[c] * ctxs[c]->p.pl.stride * sizeof(double)) != cudaSuccess) {
            pnamp_multi_free(m);
            return PNAMP_ERR_NOMEM;
        }
        m->pairbuf.push_back(pb);
        m->args.pairbuf[c] = pb;
    }
    for (int c = nctx; c < kMultiCtx; ++c) {   // unused slots: copies of context 0, never dispatched
        m->args.pairbuf[c] = m->args.pairbuf[0];
        m->args.zres[c] = m->args.zres[0];
        m->args.status[c] = m->args.status[0];
    }
    if (nitems > 0x7fffffffLL) {
        pnamp_multi_free(m);
        return PNAMP_ERR_UNSUPPORTED;
    }
    m->nitems = (int)nitems;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&m->nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&m->optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        pnamp_multi_free(m);
        return PNAMP_ERR_CUDA;
    }
    if (cudaMalloc(&m->d_items, (size_t)m->nitems * sizeof(int4)) != cudaSuccess ||
        cudaMalloc(&m->counter, sizeof(int)) != cudaSuccess) {
        pnamp_multi_free(m);
        return PNAMP_ERR_NOMEM;
    }
    int rc0 = pnamp_multi_placement(m, 0, nullptr);
    if (rc0) {
        pnamp_multi_free(m);
        return rc0;
    }
    const int rc = pnamp_multi_schedule(m, 1, 1, 0);
    if (rc) {
        pnamp_multi_free(m);
        return rc;
    }
    *out = m;
    return PNAMP_OK;
}

int pnamp_multi_launch(pnamp_multi *m, void *stream) {
    if (!m) return PNAMP_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;  // NULL: legacy default stream
    for (int c = 0; c < m->nctx; ++c) CK(launch_setup(m->ctxs[c]->p, m->npairs[c], m->uv[c], m->pairbuf[c], st));
    CK(launch_multi(m->form, m->args, m->d_items, m->nitems, m->grab, m->counter, m->scratch, m->grid, m->smem,
                    st));
    return PNAMP_OK;
}

int pnamp_multi_items(const pnamp_multi *m) { return m ? m->nitems : -1; }

}  // extern "C"
