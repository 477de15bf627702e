// mw_apply.cpp -- host drivers of the hot path: adaptive NS-form apply
// (single, batched, fixed grid), tree multiply and add.
//
// mrcpp::apply(prec, out, oper, inp[, precTrees], maxIter, absPrec) is called at
// src/qmoperators/two_electron/CoulombPotential.cpp:131,156,
// src/scf_solver/HelmholtzVector.cpp:149,154 and
// src/qmoperators/two_electron/ExchangePotential.cpp:200,204.  The algorithm
// (published method: Frediani et al., Mol. Phys. 111 (2013) 1143):
//   - the output grid grows from the root nodes one scale per iteration; the
//     split decision and the screening are host logic on FP64 norms;
//   - an item (output node o, input node i, term t) contributes
//     c_t (A_z (x) A_y (x) A_x) in_i to o for every component pair except the
//     scaling-scaling pair below the root scale; it is skipped when
//         b = sum_{(ft,gt)} |in_ft| prod_d |A_d^{g_d f_d}|_F  <  0.01 thr(o);
//   - o is split when |wavelet part| * w(o) > thr(o) = prec R 2^{-(n+1)/2};
//   - afterwards the scales are summed top-down and the tree is compressed.
// The contractions run on the GPU in deterministic per-node order; with
// MW_PREC_MIXED the items are split into FP64 / FP32 tiers by their bound b
// (MW_PREC_MIXED_NEARFP64 also keeps every |l|_inf <= 1 item in FP64).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "mw_internal.h"
#include "mw_tc05_layout.h"

namespace mwg {

namespace {

// An item computed in FP32 (inputs, operator blocks and three passes of 2K-term sums rounded to
// FP32) is off by at most about (4 + 6K) 2^-24 b <= 4e-6 b for K <= 10.  Items with
// b <= TIER_FP64 * screening threshold = 2e4 * thr(o) therefore err by at most 0.08 thr(o),
// a tenth of the refinement tolerance; larger items run in FP64.
constexpr double TIER_FP64 = 2e6;
// An item on the TF32 tensor cores (input values, operator blocks and the two intermediates
// rounded to TF32, unit roundoff 2^-11; FP32 accumulation) is off by at most about
// 6 * 2^-11 b = 2.9e-3 b.  Items with b <= TIER_TF32 * screening threshold err by at most
// 0.06 thr(o), the same per-item bound as the FP32 tier.  Root-scale items never take this tier:
// nothing is screened there and, with precision-steering trees, the threshold is divided by the
// small weight of the large root boxes, so many items just under it would add up to more than
// prec relative to a small output.
constexpr double TIER_TF32 = 2e3;
// An item in double-FP32 (values as unevaluated FP32 pairs, error-free products and sums) is off
// by at most about 3e-13 b, so items with TIER_FP64 < b / tau <= TIER_DF err by at most 0.03 tau;
// larger ones, and root-scale items under relative precision, run in FP64.
constexpr double TIER_DF = 1e11;
constexpr int NTIER = 4;  // 0 FP64, 1 FP32, 2 TF32 tensor cores, 3 double-FP32
constexpr double BOUND_PRUNE = 8.0 * 2.8285;  // (sum_f |in_f|) / |block| <= sqrt(8); 8 output components

double split_thr(double prec, double R, int n) { return prec * R * std::pow(2.0, -0.5 * (n + 1)); }

// b = sum_ft |in_ft| s(ft), s(ft) = sum_gt prod_d |A_d^{g_d f_d}|.  For ft != 0 (and at the root)
// the sum over gt factorises into prod_d (|A_d^{0 f_d}| + |A_d^{1 f_d}|); for ft = 0 below the root
// the (0,0) pair is left out and the 7 other products are summed one by one (no cancellation).
inline double item_bound(const double *nx, const double *ny, const double *nz, const double *cn, bool root) {
    const double cx[2] = {nx[0] + nx[2], nx[1] + nx[3]}, cy[2] = {ny[0] + ny[2], ny[1] + ny[3]},
                 cz[2] = {nz[0] + nz[2], nz[1] + nz[3]};
    double b = 0.0;
    if (cn[0] != 0.0) {
        double s = 0.0;
        if (root) {
            s = cx[0] * cy[0] * cz[0];
        } else {
            for (int gt = 1; gt < 8; gt++) s += nx[2 * (gt & 1)] * ny[2 * ((gt >> 1) & 1)] * nz[2 * (gt >> 2)];
        }
        b += cn[0] * s;
    }
    for (int ft = 1; ft < 8; ft++)
        if (cn[ft] != 0.0) b += cn[ft] * (cx[ft & 1] * cy[(ft >> 1) & 1] * cz[ft >> 2]);
    return b;
}

// component pairs with a non-zero contraction (the algorithmic work unit, 6 K^4 flops each)
inline int item_pairs(const double *nx, const double *ny, const double *nz, const double *cn, bool root) {
    // non-zero sub-blocks per dimension and input half, multiplied over the dimensions
    const int ex[2] = {(nx[0] != 0.0) + (nx[2] != 0.0), (nx[1] != 0.0) + (nx[3] != 0.0)},
              ey[2] = {(ny[0] != 0.0) + (ny[2] != 0.0), (ny[1] != 0.0) + (ny[3] != 0.0)},
              ez[2] = {(nz[0] != 0.0) + (nz[2] != 0.0), (nz[1] != 0.0) + (nz[3] != 0.0)};
    int p = 0;
    for (int ft = 0; ft < 8; ft++) {
        if (cn[ft] == 0.0) continue;
        p += ex[ft & 1] * ey[(ft >> 1) & 1] * ez[ft >> 2];
        if (!root && ft == 0 && nx[0] != 0.0 && ny[0] != 0.0 && nz[0] != 0.0) p--;
    }
    return p;
}

inline double block_norm8(const double *cn) {
    double s = 0.0;
    for (int c = 0; c < 8; c++) s += cn[c] * cn[c];
    return std::sqrt(s);
}

inline double wavelet_norm8(const double *cn) {
    double s = 0.0;
    for (int c = 1; c < 8; c++) s += cn[c] * cn[c];
    return std::sqrt(s);
}

double prec_weight(const std::vector<Tree *> &pt, int n, const int *l) {
    double w = 0.0;
    for (const Tree *t : pt) {
        int idx = t->find(n, l), an = n;
        if (idx < 0) idx = find_ancestor(*t, n, l, &an);
        if (idx < 0) continue;
        w += block_norm8(&t->cn[8 * (size_t)idx]) * std::pow(2.0, 1.5 * an);
    }
    return w;
}

struct Cand {
    int t, lx, ly, lz;
    int src;   // input node index, or generated slot
    int gen;   // 1: src is a generated slot (ancestor index before generation)
    int tier;  // after screening: -1 skipped, 0 FP64, 1 FP32, 2 TF32 tensor cores, 3 double-FP32
    double bd; // bound: exact for real inputs, from the ancestor's norm for generated ones
};

struct JobState {
    ApplyJob *job = nullptr;
    double R = 1.0, fmax = 0.0;
    // per level (scale - root scale): the largest block norm an input candidate at that scale can
    // have, i.e. of the input nodes at that scale and of the coarser leaves (generated inputs)
    std::vector<double> fmax_lv;
    double fmax_at(int lv) const { return lv < (int)fmax_lv.size() ? fmax_lv[lv] : fmax; }
    void set_fmax(const Tree &t, int n0) {
        fmax = 0.0;
        int nl = 1;
        for (const NodeInfo &ni : t.nodes) nl = std::max(nl, ni.n - n0 + 2);
        std::vector<double> at(nl, 0.0), leaf(nl, 0.0);
        for (int i = 0; i < t.nn(); i++) {
            const int lv = t.nodes[i].n - n0;
            const double v = block_norm8(&t.cn[8 * (size_t)i]);
            fmax = std::max(fmax, v);
            at[lv] = std::max(at[lv], v);
            if (t.nodes[i].child0 < 0) leaf[lv] = std::max(leaf[lv], v);
        }
        fmax_lv.assign(nl, 0.0);
        double coarser_leaf = 0.0;
        for (int lv = 0; lv < nl; lv++) {
            fmax_lv[lv] = std::max(at[lv], coarser_leaf);
            coarser_leaf = std::max(coarser_leaf, leaf[lv]);
        }
    }
    std::vector<int> work;
    std::vector<double> wgt;
    int iter = 0;
    GenSet gens;
    double *gbase = nullptr;
    float *gbase32 = nullptr;
    float *gbase_tc = nullptr;  // generated blocks in the tensor-core tier's x-pass layout
    std::vector<double> gcn;
    std::vector<std::vector<Cand>> cand;
};

struct LookupCache {
    int L = -1, side = 0;
    unsigned stamp = 0;          // entries whose stamp differs are unknown (reset in O(1))
    std::vector<unsigned> st;
    std::vector<int> idx;      // -3 unknown, -2 outside, >= 0 node, <= -4 generated with ancestor -(v+4)
    std::vector<double> anorm;
    void reset(int Lm) {
        if (Lm != L || ++stamp == 0) {
            L = Lm;
            side = 2 * Lm + 1;
            const size_t n = (size_t)side * side * side;
            st.assign(n, 0u);
            idx.assign(n, -3);
            anorm.assign(n, 0.0);
            stamp = 1;
        }
    }
    int &entry(size_t ci) {
        if (st[ci] != stamp) {
            st[ci] = stamp;
            idx[ci] = -3;
        }
        return idx[ci];
    }
};

// phase A for one output node: candidate items with bounds from real norms or ancestor norms
void enumerate_node(JobState &js, int w, int s, bool root, double thr, LookupCache &cache) {
    const Tree &inp = *js.job->inp;
    const Oper &op = *js.job->op;
    const Basis &b = inp.ctx->basis;
    const NodeInfo &o = js.job->out->nodes[js.work[w]];
    std::vector<Cand> &out = js.cand[w];
    out.clear();
    const double fm = BOUND_PRUNE * js.fmax_at(s);
    int Lm = 0;
    for (int t = 0; t < op.T; t++) Lm = std::max(Lm, op.band[t * op.S + s]);
    cache.reset(Lm);
    for (int t = 0; t < op.T; t++) {
        int L = op.band[t * op.S + s];
        if (L < 0) continue;
        double A = op.amax[t * op.S + s], X = op.xmax[t * op.S + s];
        if (!root && fm * 3.0 * X * A * A < thr) continue;
        for (int lz = -L; lz <= L; lz++) {
            const double *nz = op.norm(t, s, lz);
            double az = std::max(std::max(nz[0], nz[1]), std::max(nz[2], nz[3]));
            double xz = std::max(nz[1], std::max(nz[2], nz[3]));
            if (!root && fm * (xz * A * A + 2.0 * az * X * A) < thr) continue;
            for (int ly = -L; ly <= L; ly++) {
                const double *ny = op.norm(t, s, ly);
                double ay = std::max(std::max(ny[0], ny[1]), std::max(ny[2], ny[3]));
                double xy = std::max(ny[1], std::max(ny[2], ny[3]));
                if (!root && fm * (xz * ay * A + az * xy * A + az * ay * X) < thr) continue;
                for (int lx = -L; lx <= L; lx++) {
                    size_t ci = ((size_t)(lz + Lm) * cache.side + (ly + Lm)) * cache.side + (lx + Lm);
                    int &ce = cache.entry(ci);
                    if (ce == -3) {
                        int p[3] = {o.l[0] - lx, o.l[1] - ly, o.l[2] - lz};
                        if (!b.in_world(o.n, p)) {
                            ce = -2;
                        } else {
                            int i = inp.find(o.n, p);
                            if (i >= 0) {
                                ce = i;
                            } else {
                                int a = find_ancestor(inp, o.n, p, nullptr);
                                ce = -(a + 4);
                                cache.anorm[ci] = block_norm8(&inp.cn[8 * (size_t)a]);
                            }
                        }
                    }
                    if (ce == -2) continue;
                    const double *nx = op.norm(t, s, lx);
                    double cnb[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                    const double *cn;
                    if (ce >= 0) {
                        cn = &inp.cn[8 * (size_t)ce];
                    } else {
                        cnb[0] = cache.anorm[ci];
                        cn = cnb;
                    }
                    double bd = item_bound(nx, ny, nz, cn, root);
                    if (!root && bd < thr) continue;
                    out.push_back(Cand{t, lx, ly, lz, ce >= 0 ? ce : -(ce + 4), ce >= 0 ? 0 : 1, -1, bd});
                }
            }
        }
    }
}

struct LevelItems {
    // per tier: node list, begin offsets, item SoA.  The arrays only grow; `nodes` and `items`
    // are the level's counts, and the fill writes every entry below them.
    long nodes = 0;
    long long items = 0;
    std::vector<double *> out;
    std::vector<long long> begin;
    std::vector<const void *> in, ax, ay, az;
    std::vector<double> coef;
    void resize(long n, long long m) {
        nodes = n;
        items = m;
        if ((long)out.size() < n) out.resize(n);
        if ((long)begin.size() < n + 1) begin.resize(n + 1);
        begin[0] = 0;
        if ((long long)in.size() < m) {
            in.resize(m);
            ax.resize(m);
            ay.resize(m);
            az.resize(m);
            coef.resize(m);
        }
    }
};

// tier: 0 FP64, 1 FP32 CUDA cores, 2 TF32 tensor cores, 3 double-FP32.  Returns the pinned host copy of the
// launch's status word and row count (two ints; read them after the stream has been synchronised),
// or nullptr when the level has no node in the tier.
// item arrays written on the GPU by the screening kernels (mw_screen.cu): the tiers one after the
// other, tier k from base[k]
struct DevItems {
    const void **in = nullptr, **ax = nullptr, **ay = nullptr, **az = nullptr;
    double *coef = nullptr;
    long long base[NTIER] = {0, 0, 0, 0};
};

int *launch_tier(Ctx &ctx, Arena &arena, LevelItems &li, bool root, bool set, int tier, long long chunk,
                 mw_stats &st, const DevItems *dv = nullptr, bool split_tc = false) {
    const int nn = (int)li.nodes;
    const size_t ni = (size_t)li.items;
    if (nn == 0) return nullptr;
    // A node with many items runs as several chunks of about CHUNK items, each a CTA task that
    // writes a partial block; the CTA that ends a node's last chunk sums its partials in chunk
    // order (mw_chunks.cuh).
    // The split depends only on the tier and the node's own item count, so results do not depend
    // on which nodes share the launch.  CHUNK (Ctx::Tuning; by default 4, 32, 96 and 8 items) is
    // about half a millisecond of one CTA's work: an item costs ~200 us (FP64), ~20 us (FP32),
    // ~3 us (TF32) and ~70 us (double-FP32).
    const long long CHUNK = chunk > 0 ? chunk : 1;
    const int bs = ctx.basis.bs;
    std::vector<double *> vout;
    std::vector<long long> vbeg, vend;
    std::vector<int> vred;  // per task: its node's ReduceTask, or -1
    std::vector<ReduceTask> red;
    long nsplit = 0;
    for (int i = 0; i < nn; i++) {
        const long long m = li.begin[i + 1] - li.begin[i];
        if (m > CHUNK + CHUNK / 2) nsplit += (m + CHUNK / 2) / CHUNK;
    }
    double *scratch = nsplit ? (double *)arena.alloc(sizeof(double) * (size_t)bs * nsplit) : nullptr;
    if (scratch && !set) MWG_CUDA(cudaMemsetAsync(scratch, 0, sizeof(double) * (size_t)bs * nsplit, ctx.stream));
    long used = 0;
    for (int i = 0; i < nn; i++) {
        const long long b0 = li.begin[i], m = li.begin[i + 1] - b0;
        const long long pieces = m > CHUNK + CHUNK / 2 ? (m + CHUNK / 2) / CHUNK : 1;
        if (pieces == 1) {
            vout.push_back(li.out[i]);
            vbeg.push_back(b0);
            vend.push_back(b0 + m);
            vred.push_back(-1);
            continue;
        }
        for (long long k = 0; k < pieces; k++) {
            vout.push_back(scratch + (size_t)(used + k) * bs);
            vbeg.push_back(b0 + m * k / pieces);
            vend.push_back(b0 + m * (k + 1) / pieces);
            vred.push_back((int)red.size());
        }
        red.push_back(ReduceTask{li.out[i], scratch + (size_t)used * bs, (int)pieces, set ? 1 : 0});
        used += (long)pieces;
    }
    // tasks in decreasing item count (longest first) for the persistent grid's dynamic
    // scheduler; each task's own items keep their order, so results do not change
    const int nv = (int)vout.size();
    std::vector<int> ord(nv);
    for (int i = 0; i < nv; i++) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int a, int b) { return vend[a] - vbeg[a] > vend[b] - vbeg[b]; });
    std::vector<double *> outp(nv);
    std::vector<long long> beg(nv), end(nv);
    std::vector<int> redof(nv);
    for (int i = 0; i < nv; i++) {
        outp[i] = vout[ord[i]];
        beg[i] = vbeg[ord[i]];
        end[i] = vend[ord[i]];
        redof[i] = vred[ord[i]];
    }
    Packer pk;
    pk.add(outp.data(), outp.size() * sizeof(double *));
    pk.add(beg.data(), beg.size() * sizeof(long long));
    pk.add(end.data(), end.size() * sizeof(long long));
    const size_t nh = dv ? 0 : ni;  // item arrays shipped from the host (none when the GPU wrote them)
    pk.add(li.in.data(), nh * sizeof(void *));
    pk.add(li.ax.data(), nh * sizeof(void *));
    pk.add(li.ay.data(), nh * sizeof(void *));
    pk.add(li.az.data(), nh * sizeof(void *));
    pk.add(li.coef.data(), nh * sizeof(double));
    pk.add(red.data(), red.size() * sizeof(ReduceTask));
    pk.add(redof.data(), redof.size() * sizeof(int));
    // the task counter, the status word, the row count and the chunk counters start at zero: they
    // travel with the pack instead of being cleared by separate launches
    std::vector<int> zeros(3 + red.size(), 0);
    pk.add(zeros.data(), zeros.size() * sizeof(int));
    pk.ship(ctx, arena);
    int *counter = (int *)pk.ptr(10);
    int *red_cnt = red.empty() ? nullptr : counter + 3;
    ApplyLaunch L;
    L.nnodes = nv;
    L.root = root ? 1 : 0;
    L.set = set ? 1 : 0;
    L.out = (double *const *)pk.ptr(0);
    L.begin = (const long long *)pk.ptr(1);
    L.end = (const long long *)pk.ptr(2);
    L.in = (const void *const *)pk.ptr(3);
    L.ax = (const void *const *)pk.ptr(4);
    L.ay = (const void *const *)pk.ptr(5);
    L.az = (const void *const *)pk.ptr(6);
    L.coef = (const double *)pk.ptr(7);
    if (dv) {
        const long long b0 = dv->base[tier];
        L.in = (const void *const *)(dv->in + b0);
        L.ax = (const void *const *)(dv->ax + b0);
        L.ay = (const void *const *)(dv->ay + b0);
        L.az = (const void *const *)(dv->az + b0);
        L.coef = dv->coef + b0;
    }
    L.counter = counter;
    L.status = counter + 1;
    L.rows = counter + 2;
    if (!red.empty()) {
        L.red = (const ReduceTask *)pk.ptr(8);
        L.red_of = (const int *)pk.ptr(9);
        L.red_cnt = red_cnt;
    }
    st.launches++;
    int *hs = nullptr;
    // tier 1 in the tensor-core modes: the split-TF32 tcgen05 kernel (FP32 accuracy); else the
    // FP32 CUDA-core kernel
    const bool tc = tier == 2 || (tier == 1 && split_tc);
    if (tier == 3) {
        k_apply_df(ctx.dbasis, L, ctx.nsm, ctx.stream);
    } else {
        if (tc)
            k_apply_tc05(ctx.dbasis, L, tier == 1, ctx.stream);
        else
            k_apply(ctx.dbasis, L, tier, ctx.nsm, ctx.stream);
    }
    // the status word (the tensor-core kernels wait for bulk copies with a bound) and the row count
    hs = (int *)arena.halloc(2 * sizeof(int));
    hs[0] = hs[1] = 0;
    MWG_CUDA(cudaMemcpyAsync(hs, L.status, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
    return hs;
}

// runs host code with the context's stream pointing at another stream
struct StreamSwap {
    Ctx &c;
    cudaStream_t saved;
    StreamSwap(Ctx &c_, cudaStream_t s) : c(c_), saved(c_.stream) { c.stream = s; }
    ~StreamSwap() { c.stream = saved; }
};

// ------------------------------------------------------------------ screening on the GPU
// Per-apply tables of the GPU screening (mw_screen.cu): each operator's bands, offsets and
// sub-block norms (uploaded once per operator), and per job the input tree's hash table and the
// norms the host screens with.
struct DevScreen {
    bool on = false;
    std::vector<double> op_max;  // per job: its operator's largest sub-block norm
    int levels = 0;  // levels 0 .. levels-1 are screened on the GPU
    int maxT = 0;
    ScreenJob *djobs = nullptr;
    cudaEvent_t ev_counts = nullptr;  // the write pass's per-node tier counts have reached the host
};

// layout of Oper::d_screen: int band[TS], int off[TS] | double amax[TS], xmax[TS], c[T], norms[4 nb]
// | float amax32[TS], xmax32[TS], norms32[4 nb]   (TS = T * S, nb = blocks)
struct OperScreenLayout {
    size_t TS, nb, ib, db, fb;
    explicit OperScreenLayout(const Oper &op) {
        TS = (size_t)op.T * op.S;
        nb = (size_t)std::max<long>(op.nblocks, 1);
        ib = ((2 * TS * sizeof(int)) + 255) & ~size_t(255);
        db = ((sizeof(double) * (2 * TS + (size_t)op.T + 4 * nb)) + 255) & ~size_t(255);
        fb = sizeof(float) * (2 * TS + 4 * nb);
    }
};

bool oper_screen_tables(Oper &op) {
    if (op.d_screen) return true;
    const OperScreenLayout ly(op);
    const size_t TS = ly.TS;
    for (size_t i = 0; i < TS; i++)
        if (op.band[i] > 32767 || op.off[i] > 0x3fffffffL) return false;
    if (op.nblocks > 0x3fffffffL) return false;
    std::vector<char> h(ly.ib + ly.db + ly.fb, 0);
    int *iv = (int *)h.data();
    double *dd = (double *)(h.data() + ly.ib);
    float *ff = (float *)(h.data() + ly.ib + ly.db);
    for (size_t i = 0; i < TS; i++) {
        iv[i] = op.band[i];
        iv[TS + i] = (int)op.off[i];
        dd[i] = op.amax[i];
        dd[TS + i] = op.xmax[i];
        ff[i] = (float)op.amax[i];
        ff[TS + i] = (float)op.xmax[i];
    }
    for (int t = 0; t < op.T; t++) dd[2 * TS + t] = op.c[t];
    for (size_t i = 0; i < op.norms.size(); i++) {
        dd[2 * TS + op.T + i] = op.norms[i];
        ff[2 * TS + i] = (float)op.norms[i];
    }
    MWG_CUDA(cudaMalloc(&op.d_screen, h.size()));
    MWG_CUDA(cudaMemcpy(op.d_screen, h.data(), h.size(), cudaMemcpyHostToDevice));
    return true;
}

ScreenOp oper_screen_view(const Oper &op) {
    const OperScreenLayout ly(op);
    const size_t TS = ly.TS;
    const int *iv = (const int *)op.d_screen;
    const double *dd = (const double *)((const char *)op.d_screen + ly.ib);
    const float *ff = (const float *)((const char *)op.d_screen + ly.ib + ly.db);
    ScreenOp so;
    so.band = iv;
    so.off = iv + TS;
    so.amax = dd;
    so.xmax = dd + TS;
    so.c = dd + 2 * TS;
    so.norms = dd + 2 * TS + op.T;
    so.amax32 = ff;
    so.xmax32 = ff + TS;
    so.norms32 = ff + 2 * TS;
    so.b64 = op.d_blocks;
    so.b32 = op.d_blocks32;
    so.btc = op.d_blocks_tc;
    so.btc2 = op.split_blocks();
    so.T = op.T;
    so.S = op.S;
    return so;
}

// the largest sub-block norm of an operator (the FP32 estimates need it well inside FP32's range)
double oper_norm_max(const Oper &op) {
    double m = 0.0;
    for (double v : op.amax) m = std::max(m, v);
    return m;
}

// The per-job tables that need the input trees' norms: a hash table of each input tree's keys and
// its component and block norms (FP64 and FP32), and the jobs' ScreenJob entries, uploaded on the
// context's current stream.  `idx`: the jobs to set up (all of them, or one job group's when the
// group's inputs arrive during the apply).
void screen_setup_inputs(Ctx &ctx, std::vector<ApplyJob> &jobs, const std::vector<int> &idx, DevScreen &ds) {
    std::vector<const Tree *> trees;
    std::unordered_map<const Tree *, int> tix;
    for (int j : idx)
        if (tix.emplace(jobs[j].inp, (int)trees.size()).second) trees.push_back(jobs[j].inp);
    std::vector<size_t> cap(trees.size()), off(trees.size() + 1, 0);
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    for (size_t i = 0; i < trees.size(); i++) {
        size_t c = 64;
        while (c < 2 * (size_t)trees[i]->nn()) c <<= 1;
        cap[i] = c;
        off[i + 1] = off[i] + al(c * sizeof(int4)) + al(c * sizeof(int)) + al(sizeof(double) * 9 * trees[i]->nn()) +
                     al(sizeof(float) * 9 * trees[i]->nn());
    }
    const size_t total = off.back() + al(sizeof(ScreenJob) * idx.size());
    char *h = (char *)ctx.sarena.halloc(total);
    char *d = (char *)ctx.sarena.alloc(total);
    for (size_t i = 0; i < trees.size(); i++) {
        const Tree &t = *trees[i];
        const size_t c = cap[i];
        int4 *hk = (int4 *)(h + off[i]);
        int *hv = (int *)(h + off[i] + al(c * sizeof(int4)));
        double *cn = (double *)(h + off[i] + al(c * sizeof(int4)) + al(c * sizeof(int)));
        for (size_t e = 0; e < c; e++) {
            hk[e] = make_int4(HASH_EMPTY, 0, 0, 0);
            hv[e] = -1;
        }
        for (int n = 0; n < t.nn(); n++) {
            const NodeInfo &ni = t.nodes[n];
            unsigned e = key_hash(ni.n, ni.l[0], ni.l[1], ni.l[2]) & (unsigned)(c - 1);
            while (hk[e].x != HASH_EMPTY) e = (e + 1) & (unsigned)(c - 1);
            hk[e] = make_int4(ni.n, ni.l[0], ni.l[1], ni.l[2]);
            hv[e] = n;
        }
        std::memcpy(cn, t.cn.data(), sizeof(double) * 8 * t.nn());
        for (int n = 0; n < t.nn(); n++) cn[8 * (size_t)t.nn() + n] = block_norm8(&t.cn[8 * (size_t)n]);
        float *cn32 = (float *)((char *)cn + al(sizeof(double) * 9 * t.nn()));
        for (size_t e = 0; e < 9 * (size_t)t.nn(); e++) cn32[e] = (float)cn[e];
    }
    ScreenJob *hj = (ScreenJob *)(h + off.back());
    for (size_t q = 0; q < idx.size(); q++) {
        const int j = idx[q];
        const int i = tix[jobs[j].inp];
        const Tree &t = *trees[i];
        const size_t c = cap[i];
        ScreenJob &J = hj[q];
        J.op = oper_screen_view(*jobs[j].op);
        J.hkey = (const int4 *)(d + off[i]);
        J.hval = (const int *)(d + off[i] + al(c * sizeof(int4)));
        J.hmask = (int)(c - 1);
        J.pad = 0;
        J.cn = (const double *)(d + off[i] + al(c * sizeof(int4)) + al(c * sizeof(int)));
        J.bn = J.cn + 8 * (size_t)t.nn();
        J.cn32 = (const float *)((const char *)J.cn + al(sizeof(double) * 9 * t.nn()));
        J.bn32 = J.cn32 + 8 * (size_t)t.nn();
        J.in64 = t.d_coefs;
        J.in32 = t.d_coefs32;
        J.intc = t.d_coefs_tc;
    }
    // read by kernels from the pinned staging: with host inputs these tables go up while the later
    // job groups' input blocks still occupy the copy engines
    k_fetch(d, h, off.back(), ctx.stream);
    ctx.fetch_launches++;
    // the entries go to their jobs' places in the apply's ScreenJob array (contiguous runs copied
    // together)
    for (size_t q = 0; q < idx.size();) {
        size_t r = q + 1;
        while (r < idx.size() && idx[r] == idx[r - 1] + 1) r++;
        k_fetch(ds.djobs + idx[q], hj + q, sizeof(ScreenJob) * (r - q), ctx.stream);
        ctx.fetch_launches++;
        q = r;
    }
}

// The per-apply part that needs no input data: the levels the GPU screens, the operators' tables,
// and the ScreenJob array; false when an operator falls outside what the kernels encode (bands
// above 32767), and the host screens instead.  With `inputs_now` the input tables are built too.
bool screen_setup(Ctx &ctx, std::vector<ApplyJob> &jobs, DevScreen &ds, bool inputs_now) {
    const Basis &b = ctx.basis;
    // levels whose translations fit the generation tables' 21-bit fields (deeper levels, about
    // 20 scales below the root, are screened on the host)
    ds.levels = 0;
    while (ds.levels < 40) {
        bool fits = true;
        for (int d = 0; d < 3; d++) fits &= ((long)b.boxes[d] << ds.levels) < (1L << 21);
        if (!fits) break;
        ds.levels++;
    }
    for (ApplyJob &job : jobs)
        if (!oper_screen_tables(*job.op)) return false;
    for (ApplyJob &job : jobs) {
        ds.op_max.push_back(oper_norm_max(*job.op));
        ds.maxT = std::max(ds.maxT, job.op->T);
    }
    ds.djobs = (ScreenJob *)ctx.sarena.alloc(sizeof(ScreenJob) * jobs.size());
    if (!ds.ev_counts) MWG_CUDA(cudaEventCreateWithFlags(&ds.ev_counts, cudaEventDisableTiming));
    if (inputs_now) {
        std::vector<int> all(jobs.size());
        for (size_t j = 0; j < jobs.size(); j++) all[j] = (int)j;
        screen_setup_inputs(ctx, jobs, all, ds);
    }
    ds.on = true;
    return true;
}

struct TierRule {  // the apply's precision mode, as the tier choice reads it
    bool mixed, near_fp64, df_only, dfp, tensor;
};

// the walk kernels' (t, lz) rows at a scale: the most over the group's operators
int level_zrows(const std::vector<JobState *> &jp, int sidx) {
    int zmax = 1;
    for (const JobState *sp : jp) {
        const Oper &op = *sp->job->op;
        int z = 0;
        for (int t = 0; t < op.T; t++) {
            const int L = op.band[t * op.S + sidx];
            if (L >= 0) z += 2 * L + 1;
        }
        zmax = std::max(zmax, z);
    }
    return zmax;
}
constexpr size_t SCREEN_SMEM_MAX = 96 * 1024;  // larger walks (very wide bands) are screened on the host

// One level of a job group screened on the GPU (mw_screen.cu).  The walk, the generation of
// missing inputs, the exact screening, the tiers and the item arrays run on the high-priority
// stream; the host reads back two small arrays (per-node candidate counts, then per-node tier
// counts), from which it sizes the buffers and builds each tier's node list exactly as the host
// screening does.  The group's stream waits for the item arrays with an event.
void screen_level_gpu(Ctx &ctx, Arena &ar, DevScreen &ds, const std::vector<JobState *> &jp,
                      const std::vector<int> &jglob, int level, int zmax, const TierRule &rule, LevelItems *lt,
                      DevItems &dv, mw_stats &st, double &t_enum, double &t_gen, double &t_items) {
    const Basis &b = ctx.basis;
    const int K = b.K, bs = b.bs, bsz = 4 * K * K;
    const double K4 = (double)K * K * K * K;
    const int n = b.n0 + level, sidx = level;
    const bool root = level == 0;
    auto now = [] { return std::chrono::steady_clock::now(); };
    auto ms = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point c) {
        return std::chrono::duration<double, std::milli>(c - a).count();
    };
    const auto tA = now();
    cudaStream_t gstream = ctx.stream;
    // node records in the host's order (jobs of the group, then their work lists)
    std::vector<ScreenNode> nodes;
    std::vector<double *> outb;
    std::vector<long> gcap(jp.size(), 0);
    long gtot = 0;
    for (size_t j = 0; j < jp.size(); j++) {
        JobState &s = *jp[j];
        long c = 256;
        while (c < 16 * (long)s.work.size()) c <<= 1;
        if (ctx.screen_gen_slots > 0) {
            c = 1;
            while (c < ctx.screen_gen_slots) c <<= 1;
        }
        gcap[j] = c;
        const double fm = BOUND_PRUNE * s.fmax_at(sidx);
        const double base = SCREEN_FAC * split_thr(s.job->prec, s.R, n);
        for (size_t w = 0; w < s.work.size(); w++) {
            ScreenNode nd;
            const double wg = s.wgt[w], wgc = std::max(wg, 1e-300);
            nd.thr = root ? 0.0 : (wg > 0.0 ? base / wg : 0.0);
            nd.thr2 = root ? 0.0 : base / wgc;
            nd.tthr = !root ? nd.thr2
                      : s.job->abs_prec ? SCREEN_FAC * split_thr(s.job->prec, 1.0, n) / wgc
                                        : -1.0;
            nd.fm = fm;
            nd.job = jglob[j];
            const NodeInfo &o = s.job->out->nodes[s.work[w]];
            for (int d = 0; d < 3; d++) nd.l[d] = o.l[d];
            nd.flags = ((!root && wg <= 0.0) ? 1 : 0) | ((!root || (s.job->abs_prec && s.job->prec_trees.empty())) ? 2 : 0);
            nd.gtab = (int)gtot;
            nd.gmask = (int)(gcap[j] - 1);
            // FP32 estimates decide clear cases when every factor of a bound is at most 1e6 (input
            // norms are at most fm) and the thresholds are at least 1e-14: then FP32 rounding (2e-6
            // relative) and products flushed below FP32's range (< 1e-24 in all) stay well inside
            // the 1e-4 relative bands, and FP64 decides inside them
            constexpr double BAND = 1e-4, BIG = 1e6, SMALL = 1e-14;
            const bool fast = fm <= BIG && ds.op_max[nd.job] <= BIG &&
                              (root || (nd.thr >= SMALL && nd.thr2 >= SMALL)) &&
                              (nd.tthr < 0.0 || nd.tthr >= SMALL);
            if (fast) nd.flags |= 4;
            nd.thr_lo = (float)(nd.thr * (1.0 - BAND));
            nd.thr_hi = (float)(nd.thr * (1.0 + BAND));
            nd.thr2_lo = (float)(nd.thr2 * (1.0 - BAND));
            nd.thr2_hi = (float)(nd.thr2 * (1.0 + BAND));
            const double tb[3] = {TIER_TF32, TIER_FP64, TIER_DF};
            for (int k = 0; k < 3; k++) {
                const double B = nd.tthr >= 0.0 ? tb[k] * nd.tthr : 0.0;
                nd.tier_lo[k] = (float)(B * (1.0 - BAND));
                nd.tier_hi[k] = (float)(B * (1.0 + BAND));
            }
            nd.fm32 = (float)fm;
            nd.prune32 = (float)(nd.thr * (1.0 - BAND));
            nodes.push_back(nd);
            outb.push_back(s.job->out->block(s.work[w]));
        }
        gtot += gcap[j];
    }
    const int NN = (int)nodes.size();
    ScreenLevel P{};
    P.jobs = ds.djobs;
    P.nn = NN;
    P.n = n;
    P.sidx = sidx;
    P.root = root ? 1 : 0;
    P.n0 = b.n0;
    P.bs = bs;
    P.bsz = bsz;
    for (int d = 0; d < 3; d++) {
        P.lo[d] = (int)((long)b.corner[d] * (1L << (n - b.n0)));
        P.hi[d] = (int)((long)(b.corner[d] + b.boxes[d]) * (1L << (n - b.n0)));
    }
    P.mixed = rule.mixed;
    P.near_fp64 = rule.near_fp64;
    P.df_only = rule.df_only;
    P.dfp = rule.dfp;
    P.tensor = rule.tensor;
    P.tier_fp64 = TIER_FP64;
    P.tier_tf32 = TIER_TF32;
    P.tier_df = TIER_DF;
    P.tx = tc5_x_stride(K);
    P.tb = tc5_b_stride(K);
    // walk 1: candidate counts and generation requests (tables grown and the walk repeated if a
    // job's generation table fills up)
    int *hc = nullptr;
    int ngen = 0;
    {
        StreamSwap fast(ctx, ctx.fast);
        for (int attempt = 0;; attempt++) {
            if (attempt > 0) st.screen_regrows++;
            if (gtot > (1L << 26)) throw Error(MW_ERR_STATE, "apply: generation tables of the GPU screening overflowed");
            if (attempt > 0) {
                gtot = 0;
                for (size_t j = 0, q = 0; j < jp.size(); j++) {
                    gcap[j] *= 8;
                    for (size_t w = 0; w < jp[j]->work.size(); w++, q++) {
                        nodes[q].gtab = (int)gtot;
                        nodes[q].gmask = (int)(gcap[j] - 1);
                    }
                    gtot += gcap[j];
                }
            }
            std::vector<unsigned long long> zeros((size_t)gtot + 1, 0ull);  // keys, then the counter and flag
            Packer pk;
            pk.add(nodes.data(), sizeof(ScreenNode) * NN);
            pk.add(zeros.data(), sizeof(unsigned long long) * zeros.size());
            pk.ship(ctx, ar);
            P.nodes = (const ScreenNode *)pk.ptr(0);
            P.gkey = (unsigned long long *)pk.ptr(1);
            P.gen_cnt = (int *)(P.gkey + gtot);
            P.overflow = P.gen_cnt + 1;
            P.gval = (int *)ar.alloc(sizeof(int) * (size_t)gtot);
            P.gen_cap = (int)gtot;
            P.gen_info = (int *)ar.alloc(sizeof(int) * 6 * (size_t)gtot);
            P.cnt = (int *)ar.alloc(sizeof(int) * (size_t)NN);
            k_screen_count(P, ds.maxT, zmax, ctx.stream);
            st.launches++;
            hc = (int *)ar.halloc(sizeof(int) * ((size_t)NN + 2));
            MWG_CUDA(cudaMemcpyAsync(hc, P.cnt, sizeof(int) * NN, cudaMemcpyDeviceToHost, ctx.stream));
            MWG_CUDA(cudaMemcpyAsync(hc + NN, P.gen_cnt, sizeof(int) * 2, cudaMemcpyDeviceToHost, ctx.stream));
            MWG_CUDA(cudaStreamSynchronize(ctx.stream));
            if (hc[NN + 1] == 0) break;
        }
        ngen = hc[NN];
    }
    const auto tB = now();
    t_enum += ms(tA, tB);
    // buffers sized by the counts; generation of the missing inputs
    std::vector<long long> coff(NN);
    long long ctot = 0;
    for (int q = 0; q < NN; q++) {
        coff[q] = ctot;
        ctot += hc[q];
    }
    const size_t cap = (size_t)std::max<long long>(ctot, 1);
    P.cand = (ScreenCand *)ar.alloc(sizeof(ScreenCand) * cap);
    dv.in = (const void **)ar.alloc(sizeof(void *) * cap);
    dv.ax = (const void **)ar.alloc(sizeof(void *) * cap);
    dv.ay = (const void **)ar.alloc(sizeof(void *) * cap);
    dv.az = (const void **)ar.alloc(sizeof(void *) * cap);
    dv.coef = (double *)ar.alloc(sizeof(double) * cap);
    P.in = dv.in;
    P.ax = dv.ax;
    P.ay = dv.ay;
    P.az = dv.az;
    P.coef = dv.coef;
    P.tcnt = (int *)ar.alloc(sizeof(int) * 8 * (size_t)NN);
    P.tier_off = (long long *)ar.alloc(sizeof(long long) * 4 * (size_t)NN);
    P.tier_tot = (long long *)ar.alloc(sizeof(long long) * 4);
    const size_t ng = (size_t)std::max(ngen, 1);
    P.gcn = (double *)ar.alloc(sizeof(double) * 8 * ng);
    P.gcn32 = (float *)ar.alloc(sizeof(float) * 8 * ng);
    P.g64 = (double *)ar.alloc(sizeof(double) * (size_t)bs * ng);
    P.g32 = rule.mixed ? (float *)ar.alloc(sizeof(float) * 2 * (size_t)bs * ng) : nullptr;
    P.gtc = rule.tensor ? (float *)ar.alloc(sizeof(float) * P.tx * ng) : nullptr;
    int *hs = (int *)ar.halloc(sizeof(int) * (8 * (size_t)NN + 1));
    {
        StreamSwap fast(ctx, ctx.fast);
        Packer pk;
        pk.add(coff.data(), sizeof(long long) * NN);
        pk.ship(ctx, ar);
        P.cand_off = (const long long *)pk.ptr(0);
        if (ngen > 0) {
            GenTask *tasks = (GenTask *)ar.alloc(sizeof(GenTask) * (size_t)ngen);
            k_screen_gen_tasks(P, tasks, ngen, ctx.stream);
            const int ggrid = std::min(ngen, 4 * std::max(ctx.nsm, 1));
            double *gscratch = (K >= 4 && K <= KMAX)
                                   ? nullptr
                                   : (double *)ar.alloc(sizeof(double) * generate_scratch_doubles(K) * ggrid);
            k_generate(ctx.dbasis, tasks, ngen, gscratch, ggrid, ctx.nsm, ctx.stream);
            k_screen_gen_norms32(P, ngen, ctx.stream);
            st.launches += 3;
            st.generated += ngen;
            if (rule.mixed) {
                k_to_fp32_cube(P.g64, P.g32, (size_t)ngen, K, ctx.stream);
                st.launches++;
                if (rule.tensor) {
                    k_to_tc_x(P.g32, P.gtc, (size_t)ngen, K, ctx.stream);
                    st.launches++;
                }
            }
        }
        const auto tC = now();
        t_gen += ms(tB, tC);
        // walk 2: items with their tiers, per-node tier counts back to the host, then the item arrays
        k_screen_write(P, ds.maxT, zmax, ctx.stream);
        st.launches += 2;
        MWG_CUDA(cudaMemcpyAsync(hs, P.tcnt, sizeof(int) * 8 * NN, cudaMemcpyDeviceToHost, ctx.stream));
        MWG_CUDA(cudaMemcpyAsync(hs + 8 * NN, P.overflow, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
        MWG_CUDA(cudaEventRecord(ds.ev_counts, ctx.stream));
        k_screen_fill(P, ctx.stream);
        st.launches++;
        MWG_CUDA(cudaEventRecord(ctx.fast_done, ctx.stream));
    }
    MWG_CUDA(cudaStreamWaitEvent(gstream, ctx.fast_done, 0));
    MWG_CUDA(cudaEventSynchronize(ds.ev_counts));
    if (hs[8 * NN] != 0) throw Error(MW_ERR_STATE, "apply: a generated input was missing from the GPU screening's tables");
    const auto tD = now();
    // each tier's node list in node order, as the host screening builds it
    long long tot[NTIER] = {0, 0, 0, 0}, pairs[NTIER] = {0, 0, 0, 0};
    long nnt[NTIER] = {0, 0, 0, 0};
    for (int q = 0; q < NN; q++)
        for (int k = 0; k < NTIER; k++) {
            if (hs[8 * q + k] > 0) nnt[k]++;
            tot[k] += hs[8 * q + k];
            pairs[k] += hs[8 * q + 4 + k];
        }
    long long base = 0;
    for (int k = 0; k < NTIER; k++) {
        dv.base[k] = base;
        base += tot[k];
        LevelItems &T = lt[k];
        T.nodes = nnt[k];
        T.items = tot[k];
        if ((long)T.out.size() < nnt[k]) T.out.resize(nnt[k]);
        if ((long)T.begin.size() < nnt[k] + 1) T.begin.resize(nnt[k] + 1);
        T.begin[0] = 0;
        long slot = 0;
        long long run = 0;
        for (int q = 0; q < NN; q++) {
            const int c = hs[8 * q + k];
            if (c <= 0) continue;
            run += c;
            T.out[slot] = outb[q];
            T.begin[++slot] = run;
        }
    }
    st.items += tot[0] + tot[1] + tot[2] + tot[3];
    st.items_fp64 += tot[0];
    st.items_fp32 += tot[1];
    st.items_tf32 += tot[2];
    st.items_df += tot[3];
    st.flops += 6.0 * K4 * (double)(pairs[0] + pairs[1] + pairs[2] + pairs[3]);
    st.flops_issued += 96.0 * K4 * (double)(tot[0] + tot[1] + tot[2] + tot[3]);
    st.flops_fp64 += 6.0 * K4 * (double)pairs[0];
    st.flops_fp32 += 6.0 * K4 * (double)pairs[1];
    st.flops_tf32 += 6.0 * K4 * (double)pairs[2];
    st.flops_df += 6.0 * K4 * (double)pairs[3];
    t_items += ms(tD, now());
}

void check_status(const int *hs) {
    if (hs && *hs != 0)
        throw Error(MW_ERR_TIMEOUT,
                    "apply: a bounded wait for an asynchronous copy or MMA ran out (status " + std::to_string(*hs) + ")");
}

}  // namespace

void apply_batch(std::vector<ApplyJob> &jobs, int precision_mode, bool fixed_grid, mw_stats &st,
                 const HostInputs *hin) {
    if (jobs.empty()) return;
    Ctx &ctx = *jobs[0].out->ctx;
    const Basis &b = ctx.basis;
    const int K = b.K, bs = b.bs, bsz = 4 * K * K;
    const double K4 = (double)K * K * K * K;
    const bool mixed = precision_mode != MW_PREC_FP64;
    const bool near_fp64 = precision_mode == MW_PREC_MIXED_NEARFP64;
    const bool tensor = mixed && precision_mode != MW_PREC_MIXED_FP32 && precision_mode != MW_PREC_DF;
    const bool dfp = tensor;  // the double-FP32 tier comes with the tensor-core tier
    const bool df_only = precision_mode == MW_PREC_DF;
    auto t_start = std::chrono::steady_clock::now();
    const long long fetch0 = ctx.fetch_launches;
    Arena &arena = ctx.arena;
    // copies into the arenas that an apply which failed part-way left in flight end first
    if (ctx.ustream) MWG_CUDA(cudaStreamSynchronize(ctx.ustream));
    arena.reset();
    float kernel_ms = 0.0f;
    // GPU spans: set-up + levels, and the post-processing after them
    cudaEvent_t ev_span[3];
    for (auto &e : ev_span) MWG_CUDA(cudaEventCreate(&e));
    MWG_CUDA(cudaEventRecord(ev_span[0], ctx.stream));

    // the reduced tiers' copies of an input tree's blocks (FP32 cube-order shadows, and the TF32
    // tier's x-pass operand), on the context's current stream
    auto convert_input = [&](Tree &in) {
        k_to_fp32_cube(in.d_coefs, in.d_coefs32, (size_t)in.nn(), b.K, ctx.stream);
        st.launches++;
        if (tensor) {
            k_to_tc_x(in.d_coefs32, in.d_coefs_tc, (size_t)in.nn(), b.K, ctx.stream);
            st.launches++;
        }
    };
    // The jobs are split into up to four groups that take turns: while the GPU runs the other
    // groups' levels, the host enumerates, screens and builds the items of one group's level.
    // Group 0 works on the context's stream and arena, the others on extra streams and arenas of
    // the context.  A single job runs as one group.
    struct Group {
        std::vector<int> jobs;
        cudaStream_t stream = nullptr;
        Arena *arena = nullptr;
        int level = 0;
        bool pending = false, done = false;
        LevelItems lt[NTIER];
        cudaEvent_t ev[NTIER + 1];
        std::vector<std::pair<int, int *>> status;  // per launch: tier, pinned copy of (status, rows)
        std::vector<double *> h_cn;  // pinned staging of each job's component norms
        cudaEvent_t ev_up = nullptr;  // host inputs: the group's input blocks are on the device ...
        double *in_blocks = nullptr;  // ... here, in the caller's order
        cudaEvent_t ev_in = nullptr;  // ... are in the trees, with their norms on the host
        double *in_cn = nullptr;      // ... here
        cudaStream_t pstream = nullptr;  // ... the high-priority stream that prepares them
        cudaEvent_t ev_prep = nullptr;   // ... reduced copies and screening tables written
    };
    // launch settings: the autotuner's for this (order, jobs, mode) if it ran, else the context's
    Ctx::Tuning tune;
    tune.groups = ctx.groups;
    {
        auto it = ctx.tuned.find(std::make_tuple(b.K, (int)jobs.size(), precision_mode));
        if (it != ctx.tuned.end() && ctx.groups > 1) tune = it->second;
    }
    const int ngroups = std::max(1, std::min<int>(tune.groups, (int)jobs.size()));
    std::vector<Group> groups(ngroups);
    {
        // balance the groups by input size, largest jobs first into the lightest group
        auto in_nn = [&](int j) -> long { return hin ? hin->nnodes[j] : jobs[j].inp->nn(); };
        std::vector<int> ord(jobs.size());
        for (size_t j = 0; j < jobs.size(); j++) ord[j] = (int)j;
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) { return in_nn(a) > in_nn(c); });
        std::vector<long> load(ngroups, 0);
        for (int j : ord) {
            int g = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            groups[g].jobs.push_back(j);
            load[g] += in_nn(j);
        }
        for (auto &g : groups) std::sort(g.jobs.begin(), g.jobs.end());
    }
    groups[0].stream = ctx.stream;
    groups[0].arena = &arena;
    for (int g = 1; g < ngroups; g++) {
        ctx.xarena[g - 1].reset();
        groups[g].arena = &ctx.xarena[g - 1];
    }
    // host inputs: every group's blocks start up on the copy stream, in group order, and the host
    // builds the input trees' structures while they move; each group's blocks are permuted into
    // its trees on the group's stream below
    std::vector<std::vector<int>> in_maps;
    if (hin) {
        const auto tS = std::chrono::steady_clock::now();
        if (!ctx.ustream) MWG_CUDA(cudaStreamCreateWithFlags(&ctx.ustream, cudaStreamNonBlocking));
        for (Group &G : groups) {
            size_t tot = 0;
            for (int j : G.jobs) tot += (size_t)hin->nnodes[j];
            G.in_blocks = (double *)G.arena->alloc(sizeof(double) * (size_t)bs * tot);
            size_t off = 0;
            for (int j : G.jobs) {
                MWG_CUDA(cudaMemcpyAsync(G.in_blocks + off * bs, hin->coefs[j], sizeof(double) * (size_t)bs * hin->nnodes[j],
                                         cudaMemcpyHostToDevice, ctx.ustream));
                off += (size_t)hin->nnodes[j];
            }
            MWG_CUDA(cudaEventCreateWithFlags(&G.ev_up, cudaEventDisableTiming));
            MWG_CUDA(cudaEventRecord(G.ev_up, ctx.ustream));
        }
        std::vector<Tree *> itrees;
        for (ApplyJob &job : jobs) itrees.push_back(job.inp);
        in_maps = upload_structures(itrees, hin->nnodes.data(), hin->keys.data());
        st.host_io_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tS).count();
    }
    std::vector<JobState> js(jobs.size());
    int max_levels = 0;
    for (size_t j = 0; j < jobs.size(); j++) {
        ApplyJob &job = jobs[j];
        JobState &s = js[j];
        s.job = &job;
        if (job.inp->ctx != &ctx || job.out->ctx != &ctx || job.op->ctx != &ctx)
            throw Error(MW_ERR_ARG, "apply: trees and operator must belong to one context");
        if (!hin) s.set_fmax(*job.inp, b.n0);  // with host inputs: when the job's group has them
        if (!fixed_grid && job.out->nn() != job.out->nroots)
            throw Error(MW_ERR_STATE, "apply: output tree must be empty");
        // every tier adds into the output blocks: they start at zero (on a fixed grid too, whose
        // coefficients the apply replaces)
        tree_zero(*job.out, 0, job.out->nn());
        if (mixed) {
            Tree &in = *job.inp;
            if (in.cap32 < (size_t)in.nn()) {
                if (in.d_coefs32) cudaFree(in.d_coefs32);
                MWG_CUDA(cudaMalloc(&in.d_coefs32, sizeof(float) * 2 * (size_t)bs * in.cap));
                in.cap32 = in.cap;
            }
            if (tensor && in.cap_tc < (size_t)in.nn()) {
                if (in.d_coefs_tc) cudaFree(in.d_coefs_tc);
                MWG_CUDA(cudaMalloc(&in.d_coefs_tc, sizeof(float) * tc5_x_stride(b.K) * in.cap));
                in.cap_tc = in.cap;
            }
            if (!hin) convert_input(in);
        }
        for (int i = 0; i < job.out->nroots; i++) s.work.push_back(i);
        if (fixed_grid) max_levels = std::max(max_levels, job.out->max_scale() - b.n0 + 1);
        s.R = 1.0;
    }
    // screening on the GPU (mw_screen.cu) when the context asks for it and the jobs fit its tables
    const TierRule rule{mixed, near_fp64, df_only, dfp, tensor};
    DevScreen ds;
    if (ctx.screening == 1) {
        ctx.sarena.reset();
        screen_setup(ctx, jobs, ds, hin == nullptr);
    }
    // fixed grid: per level, the output's nodes at that scale
    auto fixed_level_nodes = [&](JobState &s, int n) {
        s.work.clear();
        for (int i = 0; i < s.job->out->nn(); i++)
            if (s.job->out->nodes[i].n == n) s.work.push_back(i);
    };

    if (!ctx.fast) {
        int least = 0, greatest = 0;
        MWG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        MWG_CUDA(cudaStreamCreateWithPriority(&ctx.fast, cudaStreamNonBlocking, greatest));
        MWG_CUDA(cudaEventCreateWithFlags(&ctx.fast_done, cudaEventDisableTiming));
    }
    cudaEvent_t ev_start = nullptr;
    std::vector<cudaEvent_t> ev_end(ngroups, nullptr);
    // the generation stream and groups 1.. start after everything queued on the context's stream
    // so far (input uploads, FP32 shadows, zeroed roots)
    MWG_CUDA(cudaEventCreateWithFlags(&ev_start, cudaEventDisableTiming));
    MWG_CUDA(cudaEventRecord(ev_start, ctx.stream));
    MWG_CUDA(cudaStreamWaitEvent(ctx.fast, ev_start, 0));
    if (ngroups > 1) {
        for (int g = 1; g < ngroups; g++) {
            cudaStream_t &xs = ctx.xstream[g - 1];
            if (!xs) MWG_CUDA(cudaStreamCreateWithFlags(&xs, cudaStreamNonBlocking));
            groups[g].stream = xs;
            MWG_CUDA(cudaStreamWaitEvent(xs, ev_start, 0));
            MWG_CUDA(cudaEventCreateWithFlags(&ev_end[g], cudaEventDisableTiming));
        }
    }
    for (auto &g : groups)
        for (auto &e : g.ev) MWG_CUDA(cudaEventCreate(&e));
    // host inputs: each group's blocks go into its trees on the group's high-priority stream once
    // they are on the device, so that the first groups compute while the copy engine still moves
    // the later groups' blocks
    if (hin)
        for (int g = 0; g < ngroups; g++) {
            Group &G = groups[g];
            cudaStream_t &ps = ctx.pstream[g];
            if (!ps) {
                int least = 0, greatest = 0;
                MWG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
                MWG_CUDA(cudaStreamCreateWithPriority(&ps, cudaStreamNonBlocking, greatest));
            }
            G.pstream = ps;
            MWG_CUDA(cudaStreamWaitEvent(ps, ev_start, 0));
            StreamSwap swap(ctx, ps);
            MWG_CUDA(cudaStreamWaitEvent(ctx.stream, G.ev_up, 0));
            std::vector<Tree *> trees;
            std::vector<const int *> maps;
            for (int j : G.jobs) {
                trees.push_back(jobs[j].inp);
                maps.push_back(in_maps[j].data());
            }
            G.in_cn = upload_enqueue(trees, maps, G.in_blocks, *G.arena);
            MWG_CUDA(cudaEventCreateWithFlags(&G.ev_in, cudaEventDisableTiming));
            MWG_CUDA(cudaEventRecord(G.ev_in, ctx.stream));
        }

    // host phases of the group's next level and its launches; false when the group has no work left
    auto launch_level = [&](Group &G) -> bool {
        StreamSwap swap(ctx, G.stream);
        Arena &ar = *G.arena;
        const int level = G.level;
        const int n = b.n0 + level, sidx = level;
        std::vector<JobState *> jp;
        for (int j : G.jobs) jp.push_back(&js[j]);
        if (fixed_grid) {
            if (level >= max_levels) return false;
            for (JobState *sp : jp) fixed_level_nodes(*sp, n);
        }
        if (hin && level == 0) {
            // the group's inputs have landed: their norms to the host, then what the apply derives
            // from them (pruning norms per level; reduced-precision copies and screening tables on
            // the group's high-priority stream, which the group's stream and the screening stream
            // wait for on the GPU)
            const auto tI = std::chrono::steady_clock::now();
            MWG_CUDA(cudaEventSynchronize(G.ev_in));
            {
                StreamSwap pswap(ctx, G.pstream);
                size_t off = 0;
                for (int j : G.jobs) {
                    Tree &in = *jobs[j].inp;
                    std::copy(G.in_cn + off, G.in_cn + off + 8 * (size_t)in.nn(), in.cn.begin());
                    off += 8 * (size_t)in.nn();
                    js[j].set_fmax(in, b.n0);
                    if (mixed) convert_input(in);
                }
                if (ds.on) screen_setup_inputs(ctx, jobs, G.jobs, ds);
                MWG_CUDA(cudaEventCreateWithFlags(&G.ev_prep, cudaEventDisableTiming));
                MWG_CUDA(cudaEventRecord(G.ev_prep, ctx.stream));
            }
            MWG_CUDA(cudaStreamWaitEvent(ctx.stream, G.ev_prep, 0));
            MWG_CUDA(cudaStreamWaitEvent(ctx.fast, G.ev_prep, 0));
            st.host_io_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tI).count();
        }
        bool any = false;
        for (JobState *sp : jp) any |= !sp->work.empty();
        if (!any) return false;
        const bool root = (level == 0);
        // thresholds and precision-steering weights
        for (JobState *sp : jp) {
            JobState &s = *sp;
            s.wgt.assign(s.work.size(), 1.0);
            if (!s.job->prec_trees.empty())
                for (size_t w = 0; w < s.work.size(); w++)
                    s.wgt[w] = prec_weight(s.job->prec_trees, n, s.job->out->nodes[s.work[w]].l);
            s.cand.assign(s.work.size(), {});
        }
        LevelItems *lt = G.lt;
        DevItems dv;
        const int zmax = ds.on ? level_zrows(jp, sidx) : 0;
        const bool dscreen = ds.on && level < ds.levels && screen_smem(ds.maxT, zmax) <= SCREEN_SMEM_MAX;
        if (dscreen) {
            screen_level_gpu(ctx, ar, ds, jp, G.jobs, level, zmax, rule, G.lt, dv, st, st.host_enum_ms,
                             st.host_gen_ms, st.host_items_ms);
        } else {
            // phase A: candidate enumeration (host, all the group's nodes in parallel)
            auto tA = std::chrono::steady_clock::now();
            std::vector<std::pair<int, int>> flat;
            for (size_t j = 0; j < jp.size(); j++)
                for (size_t w = 0; w < jp[j]->work.size(); w++) flat.push_back({(int)j, (int)w});
    #pragma omp parallel
            {
                LookupCache cache;
    #pragma omp for schedule(dynamic, 4)
                for (long q = 0; q < (long)flat.size(); q++) {
                    JobState &s = *jp[flat[q].first];
                    int w = flat[q].second;
                    if (!root && s.wgt[w] <= 0.0) {
                        s.cand[w].clear();
                        continue;
                    }
                    double thr = root ? 0.0 : SCREEN_FAC * split_thr(s.job->prec, s.R, n) / s.wgt[w];
                    enumerate_node(s, w, sidx, root, thr, cache);
                }
            }
            auto tB = std::chrono::steady_clock::now();
            st.host_enum_ms += std::chrono::duration<double, std::milli>(tB - tA).count();
            // phase B: generated input nodes (each job has its own set: jobs in parallel, each in order)
    #pragma omp parallel for schedule(dynamic, 1)
            for (long j = 0; j < (long)jp.size(); j++) {
                JobState &s = *jp[j];
                s.gens.clear();
                for (size_t w = 0; w < s.work.size(); w++) {
                    const NodeInfo &o = s.job->out->nodes[s.work[w]];
                    for (Cand &c : s.cand[w]) {
                        if (!c.gen) continue;
                        int p[3] = {o.l[0] - c.lx, o.l[1] - c.ly, o.l[2] - c.lz};
                        c.src = s.gens.request(*s.job->inp, n, p, c.src);
                    }
                }
            }
            {
                // one generation launch for the group; the blocks are contiguous in job order
                std::vector<std::pair<GenSet *, const Tree *>> sets;
                size_t total = 0;
                for (JobState *sp : jp) {
                    sets.push_back({&sp->gens, sp->job->inp});
                    total += sp->gens.keys.size();
                }
                {
                    // generation on the high-priority stream: its kernel and norm download are what
                    // the host waits for before the exact screening; the group's stream then waits
                    // for the generated blocks with an event
                    StreamSwap fast(ctx, ctx.fast);
                    generate_all(sets, ar, &st);
                    MWG_CUDA(cudaEventRecord(ctx.fast_done, ctx.fast));
                }
                MWG_CUDA(cudaStreamWaitEvent(ctx.stream, ctx.fast_done, 0));
                double *first = nullptr;
                for (JobState *sp : jp)
                    if (sp->gens.base && !first) first = sp->gens.base;
                float *first32 = nullptr, *firsttc = nullptr;
                if (mixed && total > 0) {
                    first32 = (float *)ar.alloc(sizeof(float) * 2 * (size_t)bs * total);
                    k_to_fp32_cube(first, first32, total, b.K, ctx.stream);
                    st.launches++;
                    if (tensor) {
                        firsttc = (float *)ar.alloc(sizeof(float) * tc5_x_stride(b.K) * total);
                        k_to_tc_x(first32, firsttc, total, b.K, ctx.stream);
                        st.launches++;
                    }
                }
                for (JobState *sp : jp) {
                    JobState &s = *sp;
                    s.gbase = s.gens.base;
                    s.gcn.swap(s.gens.cn);
                    s.gbase32 = (first32 && s.gbase) ? first32 + 2 * (s.gbase - first) : nullptr;
                    s.gbase_tc = (firsttc && s.gbase) ? firsttc + tc5_x_stride(b.K) * (size_t)((s.gbase - first) / bs) : nullptr;
                }
            }
            auto tC = std::chrono::steady_clock::now();
            st.host_gen_ms += std::chrono::duration<double, std::milli>(tC - tB).count();
            // phase C: exact screening and tier per candidate (parallel), then the
            // per-tier item lists in node order (prefix sums + parallel fill)
            std::vector<std::pair<int, int>> nodes_flat;  // (job, work index) in launch order
            for (size_t j = 0; j < jp.size(); j++)
                for (size_t w = 0; w < jp[j]->work.size(); w++) nodes_flat.push_back({(int)j, (int)w});
            const long NN = (long)nodes_flat.size();
            // per tier (0 FP64, 1 FP32, 2 TF32): per-node item counts, then prefix sums
            std::vector<long long> cnt[NTIER];
            for (int k = 0; k < NTIER; k++) cnt[k].assign(NN + 1, 0);
            long long pairs_tot = 0, pairs_t0 = 0, pairs_t1 = 0, pairs_t2 = 0, pairs_t3 = 0;
    #pragma omp parallel for schedule(dynamic, 4) reduction(+ : pairs_tot, pairs_t0, pairs_t1, pairs_t2, pairs_t3)
            for (long q = 0; q < NN; q++) {
                JobState &s = *jp[nodes_flat[q].first];
                int w = nodes_flat[q].second;
                const Tree &inp = *s.job->inp;
                const Oper &op = *s.job->op;
                double thr = root ? 0.0 : SCREEN_FAC * split_thr(s.job->prec, s.R, n) / std::max(s.wgt[w], 1e-300);
                // tier threshold: the screening threshold; at the root scale (no screening) it is known in
                // advance only for absolute precision, otherwise root items stay in FP64
                double tthr = !root ? thr
                              : s.job->abs_prec ? SCREEN_FAC * split_thr(s.job->prec, 1.0, n) / std::max(s.wgt[w], 1e-300)
                                                : -1.0;
                // TF32 at the root scale only where its threshold is the plain one: absolute precision
                // and no precision-steering trees (their weights shrink on the huge root boxes)
                const bool tf32_here = !root || (s.job->abs_prec && s.job->prec_trees.empty());
                long long c[NTIER] = {0, 0, 0, 0};
                for (Cand &cd : s.cand[w]) {
                    const double *cn = cd.gen ? &s.gcn[8 * (size_t)cd.src] : &inp.cn[8 * (size_t)cd.src];
                    const double *nx = op.norm(cd.t, sidx, cd.lx), *ny = op.norm(cd.t, sidx, cd.ly),
                                 *nz = op.norm(cd.t, sidx, cd.lz);
                    // real inputs keep their bound from the enumeration; generated ones get their own
                    const double bd = cd.gen ? item_bound(nx, ny, nz, cn, root) : cd.bd;
                    if (!root && bd < thr) {
                        cd.tier = -1;
                        continue;
                    }
                    int np_ = item_pairs(nx, ny, nz, cn, root);
                    pairs_tot += np_;
                    bool near = std::max(std::abs(cd.lx), std::max(std::abs(cd.ly), std::abs(cd.lz))) <= 1;
                    int tier;
                    if (!mixed || tthr < 0.0 || (near_fp64 && near))
                        tier = 0;
                    else if (df_only)
                        tier = bd <= TIER_DF * tthr ? 3 : 0;
                    else if (bd > TIER_FP64 * tthr)
                        tier = (dfp && bd <= TIER_DF * tthr) ? 3 : 0;
                    else if (tensor && tf32_here && bd <= TIER_TF32 * tthr)
                        tier = 2;
                    else
                        tier = 1;
                    cd.tier = tier;
                    c[tier]++;
                    (tier == 0 ? pairs_t0 : tier == 1 ? pairs_t1 : tier == 2 ? pairs_t2 : pairs_t3) += np_;
                }
                for (int k = 0; k < NTIER; k++) cnt[k][q + 1] = c[k];
            }
            // every tier adds to the output blocks (zeroed when their nodes were created), so each
            // tier launches only the nodes that have items in it
            std::vector<long> slot[NTIER];
            long nnt[NTIER] = {0, 0, 0, 0};
            for (int k = 0; k < NTIER; k++) slot[k].assign(NN, -1);
            for (long q = 0; q < NN; q++) {
                for (int k = 0; k < NTIER; k++)
                    if (cnt[k][q + 1] > 0) slot[k][q] = nnt[k]++;
                for (int k = 0; k < NTIER; k++) cnt[k][q + 1] += cnt[k][q];
            }
            long long ntot[NTIER];
            for (int k = 0; k < NTIER; k++) {
                ntot[k] = cnt[k][NN];
                lt[k].resize(nnt[k], ntot[k]);
            }
    #pragma omp parallel for schedule(dynamic, 4)
            for (long q = 0; q < NN; q++) {
                JobState &s = *jp[nodes_flat[q].first];
                int w = nodes_flat[q].second;
                const Tree &inp = *s.job->inp;
                const Oper &op = *s.job->op;
                double *ob = s.job->out->block(s.work[w]);
                long long p[NTIER];
                for (int k = 0; k < NTIER; k++) {
                    p[k] = cnt[k][q];
                    if (slot[k][q] >= 0) {
                        lt[k].out[slot[k][q]] = ob;
                        lt[k].begin[slot[k][q] + 1] = cnt[k][q + 1];
                    }
                }
                for (const Cand &cd : s.cand[w]) {
                    if (cd.tier < 0) continue;
                    long bxi = op.block_index(cd.t, sidx, cd.lx), byi = op.block_index(cd.t, sidx, cd.ly),
                         bzi = op.block_index(cd.t, sidx, cd.lz);
                    LevelItems &T = lt[cd.tier];
                    long long &pi = p[cd.tier];
                    if (cd.tier == 0) {
                        T.in[pi] = cd.gen ? (const void *)(s.gbase + (size_t)cd.src * bs) : (const void *)inp.block(cd.src);
                        T.ax[pi] = op.d_blocks + (size_t)bxi * bsz;
                        T.ay[pi] = op.d_blocks + (size_t)byi * bsz;
                        T.az[pi] = op.d_blocks + (size_t)bzi * bsz;
                    } else if (cd.tier == 2 || (cd.tier == 1 && tensor)) {
                        // the tensor-core tiers read their own operand layouts (mw_tc05_layout.h)
                        const size_t tx = tc5_x_stride(b.K), tb = tc5_b_stride(b.K);
                        T.in[pi] = cd.gen ? (const void *)(s.gbase_tc + tx * (size_t)cd.src)
                                          : (const void *)(inp.d_coefs_tc + tx * (size_t)cd.src);
                        const float *bt = cd.tier == 1 ? op.split_blocks() : op.d_blocks_tc;
                        T.ax[pi] = bt + tb * (size_t)bxi;
                        T.ay[pi] = bt + tb * (size_t)byi;
                        T.az[pi] = bt + tb * (size_t)bzi;
                    } else {
                        // the reduced tiers read the FP32 cube-order shadows and the FP32 operator blocks
                        // (high part first, low part after it)
                        T.in[pi] = cd.gen ? (const void *)(s.gbase32 + 2 * (size_t)cd.src * bs)
                                          : (const void *)(inp.d_coefs32 + 2 * (size_t)cd.src * bs);
                        T.ax[pi] = op.d_blocks32 + 2 * (size_t)bxi * bsz;
                        T.ay[pi] = op.d_blocks32 + 2 * (size_t)byi * bsz;
                        T.az[pi] = op.d_blocks32 + 2 * (size_t)bzi * bsz;
                    }
                    T.coef[pi] = op.c[cd.t];
                    pi++;
                }
            }
            st.items += ntot[0] + ntot[1] + ntot[2] + ntot[3];
            st.items_fp64 += ntot[0];
            st.items_fp32 += ntot[1];
            st.items_tf32 += ntot[2];
            st.items_df += ntot[3];
            st.flops += 6.0 * K4 * (double)pairs_tot;
            st.flops_issued += 96.0 * K4 * (double)(ntot[0] + ntot[1] + ntot[2] + ntot[3]);
            st.flops_fp64 += 6.0 * K4 * (double)pairs_t0;
            st.flops_fp32 += 6.0 * K4 * (double)pairs_t1;
            st.flops_tf32 += 6.0 * K4 * (double)pairs_t2;
            st.flops_df += 6.0 * K4 * (double)pairs_t3;
            st.host_items_ms +=
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tC).count();
        }
        const auto tD = std::chrono::steady_clock::now();
        MWG_CUDA(cudaEventRecord(G.ev[0], ctx.stream));
        G.status.clear();
        for (int k = 0; k < NTIER; k++) {
            int *hs = launch_tier(ctx, ar, lt[k], root, false, k, tune.chunk[k], st, dscreen ? &dv : nullptr,
                                  tensor && k == 1);
            if (hs) G.status.push_back({k, hs});
            MWG_CUDA(cudaEventRecord(G.ev[k + 1], ctx.stream));
        }
        // norms of the level's output nodes, downloaded into pinned staging
        std::vector<double *> bl, cnp;
        for (JobState *sp : jp)
            for (int oi : sp->work) {
                bl.push_back(sp->job->out->block(oi));
                cnp.push_back(sp->job->out->d_cn + (size_t)8 * oi);
            }
        {
            Packer pk;
            pk.add(bl.data(), bl.size() * sizeof(double *));
            pk.add(cnp.data(), cnp.size() * sizeof(double *));
            pk.ship(ctx, ar);
            k_norms(ctx.dbasis, (double *const *)pk.ptr(0), (double *const *)pk.ptr(1), (int)bl.size(), ctx.stream);
            st.launches++;
        }
        G.h_cn.assign(jp.size(), nullptr);
        for (size_t j = 0; j < jp.size(); j++) {
            Tree &out = *jp[j]->job->out;
            G.h_cn[j] = (double *)ar.halloc(sizeof(double) * 8 * out.nn());
            MWG_CUDA(cudaMemcpyAsync(G.h_cn[j], out.d_cn, sizeof(double) * 8 * out.nn(), cudaMemcpyDeviceToHost,
                                     ctx.stream));
        }
        st.host_launch_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tD).count();
        return true;
    };

    // waits for the group's level, then the refinement decisions on its norms
    auto finish_level = [&](Group &G) {
        StreamSwap swap(ctx, G.stream);
        const int n = b.n0 + G.level;
        const bool root = (G.level == 0);
        auto tW = std::chrono::steady_clock::now();
        ctx.sync();
        auto tR = std::chrono::steady_clock::now();
        st.host_wait_ms += std::chrono::duration<double, std::milli>(tR - tW).count();
        for (const auto &ts : G.status) {
            check_status(ts.second);
            long long &rows = ts.first == 0 ? st.rows_fp64 : ts.first == 1 ? st.rows_fp32 : ts.first == 2 ? st.rows_tf32 : st.rows_df;
            rows += ts.second[1];
        }
        float ms_t[NTIER];
        for (int k = 0; k < NTIER; k++) MWG_CUDA(cudaEventElapsedTime(&ms_t[k], G.ev[k], G.ev[k + 1]));
        kernel_ms += ms_t[0] + ms_t[1] + ms_t[2] + ms_t[3];
        st.kernel_ms_fp64 += ms_t[0];
        st.kernel_ms_fp32 += ms_t[1];
        st.kernel_ms_tf32 += ms_t[2];
        st.kernel_ms_df += ms_t[3];
        for (size_t j = 0; j < G.jobs.size(); j++) {
            JobState &s = js[G.jobs[j]];
            Tree &out = *s.job->out;
            std::copy(G.h_cn[j], G.h_cn[j] + (size_t)8 * out.nn(), out.cn.begin());
            st.out_nodes += (long long)s.work.size();
            st.bytes += 8.0 * bs * (double)s.work.size();
            if (root && !s.job->abs_prec) {
                double r2 = 0.0;
                for (int oi : s.work) r2 += std::pow(block_norm8(&out.cn[8 * (size_t)oi]), 2);
                s.R = r2 > 0.0 ? std::sqrt(r2) : 1.0;
            }
            std::vector<int> next;
            if (!fixed_grid && (s.job->max_iter < 0 || s.iter < s.job->max_iter) && n < b.max_scale()) {
                double thr = split_thr(s.job->prec, s.R, n);
                for (size_t w = 0; w < s.work.size(); w++) {
                    int oi = s.work[w];
                    if (wavelet_norm8(&out.cn[8 * (size_t)oi]) * s.wgt[w] > thr) {
                        int c0 = out.split(oi);
                        for (int c = 0; c < 8; c++) next.push_back(c0 + c);
                    }
                }
                tree_zero(out, out.nn() - (int)next.size(), (int)next.size());
            }
            s.work.swap(next);
            s.iter++;
        }
        st.levels++;
        G.arena->reset();
        G.level++;
        st.host_refine_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tR).count();
    };

    // post-processing of a set of jobs on the context's current stream: top-down sum over scales,
    // bottom-up compression, leaf norms, and the norms' download into pinned staging (copied into
    // the trees after the final synchronisation)
    std::vector<std::pair<Tree *, double *>> cn_staging;
    auto post_process = [&](const std::vector<JobState *> &jset, Arena &ar) {
        int maxn = b.n0;
        for (JobState *sp : jset) maxn = std::max(maxn, sp->job->out->max_scale());
        for (int n = b.n0; n < maxn; n++) {
            std::vector<PairTask> tasks;
            for (JobState *sp : jset) {
                Tree &out = *sp->job->out;
                for (int i = 0; i < out.nn(); i++)
                    if (out.nodes[i].n == n && out.nodes[i].child0 >= 0)
                        tasks.push_back({out.block(i), out.block(out.nodes[i].child0)});
            }
            if (tasks.empty()) continue;
            Packer pk;
            pk.add(tasks.data(), tasks.size() * sizeof(PairTask));
            pk.ship(ctx, ar);
            if (mixed)
                k_topdown_df(ctx.dbasis, (const PairTask *)pk.ptr(0), (int)tasks.size(), ctx.stream);
            else
                k_topdown(ctx.dbasis, (const PairTask *)pk.ptr(0), (int)tasks.size(), ctx.stream);
            st.launches++;
        }
        for (int n = maxn - 1; n >= b.n0; n--) {
            std::vector<PairTask> tasks;
            std::vector<double *> cnp;
            for (JobState *sp : jset) {
                Tree &out = *sp->job->out;
                for (int i = 0; i < out.nn(); i++)
                    if (out.nodes[i].n == n && out.nodes[i].child0 >= 0) {
                        tasks.push_back({out.block(i), out.block(out.nodes[i].child0)});
                        cnp.push_back(out.d_cn + (size_t)8 * i);
                    }
            }
            if (tasks.empty()) continue;
            Packer pk;
            pk.add(tasks.data(), tasks.size() * sizeof(PairTask));
            pk.add(cnp.data(), cnp.size() * sizeof(double *));
            pk.ship(ctx, ar);
            if (mixed)
                k_compress_df(ctx.dbasis, (const PairTask *)pk.ptr(0), (double *const *)pk.ptr(1),
                              (int)tasks.size(), ctx.stream);
            else
                k_compress(ctx.dbasis, (const PairTask *)pk.ptr(0), (double *const *)pk.ptr(1), (int)tasks.size(),
                           ctx.stream);
            st.launches++;
        }
        // leaf norms after the top-down pass
        std::vector<double *> bl, cnp;
        for (JobState *sp : jset) {
            Tree &out = *sp->job->out;
            for (int i = 0; i < out.nn(); i++)
                if (out.nodes[i].child0 < 0) {
                    bl.push_back(out.block(i));
                    cnp.push_back(out.d_cn + (size_t)8 * i);
                }
        }
        if (!bl.empty()) {
            Packer pk;
            pk.add(bl.data(), bl.size() * sizeof(double *));
            pk.add(cnp.data(), cnp.size() * sizeof(double *));
            pk.ship(ctx, ar);
            k_norms(ctx.dbasis, (double *const *)pk.ptr(0), (double *const *)pk.ptr(1), (int)bl.size(), ctx.stream);
            st.launches++;
        }
        for (JobState *sp : jset) {
            Tree &out = *sp->job->out;
            double *h = (double *)ar.halloc(sizeof(double) * 8 * out.nn());
            MWG_CUDA(cudaMemcpyAsync(h, out.d_cn, sizeof(double) * 8 * out.nn(), cudaMemcpyDeviceToHost, ctx.stream));
            cn_staging.push_back({&out, h});
        }
    };

    // the levels of the job groups, pipelined; a group's post-processing starts on its own stream
    // as soon as its last level is launched, beside the other groups' levels
    std::vector<cudaEvent_t> ev_post(2 * ngroups, nullptr);
    for (auto &e : ev_post) MWG_CUDA(cudaEventCreate(&e));
    while (true) {
        bool active = false;
        for (int g = 0; g < ngroups; g++) {
            Group &G = groups[g];
            if (G.pending) {
                finish_level(G);
                G.pending = false;
            }
            if (!G.done) {
                G.done = !launch_level(G);
                if (G.done) {
                    StreamSwap swap(ctx, G.stream);
                    std::vector<JobState *> jset;
                    for (int j : G.jobs) jset.push_back(&js[j]);
                    MWG_CUDA(cudaEventRecord(ev_post[2 * g], ctx.stream));
                    post_process(jset, *G.arena);
                    MWG_CUDA(cudaEventRecord(ev_post[2 * g + 1], ctx.stream));
                    if (hin && hin->out_nnodes) {
                        const auto tO = std::chrono::steady_clock::now();
                        // the group's outputs that fit go down now, beside the other groups' levels
                        std::vector<Tree *> trees;
                        std::vector<int *> k;
                        std::vector<double *> c;
                        std::vector<unsigned char *> l;
                        for (int j : G.jobs) {
                            Tree &out = *jobs[j].out;
                            const bool fits = out.nn() <= hin->out_cap[j] && hin->out_coefs[j];
                            hin->out_nnodes[j] = fits ? out.nn() : -out.nn();
                            if (!fits) continue;
                            trees.push_back(&out);
                            k.push_back(hin->out_keys[j]);
                            c.push_back(hin->out_coefs[j]);
                            l.push_back(hin->out_leaf[j]);
                        }
                        download_enqueue(trees, k.data(), c.data(), l.data(), *G.arena);
                        st.host_io_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tO).count();
                    }
                }
            }
            if (!G.done) {
                G.pending = true;
                active = true;
            }
        }
        if (!active) break;
    }
    // the context's stream follows every group's last work
    for (int g = 1; g < ngroups; g++) {
        MWG_CUDA(cudaEventRecord(ev_end[g], groups[g].stream));
        MWG_CUDA(cudaStreamWaitEvent(ctx.stream, ev_end[g], 0));
    }
    for (auto &g : groups)
        for (auto &e : g.ev) cudaEventDestroy(e);
    if (ev_start) cudaEventDestroy(ev_start);
    for (auto &e : ev_end)
        if (e) cudaEventDestroy(e);
    // input bytes: every distinct input block read once per apply (FP64 or FP32 shadow) + operator blocks
    for (auto &s : js) st.bytes += 8.0 * bs * (double)s.job->inp->nn();
    MWG_CUDA(cudaEventRecord(ev_span[1], ctx.stream));
    MWG_CUDA(cudaEventRecord(ev_span[2], ctx.stream));
    ctx.sync();
    for (auto &p : cn_staging) std::copy(p.second, p.second + 8 * (size_t)p.first->nn(), p.first->cn.begin());
    arena.reset();
    for (int g = 1; g < ngroups; g++) ctx.xarena[g - 1].reset();
    {
        // levels: from the start to the last group's end; post: the groups' post-processing
        // spans summed (they overlap other groups' levels)
        float a = 0.0f, c = 0.0f;
        MWG_CUDA(cudaEventElapsedTime(&a, ev_span[0], ev_span[1]));
        st.gpu_levels_ms += a;
        for (int g = 0; g < ngroups; g++) {
            MWG_CUDA(cudaEventElapsedTime(&c, ev_post[2 * g], ev_post[2 * g + 1]));
            st.gpu_post_ms += c;
        }
    }
    for (auto &e : ev_post) cudaEventDestroy(e);
    for (auto &G : groups) {
        if (G.ev_in) cudaEventDestroy(G.ev_in);
        if (G.ev_up) cudaEventDestroy(G.ev_up);
        if (G.ev_prep) cudaEventDestroy(G.ev_prep);
    }
    for (auto &e : ev_span) cudaEventDestroy(e);
    if (ds.ev_counts) cudaEventDestroy(ds.ev_counts);
    st.kernel_ms += kernel_ms;
    st.launches += ctx.fetch_launches - fetch0;
    st.host_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
}

// ------------------------------------------------------------------ multiply
// bottom-up compression of several trees, one launch per scale
void compress_batch(const std::vector<Tree *> &trees, Arena &arena, mw_stats *st, bool df) {
    if (trees.empty()) return;
    Ctx &ctx = *trees[0]->ctx;
    int maxn = ctx.basis.n0;
    for (Tree *t : trees) maxn = std::max(maxn, t->max_scale());
    for (int n = maxn - 1; n >= ctx.basis.n0; n--) {
        std::vector<PairTask> tasks;
        std::vector<double *> cnp;
        for (Tree *t : trees)
            for (int i = 0; i < t->nn(); i++)
                if (t->nodes[i].n == n && t->nodes[i].child0 >= 0) {
                    tasks.push_back({t->block(i), t->block(t->nodes[i].child0)});
                    cnp.push_back(t->d_cn + (size_t)8 * i);
                }
        if (tasks.empty()) continue;
        Packer pk;
        pk.add(tasks.data(), tasks.size() * sizeof(PairTask));
        pk.add(cnp.data(), cnp.size() * sizeof(double *));
        pk.ship(ctx, arena);
        if (df)
            k_compress_df(ctx.dbasis, (const PairTask *)pk.ptr(0), (double *const *)pk.ptr(1), (int)tasks.size(),
                          ctx.stream);
        else
            k_compress(ctx.dbasis, (const PairTask *)pk.ptr(0), (double *const *)pk.ptr(1), (int)tasks.size(),
                       ctx.stream);
        if (st) st->launches++;
    }
    // every tree's norms in one download (gathered on the device into pinned memory)
    std::vector<const double *> gsrc;
    std::vector<long long> goff;
    std::vector<int> glen;
    long long gtot = 0;
    for (Tree *t : trees) {
        gsrc.push_back(t->d_cn);
        goff.push_back(gtot);
        glen.push_back(8 * t->nn());
        gtot += 8LL * t->nn();
    }
    double *hnorm = nullptr;
    if (gtot > 0) {
        Packer pg;
        pg.add(gsrc.data(), gsrc.size() * sizeof(const double *));
        pg.add(goff.data(), goff.size() * sizeof(long long));
        pg.add(glen.data(), glen.size() * sizeof(int));
        pg.ship(ctx, arena);
        double *dnorm = (double *)arena.alloc(sizeof(double) * (size_t)gtot);
        k_gather_ranges((const double *const *)pg.ptr(0), (const long long *)pg.ptr(1), (const int *)pg.ptr(2),
                        (int)gsrc.size(), dnorm, ctx.stream);
        if (st) st->launches++;
        hnorm = (double *)arena.halloc(sizeof(double) * (size_t)gtot);
        MWG_CUDA(cudaMemcpyAsync(hnorm, dnorm, sizeof(double) * (size_t)gtot, cudaMemcpyDeviceToHost, ctx.stream));
    }
    ctx.sync();
    for (size_t r = 0; r < trees.size(); r++) std::copy(hnorm + goff[r], hnorm + goff[r] + glen[r], trees[r]->cn.data());
}

namespace {

// unresolved detail below each node: tail^2 = sum over children (|w|^2 + tail^2)
std::vector<double> detail_tails(const Tree &t) {
    std::vector<double> tl(t.nn(), 0.0);
    std::vector<int> order(t.nn());
    for (int i = 0; i < t.nn(); i++) order[i] = i;
    std::sort(order.begin(), order.end(), [&](int x, int y) { return t.nodes[x].n > t.nodes[y].n; });
    for (int i : order) {
        if (t.nodes[i].child0 < 0) continue;
        double s = 0.0;
        for (int c = 0; c < 8; c++) {
            int ci = t.nodes[i].child0 + c;
            double w = wavelet_norm8(&t.cn[8 * (size_t)ci]);
            s += w * w + tl[ci] * tl[ci];
        }
        tl[i] = std::sqrt(s);
    }
    return tl;
}

struct MulState {
    MulJob *job;
    const std::vector<double> *ta = nullptr, *tb = nullptr;  // the inputs' detail tails (useMaxNorms)
    std::vector<int> work;
    int iter = 0;
    int tia = 0, tib = 0;                  // the inputs' indices among the batch's distinct trees
    std::vector<Key> ra, rb;               // this level's missing input nodes of a and b ...
    std::vector<int> aa, ab;               // ... and their leaf ancestors
    std::vector<MulTask> tasks;  // this level's node tasks
    std::vector<double> crit;    // ... and their max-norm criteria
    std::vector<const float2 *> va, vb;  // ... their inputs' cached value cubes (nullptr: none)
};

}  // namespace

// Level-synchronous multiply of several (out, a, b) products: per refinement
// iteration one generation launch, one product launch and one norm download
// for all products.  Each product follows mrcpp::multiply: the output's current
// grid is the start grid (end nodes computed), refined while the product's
// wavelet norm (or, with useMaxNorms, the inputs' unresolved detail times the
// other input's RMS value) exceeds prec * R * 2^{-(n+1)/2}.
void multiply_batch(std::vector<MulJob> &jobs, mw_stats &st) {
    if (jobs.empty()) return;
    Ctx &ctx = *jobs[0].out->ctx;
    const Basis &bsis = ctx.basis;
    Arena &arena = ctx.arena;
    auto t_start = std::chrono::steady_clock::now();
    const long long fetch0 = ctx.fetch_launches;
    using clk = std::chrono::steady_clock;
    auto since = [](clk::time_point t0) { return std::chrono::duration<double, std::milli>(clk::now() - t0).count(); };
    std::vector<MulState> ms(jobs.size());
    // the inputs' unresolved detail, once per distinct input tree (the exchange products share
    // their 32 orbitals among 528 jobs)
    std::vector<std::pair<const Tree *, std::vector<double>>> tails;
    {
        std::unordered_map<const Tree *, int> idx;
        for (auto &j : jobs)
            if (j.use_max_norms)
                for (const Tree *t : {j.a, j.b})
                    if (idx.emplace(t, (int)tails.size()).second) tails.push_back({t, {}});
#pragma omp parallel for schedule(dynamic, 1)
        for (long i = 0; i < (long)tails.size(); i++) tails[i].second = detail_tails(*tails[i].first);
        for (size_t j = 0; j < jobs.size(); j++)
            if (jobs[j].use_max_norms) {
                ms[j].ta = &tails[idx.at(jobs[j].a)].second;
                ms[j].tb = &tails[idx.at(jobs[j].b)].second;
            }
    }
    for (size_t j = 0; j < jobs.size(); j++) {
        MulState &s = ms[j];
        s.job = &jobs[j];
        Tree &out = *jobs[j].out;
        // a product's grid rarely outgrows the smaller input's: sized once for that
        out.reserve(std::max((size_t)out.nn(), (size_t)std::min(jobs[j].a->nn(), jobs[j].b->nn())));
        for (int i = 0; i < out.nn(); i++)
            if (out.nodes[i].child0 < 0) s.work.push_back(i);
    }
    // The node kernel works from the inputs' value cubes (mw_multiply_df.cu).  An input tree that
    // feeds several products gets the value cube of every node once, up front (stream-ordered
    // allocation, freed at the end); the other inputs' blocks at a level's nodes (generated ones,
    // nodes of trees used once) get theirs per level.
    const size_t VS = mul_value_floats(bsis.K);
    std::vector<std::pair<const Tree *, float2 *>> vcache;
    std::vector<const double *> cblk;  // the cached trees' blocks and their value cubes, computed
    std::vector<float2 *> cval;        // with the first level's launches (its pack, its arena)
    {
        std::vector<const Tree *> order;
        std::unordered_map<const Tree *, int> uses;
        for (auto &j : jobs)
            for (const Tree *t : {j.a, j.b})
                if (uses[t]++ == 0) order.push_back(t);
        size_t bytes = 0;
        for (const Tree *t : order)
            if (uses[t] >= 2) bytes += sizeof(float) * VS * (size_t)t->nn();
        size_t free_b = 0, total_b = 0;
        MWG_CUDA(cudaMemGetInfo(&free_b, &total_b));
        if (bytes > 0 && bytes <= free_b / 4) {
            for (const Tree *t : order) {
                if (uses[t] < 2) continue;
                float2 *p = nullptr;
                MWG_CUDA(cudaMallocAsync(&p, sizeof(float) * VS * (size_t)t->nn(), ctx.stream));
                vcache.push_back({t, p});
                for (int i = 0; i < t->nn(); i++) {
                    cblk.push_back(t->block(i));
                    cval.push_back(p + (VS / 2) * (size_t)i);
                }
            }
        }
    }
    auto cached = [&](const Tree *t) -> float2 * {
        for (auto &c : vcache)
            if (c.first == t) return c.second;
        return nullptr;
    };
    for (auto &s : ms) {
        s.va.clear();
        s.vb.clear();
    }
    // the batch's distinct input trees and, per tree, the (job, side) pairs that read it: a block
    // missing from a tree is generated once per level however many products need it
    std::vector<const Tree *> dtrees;
    std::vector<std::vector<std::pair<int, int>>> readers;
    {
        std::unordered_map<const Tree *, int> tix;
        for (size_t j = 0; j < ms.size(); j++)
            for (int side = 0; side < 2; side++) {
                const Tree *t = side ? jobs[j].b : jobs[j].a;
                auto it = tix.emplace(t, (int)dtrees.size());
                if (it.second) {
                    dtrees.push_back(t);
                    readers.emplace_back();
                }
                readers[it.first->second].push_back({(int)j, side});
                (side ? ms[j].tib : ms[j].tia) = it.first->second;
            }
    }
    std::vector<GenSet> tgs(dtrees.size());
    while (true) {
        bool any = false;
        for (auto &s : ms) any |= !s.work.empty();
        if (!any) break;
        arena.reset();
        if (!cblk.empty()) {  // the cached value cubes, ahead of the first level's launches
            Packer pc;
            pc.add(cblk.data(), cblk.size() * sizeof(const double *));
            pc.add(cval.data(), cval.size() * sizeof(float2 *));
            pc.ship(ctx, arena);
            k_values_df(ctx.dbasis, (const double *const *)pc.ptr(0), (float2 *const *)pc.ptr(1), (int)cblk.size(),
                        ctx.nsm, ctx.stream);
            st.launches++;
            cblk.clear();
        }
        auto tA = clk::now();
        // input blocks to generate at this level's output nodes: each job's missing nodes (jobs in
        // parallel), then per input tree its readers' requests in job order (trees in parallel)
#pragma omp parallel for schedule(dynamic, 4)
        for (long j = 0; j < (long)ms.size(); j++) {
            MulState &s = ms[j];
            s.ra.clear();
            s.rb.clear();
            s.aa.clear();
            s.ab.clear();
            Tree &out = *s.job->out, &a = *s.job->a, &b = *s.job->b;
            for (int oi : s.work) {
                const NodeInfo &o = out.nodes[oi];
                const Key k{o.n, {o.l[0], o.l[1], o.l[2]}};
                if (a.find(o.n, o.l) < 0) {
                    s.ra.push_back(k);
                    s.aa.push_back(find_ancestor(a, o.n, o.l, nullptr));
                }
                if (b.find(o.n, o.l) < 0) {
                    s.rb.push_back(k);
                    s.ab.push_back(find_ancestor(b, o.n, o.l, nullptr));
                }
            }
        }
#pragma omp parallel for schedule(dynamic, 1)
        for (long t = 0; t < (long)dtrees.size(); t++) {
            GenSet &gs = tgs[t];
            gs.clear();
            for (const auto &rd : readers[t]) {
                const MulState &s = ms[rd.first];
                const std::vector<Key> &keys = rd.second ? s.rb : s.ra;
                const std::vector<int> &anc = rd.second ? s.ab : s.aa;
                for (size_t r = 0; r < keys.size(); r++) gs.request(*dtrees[t], keys[r].n, keys[r].l, anc[r]);
            }
        }
        std::vector<std::pair<GenSet *, const Tree *>> sets;
        for (size_t t = 0; t < dtrees.size(); t++) sets.push_back({&tgs[t], dtrees[t]});
        st.host_enum_ms += since(tA);
        auto tB = clk::now();
        generate_all(sets, arena, &st);
        st.host_gen_ms += since(tB);
        // the generated blocks' value cubes, once per block: tree t's block g at gvoff[t] + g
        std::vector<size_t> gvoff(dtrees.size() + 1, 0);
        for (size_t t = 0; t < dtrees.size(); t++) gvoff[t + 1] = gvoff[t] + tgs[t].keys.size();
        float2 *gvals = gvoff.back() ? (float2 *)arena.alloc(sizeof(float) * VS * gvoff.back()) : nullptr;
        auto tC = clk::now();
        // node tasks and max-norm criteria, jobs in parallel, then concatenated in job order
#pragma omp parallel for schedule(dynamic, 4)
        for (long j = 0; j < (long)ms.size(); j++) {
            MulState &s = ms[j];
            Tree &out = *s.job->out, &a = *s.job->a, &b = *s.job->b;
            s.tasks.resize(s.work.size());
            s.crit.assign(s.work.size(), 0.0);
            s.va.assign(s.work.size(), nullptr);
            s.vb.assign(s.work.size(), nullptr);
            float2 *ca = cached(&a), *cb = cached(&b);
            const GenSet &ga = tgs[s.tia], &gb = tgs[s.tib];
            for (size_t w = 0; w < s.work.size(); w++) {
                const NodeInfo &o = out.nodes[s.work[w]];
                const Key k{o.n, {o.l[0], o.l[1], o.l[2]}};
                int ia = a.find(o.n, o.l), ib = b.find(o.n, o.l);
                if (ia < 0) s.va[w] = gvals + (VS / 2) * (gvoff[s.tia] + (size_t)ga.slot.at(k));
                else if (ca) s.va[w] = ca + (VS / 2) * (size_t)ia;
                if (ib < 0) s.vb[w] = gvals + (VS / 2) * (gvoff[s.tib] + (size_t)gb.slot.at(k));
                else if (cb) s.vb[w] = cb + (VS / 2) * (size_t)ib;
                MulTask &tk = s.tasks[w];
                tk.a = block_at(a, ga, ga.base, o.n, o.l);
                tk.b = block_at(b, gb, gb.base, o.n, o.l);
                tk.out = out.block(s.work[w]);
                tk.cn = out.d_cn + (size_t)8 * s.work[w];
                tk.scale = s.job->coef * std::pow(2.0, 1.5 * (o.n + 1));
                if (s.job->use_max_norms) {
                    const double *cna = ia >= 0 ? &a.cn[8 * (size_t)ia] : &ga.cn[8 * (size_t)ga.slot.at(k)];
                    const double *cnb = ib >= 0 ? &b.cn[8 * (size_t)ib] : &gb.cn[8 * (size_t)gb.slot.at(k)];
                    double sc = std::pow(2.0, 1.5 * o.n);
                    s.crit[w] = (ia >= 0 ? (*s.ta)[ia] : 0.0) * block_norm8(cnb) * sc +
                                (ib >= 0 ? (*s.tb)[ib] : 0.0) * block_norm8(cna) * sc;
                }
            }
        }
        // the level's inputs without a cached value cube get theirs into level scratch: per job
        // its count, then the blocks and the value pointers in job order
        std::vector<size_t> voff(ms.size() + 1, 0), toff(ms.size() + 1, 0);
        for (size_t j = 0; j < ms.size(); j++) {
            size_t c = 0;
            for (size_t w = 0; w < ms[j].tasks.size(); w++) c += (ms[j].va[w] ? 0 : 1) + (ms[j].vb[w] ? 0 : 1);
            voff[j + 1] = voff[j] + c;
            toff[j + 1] = toff[j] + ms[j].tasks.size();
        }
        const size_t ng = gvoff.back();
        const size_t nv = voff.back() + ng, nt = toff.back();
        float2 *lvals = voff.back() ? (float2 *)arena.alloc(sizeof(float) * VS * voff.back()) : nullptr;
        std::vector<const double *> vblk(nv);
        std::vector<float2 *> vdst(nv);
        // the generated blocks first, then the per-task blocks
        for (size_t t = 0; t < dtrees.size(); t++)
            for (size_t g = 0; g < tgs[t].keys.size(); g++) {
                vblk[gvoff[t] + g] = tgs[t].base + (size_t)g * bsis.bs;
                vdst[gvoff[t] + g] = gvals + (VS / 2) * (gvoff[t] + g);
            }
        std::vector<MulVTask> tasks(nt);
#pragma omp parallel for schedule(dynamic, 4)
        for (long j = 0; j < (long)ms.size(); j++) {
            MulState &s = ms[j];
            size_t k = voff[j];
            for (size_t w = 0; w < s.tasks.size(); w++) {
                const MulTask &tk = s.tasks[w];
                MulVTask &vt = tasks[toff[j] + w];
                auto value_of = [&](const float2 *v, const double *blk) -> const float2 * {
                    if (v) return v;
                    vblk[ng + k] = blk;
                    vdst[ng + k] = lvals + (VS / 2) * k;
                    return vdst[ng + k++];
                };
                vt.a = value_of(s.va[w], tk.a);
                vt.b = value_of(s.vb[w], tk.b);
                vt.out = tk.out;
                vt.cn = tk.cn;
                vt.scale = tk.scale;
            }
        }
        st.host_items_ms += since(tC);
        auto tD = clk::now();
        Packer pk;
        pk.add(tasks.data(), tasks.size() * sizeof(MulVTask));
        pk.add(vblk.data(), vblk.size() * sizeof(const double *));
        pk.add(vdst.data(), vdst.size() * sizeof(float2 *));
        pk.ship(ctx, arena);
        if (nv) {
            k_values_df(ctx.dbasis, (const double *const *)pk.ptr(1), (float2 *const *)pk.ptr(2), (int)nv, ctx.nsm,
                        ctx.stream);
            st.launches++;
        }
        k_multiply_values_df(ctx.dbasis, (const MulVTask *)pk.ptr(0), (int)tasks.size(), ctx.nsm, ctx.stream);
        st.launches++;
        st.out_nodes += (long long)tasks.size();
        // the norms of the nodes computed at this level (each job's index range: the children
        // appended by the last refinement, or the whole array when not contiguous), gathered on
        // the device and downloaded with one copy into pinned memory: a copy per tree into its
        // pageable norm array cost several microseconds each, hundreds of trees per level
        std::vector<const double *> gsrc;
        std::vector<long long> goff;
        std::vector<int> glen;
        std::vector<std::pair<Tree *, size_t>> gdst;  // (tree, first node)
        long long gtot = 0;
        for (auto &s : ms) {
            Tree &out = *s.job->out;
            if (s.work.empty()) continue;
            const auto mm = std::minmax_element(s.work.begin(), s.work.end());
            size_t first = 0, count = (size_t)out.nn();
            if ((size_t)(*mm.second - *mm.first + 1) == s.work.size()) {
                first = (size_t)*mm.first;
                count = s.work.size();
            }
            gsrc.push_back(out.d_cn + 8 * first);
            goff.push_back(gtot);
            glen.push_back((int)(8 * count));
            gdst.push_back({&out, first});
            gtot += (long long)(8 * count);
        }
        double *hnorm = nullptr;
        if (gtot > 0) {
            Packer pg;
            pg.add(gsrc.data(), gsrc.size() * sizeof(const double *));
            pg.add(goff.data(), goff.size() * sizeof(long long));
            pg.add(glen.data(), glen.size() * sizeof(int));
            pg.ship(ctx, arena);
            double *dnorm = (double *)arena.alloc(sizeof(double) * (size_t)gtot);
            k_gather_ranges((const double *const *)pg.ptr(0), (const long long *)pg.ptr(1), (const int *)pg.ptr(2),
                            (int)gsrc.size(), dnorm, ctx.stream);
            st.launches++;
            hnorm = (double *)arena.halloc(sizeof(double) * (size_t)gtot);
            MWG_CUDA(cudaMemcpyAsync(hnorm, dnorm, sizeof(double) * (size_t)gtot, cudaMemcpyDeviceToHost, ctx.stream));
        }
        ctx.sync();
        for (size_t r = 0; r < gdst.size(); r++)
            std::copy(hnorm + goff[r], hnorm + goff[r] + glen[r], gdst[r].first->cn.data() + 8 * gdst[r].second);
        st.host_wait_ms += since(tD);
        auto tE = clk::now();
        // refinement, jobs in parallel (each splits its own tree); the new children need no
        // zeroing: the next level's kernel writes their blocks
#pragma omp parallel for schedule(dynamic, 4)
        for (long j = 0; j < (long)ms.size(); j++) {
            MulState &s = ms[j];
            Tree &out = *s.job->out;
            double R = s.job->abs_prec ? 1.0 : std::sqrt(out.sqnorm_leaves());
            std::vector<int> next;
            if (s.job->max_iter < 0 || s.iter < s.job->max_iter) {
                for (size_t w = 0; w < s.work.size(); w++) {
                    int oi = s.work[w];
                    int n = out.nodes[oi].n;
                    if (n >= bsis.max_scale()) continue;
                    double thr = split_thr(s.job->prec, R, n);
                    if (wavelet_norm8(&out.cn[8 * (size_t)oi]) > thr || s.crit[w] > thr) {
                        int c0 = out.split(oi);
                        for (int c = 0; c < 8; c++) next.push_back(c0 + c);
                    }
                }
            }
            s.work.swap(next);
            s.iter++;
        }
        st.host_refine_ms += since(tE);
        st.levels++;
    }
    for (auto &c : vcache) MWG_CUDA(cudaFreeAsync(c.second, ctx.stream));
    std::vector<Tree *> outs;
    for (auto &j : jobs) outs.push_back(j.out);
    arena.reset();
    auto tF = clk::now();
    compress_batch(outs, arena, &st, true);
    st.gpu_post_ms += since(tF);
    st.launches += ctx.fetch_launches - fetch0;
    st.host_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
}

// ------------------------------------------------------------------ adjoint apply
// L2-adjoint of the fixed-grid apply y = A x (output grid = y's grid, input x,
// absolute precision, FP64).  The forward output is the function
//     A x = sum_o (s_o phi_o + d_o psi_o),   (s_o, d_o) = sum_{items (o,i,t)} c_t B_t(l_o - l_i) x_i,
// with x_i the block of x at input position i (a node or a generated node), so
//     <y, A x> = sum_items <c_t B_t(l)^T y_o, x_i>,   y_o = y's block at o.
// The adjoint function is therefore A^T y = sum_i (g_i^s phi_i + g_i^d psi_i) with
// g_i = sum_{items at i} c_t B_t(-l) y_o (NS(-l) = NS(l)^T), i.e. the same contraction
// with the roles of output and input swapped ("scatter turned into gather": items are
// grouped by input position), followed by the forward's top-down sum and compression,
// and the projection onto x's grid (the space the forward map acts on).  The item set is
// the forward's, screened with x's norms.
void apply_adjoint(double prec, Tree &res, Oper &op, Tree &x, Tree &y, mw_stats &st) {
    Ctx &ctx = *res.ctx;
    const Basis &b = ctx.basis;
    const int bsz = 4 * b.K * b.K;
    const double K4 = (double)b.K * b.K * b.K * b.K;
    Arena &arena = ctx.arena;
    auto t_start = std::chrono::steady_clock::now();
    if (x.ctx != &ctx || y.ctx != &ctx || op.ctx != &ctx) throw Error(MW_ERR_ARG, "adjoint: mixed contexts");
    // extended result grid: x's grid, grown below x's leaves where generated input positions occur
    Tree ext;
    ext.ctx = &ctx;
    copy_grid(ext, x);
    ApplyJob job{&y, &op, &x, prec, true, 0, {}};
    JobState s;
    s.job = &job;
    for (int i = 0; i < x.nn(); i++) s.fmax = std::max(s.fmax, block_norm8(&x.cn[8 * (size_t)i]));
    LevelItems li;
    const int maxn = y.max_scale();
    for (int n = b.n0; n <= maxn; n++) {
        const int sidx = n - b.n0;
        const bool root = (n == b.n0);
        arena.reset();
        s.work.clear();
        for (int i = 0; i < y.nn(); i++)
            if (y.nodes[i].n == n) s.work.push_back(i);
        if (s.work.empty()) continue;
        s.wgt.assign(s.work.size(), 1.0);
        s.cand.assign(s.work.size(), {});
        const double thr = root ? 0.0 : SCREEN_FAC * split_thr(prec, 1.0, n);
#pragma omp parallel
        {
            LookupCache cache;
#pragma omp for schedule(dynamic, 4)
            for (long w = 0; w < (long)s.work.size(); w++) enumerate_node(s, (int)w, sidx, root, thr, cache);
        }
        s.gens.clear();
        for (size_t w = 0; w < s.work.size(); w++) {
            const NodeInfo &o = y.nodes[s.work[w]];
            for (Cand &c : s.cand[w]) {
                if (!c.gen) continue;
                int p[3] = {o.l[0] - c.lx, o.l[1] - c.ly, o.l[2] - c.lz};
                c.src = s.gens.request(x, n, p, c.src);
            }
        }
        generate_all({{&s.gens, &x}}, arena, &st);
        // surviving items, each with its input position; grow the result grid to hold every position
        struct TItem {
            int target, o;
            const Cand *c;
        };
        std::vector<TItem> items;
        for (size_t w = 0; w < s.work.size(); w++) {
            const NodeInfo &o = y.nodes[s.work[w]];
            for (const Cand &c : s.cand[w]) {
                const double *cn = c.gen ? &s.gens.cn[8 * (size_t)c.src] : &x.cn[8 * (size_t)c.src];
                const double *nx = op.norm(c.t, sidx, c.lx), *ny = op.norm(c.t, sidx, c.ly),
                             *nz = op.norm(c.t, sidx, c.lz);
                if (!root && item_bound(nx, ny, nz, cn, root) < thr) continue;
                int p[3] = {o.l[0] - c.lx, o.l[1] - c.ly, o.l[2] - c.lz};
                int t = ext.find(n, p);
                while (t < 0) {  // split the deepest existing ancestor until the position exists
                    int an = n, al[3] = {p[0], p[1], p[2]}, a = -1;
                    while (a < 0) {
                        an--;
                        for (int d = 0; d < 3; d++) al[d] = floordiv2(al[d]);
                        a = ext.find(an, al);
                    }
                    int first = ext.nn();
                    ext.split(a);
                    tree_zero(ext, first, 8);
                    t = ext.find(n, p);
                }
                items.push_back({t, s.work[w], &c});
                st.flops += 6.0 * K4 * item_pairs(nx, ny, nz, cn, root);
            }
        }
        std::stable_sort(items.begin(), items.end(), [](const TItem &a, const TItem &b2) { return a.target < b2.target; });
        li = LevelItems();
        li.begin.assign(1, 0);
        for (size_t q = 0; q < items.size(); q++) {
            const TItem &it = items[q];
            if (q == 0 || it.target != items[q - 1].target) {
                if (q > 0) li.begin.push_back((long long)q);
                li.out.push_back(ext.block(it.target));
            }
            li.in.push_back(y.block(it.o));
            li.ax.push_back(op.d_blocks + (size_t)op.block_index(it.c->t, sidx, -it.c->lx) * bsz);
            li.ay.push_back(op.d_blocks + (size_t)op.block_index(it.c->t, sidx, -it.c->ly) * bsz);
            li.az.push_back(op.d_blocks + (size_t)op.block_index(it.c->t, sidx, -it.c->lz) * bsz);
            li.coef.push_back(op.c[it.c->t]);
        }
        if (!items.empty()) li.begin.push_back((long long)items.size());
        li.nodes = (long)li.out.size();
        li.items = (long long)items.size();
        st.items += (long long)items.size();
        st.items_fp64 += (long long)items.size();
        st.out_nodes += (long long)li.out.size();
        launch_tier(ctx, ctx.arena, li, root, true, 0, Ctx::Tuning().chunk[0], st);
        ctx.sync();
        st.levels++;
    }
    // the forward's post-processing: top-down sum over scales, bottom-up compression
    arena.reset();
    for (int n = b.n0; n < ext.max_scale(); n++) {
        std::vector<PairTask> tasks;
        for (int i = 0; i < ext.nn(); i++)
            if (ext.nodes[i].n == n && ext.nodes[i].child0 >= 0)
                tasks.push_back({ext.block(i), ext.block(ext.nodes[i].child0)});
        if (tasks.empty()) continue;
        Packer pk;
        pk.add(tasks.data(), tasks.size() * sizeof(PairTask));
        pk.ship(ctx, arena);
        k_topdown(ctx.dbasis, (const PairTask *)pk.ptr(0), (int)tasks.size(), ctx.stream);
        st.launches++;
    }
    compress_batch({&ext}, arena, &st);
    // projection onto x's grid: keep x's nodes (their blocks now carry the finer parts)
    copy_grid(res, x);
    arena.reset();
    combine_on_grid(res, {&ext}, {1.0}, arena, &st);
    ext.free_device();
    arena.reset();
    st.host_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
}

void add(Tree &out, const std::vector<const Tree *> &trees, const std::vector<double> &coefs, mw_stats &st) {
    Ctx &ctx = *out.ctx;
    auto t_start = std::chrono::steady_clock::now();
    build_grid(out, trees);
    ctx.arena.reset();
    combine_on_grid(out, trees, coefs, ctx.arena, &st);
    ctx.arena.reset();
    st.out_nodes += out.nn();
    st.host_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
}

// Electron density rho = sum_i occ_i |phi_i|^2 kept on the device, following
// density::compute (src/qmfunctions/density_utils.cpp:64-150): every square on a copy of the
// orbital's grid (refined adaptively at prec), the squares added on their union grid, and the
// sum cropped at prec / N_el when crop is set.  The squares of all orbitals run as one batched
// multiply.
// ------------------------------------------------------------------ adjoint multiply
// L2-adjoint of the fixed-grid product h = coef a b in its first factor.  The forward map
// a -> h represents a at h's end nodes (generated from a's coarser leaves, or with a's finer
// detail left out), multiplies the values at the children's quadrature points by b's and maps
// them back; the value <-> coefficient maps are orthogonal, so the transpose is the same
// product with the seed in place of a, on h's grid (the seed's), followed by the transpose of
// the representation step: the projection onto a's grid (copy_func: compression where a's grid
// is coarser, exact injection where it is finer).  out <- coef P_a (seed b), on a's grid.
void multiply_adjoint(double prec, Tree &out, double coef, const Tree &a, Tree &b, Tree &seed, mw_stats &st) {
    Ctx &ctx = *out.ctx;
    if (a.ctx != &ctx || b.ctx != &ctx || seed.ctx != &ctx) throw Error(MW_ERR_ARG, "multiply adjoint: mixed contexts");
    Tree t;
    t.ctx = &ctx;
    copy_grid(t, seed);
    std::vector<MulJob> jobs{MulJob{&t, &seed, &b, coef, prec, 0, true, false}};
    multiply_batch(jobs, st);
    copy_grid(out, a);
    copy_func(out, t, ctx.arena);
    ctx.sync();
    t.free_device();
}

void density(double prec, Tree &rho, const std::vector<Tree *> &orbs, const std::vector<double> &occ, bool crop_sum,
             mw_stats &st) {
    Ctx &ctx = *rho.ctx;
    std::vector<Tree> sq(orbs.size());
    std::vector<MulJob> jobs(orbs.size());
    for (size_t i = 0; i < orbs.size(); i++) {
        sq[i].ctx = &ctx;
        copy_grid(sq[i], *orbs[i]);
        jobs[i] = MulJob{&sq[i], orbs[i], orbs[i], 1.0, prec, -1, false, false};
    }
    multiply_batch(jobs, st);
    std::vector<const Tree *> v;
    for (auto &t : sq) v.push_back(&t);
    tree_clear(rho);
    add(rho, v, occ, st);
    if (crop_sum) {
        double nel = 0.0;
        for (double o : occ) nel += o;
        crop(rho, prec / std::max(nel, 1.0), true, ctx.arena);
    }
    for (auto &t : sq) t.free_device();
}

// Linear combinations out_i = sum_j U_ij in_j for many outputs at once (orbital rotation,
// src/qmfunctions/orbital_utils.cpp:242-248): every output gets the union grid of the inputs,
// and each node block is a small matrix product over the inputs' blocks at that node.
void rotate(const std::vector<Tree *> &outs, const std::vector<const Tree *> &ins, const double *U, mw_stats &st) {
    Ctx &ctx = *outs[0]->ctx;
    auto t_start = std::chrono::steady_clock::now();
    Tree grid;
    grid.ctx = &ctx;
    tree_clear(grid);
    build_grid(grid, ins);
    const size_t nj = ins.size();
    for (size_t i = 0; i < outs.size(); i++) {
        copy_grid(*outs[i], grid);
        std::vector<double> row(U + i * nj, U + (i + 1) * nj);
        ctx.arena.reset();
        combine_on_grid(*outs[i], ins, row, ctx.arena, &st);
        st.out_nodes += outs[i]->nn();
    }
    grid.free_device();
    ctx.arena.reset();
    st.host_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
}

}  // namespace mwg
