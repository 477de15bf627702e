// mw_tree.cpp -- device-resident function trees: structure, transfers,
// projection, grids, norms, dot, evaluation, crop.
//
// Reference call surface: mrcpp::FunctionTree<3> inside ComplexFunction
// (src/qmfunctions/Orbital.h:51); copy_grid / build_grid / copy_func / clear
// (src/qmfunctions/density_utils.cpp:72,85,87); crop
// (density_utils.cpp:147); dot (src/qmfunctions/orbital_utils.cpp:79-82).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>

#include "mw_internal.h"

namespace mwg {

// ------------------------------------------------------------------ arena
void *Arena::alloc(size_t bytes) {
    bytes = (bytes + 255) & ~size_t(255);
    if (bytes == 0) bytes = 256;
    if (!chunks.empty() && chunks.back().used + bytes <= chunks.back().size) {
        Chunk &c = chunks.back();
        void *p = (char *)c.ptr + c.used;
        c.used += bytes;
        total += bytes;
        return p;
    }
    size_t sz = std::max(bytes, chunks.empty() ? (size_t)64 << 20 : chunks.back().size * 2);
    Chunk c;
    c.size = sz;
    MWG_CUDA(cudaMalloc(&c.ptr, sz));
    c.used = bytes;
    chunks.push_back(c);
    total += bytes;
    return c.ptr;
}

void *Arena::halloc(size_t bytes) {
    bytes = (bytes + 255) & ~size_t(255);
    if (bytes == 0) bytes = 256;
    if (!hchunks.empty() && hchunks.back().used + bytes <= hchunks.back().size) {
        Chunk &c = hchunks.back();
        void *p = (char *)c.ptr + c.used;
        c.used += bytes;
        return p;
    }
    size_t sz = std::max(bytes, hchunks.empty() ? (size_t)64 << 20 : hchunks.back().size * 2);
    Chunk c;
    c.size = sz;
    MWG_CUDA(cudaMallocHost(&c.ptr, sz));
    c.used = bytes;
    hchunks.push_back(c);
    return c.ptr;
}

void Arena::reset() {
    if (chunks.size() > 1) {
        size_t need = 0;
        for (auto &c : chunks) need += c.size;
        for (auto &c : chunks) cudaFree(c.ptr);
        chunks.clear();
        Chunk c;
        c.size = need;
        MWG_CUDA(cudaMalloc(&c.ptr, need));
        c.used = 0;
        chunks.push_back(c);
    } else if (!chunks.empty()) {
        chunks.back().used = 0;
    }
    if (hchunks.size() > 1) {
        size_t need = 0;
        for (auto &c : hchunks) need += c.size;
        for (auto &c : hchunks) cudaFreeHost(c.ptr);
        hchunks.clear();
        Chunk c;
        c.size = need;
        MWG_CUDA(cudaMallocHost(&c.ptr, need));
        c.used = 0;
        hchunks.push_back(c);
    } else if (!hchunks.empty()) {
        hchunks.back().used = 0;
    }
    total = 0;
}

void Arena::release() {
    for (auto &c : chunks) cudaFree(c.ptr);
    for (auto &c : hchunks) cudaFreeHost(c.ptr);
    chunks.clear();
    hchunks.clear();
    total = 0;
}

void *Ctx::pinned(size_t bytes) {
    if (bytes > pinned_bytes) {
        if (h_pinned) cudaFreeHost(h_pinned);
        h_pinned = nullptr;
        size_t sz = std::max(bytes, pinned_bytes * 2);
        MWG_CUDA(cudaMallocHost(&h_pinned, sz));
        pinned_bytes = sz;
    }
    return h_pinned;
}

void Ctx::sync() { MWG_CUDA(cudaStreamSynchronize(stream)); }

void Ctx::release_retired() {
    if (retired.empty()) return;
    cudaStreamSynchronize(stream);
    for (auto &xs : xstream)
        if (xs) cudaStreamSynchronize(xs);
    if (fast) cudaStreamSynchronize(fast);
    for (void *p : retired) cudaFreeAsync(p, stream);  // back to the pool, which keeps it for reuse
    retired.clear();
}

// Packs several host arrays into one pinned buffer and ships them with one copy.
void *Packer::add(const void *src, size_t bytes) {
    size_t o = (size.size() ? offs.back() + size.back() : 0);
    o = (o + 255) & ~size_t(255);
    offs.push_back(o);
    size.push_back(bytes);
    srcs.push_back(src);
    return (void *)o;  // placeholder offset, resolved by ptr()
}

void Packer::ship(Ctx &ctx, Arena &arena) {
    size_t total = size.empty() ? 0 : offs.back() + size.back();
    if (total == 0) return;
    // staging lives in the arena's pinned chunks until the arena is reset, so packing never
    // waits for earlier copies or kernels
    char *h = (char *)arena.halloc(total);
    if (total < ((size_t)1 << 20)) {
        for (size_t i = 0; i < srcs.size(); i++)
            if (size[i]) std::memcpy(h + offs[i], srcs[i], size[i]);
    } else {
        // large packs (the item lists of a level): 256 KiB pieces copied by all host threads
        constexpr size_t PIECE = (size_t)1 << 18;
        std::vector<std::pair<size_t, size_t>> pieces;  // (array, offset in it)
        for (size_t i = 0; i < srcs.size(); i++)
            for (size_t o = 0; o < size[i]; o += PIECE) pieces.push_back({i, o});
#pragma omp parallel for schedule(dynamic, 1)
        for (long p = 0; p < (long)pieces.size(); p++) {
            const size_t i = pieces[p].first, o = pieces[p].second;
            std::memcpy(h + offs[i] + o, (const char *)srcs[i] + o, std::min(PIECE, size[i] - o));
        }
    }
    dev = (char *)arena.alloc(total);
    // packs up to a few MB are read by a kernel, so that they never wait behind bulk copies on the
    // copy engines; larger ones take a copy engine
    if (total <= ((size_t)4 << 20)) {
        k_fetch(dev, h, total, ctx.stream);
        ctx.fetch_launches++;
    } else
        MWG_CUDA(cudaMemcpyAsync(dev, h, total, cudaMemcpyHostToDevice, ctx.stream));
}

// ------------------------------------------------------------------ tree
double *Tree::block(int i) const { return d_coefs + (size_t)i * ctx->basis.bs; }

// Grows the device arrays geometrically.  The new arrays come from the device's stream-ordered
// pool on the context's current stream, which also copies the old contents, so a growth neither
// waits for the GPU nor synchronises the device (as cudaMalloc / cudaFree may): the refinement of
// hundreds of trees per call (the exchange pair products) grows each a few times.  The old arrays
// are retired, not freed: kernels queued before the growth may still read them.
void Tree::reserve(size_t n) {
    if (n <= cap) return;
    size_t nc = std::max(n, std::max(cap * 2, (size_t)64));
    int bs = ctx->basis.bs;
    double *nd = nullptr, *ncn = nullptr;
    MWG_CUDA(cudaMallocAsync(&nd, sizeof(double) * bs * nc, ctx->stream));
    MWG_CUDA(cudaMallocAsync(&ncn, sizeof(double) * 8 * nc, ctx->stream));
    if (d_coefs) {
        MWG_CUDA(cudaMemcpyAsync(nd, d_coefs, sizeof(double) * bs * nodes.size(), cudaMemcpyDeviceToDevice,
                                 ctx->stream));
        MWG_CUDA(cudaMemcpyAsync(ncn, d_cn, sizeof(double) * 8 * nodes.size(), cudaMemcpyDeviceToDevice,
                                 ctx->stream));
        std::lock_guard<std::mutex> lock(ctx->retired_mu);
        ctx->retired.push_back(d_coefs);
        ctx->retired.push_back(d_cn);
    }
    d_coefs = nd;
    d_cn = ncn;
    cap = nc;
}

int Tree::add(int n, const int *l, int parent) {
    reserve(nodes.size() + 1);
    NodeInfo ni;
    ni.n = n;
    for (int d = 0; d < 3; d++) ni.l[d] = l[d];
    ni.parent = parent;
    ni.child0 = -1;
    int i = (int)nodes.size();
    nodes.push_back(ni);
    map[Key{n, {l[0], l[1], l[2]}}] = i;
    cn.insert(cn.end(), 8, 0.0);
    return i;
}

int Tree::split(int i) {
    if (nodes[i].child0 >= 0) return nodes[i].child0;
    reserve(nodes.size() + 8);
    NodeInfo p = nodes[i];
    int first = (int)nodes.size();
    for (int c = 0; c < 8; c++) {
        int cl[3] = {2 * p.l[0] + (c & 1), 2 * p.l[1] + ((c >> 1) & 1), 2 * p.l[2] + ((c >> 2) & 1)};
        add(p.n + 1, cl, i);
    }
    nodes[i].child0 = first;
    return first;
}

void Tree::reset_roots() {
    nodes.clear();
    map.clear();
    cn.clear();
    const Basis &b = ctx->basis;
    for (int bz = 0; bz < b.boxes[2]; bz++)
        for (int by = 0; by < b.boxes[1]; by++)
            for (int bx = 0; bx < b.boxes[0]; bx++) {
                int l[3] = {b.corner[0] + bx, b.corner[1] + by, b.corner[2] + bz};
                add(b.n0, l, -1);
            }
    nroots = (int)nodes.size();
}

void Tree::download_norms(int first, int count) {
    if (count <= 0) return;
    MWG_CUDA(cudaMemcpyAsync(&cn[(size_t)first * 8], d_cn + (size_t)first * 8, sizeof(double) * 8 * count,
                             cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
}

double Tree::sqnorm_leaves() const {
    double s = 0.0;
    for (size_t i = 0; i < nodes.size(); i++) {
        if (nodes[i].child0 >= 0) continue;
        for (int c = 0; c < 8; c++) s += cn[8 * i + c] * cn[8 * i + c];
    }
    return s;
}

int Tree::max_scale() const {
    int m = ctx->basis.n0;
    for (auto &nd : nodes) m = std::max(m, nd.n);
    return m;
}

void Tree::free_device() {
    if (d_coefs) cudaFree(d_coefs);
    if (d_cn) cudaFree(d_cn);
    if (d_coefs32) cudaFree(d_coefs32);
    if (d_coefs_tc) cudaFree(d_coefs_tc);
    d_coefs = nullptr;
    d_cn = nullptr;
    d_coefs32 = nullptr;
    d_coefs_tc = nullptr;
    cap = cap32 = cap_tc = 0;
}

void tree_zero(Tree &t, int first, int count) {
    if (count <= 0) return;
    int bs = t.ctx->basis.bs;
    MWG_CUDA(cudaMemsetAsync(t.block(first), 0, sizeof(double) * bs * count, t.ctx->stream));
    MWG_CUDA(cudaMemsetAsync(t.d_cn + (size_t)first * 8, 0, sizeof(double) * 8 * count, t.ctx->stream));
    std::fill(t.cn.begin() + (size_t)first * 8, t.cn.begin() + (size_t)(first + count) * 8, 0.0);
}

void tree_clear(Tree &t) {
    t.reset_roots();
    tree_zero(t, 0, t.nn());
}

// Morton order (z most significant) of translations shifted to be non-negative
static bool less_msb(unsigned a, unsigned b) { return a < b && a < (a ^ b); }

bool key_less(const Basis &b, const NodeInfo &x, const NodeInfo &y) {
    if (x.n != y.n) return x.n < y.n;
    int sh = x.n - b.n0;
    unsigned ux[3], uy[3];
    for (int d = 0; d < 3; d++) {
        ux[d] = (unsigned)(x.l[d] - b.corner[d] * (1 << sh));
        uy[d] = (unsigned)(y.l[d] - b.corner[d] * (1 << sh));
    }
    int dim = 2;
    unsigned xm = ux[2] ^ uy[2];
    for (int d = 1; d >= 0; d--) {
        unsigned v = ux[d] ^ uy[d];
        if (less_msb(xm, v)) {
            dim = d;
            xm = v;
        }
    }
    return ux[dim] < uy[dim];
}

std::vector<int> canonical_order(const Tree &t) {
    std::vector<int> idx(t.nn());
    std::iota(idx.begin(), idx.end(), 0);
    const Basis &b = t.ctx->basis;
    std::sort(idx.begin(), idx.end(), [&](int i, int j) { return key_less(b, t.nodes[i], t.nodes[j]); });
    return idx;
}

// bottom-up: every branch node's block <- compress(children scaling parts)
void tree_compress(Tree &t, Arena &arena, mw_stats *st) {
    Ctx &ctx = *t.ctx;
    int maxn = t.max_scale();
    for (int n = maxn - 1; n >= ctx.basis.n0; n--) {
        std::vector<PairTask> tasks;
        std::vector<double *> cnp;
        for (int i = 0; i < t.nn(); i++) {
            const NodeInfo &nd = t.nodes[i];
            if (nd.n != n || nd.child0 < 0) continue;
            tasks.push_back({t.block(i), t.block(nd.child0)});
            cnp.push_back(t.d_cn + (size_t)i * 8);
        }
        if (tasks.empty()) continue;
        Packer pk;
        pk.add(tasks.data(), tasks.size() * sizeof(PairTask));
        pk.add(cnp.data(), cnp.size() * sizeof(double *));
        pk.ship(ctx, arena);
        k_compress(ctx.dbasis, (const PairTask *)pk.ptr(0), (double *const *)pk.ptr(1), (int)tasks.size(), ctx.stream);
        if (st) st->launches++;
    }
    MWG_CUDA(cudaMemcpyAsync(t.cn.data(), t.d_cn, sizeof(double) * 8 * t.nn(), cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
}

void tree_norms_all(Tree &t, Arena &arena) {
    Ctx &ctx = *t.ctx;
    std::vector<double *> bl(t.nn()), cnp(t.nn());
    for (int i = 0; i < t.nn(); i++) {
        bl[i] = t.block(i);
        cnp[i] = t.d_cn + (size_t)i * 8;
    }
    Packer pk;
    pk.add(bl.data(), bl.size() * sizeof(double *));
    pk.add(cnp.data(), cnp.size() * sizeof(double *));
    pk.ship(ctx, arena);
    k_norms(ctx.dbasis, (double *const *)pk.ptr(0), (double *const *)pk.ptr(1), t.nn(), ctx.stream);
    MWG_CUDA(cudaMemcpyAsync(t.cn.data(), t.d_cn, sizeof(double) * 8 * t.nn(), cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
}

// ------------------------------------------------------------------ generated blocks
void GenSet::clear() {
    slot.clear();
    tasks.clear();
    keys.clear();
    anc.clear();
}

int GenSet::request(const Tree &src, int n, const int *l, int ancestor) {
    Key k{n, {l[0], l[1], l[2]}};
    auto it = slot.find(k);
    if (it != slot.end()) return it->second;
    int g = (int)keys.size();
    slot.emplace(k, g);
    keys.push_back(k);
    anc.push_back(ancestor);
    (void)src;
    return g;
}

int find_ancestor(const Tree &t, int n, const int *l, int *an_out) {
    int an = n, al[3] = {l[0], l[1], l[2]};
    int a = -1;
    while (a < 0 && an > t.ctx->basis.n0) {
        an--;
        for (int d = 0; d < 3; d++) al[d] = floordiv2(al[d]);
        a = t.find(an, al);
    }
    if (an_out) *an_out = an;
    return a;
}

// Generates the requested blocks of several (set, source tree) pairs with one
// launch and one norm download; each set gets its device base and host norms.
void generate_all(const std::vector<std::pair<GenSet *, const Tree *>> &sets, Arena &arena, mw_stats *st) {
    if (sets.empty()) return;
    Ctx &ctx = *sets[0].second->ctx;
    const int bs = ctx.basis.bs;
    long total = 0;
    for (auto &p : sets) total += (long)p.first->keys.size();
    for (auto &p : sets) {
        p.first->base = nullptr;
        p.first->cn.assign(8 * p.first->keys.size(), 0.0);
    }
    if (total == 0) return;
    double *blocks = (double *)arena.alloc(sizeof(double) * (size_t)bs * total);
    double *cnd = (double *)arena.alloc(sizeof(double) * 8 * (size_t)total);
    std::vector<GenTask> tasks(total);
    long off = 0;
    for (auto &p : sets) {
        GenSet &gs = *p.first;
        const Tree &src = *p.second;
        gs.base = blocks + (size_t)off * bs;
        for (size_t g = 0; g < gs.keys.size(); g++) {
            const Key &k = gs.keys[g];
            int a = gs.anc[g];
            int an = src.nodes[a].n;
            GenTask &tk = tasks[off + g];
            tk.anc = src.block(a);
            tk.out = blocks + (size_t)(off + g) * bs;
            tk.cn = cnd + (size_t)8 * (off + g);
            tk.steps = k.n - an;
            tk.path = 0;
            for (int s = 0; s < tk.steps; s++) {
                int sh = k.n - (an + s + 1);
                uint64_t c = 0;
                for (int d = 0; d < 3; d++) c |= (uint64_t)((k.l[d] >> sh) & 1) << d;
                tk.path |= c << (3 * s);
            }
            tk.pad = 0;
        }
        off += (long)gs.keys.size();
    }
    Packer pk;
    pk.add(tasks.data(), tasks.size() * sizeof(GenTask));
    pk.ship(ctx, arena);
    const int ggrid = (int)std::min<long>(total, 4L * std::max(ctx.nsm, 1));
    const int K = ctx.basis.K;
    double *gscratch =
        (K >= 4 && K <= KMAX) ? nullptr : (double *)arena.alloc(sizeof(double) * generate_scratch_doubles(K) * ggrid);
    k_generate(ctx.dbasis, (const GenTask *)pk.ptr(0), (int)total, gscratch, ggrid, ctx.nsm, ctx.stream);
    if (st) {
        st->launches++;
        st->generated += total;
    }
    std::vector<double> h((size_t)8 * total);
    MWG_CUDA(cudaMemcpyAsync(h.data(), cnd, sizeof(double) * 8 * total, cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    off = 0;
    for (auto &p : sets) {
        std::copy(h.begin() + 8 * off, h.begin() + 8 * (off + (long)p.first->keys.size()), p.first->cn.begin());
        off += (long)p.first->keys.size();
    }
}

// Generates the requested blocks of `src` into arena memory; returns device base.
double *GenSet::generate(const Tree &src, Arena &arena, std::vector<double> &cn_out, mw_stats *st) {
    generate_all({{this, &src}}, arena, st);
    cn_out = cn;
    return base;
}

// block pointer of src at (n,l): the node's block or a generated one (gens must be generated)
const double *block_at(const Tree &src, const GenSet &gs, const double *gbase, int n, const int *l) {
    int i = src.find(n, l);
    if (i >= 0) return src.block(i);
    auto it = gs.slot.find(Key{n, {l[0], l[1], l[2]}});
    return gbase + (size_t)it->second * src.ctx->basis.bs;
}

// ------------------------------------------------------------------ projection
namespace {

struct HostFunc {
    int kind = 0;
    std::vector<mw_gterm> terms;
    int hn = 1, hl = 0, hm = 0;
    double Z = 1.0, origin[3] = {0, 0, 0}, hnorm = 1.0;
};

double box_dist(const double *lo, const double *hi, const double *p) {
    double s = 0.0;
    for (int d = 0; d < 3; d++) {
        double e = 0.0;
        if (p[d] < lo[d]) e = lo[d] - p[d];
        if (p[d] > hi[d]) e = p[d] - hi[d];
        s += e * e;
    }
    return std::sqrt(s);
}

// zero: all terms negligible on the box; forced: a term narrower than the children's quadrature resolves
void box_flags(const HostFunc &f, int K, int n, const int *l, int &zero, int &forced) {
    double h = std::ldexp(1.0, -n), lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
        lo[d] = h * l[d];
        hi[d] = h * (l[d] + 1);
    }
    zero = 1;
    forced = 0;
    if (f.kind == 0) {
        for (const auto &g : f.terms) {
            double dist = box_dist(lo, hi, g.pos);
            if (g.alpha * dist * dist > ZERO_EXP) continue;
            zero = 0;
            double sigma = 1.0 / std::sqrt(2.0 * g.alpha);
            if (0.5 * h > 0.5 * K * sigma) forced = 1;
        }
    } else {
        double dist = box_dist(lo, hi, f.origin), decay = f.Z / f.hn;
        if (decay * dist < ZERO_EXP) {
            zero = 0;
            if (0.5 * h > 0.5 * K / decay) forced = 1;
        }
    }
}

double split_thr(double prec, double R, int n) { return prec * R * std::pow(2.0, -0.5 * (n + 1)); }

void project(double prec, Tree &t, const HostFunc &f, bool abs_prec, Arena &arena) {
    Ctx &ctx = *t.ctx;
    const Basis &b = ctx.basis;
    arena.reset();
    t.reset_roots();
    ProjFunc pf{};
    pf.kind = f.kind;
    pf.nterms = (int)f.terms.size();
    pf.hn = f.hn;
    pf.hl = f.hl;
    pf.hm = f.hm;
    pf.Z = f.Z;
    for (int d = 0; d < 3; d++) pf.origin[d] = f.origin[d];
    pf.hnorm = f.hnorm;
    if (!f.terms.empty()) {
        Packer pk;
        pk.add(f.terms.data(), f.terms.size() * sizeof(mw_gterm));
        pk.ship(ctx, arena);
        pf.terms = (const mw_gterm *)pk.ptr(0);
    }
    int first = 0, count = t.nn();
    int maxn = b.max_scale();
    while (count > 0) {
        std::vector<ProjTask> tasks(count);
        std::vector<char> forced(count);
        for (int w = 0; w < count; w++) {
            int i = first + w;
            const NodeInfo &nd = t.nodes[i];
            int zero, frc;
            box_flags(f, b.K, nd.n, nd.l, zero, frc);
            forced[w] = (char)(frc && !zero);
            ProjTask &tk = tasks[w];
            tk.n = nd.n;
            for (int d = 0; d < 3; d++) tk.l[d] = nd.l[d];
            tk.out = t.block(i);
            tk.cn = t.d_cn + (size_t)8 * i;
            tk.zero = zero;
            tk.pad = 0;
        }
        Packer pk;
        pk.add(tasks.data(), tasks.size() * sizeof(ProjTask));
        pk.ship(ctx, arena);
        k_project(ctx.dbasis, pf, (const ProjTask *)pk.ptr(0), count, ctx.stream);
        t.download_norms(first, count);
        double R = abs_prec ? 1.0 : std::sqrt(t.sqnorm_leaves());
        int next_first = t.nn(), next_count = 0;
        for (int w = 0; w < count; w++) {
            int i = first + w;
            int n = t.nodes[i].n;
            if (n >= maxn) continue;
            double wn = 0.0;
            for (int c = 1; c < 8; c++) wn += t.cn[8 * i + c] * t.cn[8 * i + c];
            if (forced[w] || std::sqrt(wn) > split_thr(prec, R, n)) {
                t.split(i);
                next_count += 8;
            }
        }
        first = next_first;
        count = next_count;
    }
    tree_compress(t, arena, nullptr);
}

}  // namespace

void project_gauss(double prec, Tree &t, int nterms, const mw_gterm *terms, bool abs_prec, Arena &arena) {
    HostFunc f;
    f.kind = 0;
    f.terms.assign(terms, terms + nterms);
    project(prec, t, f, abs_prec, arena);
}

static double factorial(int n) {
    double f = 1.0;
    for (int i = 2; i <= n; i++) f *= i;
    return f;
}

void project_hydrogen(double prec, Tree &t, int n, int l, int m, double Z, const double *origin, bool abs_prec,
                      Arena &arena) {
    if (n < 1 || l < 0 || l > 1 || l >= n || m < 0 || m > 2 * l)
        throw Error(MW_ERR_ARG, "hydrogen orbital: need n >= 1, 0 <= l <= 1, l < n, 0 <= m <= 2l");
    HostFunc f;
    f.kind = 1;
    f.hn = n;
    f.hl = l;
    f.hm = m;
    f.Z = Z;
    for (int d = 0; d < 3; d++) f.origin[d] = origin ? origin[d] : 0.0;
    f.hnorm = std::sqrt(std::pow(2.0 * Z / n, 3) * factorial(n - l - 1) / (2.0 * n * factorial(n + l)));
    project(prec, t, f, abs_prec, arena);
}

// ------------------------------------------------------------------ transfers
// the tree structure of a key list; returns, per tree node, its position in the list
static std::vector<int> upload_structure(Tree &t, int nnodes, const int *keys) {
    std::unordered_map<Key, int, KeyHash> src;
    src.reserve(nnodes * 2);
    for (int i = 0; i < nnodes; i++) src[Key{keys[4 * i], {keys[4 * i + 1], keys[4 * i + 2], keys[4 * i + 3]}}] = i;
    t.reset_roots();
    std::vector<int> from;
    for (int i = 0; i < t.nn(); i++) {
        const NodeInfo nd = t.nodes[i];
        auto it = src.find(Key{nd.n, {nd.l[0], nd.l[1], nd.l[2]}});
        if (it == src.end()) throw Error(MW_ERR_ARG, "upload: keys do not contain every root / sibling node");
        from.push_back(it->second);
        int cl[3] = {2 * nd.l[0], 2 * nd.l[1], 2 * nd.l[2]};
        if (src.count(Key{nd.n + 1, {cl[0], cl[1], cl[2]}})) t.split(i);
    }
    if (t.nn() != nnodes) throw Error(MW_ERR_ARG, "upload: keys do not form a complete tree");
    return from;
}

void tree_upload(Tree &t, int nnodes, const int *keys, const double *coefs, Arena &arena) {
    Ctx &ctx = *t.ctx;
    int bs = ctx.basis.bs;
    std::vector<int> from = upload_structure(t, nnodes, keys);
    ctx.sync();
    double *h = (double *)ctx.pinned(sizeof(double) * (size_t)bs * nnodes);
    // gather into tree order with all host threads (the blocks are tens of MB per tree)
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nnodes; i++) std::memcpy(h + (size_t)i * bs, coefs + (size_t)from[i] * bs, sizeof(double) * bs);
    MWG_CUDA(cudaMemcpyAsync(t.d_coefs, h, sizeof(double) * (size_t)bs * nnodes, cudaMemcpyHostToDevice, ctx.stream));
    arena.reset();
    tree_norms_all(t, arena);
}

// Several trees of one context in one pass: all structures first, then one gather of every
// block into pinned staging with all host threads, the copies, one norms launch and one
// synchronisation (instead of one per tree).
bool host_is_pinned(const void *p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

std::vector<std::vector<int>> upload_structures(const std::vector<Tree *> &trees, const int *nnodes,
                                                const int *const *keys) {
    const int n = (int)trees.size();
    std::vector<std::vector<int>> from(n);
    if (n == 0) return from;
    // sized first, so that building the structures is host work only and runs in parallel
    for (int i = 0; i < n; i++) trees[i]->reserve((size_t)nnodes[i]);
    trees[0]->ctx->sync();
    std::vector<std::string> err(n);
    std::vector<int> code(n, MW_OK);
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < n; i++) {
        try {
            from[i] = upload_structure(*trees[i], nnodes[i], keys[i]);
        } catch (const Error &e) {
            code[i] = e.code;
            err[i] = e.what();
        }
    }
    for (int i = 0; i < n; i++)
        if (code[i] != MW_OK) throw Error(code[i], err[i]);
    return from;
}

double *upload_enqueue(const std::vector<Tree *> &trees, const std::vector<const int *> &maps,
                       const double *staged, Arena &arena) {
    Ctx &ctx = *trees[0]->ctx;
    const int bs = ctx.basis.bs, n = (int)trees.size();
    std::vector<size_t> first(n + 1, 0);
    for (int i = 0; i < n; i++) first[i + 1] = first[i] + (size_t)trees[i]->nn();
    std::vector<int> m;
    std::vector<double *> bl, cnp;
    m.reserve(first[n]);
    for (int i = 0; i < n; i++) {
        m.insert(m.end(), maps[i], maps[i] + trees[i]->nn());
        for (int j = 0; j < trees[i]->nn(); j++) {
            bl.push_back(trees[i]->block(j));
            cnp.push_back(trees[i]->d_cn + (size_t)8 * j);
        }
    }
    Packer pk;
    pk.add(m.data(), m.size() * sizeof(int));
    pk.add(bl.data(), bl.size() * sizeof(double *));
    pk.add(cnp.data(), cnp.size() * sizeof(double *));
    pk.ship(ctx, arena);
    const int *dmap = (const int *)pk.ptr(0);
    for (int i = 0; i < n; i++)
        k_permute_blocks(trees[i]->d_coefs, staged + first[i] * bs, dmap + first[i], trees[i]->nn(), bs, ctx.stream);
    k_norms(ctx.dbasis, (double *const *)pk.ptr(1), (double *const *)pk.ptr(2), (int)bl.size(), ctx.stream);
    double *h = (double *)arena.halloc(sizeof(double) * 8 * first[n]);
    for (int i = 0; i < n; i++)
        MWG_CUDA(cudaMemcpyAsync(h + 8 * first[i], trees[i]->d_cn, sizeof(double) * 8 * trees[i]->nn(),
                                 cudaMemcpyDeviceToHost, ctx.stream));
    return h;
}

void download_enqueue(const std::vector<Tree *> &trees, int *const *keys, double *const *coefs,
                      unsigned char *const *leaf, Arena &arena) {
    const int n = (int)trees.size();
    if (n == 0) return;
    Ctx &ctx = *trees[0]->ctx;
    const int bs = ctx.basis.bs;
    std::vector<std::vector<int>> idx(n);
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < n; i++) idx[i] = canonical_order(*trees[i]);
    std::vector<size_t> first(n + 1, 0);
    for (int i = 0; i < n; i++) first[i + 1] = first[i] + (size_t)trees[i]->nn();
    double *scratch = (double *)arena.alloc(sizeof(double) * (size_t)bs * first[n]);
    std::vector<int> maps;
    maps.reserve(first[n]);
    for (int i = 0; i < n; i++) maps.insert(maps.end(), idx[i].begin(), idx[i].end());
    Packer pk;
    pk.add(maps.data(), maps.size() * sizeof(int));
    pk.ship(ctx, arena);
    const int *dmap = (const int *)pk.ptr(0);
    for (int i = 0; i < n; i++) {
        k_permute_blocks(scratch + first[i] * bs, trees[i]->d_coefs, dmap + first[i], trees[i]->nn(), bs, ctx.stream);
        MWG_CUDA(cudaMemcpyAsync(coefs[i], scratch + first[i] * bs, sizeof(double) * (size_t)bs * trees[i]->nn(),
                                 cudaMemcpyDeviceToHost, ctx.stream));
    }
    // keys and leaf flags are host data: written now
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < n; i++)
        for (int j = 0; j < trees[i]->nn(); j++) {
            const NodeInfo &nd = trees[i]->nodes[idx[i][j]];
            if (keys[i]) {
                keys[i][4 * j] = nd.n;
                for (int d = 0; d < 3; d++) keys[i][4 * j + 1 + d] = nd.l[d];
            }
            if (leaf[i]) leaf[i][j] = nd.child0 < 0;
        }
}

void tree_upload_batch(const std::vector<Tree *> &trees, const int *nnodes, const int *const *keys,
                       const double *const *coefs, Arena &arena) {
    if (trees.empty()) return;
    Ctx &ctx = *trees[0]->ctx;
    const int bs = ctx.basis.bs, n = (int)trees.size();
    std::vector<std::vector<int>> from(n);
    std::vector<size_t> first(n + 1, 0);
    for (int i = 0; i < n; i++) first[i + 1] = first[i] + (size_t)nnodes[i];
    // the trees' device arrays are sized first, so that building the structures below is host
    // work only and runs for all trees in parallel
    for (int i = 0; i < n; i++) trees[i]->reserve((size_t)nnodes[i]);
    ctx.sync();
    auto structures = [&] {
        std::vector<std::string> err(n);
        std::vector<int> code(n, MW_OK);
#pragma omp parallel for schedule(dynamic, 1)
        for (int i = 0; i < n; i++) {
            try {
                from[i] = upload_structure(*trees[i], nnodes[i], keys[i]);
            } catch (const Error &e) {
                code[i] = e.code;
                err[i] = e.what();
            }
        }
        for (int i = 0; i < n; i++)
            if (code[i] != MW_OK) throw Error(code[i], err[i]);
    };
    bool pinned = true;
    for (int i = 0; i < n && pinned; i++) pinned = host_is_pinned(coefs[i]);
    if (pinned) {
        // the caller's blocks go straight to device scratch while the host builds the trees'
        // structures; the permutation into tree order runs on the device
        arena.reset();
        double *scratch = (double *)arena.alloc(sizeof(double) * (size_t)bs * first[n]);
        for (int i = 0; i < n; i++)
            MWG_CUDA(cudaMemcpyAsync(scratch + first[i] * bs, coefs[i], sizeof(double) * (size_t)bs * nnodes[i],
                                     cudaMemcpyHostToDevice, ctx.stream));
        structures();
        std::vector<int> maps;
        maps.reserve(first[n]);
        for (int i = 0; i < n; i++) maps.insert(maps.end(), from[i].begin(), from[i].end());
        Packer pk;
        pk.add(maps.data(), maps.size() * sizeof(int));
        pk.ship(ctx, arena);
        const int *dmap = (const int *)pk.ptr(0);
        for (int i = 0; i < n; i++)
            k_permute_blocks(trees[i]->d_coefs, scratch + first[i] * bs, dmap + first[i], nnodes[i], bs, ctx.stream);
        tree_norms_batch(trees, nnodes, arena);
        return;
    }
    structures();
    double *h = (double *)ctx.pinned(sizeof(double) * (size_t)bs * first[n]);
    std::vector<std::pair<int, int>> all;  // (tree, node)
    all.reserve(first[n]);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < nnodes[i]; j++) all.push_back({i, j});
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)all.size(); q++) {
        const int i = all[q].first, j = all[q].second;
        std::memcpy(h + (first[i] + j) * bs, coefs[i] + (size_t)from[i][j] * bs, sizeof(double) * bs);
    }
    arena.reset();
    for (int i = 0; i < n; i++)
        MWG_CUDA(cudaMemcpyAsync(trees[i]->d_coefs, h + first[i] * bs, sizeof(double) * (size_t)bs * nnodes[i],
                                 cudaMemcpyHostToDevice, ctx.stream));
    tree_norms_batch(trees, nnodes, arena);
}

// component norms of every node of several trees: one launch, one download, one synchronisation
void tree_norms_batch(const std::vector<Tree *> &trees, const int *nnodes, Arena &arena) {
    Ctx &ctx = *trees[0]->ctx;
    const int n = (int)trees.size();
    std::vector<double *> bl, cnp;
    for (int i = 0; i < n; i++) {
        Tree &t = *trees[i];
        for (int j = 0; j < t.nn(); j++) {
            bl.push_back(t.block(j));
            cnp.push_back(t.d_cn + (size_t)j * 8);
        }
    }
    Packer pk;
    pk.add(bl.data(), bl.size() * sizeof(double *));
    pk.add(cnp.data(), cnp.size() * sizeof(double *));
    pk.ship(ctx, arena);
    k_norms(ctx.dbasis, (double *const *)pk.ptr(0), (double *const *)pk.ptr(1), (int)bl.size(), ctx.stream);
    std::vector<double *> hcn(n);
    for (int i = 0; i < n; i++) {
        hcn[i] = (double *)arena.halloc(sizeof(double) * 8 * nnodes[i]);
        MWG_CUDA(cudaMemcpyAsync(hcn[i], trees[i]->d_cn, sizeof(double) * 8 * nnodes[i], cudaMemcpyDeviceToHost,
                                 ctx.stream));
    }
    ctx.sync();
    for (int i = 0; i < n; i++) std::copy(hcn[i], hcn[i] + (size_t)8 * nnodes[i], trees[i]->cn.begin());
    arena.reset();
}

void tree_download_batch(const std::vector<Tree *> &trees, int *const *keys, double *const *coefs,
                         unsigned char *const *leaf) {
    if (trees.empty()) return;
    Ctx &ctx = *trees[0]->ctx;
    const int bs = ctx.basis.bs, n = (int)trees.size();
    std::vector<std::vector<int>> idx(n);
    std::vector<size_t> first(n + 1, 0);
    for (int i = 0; i < n; i++) first[i + 1] = first[i] + (size_t)trees[i]->nn();
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < n; i++) idx[i] = canonical_order(*trees[i]);
    bool pinned = true;
    for (int i = 0; i < n && pinned; i++) pinned = !coefs[i] || host_is_pinned(coefs[i]);
    double *h = nullptr;
    if (pinned) {
        // permutation into canonical order on the device, then straight into the caller's buffers
        Arena &arena = ctx.arena;
        ctx.sync();
        arena.reset();
        double *scratch = (double *)arena.alloc(sizeof(double) * (size_t)bs * first[n]);
        std::vector<int> maps;
        maps.reserve(first[n]);
        for (int i = 0; i < n; i++) maps.insert(maps.end(), idx[i].begin(), idx[i].end());
        Packer pk;
        pk.add(maps.data(), maps.size() * sizeof(int));
        pk.ship(ctx, arena);
        const int *dmap = (const int *)pk.ptr(0);
        for (int i = 0; i < n; i++) {
            if (!coefs[i]) continue;
            k_permute_blocks(scratch + first[i] * bs, trees[i]->d_coefs, dmap + first[i], trees[i]->nn(), bs,
                             ctx.stream);
            MWG_CUDA(cudaMemcpyAsync(coefs[i], scratch + first[i] * bs, sizeof(double) * (size_t)bs * trees[i]->nn(),
                                     cudaMemcpyDeviceToHost, ctx.stream));
        }
    } else {
        h = (double *)ctx.pinned(sizeof(double) * (size_t)bs * first[n]);
        for (int i = 0; i < n; i++)
            if (coefs[i])
                MWG_CUDA(cudaMemcpyAsync(h + first[i] * bs, trees[i]->d_coefs,
                                         sizeof(double) * (size_t)bs * trees[i]->nn(), cudaMemcpyDeviceToHost,
                                         ctx.stream));
    }
    ctx.sync();
    if (pinned) ctx.arena.reset();
    std::vector<std::pair<int, int>> all;
    all.reserve(first[n]);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < trees[i]->nn(); j++) all.push_back({i, j});
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)all.size(); q++) {
        const int i = all[q].first, j = all[q].second;
        const int src = idx[i][j];
        if (coefs[i] && h) std::memcpy(coefs[i] + (size_t)j * bs, h + (first[i] + src) * bs, sizeof(double) * bs);
        const NodeInfo &nd = trees[i]->nodes[src];
        if (keys[i]) {
            keys[i][4 * j] = nd.n;
            for (int d = 0; d < 3; d++) keys[i][4 * j + 1 + d] = nd.l[d];
        }
        if (leaf[i]) leaf[i][j] = nd.child0 < 0;
    }
}

void tree_download(Tree &t, int *keys, double *coefs, unsigned char *leaf) {
    Ctx &ctx = *t.ctx;
    int bs = ctx.basis.bs, n = t.nn();
    std::vector<int> idx = canonical_order(t);
    if (coefs) {
        double *h = (double *)ctx.pinned(sizeof(double) * (size_t)bs * n);
        MWG_CUDA(cudaMemcpyAsync(h, t.d_coefs, sizeof(double) * (size_t)bs * n, cudaMemcpyDeviceToHost, ctx.stream));
        ctx.sync();
#pragma omp parallel for schedule(static)
        for (int j = 0; j < n; j++) std::memcpy(coefs + (size_t)j * bs, h + (size_t)idx[j] * bs, sizeof(double) * bs);
    }
    for (int j = 0; j < n; j++) {
        const NodeInfo &nd = t.nodes[idx[j]];
        if (keys) {
            keys[4 * j] = nd.n;
            for (int d = 0; d < 3; d++) keys[4 * j + 1 + d] = nd.l[d];
        }
        if (leaf) leaf[j] = nd.child0 < 0;
    }
}

// ------------------------------------------------------------------ files
// Tree file (checkpoint of one function tree, the role of MRCPP's saveTree in
// orbital::save_orbitals, src/qmfunctions/orbital_utils.cpp:1218-1240):
//   char[8] "MWGB300T", int32 version (1), int32 order, int32 basis, int32 root_scale,
//   int32 corner[3], int32 boxes[3], int64 nnodes,
//   int32 keys[nnodes][4] (n, lx, ly, lz), float64 coefs[nnodes][8 (order+1)^3]
// little-endian, nodes in canonical order.
void tree_save(Tree &t, const char *path) {
    const Basis &b = t.ctx->basis;
    int64_t n = t.nn();
    std::vector<int> keys(4 * n);
    std::vector<double> coefs((size_t)n * b.bs);
    tree_download(t, keys.data(), coefs.data(), nullptr);
    FILE *f = std::fopen(path, "wb");
    if (!f) throw Error(MW_ERR_ARG, std::string("cannot open ") + path);
    int32_t hdr[11] = {1, b.k, b.type, b.n0, b.corner[0], b.corner[1], b.corner[2], b.boxes[0], b.boxes[1], b.boxes[2], 0};
    bool ok = std::fwrite("MWGB300T", 1, 8, f) == 8 && std::fwrite(hdr, sizeof(int32_t), 10, f) == 10 &&
              std::fwrite(&n, sizeof(n), 1, f) == 1 && std::fwrite(keys.data(), sizeof(int), keys.size(), f) == keys.size() &&
              std::fwrite(coefs.data(), sizeof(double), coefs.size(), f) == coefs.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) throw Error(MW_ERR_STATE, std::string("write failed: ") + path);
}

void tree_load(Tree &t, const char *path) {
    const Basis &b = t.ctx->basis;
    FILE *f = std::fopen(path, "rb");
    if (!f) throw Error(MW_ERR_ARG, std::string("cannot open ") + path);
    char magic[8];
    int32_t hdr[10];
    int64_t n = 0;
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "MWGB300T", 8) == 0 &&
              std::fread(hdr, sizeof(int32_t), 10, f) == 10 && std::fread(&n, sizeof(n), 1, f) == 1;
    if (ok && (hdr[0] != 1 || hdr[1] != b.k || hdr[2] != b.type || hdr[3] != b.n0 || hdr[4] != b.corner[0] ||
               hdr[5] != b.corner[1] || hdr[6] != b.corner[2] || hdr[7] != b.boxes[0] || hdr[8] != b.boxes[1] ||
               hdr[9] != b.boxes[2] || n < 1 || n > (1LL << 31))) {
        std::fclose(f);
        throw Error(MW_ERR_ARG, std::string("tree file does not match this context: ") + path);
    }
    std::vector<int> keys;
    std::vector<double> coefs;
    if (ok) {
        keys.resize(4 * n);
        coefs.resize((size_t)n * b.bs);
        ok = std::fread(keys.data(), sizeof(int), keys.size(), f) == keys.size() &&
             std::fread(coefs.data(), sizeof(double), coefs.size(), f) == coefs.size();
    }
    std::fclose(f);
    if (!ok) throw Error(MW_ERR_ARG, std::string("truncated or foreign tree file: ") + path);
    tree_upload(t, (int)n, keys.data(), coefs.data(), t.ctx->arena);
}

// ------------------------------------------------------------------ grids
void copy_grid(Tree &out, const Tree &inp) {
    out.reset_roots();
    for (int i = 0; i < out.nn(); i++) {
        const NodeInfo nd = out.nodes[i];
        int j = inp.find(nd.n, nd.l);
        if (j >= 0 && inp.nodes[j].child0 >= 0) out.split(i);
    }
    tree_zero(out, 0, out.nn());
}

void build_grid(Tree &out, const std::vector<const Tree *> &trees) {
    int before = out.nn();
    for (int i = 0; i < out.nn(); i++) {
        if (out.nodes[i].child0 >= 0) continue;
        const NodeInfo nd = out.nodes[i];
        for (const Tree *t : trees) {
            int j = t->find(nd.n, nd.l);
            if (j >= 0 && t->nodes[j].child0 >= 0) {
                out.split(i);
                break;
            }
        }
    }
    tree_zero(out, before, out.nn() - before);
}

// out <- linear combination of trees on out's current grid (generated where coarser)
void combine_on_grid(Tree &out, const std::vector<const Tree *> &trees, const std::vector<double> &coefs, Arena &arena,
                     mw_stats *st) {
    Ctx &ctx = *out.ctx;
    int N = out.nn();
    std::vector<GenSet> gens(trees.size());
    std::vector<double *> gbase(trees.size(), nullptr);
    std::vector<double> gcn;
    for (size_t k = 0; k < trees.size(); k++) {
        const Tree &src = *trees[k];
        for (int i = 0; i < N; i++) {
            const NodeInfo &nd = out.nodes[i];
            if (src.find(nd.n, nd.l) >= 0) continue;
            int a = find_ancestor(src, nd.n, nd.l, nullptr);
            if (a >= 0) gens[k].request(src, nd.n, nd.l, a);
        }
    }
    for (size_t k = 0; k < trees.size(); k++) gbase[k] = gens[k].generate(*trees[k], arena, gcn, st);
    std::vector<AddTask> tasks(N);
    std::vector<const double *> src;
    std::vector<double> cf;
    for (int i = 0; i < N; i++) {
        const NodeInfo &nd = out.nodes[i];
        tasks[i].out = out.block(i);
        tasks[i].cn = out.d_cn + (size_t)8 * i;
        tasks[i].first = (int)src.size();
        for (size_t k = 0; k < trees.size(); k++) {
            const Tree &t = *trees[k];
            int j = t.find(nd.n, nd.l);
            const double *p = nullptr;
            if (j >= 0)
                p = t.block(j);
            else if (gens[k].slot.count(Key{nd.n, {nd.l[0], nd.l[1], nd.l[2]}}))
                p = block_at(t, gens[k], gbase[k], nd.n, nd.l);
            if (!p) continue;
            src.push_back(p);
            cf.push_back(coefs[k]);
        }
        tasks[i].count = (int)src.size() - tasks[i].first;
    }
    Packer pk;
    pk.add(tasks.data(), tasks.size() * sizeof(AddTask));
    pk.add(src.data(), src.size() * sizeof(double *));
    pk.add(cf.data(), cf.size() * sizeof(double));
    pk.ship(ctx, arena);
    k_add(ctx.dbasis, (const AddTask *)pk.ptr(0), (const double *const *)pk.ptr(1), (const double *)pk.ptr(2), N,
          ctx.basis.bs, ctx.stream);
    if (st) st->launches++;
    MWG_CUDA(cudaMemcpyAsync(out.cn.data(), out.d_cn, sizeof(double) * 8 * N, cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
}

void copy_func(Tree &out, const Tree &inp, Arena &arena) {
    arena.reset();
    combine_on_grid(out, {&inp}, {1.0}, arena, nullptr);
}

// remove the children of nodes whose children are all leaves and whose combined
// wavelet norm is below prec * R * 2^{-(n+2)/2}; fine to coarse
void crop(Tree &t, double prec, bool abs_prec, Arena &arena) {
    Ctx &ctx = *t.ctx;
    double R = abs_prec ? 1.0 : std::sqrt(t.sqnorm_leaves());
    int N = t.nn();
    std::vector<char> dead(N, 0), leaf(N);
    for (int i = 0; i < N; i++) leaf[i] = t.nodes[i].child0 < 0;
    for (int n = t.max_scale() - 1; n >= ctx.basis.n0; n--)
        for (int i = 0; i < N; i++) {
            const NodeInfo &nd = t.nodes[i];
            if (nd.n != n || leaf[i]) continue;
            bool all = true;
            double s = 0.0;
            for (int c = 0; c < 8; c++) {
                int ci = nd.child0 + c;
                if (!leaf[ci]) all = false;
                for (int q = 1; q < 8; q++) s += t.cn[8 * ci + q] * t.cn[8 * ci + q];
            }
            if (all && std::sqrt(s) < split_thr(prec, R, n + 1)) {
                for (int c = 0; c < 8; c++) dead[nd.child0 + c] = 1;
                leaf[i] = 1;
            }
        }
    int keep = 0;
    for (int i = 0; i < N; i++) keep += !dead[i];
    if (keep == N) return;
    // rebuild: new structure breadth-first over surviving nodes, gather their blocks
    Tree nt;
    nt.ctx = &ctx;
    nt.reset_roots();
    std::vector<int> from;
    for (int i = 0; i < nt.nn(); i++) {
        const NodeInfo nd = nt.nodes[i];
        int j = t.find(nd.n, nd.l);
        from.push_back(j);
        int c0 = t.nodes[j].child0;
        if (c0 >= 0 && !dead[c0]) nt.split(i);
    }
    arena.reset();
    std::vector<AddTask> tasks(nt.nn());
    std::vector<const double *> src(nt.nn());
    std::vector<double> cf(nt.nn(), 1.0);
    for (int i = 0; i < nt.nn(); i++) {
        tasks[i] = AddTask{nt.block(i), nt.d_cn + (size_t)8 * i, i, 1};
        src[i] = t.block(from[i]);
    }
    Packer pk;
    pk.add(tasks.data(), tasks.size() * sizeof(AddTask));
    pk.add(src.data(), src.size() * sizeof(double *));
    pk.add(cf.data(), cf.size() * sizeof(double));
    pk.ship(ctx, arena);
    k_add(ctx.dbasis, (const AddTask *)pk.ptr(0), (const double *const *)pk.ptr(1), (const double *)pk.ptr(2),
          nt.nn(), ctx.basis.bs, ctx.stream);
    MWG_CUDA(cudaMemcpyAsync(nt.cn.data(), nt.d_cn, sizeof(double) * 8 * nt.nn(), cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    t.free_device();
    t.nodes.swap(nt.nodes);
    t.map.swap(nt.map);
    t.cn.swap(nt.cn);
    t.d_coefs = nt.d_coefs;
    t.d_cn = nt.d_cn;
    t.cap = nt.cap;
    t.nroots = nt.nroots;
    nt.d_coefs = nullptr;
    nt.d_cn = nullptr;
}

double dot(const Tree &a, const Tree &b, Arena &arena) {
    Ctx &ctx = *a.ctx;
    int K3 = ctx.basis.K * ctx.basis.K * ctx.basis.K;
    std::vector<const double *> pa, pb;
    std::vector<int> start;
    for (int i = 0; i < a.nn(); i++) {
        const NodeInfo &nd = a.nodes[i];
        int j = b.find(nd.n, nd.l);
        if (j < 0) continue;
        pa.push_back(a.block(i));
        pb.push_back(b.block(j));
        start.push_back(nd.n == ctx.basis.n0 ? 0 : K3);
    }
    int n = (int)pa.size();
    if (n == 0) return 0.0;
    arena.reset();
    Packer pk;
    pk.add(pa.data(), n * sizeof(double *));
    pk.add(pb.data(), n * sizeof(double *));
    pk.add(start.data(), n * sizeof(int));
    pk.ship(ctx, arena);
    double *part = (double *)arena.alloc(sizeof(double) * n);
    k_dot((const double *const *)pk.ptr(0), (const double *const *)pk.ptr(1), (const int *)pk.ptr(2), n, ctx.basis.bs,
          part, ctx.stream);
    std::vector<double> h(n);
    MWG_CUDA(cudaMemcpyAsync(h.data(), part, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    double s = 0.0;
    for (double v : h) s += v;
    return s;
}

double integrate(const Tree &t) {
    Ctx &ctx = *t.ctx;
    const Basis &b = ctx.basis;
    int K = b.K, K3 = K * K * K;
    std::vector<double> h((size_t)t.nroots * b.bs);
    MWG_CUDA(cudaMemcpyAsync(h.data(), t.d_coefs, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    double s = 0.0;
    for (int r = 0; r < t.nroots; r++)
        for (int i = 0; i < K3; i++) {
            int ix = i % K, iy = (i / K) % K, iz = i / (K * K);
            s += h[(size_t)r * b.bs + i] * b.integ[ix] * b.integ[iy] * b.integ[iz];
        }
    return s * std::pow(2.0, -1.5 * b.n0);
}

void rescale(Tree &t, double c) {
    Ctx &ctx = *t.ctx;
    k_scale(t.d_coefs, (size_t)t.nn() * ctx.basis.bs, c, ctx.stream);
    k_scale(t.d_cn, (size_t)t.nn() * 8, std::fabs(c), ctx.stream);
    for (double &v : t.cn) v *= std::fabs(c);
    ctx.sync();
}

void eval_points(const Tree &t, int npts, const double *xyz, double *out, Arena &arena) {
    Ctx &ctx = *t.ctx;
    const Basis &b = ctx.basis;
    std::vector<const double *> blocks;
    std::vector<int> keys;
    std::vector<double> pts;
    std::vector<int> which;
    double hr = std::ldexp(1.0, -b.n0);
    for (int p = 0; p < npts; p++) {
        out[p] = 0.0;
        const double *r = xyz + 3 * p;
        int l[3];
        bool inside = true;
        for (int d = 0; d < 3; d++) {
            l[d] = (int)std::floor(r[d] / hr);
            if (l[d] < b.corner[d] || l[d] >= b.corner[d] + b.boxes[d]) inside = false;
        }
        if (!inside) continue;
        int i = t.find(b.n0, l);
        while (t.nodes[i].child0 >= 0) {
            const NodeInfo &nd = t.nodes[i];
            double h = std::ldexp(1.0, -(nd.n + 1));
            int c = 0;
            for (int d = 0; d < 3; d++) {
                int cl = (int)std::floor(r[d] / h);
                cl = std::min(std::max(cl, 2 * nd.l[d]), 2 * nd.l[d] + 1);
                c |= (cl - 2 * nd.l[d]) << d;
            }
            i = nd.child0 + c;
        }
        blocks.push_back(t.block(i));
        keys.insert(keys.end(), {t.nodes[i].n, t.nodes[i].l[0], t.nodes[i].l[1], t.nodes[i].l[2]});
        pts.insert(pts.end(), r, r + 3);
        which.push_back(p);
    }
    int n = (int)which.size();
    if (n == 0) return;
    arena.reset();
    Packer pk;
    pk.add(blocks.data(), n * sizeof(double *));
    pk.add(keys.data(), keys.size() * sizeof(int));
    pk.add(pts.data(), pts.size() * sizeof(double));
    pk.ship(ctx, arena);
    double *d_out = (double *)arena.alloc(sizeof(double) * n);
    k_eval(ctx.dbasis, (const double *const *)pk.ptr(0), (const int *)pk.ptr(1), (const double *)pk.ptr(2), n, d_out,
           ctx.stream);
    std::vector<double> h(n);
    MWG_CUDA(cudaMemcpyAsync(h.data(), d_out, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    for (int q = 0; q < n; q++) out[which[q]] = h[q];
}

}  // namespace mwg
