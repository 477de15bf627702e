// mw_capi.cpp -- extern "C" entry points (include/mw_gb300.h).
// Every entry catches errors and returns a status; the message is kept on the
// context for mw_last_error().  Nothing here falls back to host arithmetic:
// without a usable CUDA device the calls fail with MW_ERR_CUDA.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "mw_internal.h"

struct mw_ctx_s {
    mwg::Ctx ctx;
};
struct mw_tree_s {
    mwg::Tree tree;
};
struct mw_op_s {
    mwg::Oper op;
};

namespace {

thread_local std::string g_noctx_err;

template <typename F>
int guard(mwg::Ctx *ctx, F &&f) {
    int rc = MW_OK;
    try {
        if (ctx) MWG_CUDA(cudaSetDevice(ctx->device));
        f();
    } catch (const mwg::Error &e) {
        (ctx ? ctx->err : g_noctx_err) = e.what();
        rc = e.code;
    } catch (const std::bad_alloc &) {
        (ctx ? ctx->err : g_noctx_err) = "host allocation failed";
        rc = MW_ERR_OOM;
    } catch (const std::exception &e) {
        (ctx ? ctx->err : g_noctx_err) = e.what();
        rc = MW_ERR_STATE;
    }
    // device arrays that trees outgrew during the call, released once the call's work is done
    if (ctx) ctx->release_retired();
    return rc;
}

mwg::Ctx *ctx_of(mw_tree t) { return t ? t->tree.ctx : nullptr; }

void check_same(const mwg::Tree &a, const mwg::Tree &b) {
    if (a.ctx != b.ctx) throw mwg::Error(MW_ERR_ARG, "trees belong to different contexts");
}

}  // namespace

extern "C" {

int mw_ctx_create(int device, int root_scale, const int corner[3], const int boxes[3], int order, int basis,
                  int max_depth, mw_ctx *out) {
    if (!out || !corner || !boxes) return MW_ERR_ARG;
    *out = nullptr;
    if (order + 1 < 4 || order + 1 > mwg::KMAX) {
        g_noctx_err = "order must be in [3, 9] (K = order + 1 <= 10 on the GPU)";
        return MW_ERR_ARG;
    }
    if (max_depth < 1 || max_depth > 30 || (basis != MW_BASIS_LEGENDRE && basis != MW_BASIS_INTERPOLATING)) {
        g_noctx_err = "invalid max_depth or basis";
        return MW_ERR_ARG;
    }
    for (int d = 0; d < 3; d++)
        if (boxes[d] < 1) {
            g_noctx_err = "boxes must be >= 1";
            return MW_ERR_ARG;
        }
    mw_ctx c = new mw_ctx_s;
    int rc = guard(nullptr, [&] {
        int ndev = 0;
        MWG_CUDA(cudaGetDeviceCount(&ndev));
        if (device < 0 || device >= ndev) throw mwg::Error(MW_ERR_ARG, "no such CUDA device");
        c->ctx.device = device;
        MWG_CUDA(cudaSetDevice(device));
        MWG_CUDA(cudaStreamCreateWithFlags(&c->ctx.stream, cudaStreamNonBlocking));
        MWG_CUDA(cudaDeviceGetAttribute(&c->ctx.nsm, cudaDevAttrMultiProcessorCount, device));
        mwg::Basis &b = c->ctx.basis;
        b.init(root_scale, corner, boxes, order, basis, max_depth);
        int K = b.K, K2 = 2 * K;
        size_t nd = 4 * K2 * K2 + 2 * K * K + 3 * K + K * K;
        std::vector<double> h(nd);
        double *p = h.data();
        std::memcpy(p, b.W.data(), sizeof(double) * K2 * K2);
        std::memcpy(p + K2 * K2, b.WT.data(), sizeof(double) * K2 * K2);
        std::memcpy(p + 2 * K2 * K2, b.c2v.data(), sizeof(double) * K * K);
        std::memcpy(p + 2 * K2 * K2 + K * K, b.v2c.data(), sizeof(double) * K * K);
        std::memcpy(p + 2 * K2 * K2 + 2 * K * K, b.qx.data(), sizeof(double) * K);
        std::memcpy(p + 2 * K2 * K2 + 2 * K * K + K, b.qw.data(), sizeof(double) * K);
        std::memcpy(p + 2 * K2 * K2 + 2 * K * K + 2 * K, b.legq.data(), sizeof(double) * K * K);
        MWG_CUDA(cudaMalloc(&c->ctx.d_basis, sizeof(double) * nd));
        MWG_CUDA(cudaMemcpy(c->ctx.d_basis, h.data(), sizeof(double) * nd, cudaMemcpyHostToDevice));
        double *d = c->ctx.d_basis;
        c->ctx.dbasis = mwg::DevBasis{K, basis, d, d + K2 * K2, d + 2 * K2 * K2, d + 2 * K2 * K2 + K * K,
                                      d + 2 * K2 * K2 + 2 * K * K, d + 2 * K2 * K2 + 2 * K * K + K,
                                      d + 2 * K2 * K2 + 2 * K * K + 2 * K};
        // tree growth allocates from the device's stream-ordered pool (Tree::reserve); the pool keeps
        // what is returned to it instead of handing it back to the driver at every synchronisation
        cudaMemPool_t pool = nullptr;
        MWG_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
        uint64_t keep = UINT64_MAX;
        MWG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
        // mw_dot_noalloc's fixed device array: its address is taken here, with the device current,
        // so that its module is loaded (and the array reserved) while the caller may still allocate
        mwg::noalloc_setup(device);
    });
    if (rc != MW_OK) {
        if (c->ctx.stream) cudaStreamDestroy(c->ctx.stream);
        delete c;
        return rc;
    }
    c->ctx.owner = c;
    if (const char *e = std::getenv("MW_SCREEN_GEN_SLOTS")) c->ctx.screen_gen_slots = std::max(0L, std::atol(e));
    *out = c;
    return MW_OK;
}

// A context is released only when the caller destroyed it AND no tree or operator of it is
// alive, so handles may be destroyed in any order (e.g. by a garbage collector).
static void ctx_free(mw_ctx c) {
    cudaSetDevice(c->ctx.device);
    c->ctx.release_retired();
    cudaStreamSynchronize(c->ctx.stream);
    for (auto &xs : c->ctx.xstream)
        if (xs) cudaStreamSynchronize(xs);
    if (c->ctx.fast) cudaStreamSynchronize(c->ctx.fast);
    if (c->ctx.ustream) cudaStreamSynchronize(c->ctx.ustream);
    for (auto &ps : c->ctx.pstream)
        if (ps) cudaStreamSynchronize(ps);
    c->ctx.arena.release();
    c->ctx.sarena.release();
    for (auto &xa : c->ctx.xarena) xa.release();
    if (c->ctx.h_pinned) cudaFreeHost(c->ctx.h_pinned);
    if (c->ctx.d_basis) cudaFree(c->ctx.d_basis);
    cudaStreamDestroy(c->ctx.stream);
    for (auto &xs : c->ctx.xstream)
        if (xs) cudaStreamDestroy(xs);
    if (c->ctx.fast) cudaStreamDestroy(c->ctx.fast);
    if (c->ctx.ustream) cudaStreamDestroy(c->ctx.ustream);
    for (auto &ps : c->ctx.pstream)
        if (ps) cudaStreamDestroy(ps);
    if (c->ctx.fast_done) cudaEventDestroy(c->ctx.fast_done);
    delete c;
}

static void ctx_child_gone(mwg::Ctx *ctx) {
    if (--ctx->live == 0 && ctx->closing) ctx_free(static_cast<mw_ctx>(ctx->owner));
}

int mw_ctx_destroy(mw_ctx c) {
    if (!c || c->ctx.closing) return MW_ERR_ARG;
    c->ctx.closing = true;
    if (c->ctx.live == 0) ctx_free(c);
    return MW_OK;
}

const char *mw_last_error(mw_ctx c) { return c ? c->ctx.err.c_str() : g_noctx_err.c_str(); }

int mw_ctx_basis(mw_ctx c, double *qx, double *qw, double *filter, double *c2v, double *v2c) {
    if (!c) return MW_ERR_ARG;
    const mwg::Basis &b = c->ctx.basis;
    int K = b.K;
    if (qx) std::memcpy(qx, b.qx.data(), sizeof(double) * K);
    if (qw) std::memcpy(qw, b.qw.data(), sizeof(double) * K);
    if (filter) std::memcpy(filter, b.W.data(), sizeof(double) * 4 * K * K);
    if (c2v) std::memcpy(c2v, b.c2v.data(), sizeof(double) * K * K);
    if (v2c) std::memcpy(v2c, b.v2c.data(), sizeof(double) * K * K);
    return MW_OK;
}

int mw_ctx_last_stats(mw_ctx c, mw_stats *st) {
    if (!c || !st) return MW_ERR_ARG;
    *st = c->ctx.last;
    return MW_OK;
}

int mw_ctx_synchronize(mw_ctx c) {
    if (!c) return MW_ERR_ARG;
    return guard(&c->ctx, [&] { c->ctx.sync(); });
}

int mw_ctx_set_overlap(mw_ctx c, int on) {
    if (!c || (on != 0 && on != 1)) return MW_ERR_ARG;
    c->ctx.groups = on ? mwg::Ctx::DEFAULT_GROUPS : 1;
    return MW_OK;
}

int mw_ctx_set_groups(mw_ctx c, int n) {
    if (!c || n < 1 || n > mwg::Ctx::XGROUPS + 1) return MW_ERR_ARG;
    c->ctx.groups = n;
    return MW_OK;
}

int mw_ctx_set_screening(mw_ctx c, int on) {
    if (!c || (on != 0 && on != 1)) return MW_ERR_ARG;
    c->ctx.screening = on;
    return MW_OK;
}

// ---------------------------------------------------------------- trees
int mw_tree_create(mw_ctx c, mw_tree *out) {
    if (!c || !out) return MW_ERR_ARG;
    *out = nullptr;
    mw_tree t = new mw_tree_s;
    t->tree.ctx = &c->ctx;
    int rc = guard(&c->ctx, [&] { mwg::tree_clear(t->tree); c->ctx.sync(); });
    if (rc != MW_OK) {
        t->tree.free_device();
        delete t;
        return rc;
    }
    c->ctx.live++;
    *out = t;
    return MW_OK;
}

int mw_tree_destroy(mw_tree t) {
    if (!t) return MW_ERR_ARG;
    mwg::Ctx *ctx = t->tree.ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    t->tree.free_device();
    delete t;
    ctx_child_gone(ctx);
    return MW_OK;
}

int mw_tree_nnodes(mw_tree t, int *n) {
    if (!t || !n) return MW_ERR_ARG;
    *n = t->tree.nn();
    return MW_OK;
}

int mw_tree_nleaves(mw_tree t, int *n) {
    if (!t || !n) return MW_ERR_ARG;
    int c = 0;
    for (auto &nd : t->tree.nodes) c += nd.child0 < 0;
    *n = c;
    return MW_OK;
}

int mw_tree_depth(mw_tree t, int *d) {
    if (!t || !d) return MW_ERR_ARG;
    *d = t->tree.max_scale() - t->tree.ctx->basis.n0 + 1;
    return MW_OK;
}

int mw_tree_upload(mw_tree t, int nnodes, const int *keys, const double *coefs) {
    if (!t || nnodes < 1 || !keys || !coefs) return MW_ERR_ARG;
    return guard(ctx_of(t), [&] { mwg::tree_upload(t->tree, nnodes, keys, coefs, t->tree.ctx->arena); });
}

int mw_tree_download(mw_tree t, int *keys, double *coefs, unsigned char *is_leaf) {
    if (!t) return MW_ERR_ARG;
    return guard(ctx_of(t), [&] { mwg::tree_download(t->tree, keys, coefs, is_leaf); });
}

int mw_tree_upload_batch(int n, mw_tree *trees, const int *nnodes, const int *const *keys,
                         const double *const *coefs) {
    if (n < 1 || !trees || !nnodes || !keys || !coefs) return MW_ERR_ARG;
    for (int i = 0; i < n; i++) {
        if (!trees[i] || nnodes[i] < 1 || !keys[i] || !coefs[i]) return MW_ERR_ARG;
        if (ctx_of(trees[i]) != ctx_of(trees[0])) return MW_ERR_ARG;
        for (int k = 0; k < i; k++)
            if (trees[k] == trees[i]) return MW_ERR_ARG;
    }
    mwg::Ctx *ctx = ctx_of(trees[0]);
    return guard(ctx, [&] {
        std::vector<mwg::Tree *> ts(n);
        for (int i = 0; i < n; i++) ts[i] = &trees[i]->tree;
        mwg::tree_upload_batch(ts, nnodes, keys, coefs, ctx->arena);
    });
}

int mw_tree_download_batch(int n, mw_tree *trees, int *const *keys, double *const *coefs,
                           unsigned char *const *is_leaf) {
    if (n < 1 || !trees || !keys || !coefs || !is_leaf) return MW_ERR_ARG;
    for (int i = 0; i < n; i++)
        if (!trees[i] || ctx_of(trees[i]) != ctx_of(trees[0])) return MW_ERR_ARG;
    mwg::Ctx *ctx = ctx_of(trees[0]);
    return guard(ctx, [&] {
        std::vector<mwg::Tree *> ts(n);
        for (int i = 0; i < n; i++) ts[i] = &trees[i]->tree;
        mwg::tree_download_batch(ts, keys, coefs, is_leaf);
    });
}

int mw_pin_host(mw_ctx c, void *p, size_t bytes) {
    if (!c || !p || bytes == 0) return MW_ERR_ARG;
    return guard(&c->ctx, [&] {
        MWG_CUDA(cudaSetDevice(c->ctx.device));
        MWG_CUDA(cudaHostRegister(p, bytes, cudaHostRegisterDefault));
    });
}

int mw_unpin_host(mw_ctx c, void *p) {
    if (!c || !p) return MW_ERR_ARG;
    return guard(&c->ctx, [&] {
        MWG_CUDA(cudaSetDevice(c->ctx.device));
        MWG_CUDA(cudaHostUnregister(p));
    });
}

int mw_tree_squared_norm(mw_tree t, double *out) {
    if (!t || !out) return MW_ERR_ARG;
    *out = t->tree.sqnorm_leaves();
    return MW_OK;
}

int mw_tree_integrate(mw_tree t, double *out) {
    if (!t || !out) return MW_ERR_ARG;
    return guard(ctx_of(t), [&] { *out = mwg::integrate(t->tree); });
}

int mw_tree_rescale(mw_tree t, double c) {
    if (!t) return MW_ERR_ARG;
    return guard(ctx_of(t), [&] { mwg::rescale(t->tree, c); });
}

int mw_tree_eval(mw_tree t, int npts, const double *xyz, double *out) {
    if (!t || npts < 0 || (npts > 0 && (!xyz || !out))) return MW_ERR_ARG;
    return guard(ctx_of(t), [&] { mwg::eval_points(t->tree, npts, xyz, out, t->tree.ctx->arena); });
}

int mw_tree_clear(mw_tree t) {
    if (!t) return MW_ERR_ARG;
    // the zeroing of the roots is queued on the context's stream, ahead of any later use
    return guard(ctx_of(t), [&] { mwg::tree_clear(t->tree); });
}

int mw_project_gauss(double prec, mw_tree out, int nterms, const mw_gterm *terms, int abs_prec) {
    if (!out || nterms < 1 || !terms || !(prec > 0.0)) return MW_ERR_ARG;
    return guard(ctx_of(out), [&] {
        for (int i = 0; i < nterms; i++)
            if (!(terms[i].alpha > 0.0) || terms[i].pw[0] < 0 || terms[i].pw[1] < 0 || terms[i].pw[2] < 0)
                throw mwg::Error(MW_ERR_ARG, "gaussian term needs alpha > 0 and non-negative powers");
        mwg::project_gauss(prec, out->tree, nterms, terms, abs_prec != 0, out->tree.ctx->arena);
    });
}

int mw_project_hydrogen(double prec, mw_tree out, int n, int l, int m, double Z, const double origin[3], int abs_prec) {
    if (!out || !(prec > 0.0) || !(Z > 0.0)) return MW_ERR_ARG;
    return guard(ctx_of(out),
                 [&] { mwg::project_hydrogen(prec, out->tree, n, l, m, Z, origin, abs_prec != 0, out->tree.ctx->arena); });
}

int mw_copy_grid(mw_tree out, mw_tree inp) {
    if (!out || !inp) return MW_ERR_ARG;
    return guard(ctx_of(out), [&] {
        check_same(out->tree, inp->tree);
        mwg::copy_grid(out->tree, inp->tree);
        out->tree.ctx->sync();
    });
}

int mw_build_grid(mw_tree out, int n, const mw_tree *trees) {
    if (!out || n < 0 || (n > 0 && !trees)) return MW_ERR_ARG;
    return guard(ctx_of(out), [&] {
        std::vector<const mwg::Tree *> v;
        for (int i = 0; i < n; i++) {
            if (!trees[i]) throw mwg::Error(MW_ERR_ARG, "null tree");
            check_same(out->tree, trees[i]->tree);
            v.push_back(&trees[i]->tree);
        }
        mwg::build_grid(out->tree, v);
        out->tree.ctx->sync();
    });
}

int mw_copy_func(mw_tree out, mw_tree inp) {
    if (!out || !inp) return MW_ERR_ARG;
    return guard(ctx_of(out), [&] {
        check_same(out->tree, inp->tree);
        mwg::copy_func(out->tree, inp->tree, out->tree.ctx->arena);
    });
}

int mw_crop(mw_tree t, double prec, int abs_prec) {
    if (!t || !(prec > 0.0)) return MW_ERR_ARG;
    return guard(ctx_of(t), [&] { mwg::crop(t->tree, prec, abs_prec != 0, t->tree.ctx->arena); });
}

int mw_dot(mw_tree a, mw_tree b, double *out) {
    if (!a || !b || !out) return MW_ERR_ARG;
    return guard(ctx_of(a), [&] {
        check_same(a->tree, b->tree);
        *out = mwg::dot(a->tree, b->tree, a->tree.ctx->arena);
    });
}

int mw_dot_noalloc(mw_tree a, mw_tree b, double *out) {
    if (!a || !b || !out) return MW_ERR_ARG;
    return guard(ctx_of(a), [&] {
        check_same(a->tree, b->tree);
        *out = mwg::dot_noalloc(a->tree, b->tree);
    });
}

// ---------------------------------------------------------------- operators
static int op_create(mw_ctx c, int kind, double mu, double prec, mw_op *out) {
    if (!c || !out || !(prec > 0.0) || prec >= 1.0) return MW_ERR_ARG;
    if (kind == 1 && !(mu > 0.0)) {
        c->ctx.err = "Helmholtz operator needs mu > 0";
        return MW_ERR_ARG;
    }
    *out = nullptr;
    mw_op o = new mw_op_s;
    o->op.ctx = &c->ctx;
    o->op.kind = kind;
    o->op.mu = mu;
    o->op.prec = prec;
    int rc = guard(&c->ctx, [&] { o->op.build(c->ctx.basis); });
    if (rc != MW_OK) {
        delete o;
        return rc;
    }
    c->ctx.live++;
    *out = o;
    return MW_OK;
}

int mw_op_create_poisson(mw_ctx c, double prec, mw_op *out) { return op_create(c, 0, 0.0, prec, out); }

int mw_op_create_helmholtz(mw_ctx c, double mu, double prec, mw_op *out) { return op_create(c, 1, mu, prec, out); }

int mw_op_create_helmholtz_batch(mw_ctx c, int n, const double *mu, double prec, mw_op *out) {
    if (!c || n < 1 || !mu || !out || !(prec > 0.0) || prec >= 1.0) return MW_ERR_ARG;
    for (int i = 0; i < n; i++)
        if (!(mu[i] > 0.0)) {
            c->ctx.err = "Helmholtz operator needs mu > 0";
            return MW_ERR_ARG;
        }
    std::vector<mw_op> made(n, nullptr);
    std::vector<mwg::Oper *> ops(n);
    for (int i = 0; i < n; i++) {
        made[i] = new mw_op_s;
        made[i]->op.ctx = &c->ctx;
        made[i]->op.kind = 1;
        made[i]->op.mu = mu[i];
        made[i]->op.prec = prec;
        ops[i] = &made[i]->op;
    }
    int rc = guard(&c->ctx, [&] { mwg::build_operators(ops, c->ctx.basis); });
    if (rc != MW_OK) {
        for (mw_op o : made) {
            o->op.free_device();
            delete o;
        }
        return rc;
    }
    for (int i = 0; i < n; i++) {
        c->ctx.live++;
        out[i] = made[i];
    }
    return MW_OK;
}

int mw_op_destroy(mw_op o) {
    if (!o) return MW_ERR_ARG;
    cudaSetDevice(o->op.ctx->device);
    cudaStreamSynchronize(o->op.ctx->stream);
    o->op.free_device();
    mwg::Ctx *ctx = o->op.ctx;
    delete o;
    ctx_child_gone(ctx);
    return MW_OK;
}

int mw_op_nterms(mw_op o, int *n) {
    if (!o || !n) return MW_ERR_ARG;
    *n = o->op.T;
    return MW_OK;
}

int mw_op_terms(mw_op o, double *coefs, double *exps) {
    if (!o) return MW_ERR_ARG;
    for (int t = 0; t < o->op.T; t++) {
        if (coefs) coefs[t] = o->op.c[t];
        if (exps) exps[t] = o->op.a[t];
    }
    return MW_OK;
}

int mw_op_band(mw_op o, int term, int scale, int *band) {
    if (!o || !band) return MW_ERR_ARG;
    int s = scale - o->op.ctx->basis.n0;
    if (term < 0 || term >= o->op.T || s < 0 || s >= o->op.S) return MW_ERR_ARG;
    *band = o->op.band[term * o->op.S + s];
    return MW_OK;
}

int mw_op_block(mw_op o, int term, int scale, int l, double *blk, double *norms4) {
    if (!o) return MW_ERR_ARG;
    int s = scale - o->op.ctx->basis.n0;
    if (term < 0 || term >= o->op.T || s < 0 || s >= o->op.S) return MW_ERR_ARG;
    int L = o->op.band[term * o->op.S + s];
    if (L < 0 || l < -L || l > L) return MW_ERR_ARG;
    mwg::Ctx *ctx = o->op.ctx;
    return guard(ctx, [&] {
        int K = ctx->basis.K, bsz = 4 * K * K;
        long bi = o->op.block_index(term, s, l);
        if (blk)
            MWG_CUDA(cudaMemcpy(blk, o->op.d_blocks + (size_t)bi * bsz, sizeof(double) * bsz, cudaMemcpyDeviceToHost));
        if (norms4) std::memcpy(norms4, o->op.norm(term, s, l), sizeof(double) * 4);
    });
}

// ---------------------------------------------------------------- hot path
int mw_apply(double prec, mw_tree out, mw_op op, mw_tree inp, int nprec, const mw_tree *prec_trees, int max_iter,
             int abs_prec, int precision_mode) {
    if (!out || !op || !inp || !(prec > 0.0) || nprec < 0 || (nprec > 0 && !prec_trees)) return MW_ERR_ARG;
    if (precision_mode < MW_PREC_FP64 || precision_mode > MW_PREC_DF) return MW_ERR_ARG;
    if (out == inp) return MW_ERR_ARG;
    mwg::Ctx *ctx = ctx_of(out);
    return guard(ctx, [&] {
        std::vector<mwg::ApplyJob> jobs(1);
        jobs[0] = mwg::ApplyJob{&out->tree, &op->op, &inp->tree, prec, abs_prec != 0, max_iter, {}};
        for (int i = 0; i < nprec; i++) {
            if (!prec_trees[i]) throw mwg::Error(MW_ERR_ARG, "null precision tree");
            jobs[0].prec_trees.push_back(&prec_trees[i]->tree);
        }
        mw_stats st{};
        mwg::apply_batch(jobs, precision_mode, false, st);
        ctx->last = st;
    });
}

int mw_apply_batch(int n, const double *precs, mw_tree *outs, mw_op *ops, mw_tree *inps, const int *nprec,
                   const mw_tree *prec_trees, int max_iter, int abs_prec, int precision_mode) {
    if (n < 1 || !precs || !outs || !ops || !inps) return MW_ERR_ARG;
    if (precision_mode < MW_PREC_FP64 || precision_mode > MW_PREC_DF) return MW_ERR_ARG;
    for (int i = 0; i < n; i++)
        if (!outs[i] || !ops[i] || !inps[i] || !(precs[i] > 0.0) || outs[i] == inps[i]) return MW_ERR_ARG;
    mwg::Ctx *ctx = ctx_of(outs[0]);
    return guard(ctx, [&] {
        std::vector<mwg::ApplyJob> jobs(n);
        int off = 0;
        for (int i = 0; i < n; i++) {
            jobs[i] = mwg::ApplyJob{&outs[i]->tree, &ops[i]->op, &inps[i]->tree, precs[i], abs_prec != 0, max_iter, {}};
            int np = nprec ? nprec[i] : 0;
            for (int k = 0; k < np; k++) {
                if (!prec_trees || !prec_trees[off + k]) throw mwg::Error(MW_ERR_ARG, "null precision tree");
                jobs[i].prec_trees.push_back(&prec_trees[off + k]->tree);
            }
            off += np;
        }
        mw_stats st{};
        mwg::apply_batch(jobs, precision_mode, false, st);
        ctx->last = st;
    });
}

int mw_apply_batch_host(int n, const double *precs, mw_tree *outs, mw_op *ops, mw_tree *inps, const int *in_nnodes,
                        const int *const *in_keys, const double *const *in_coefs, int max_iter, int abs_prec,
                        int precision_mode, const int *out_cap, int *const *out_keys, double *const *out_coefs,
                        unsigned char *const *out_leaf, int *out_nnodes) {
    if (out_cap && (!out_keys || !out_coefs || !out_leaf || !out_nnodes)) return MW_ERR_ARG;
    if (n < 1 || !precs || !outs || !ops || !inps || !in_nnodes || !in_keys || !in_coefs) return MW_ERR_ARG;
    if (precision_mode < MW_PREC_FP64 || precision_mode > MW_PREC_DF) return MW_ERR_ARG;
    for (int i = 0; i < n; i++)
        if (!outs[i] || !ops[i] || !inps[i] || !(precs[i] > 0.0) || outs[i] == inps[i] || in_nnodes[i] < 1 ||
            !in_keys[i] || !in_coefs[i])
            return MW_ERR_ARG;
    mwg::Ctx *ctx = ctx_of(outs[0]);
    return guard(ctx, [&] {
        std::vector<mwg::ApplyJob> jobs(n);
        std::vector<mwg::Tree *> itrees(n);
        for (int i = 0; i < n; i++) {
            check_same(outs[i]->tree, inps[i]->tree);
            jobs[i] = mwg::ApplyJob{&outs[i]->tree, &ops[i]->op, &inps[i]->tree, precs[i], abs_prec != 0, max_iter, {}};
            itrees[i] = &inps[i]->tree;
        }
        // the per-group upload needs distinct input trees, not among the outputs, and pinned blocks;
        // otherwise the inputs go up first and the apply follows (the same results)
        bool overlap = true;
        std::vector<mwg::Tree *> sorted = itrees;
        std::sort(sorted.begin(), sorted.end());
        overlap &= std::adjacent_find(sorted.begin(), sorted.end()) == sorted.end();
        for (int i = 0; i < n && overlap; i++) {
            overlap &= !std::binary_search(sorted.begin(), sorted.end(), &outs[i]->tree);
            overlap &= mwg::host_is_pinned(in_coefs[i]);
        }
        // outputs are written where they fit and their coefficient buffer is pinned
        std::vector<double *> oc(n, nullptr);
        if (out_cap)
            for (int i = 0; i < n; i++)
                if (out_coefs[i] && mwg::host_is_pinned(out_coefs[i])) oc[i] = out_coefs[i];
        mw_stats st{};
        if (overlap) {
            mwg::HostInputs hin;
            hin.nnodes.assign(in_nnodes, in_nnodes + n);
            hin.keys.assign(in_keys, in_keys + n);
            hin.coefs.assign(in_coefs, in_coefs + n);
            if (out_cap) {
                hin.out_keys.assign(out_keys, out_keys + n);
                hin.out_coefs = oc;
                hin.out_leaf.assign(out_leaf, out_leaf + n);
                hin.out_cap.assign(out_cap, out_cap + n);
                hin.out_nnodes = out_nnodes;
            }
            mwg::apply_batch(jobs, precision_mode, false, st, &hin);
        } else {
            mwg::tree_upload_batch(itrees, in_nnodes, in_keys, in_coefs, ctx->arena);
            mwg::apply_batch(jobs, precision_mode, false, st);
            if (out_cap) {
                std::vector<mwg::Tree *> ts;
                std::vector<int *> k;
                std::vector<double *> c;
                std::vector<unsigned char *> l;
                for (int i = 0; i < n; i++) {
                    const int m = outs[i]->tree.nn();
                    const bool fits = m <= out_cap[i] && oc[i];
                    out_nnodes[i] = fits ? m : -m;
                    if (!fits) continue;
                    ts.push_back(&outs[i]->tree);
                    k.push_back(out_keys[i]);
                    c.push_back(oc[i]);
                    l.push_back(out_leaf[i]);
                }
                if (!ts.empty()) mwg::tree_download_batch(ts, k.data(), c.data(), l.data());
            }
        }
        ctx->sync();
        ctx->last = st;
    });
}

int mw_apply_batch_autotune(int n, const double *precs, mw_tree *outs, mw_op *ops, mw_tree *inps, int abs_prec,
                            int precision_mode, int repeats, int *groups, long long *chunks, double *ms) {
    if (n < 1 || !precs || !outs || !ops || !inps || repeats < 1 || repeats > 20) return MW_ERR_ARG;
    if (precision_mode < MW_PREC_FP64 || precision_mode > MW_PREC_DF) return MW_ERR_ARG;
    for (int i = 0; i < n; i++)
        if (!outs[i] || !ops[i] || !inps[i] || !(precs[i] > 0.0) || outs[i] == inps[i]) return MW_ERR_ARG;
    mwg::Ctx *ctx = ctx_of(outs[0]);
    return guard(ctx, [&] {
        if (ctx->groups == 1) throw mwg::Error(MW_ERR_STATE, "autotune: job-group overlap is off");
        std::vector<mwg::ApplyJob> jobs(n);
        for (int i = 0; i < n; i++)
            jobs[i] = mwg::ApplyJob{&outs[i]->tree, &ops[i]->op, &inps[i]->tree, precs[i], abs_prec != 0, -1, {}};
        const auto key = std::make_tuple(ctx->basis.K, n, precision_mode);
        mw_stats st{};
        // median wall time of `repeats` complete batched applies with the settings t (each apply
        // ends with the device synchronised and the outputs' norms on the host)
        auto run = [&](const mwg::Ctx::Tuning &t, int reps) {
            ctx->tuned[key] = t;
            std::vector<double> v;
            for (int r = 0; r < reps; r++) {
                for (int i = 0; i < n; i++) mwg::tree_clear(outs[i]->tree);
                ctx->sync();
                const auto t0 = std::chrono::steady_clock::now();
                st = mw_stats{};
                mwg::apply_batch(jobs, precision_mode, false, st);
                v.push_back(std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
            }
            std::sort(v.begin(), v.end());
            return v[v.size() / 2];
        };
        mwg::Ctx::Tuning best;
        best.groups = ctx->groups;
        run(best, 1);  // warm-up: allocations, arenas, shadows
        double bt = run(best, repeats);
        // coordinate search: the job-group count, then each tier's chunk size.  A candidate replaces
        // the settings kept only when it is faster by more than the run-to-run noise (2%).
        const double margin = 0.98;
        for (int g : {2, 3, 4, 5, 6}) {
            mwg::Ctx::Tuning t = best;
            t.groups = g;
            const double x = run(t, repeats);
            if (x < margin * bt) bt = x, best = t;
        }
        const long long cand[4][3] = {{4, 4, 4}, {16, 32, 64}, {48, 96, 192}, {4, 8, 16}};
        for (int tier : {2, 1, 3})
            for (long long c : cand[tier]) {
                mwg::Ctx::Tuning t = best;
                t.chunk[tier] = c;
                const double x = run(t, repeats);
                if (x < margin * bt) bt = x, best = t;
            }
        run(best, 1);  // the outputs, from the settings kept
        ctx->tuned[key] = best;
        ctx->last = st;
        if (groups) *groups = best.groups;
        if (chunks)
            for (int k = 0; k < 4; k++) chunks[k] = best.chunk[k];
        if (ms) *ms = bt;
    });
}

int mw_apply_fixed(double prec, mw_tree out, mw_op op, mw_tree inp, int abs_prec, int precision_mode) {
    if (!out || !op || !inp || !(prec > 0.0) || out == inp) return MW_ERR_ARG;
    if (precision_mode < MW_PREC_FP64 || precision_mode > MW_PREC_DF) return MW_ERR_ARG;
    mwg::Ctx *ctx = ctx_of(out);
    return guard(ctx, [&] {
        std::vector<mwg::ApplyJob> jobs(1);
        jobs[0] = mwg::ApplyJob{&out->tree, &op->op, &inp->tree, prec, abs_prec != 0, 0, {}};
        mw_stats st{};
        mwg::apply_batch(jobs, precision_mode, true, st);
        ctx->last = st;
    });
}

int mw_apply_adjoint(double prec, mw_tree out, mw_op op, mw_tree x, mw_tree seed, int abs_prec) {
    if (!out || !op || !x || !seed || !(prec > 0.0) || out == x || out == seed) return MW_ERR_ARG;
    mwg::Ctx *ctx = ctx_of(out);
    if (!abs_prec) {
        ctx->err = "mw_apply_adjoint: absolute precision only (the relative threshold depends on the forward output)";
        return MW_ERR_ARG;
    }
    return guard(ctx, [&] {
        check_same(out->tree, x->tree);
        check_same(out->tree, seed->tree);
        mw_stats st{};
        mwg::apply_adjoint(prec, out->tree, op->op, x->tree, seed->tree, st);
        ctx->last = st;
    });
}

int mw_multiply_adjoint(double prec, mw_tree out, double coef, mw_tree a, mw_tree b, mw_tree seed) {
    if (!out || !a || !b || !seed || !(prec > 0.0) || out == a || out == b || out == seed) return MW_ERR_ARG;
    mwg::Ctx *ctx = ctx_of(out);
    return guard(ctx, [&] {
        check_same(out->tree, a->tree);
        check_same(out->tree, b->tree);
        check_same(out->tree, seed->tree);
        mw_stats st{};
        mwg::multiply_adjoint(prec, out->tree, coef, a->tree, b->tree, seed->tree, st);
        ctx->last = st;
    });
}

int mw_multiply(double prec, mw_tree out, double coef, mw_tree a, mw_tree b, int max_iter, int abs_prec,
                int use_max_norms) {
    return mw_multiply_batch(1, &prec, &out, &coef, &a, &b, max_iter, abs_prec, use_max_norms);
}

int mw_multiply_batch(int n, const double *precs, mw_tree *outs, const double *coefs, mw_tree *as, mw_tree *bs,
                      int max_iter, int abs_prec, int use_max_norms) {
    if (n < 1 || !precs || !outs || !coefs || !as || !bs) return MW_ERR_ARG;
    for (int i = 0; i < n; i++)
        if (!outs[i] || !as[i] || !bs[i] || !(precs[i] > 0.0) || outs[i] == as[i] || outs[i] == bs[i])
            return MW_ERR_ARG;
    mwg::Ctx *ctx = ctx_of(outs[0]);
    return guard(ctx, [&] {
        std::vector<mwg::MulJob> jobs(n);
        for (int i = 0; i < n; i++) {
            check_same(outs[i]->tree, as[i]->tree);
            check_same(outs[i]->tree, bs[i]->tree);
            jobs[i] = mwg::MulJob{&outs[i]->tree, &as[i]->tree, &bs[i]->tree, coefs[i], precs[i], max_iter,
                                  abs_prec != 0, use_max_norms != 0};
        }
        mw_stats st{};
        mwg::multiply_batch(jobs, st);
        ctx->last = st;
    });
}

int mw_square(double prec, mw_tree out, mw_tree inp, int max_iter, int abs_prec) {
    return mw_multiply(prec, out, 1.0, inp, inp, max_iter, abs_prec, 0);
}

int mw_add(double prec, mw_tree out, int n, const double *coefs, const mw_tree *trees, int max_iter) {
    (void)prec;
    (void)max_iter;
    if (!out || n < 1 || !coefs || !trees) return MW_ERR_ARG;
    mwg::Ctx *ctx = ctx_of(out);
    return guard(ctx, [&] {
        std::vector<const mwg::Tree *> v;
        std::vector<double> c(coefs, coefs + n);
        for (int i = 0; i < n; i++) {
            if (!trees[i] || trees[i] == out) throw mwg::Error(MW_ERR_ARG, "add: null tree or output among inputs");
            check_same(out->tree, trees[i]->tree);
            v.push_back(&trees[i]->tree);
        }
        mw_stats st{};
        mwg::add(out->tree, v, c, st);
        ctx->last = st;
    });
}

int mw_density(double prec, mw_tree rho, int n, const mw_tree *orbitals, const double *occ, int crop) {
    if (!rho || n < 1 || !orbitals || !occ || !(prec > 0.0)) return MW_ERR_ARG;
    mwg::Ctx *ctx = ctx_of(rho);
    return guard(ctx, [&] {
        std::vector<mwg::Tree *> v;
        for (int i = 0; i < n; i++) {
            if (!orbitals[i] || orbitals[i] == rho) throw mwg::Error(MW_ERR_ARG, "density: null orbital or output");
            check_same(rho->tree, orbitals[i]->tree);
            v.push_back(&orbitals[i]->tree);
        }
        mw_stats st{};
        mwg::density(prec, rho->tree, v, std::vector<double>(occ, occ + n), crop != 0, st);
        ctx->last = st;
    });
}

int mw_rotate(int nout, mw_tree *outs, int nin, const mw_tree *ins, const double *U) {
    if (nout < 1 || nin < 1 || !outs || !ins || !U) return MW_ERR_ARG;
    mwg::Ctx *ctx = ctx_of(outs[0]);
    return guard(ctx, [&] {
        std::vector<mwg::Tree *> o;
        std::vector<const mwg::Tree *> in;
        for (int i = 0; i < nout; i++) {
            if (!outs[i]) throw mwg::Error(MW_ERR_ARG, "rotate: null output");
            o.push_back(&outs[i]->tree);
        }
        for (int j = 0; j < nin; j++) {
            if (!ins[j]) throw mwg::Error(MW_ERR_ARG, "rotate: null input");
            for (int i = 0; i < nout; i++)
                if (ins[j] == outs[i]) throw mwg::Error(MW_ERR_ARG, "rotate: an output is also an input");
            check_same(outs[0]->tree, ins[j]->tree);
            in.push_back(&ins[j]->tree);
        }
        mw_stats st{};
        mwg::rotate(o, in, U, st);
        ctx->last = st;
    });
}

int mw_tree_save(mw_tree t, const char *path) {
    if (!t || !path) return MW_ERR_ARG;
    return guard(ctx_of(t), [&] { mwg::tree_save(t->tree, path); });
}

int mw_tree_load(mw_tree t, const char *path) {
    if (!t || !path) return MW_ERR_ARG;
    return guard(ctx_of(t), [&] { mwg::tree_load(t->tree, path); });
}

int mw_probe_mma_peak(mw_ctx c, int kind, double *tflops) {
    if (!c || !tflops || kind < 0 || kind > 3) return MW_ERR_ARG;
    return guard(&c->ctx, [&] { *tflops = mwg::probe_mma_tflops(kind, c->ctx.nsm, c->ctx.stream); });
}

int mw_probe_fma_peak(mw_ctx c, int fp64, double *tflops) {
    if (!c || !tflops) return MW_ERR_ARG;
    return guard(&c->ctx, [&] { *tflops = mwg::probe_fma_tflops(fp64, c->ctx.nsm, c->ctx.stream); });
}

}  // extern "C"
