/*
 * mw_arith.c -- oracle: tree multiply / square / add / crop.
 *
 * TEST INFRASTRUCTURE ONLY (see mworacle.h).
 *
 * multiply restates mrcpp::multiply(prec, out, coef, a, b, maxIter, absPrec,
 * useMaxNorms) (src/qmoperators/QMPotential.cpp:147,157;
 * src/qmoperators/two_electron/ExchangePotential.cpp:175,213,223; the real /
 * imaginary decomposition is documented in the unused
 * src/qmfunctions/qmfunction_utils.cpp:232-300): on every end node of the
 * output grid, both inputs are brought to the node (generated from a leaf
 * ancestor where missing), reconstructed to the children's scaling parts,
 * mapped to values at the children's Gauss-Legendre points, multiplied, mapped
 * back and compressed.  The grid is refined while the product's wavelet norm
 * (or, with useMaxNorms, the inputs' unresolved detail times the other input's
 * RMS value) exceeds prec * R * 2^{-(n+1)/2}.
 *
 * add restates mrcpp::add(prec, out, FunctionTreeVector, maxIter) on the
 * union grid (src/qmfunctions/density_utils.cpp:85-86,146-147): every union
 * node's block is the linear combination of the inputs' blocks at that node.
 */
#include "mw_internal.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* tail^2(node) = sum over children of (|wavelet part|^2 + tail^2) */
static void tree_tails(orc_tree *t) {
    int maxn = t->mra->n0;
    for (int i = 0; i < t->nn; i++) {
        t->nodes[i].aux = 0.0;
        if (t->nodes[i].n > maxn) maxn = t->nodes[i].n;
    }
    for (int n = maxn - 1; n >= t->mra->n0; n--)
        for (int i = 0; i < t->nn; i++) {
            orc_node *nd = &t->nodes[i];
            if (nd->n != n || nd->child0 < 0) continue;
            double s = 0.0;
            for (int c = 0; c < 8; c++) {
                const orc_node *ch = &t->nodes[nd->child0 + c];
                double w = orc_wavelet_norm(ch->cn);
                s += w * w + ch->aux * ch->aux;
            }
            nd->aux = sqrt(s);
        }
}

static double node_tail(const orc_tree *t, int n, const int l[3]) {
    int i = orc_hmap_get(&t->map, n, l);
    if (i < 0) return 0.0;
    return t->nodes[i].aux;
}

void orc_product_block(const orc_mra *m, double coef, int n, const double *ba, const double *bb, double *out,
                       double *work) {
    int bs = m->bs;
    double *ca = work, *cb = work + bs, *va = work + 2 * bs, *vb = work + 3 * bs;
    orc_reconstruct(m, ba, ca);
    orc_reconstruct(m, bb, cb);
    orc_map_children(m, m->c2v, ca, va);
    orc_map_children(m, m->c2v, cb, vb);
    double sc = coef * pow(2.0, 1.5 * (n + 1));
    for (int i = 0; i < bs; i++) va[i] *= vb[i] * sc;
    orc_map_children(m, m->v2c, va, ca);
    orc_compress(m, ca, out);
}

int orc_multiply(double prec, orc_tree *out, double coef, orc_tree *a, orc_tree *b, int max_iter, int abs_prec,
                 int use_max_norms) {
    const orc_mra *m = out->mra;
    if (a->mra != m || b->mra != m) return -1;
    int bs = m->bs;
    int maxn = m->n0 + m->max_depth - 1;
    if (use_max_norms) {
        tree_tails(a);
        tree_tails(b);
    }
    int nwork = 0;
    int *work = (int *)malloc(sizeof(int) * out->nn);
    for (int i = 0; i < out->nn; i++)
        if (out->nodes[i].child0 < 0) work[nwork++] = i;
    int iter = 0;
    double *crit = NULL;
    while (nwork > 0) {
        crit = (double *)realloc(crit, sizeof(double) * nwork);
#pragma omp parallel
        {
            double *wk = (double *)malloc(sizeof(double) * 6 * bs);
#pragma omp for schedule(dynamic, 4)
            for (int w = 0; w < nwork; w++) {
                orc_node *o = &out->nodes[work[w]];
                double *ga = wk + 4 * bs, *gb = wk + 5 * bs;
                int ia = orc_tree_block(a, o->n, o->l, ga, NULL);
                int ib = orc_tree_block(b, o->n, o->l, gb, NULL);
                const double *pa = ia >= 0 ? &a->coefs[(size_t)ia * bs] : ga;
                const double *pb = ib >= 0 ? &b->coefs[(size_t)ib * bs] : gb;
                double cna[8], cnb[8];
                orc_comp_norms(m, pa, cna);
                orc_comp_norms(m, pb, cnb);
                double mna = orc_block_norm(cna) * pow(2.0, 1.5 * o->n);
                double mnb = orc_block_norm(cnb) * pow(2.0, 1.5 * o->n);
                crit[w] = use_max_norms ? (node_tail(a, o->n, o->l) * mnb + node_tail(b, o->n, o->l) * mna) : 0.0;
                orc_product_block(m, coef, o->n, pa, pb, &out->coefs[(size_t)work[w] * bs], wk);
                orc_comp_norms(m, &out->coefs[(size_t)work[w] * bs], o->cn);
            }
            free(wk);
        }
        double R = abs_prec ? 1.0 : orc_tree_norm(out);
        int *next = NULL, nnext = 0;
        if (max_iter < 0 || iter < max_iter) {
            for (int w = 0; w < nwork; w++) {
                int i = work[w];
                int n = out->nodes[i].n;
                if (n >= maxn) continue;
                double thr = orc_split_thr(prec, R, n);
                if (orc_wavelet_norm(out->nodes[i].cn) > thr || crit[w] > thr) {
                    int c0 = orc_tree_split(out, i);
                    next = (int *)realloc(next, sizeof(int) * (nnext + 8));
                    for (int c = 0; c < 8; c++) next[nnext++] = c0 + c;
                }
            }
        }
        free(work);
        work = next;
        nwork = nnext;
        iter++;
    }
    free(work);
    free(crit);
    orc_tree_compress(out);
    return 0;
}

int orc_add(double prec, orc_tree *out, int n, const double *coefs, orc_tree *const *trees, int max_iter) {
    (void)prec;
    (void)max_iter;
    const orc_mra *m = out->mra;
    int bs = m->bs;
    orc_build_grid(out, n, trees);
#pragma omp parallel
    {
        double *g = (double *)malloc(sizeof(double) * bs);
#pragma omp for schedule(dynamic, 16)
        for (int i = 0; i < out->nn; i++) {
            orc_node *o = &out->nodes[i];
            double *ob = &out->coefs[(size_t)i * bs];
            memset(ob, 0, sizeof(double) * bs);
            for (int k = 0; k < n; k++) {
                int j = orc_tree_block(trees[k], o->n, o->l, g, NULL);
                const double *src = j >= 0 ? &trees[k]->coefs[(size_t)j * bs] : g;
                for (int q = 0; q < bs; q++) ob[q] += coefs[k] * src[q];
            }
            orc_comp_norms(m, ob, o->cn);
        }
        free(g);
    }
    return 0;
}

/* remove the children of nodes whose children are all leaves and carry a combined
 * wavelet norm below prec * R * 2^{-(n+2)/2}; repeated from fine to coarse */
void orc_crop(orc_tree *t, double prec, int abs_prec) {
    const orc_mra *m = t->mra;
    double R = abs_prec ? 1.0 : orc_tree_norm(t);
    unsigned char *dead = (unsigned char *)calloc(t->nn, 1);
    int maxn = m->n0;
    for (int i = 0; i < t->nn; i++)
        if (t->nodes[i].n > maxn) maxn = t->nodes[i].n;
    /* leaf status that evolves as children are removed */
    unsigned char *leaf = (unsigned char *)malloc(t->nn);
    for (int i = 0; i < t->nn; i++) leaf[i] = t->nodes[i].child0 < 0;
    for (int n = maxn - 1; n >= m->n0; n--)
        for (int i = 0; i < t->nn; i++) {
            orc_node *nd = &t->nodes[i];
            if (nd->n != n || leaf[i]) continue;
            int all = 1;
            double s = 0.0;
            for (int c = 0; c < 8; c++) {
                int ci = nd->child0 + c;
                if (!leaf[ci]) all = 0;
                double w = orc_wavelet_norm(t->nodes[ci].cn);
                s += w * w;
            }
            if (all && sqrt(s) < orc_split_thr(prec, R, n + 1)) {
                for (int c = 0; c < 8; c++) dead[nd->child0 + c] = 1;
                leaf[i] = 1;
            }
        }
    int keep = 0;
    for (int i = 0; i < t->nn; i++) keep += !dead[i];
    if (keep < t->nn) {
        int *keys = (int *)malloc(sizeof(int) * 4 * keep);
        double *co = (double *)malloc(sizeof(double) * (size_t)keep * m->bs);
        int j = 0;
        for (int i = 0; i < t->nn; i++) {
            if (dead[i]) continue;
            keys[4 * j] = t->nodes[i].n;
            memcpy(&keys[4 * j + 1], t->nodes[i].l, sizeof(int) * 3);
            memcpy(&co[(size_t)j * m->bs], &t->coefs[(size_t)i * m->bs], sizeof(double) * m->bs);
            j++;
        }
        orc_tree *nt = orc_tree_import(m, keep, keys, co);
        free(keys);
        free(co);
        if (nt) {
            orc_tree tmp = *t;
            *t = *nt;
            *nt = tmp;
            orc_tree_free(nt);
        }
    }
    free(dead);
    free(leaf);
}
