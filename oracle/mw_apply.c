/*
 * mw_apply.c -- oracle: adaptive non-standard-form convolution apply.
 *
 * TEST INFRASTRUCTURE ONLY (see mworacle.h).
 *
 * Restates mrcpp::apply(prec, out, oper, inp[, precTrees], maxIter, absPrec)
 * as called at src/qmoperators/two_electron/CoulombPotential.cpp:131,156,
 * src/scf_solver/HelmholtzVector.cpp:149,154 and
 * src/qmoperators/two_electron/ExchangePotential.cpp:200,204, following the
 * published algorithm (Frediani et al., Mol. Phys. 111 (2013) 1143):
 *
 *  1. The output grid starts at the root nodes and is refined one scale per
 *     iteration (host-side decisions), until no node is split or maxIter
 *     iterations ran.
 *  2. Output node o at scale n receives, for every term t active at n and
 *     every input node i at scale n with |l_o - l_i|_inf <= band(t, n)
 *     (missing input nodes are generated from their leaf ancestor):
 *        out[gt] += c_t (A_z (x) A_y (x) A_x) in[ft]   for all (ft, gt),
 *     except (0,0) below the root scale, with A_d the (g_d, f_d) sub-block of
 *     the 1-D NS block of term t at translation l_d.
 *  3. Screening: an item (o, i, t) is skipped when its bound
 *        b = sum_{(ft,gt)} |in_ft| prod_d |A_d^{g_d f_d}|_F
 *     is below ORC_SCREEN_FAC * thr(o); no screening at the root scale.
 *  4. Split o when |wavelet part of o| * w(o) > thr(o), where
 *     thr = prec * R * 2^{-(n+1)/2}, R = 1 (absolute) or the norm of the
 *     root-scale output blocks (relative), and w(o) = 1, or the summed
 *     RMS values of the precision-steering trees on o's box.
 *  5. Post-processing: top-down the parent's (s,d) is reconstructed into the
 *     children's scaling parts (sum over scales), then bottom-up compression.
 */
#include "mw_internal.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int t;
    int l[3];   /* l_o - l_i */
    int src;    /* input node index, or generated slot */
    int gen;    /* 1 if src is a generated slot */
} item;

typedef struct {
    item *v;
    int n, cap;
} itemvec;

static void iv_push(itemvec *iv, item it) {
    if (iv->n == iv->cap) {
        iv->cap = iv->cap ? 2 * iv->cap : 64;
        iv->v = (item *)realloc(iv->v, sizeof(item) * iv->cap);
    }
    iv->v[iv->n++] = it;
}

static const double *op_norm(const orc_oper *op, int t, int s, int l) {
    int L = op->band[t * op->nscales + s];
    return &op->norms[(size_t)(op->off[t * op->nscales + s] + l + L) * 4];
}

static const double *op_block(const orc_oper *op, int t, int s, int l) {
    int L = op->band[t * op->nscales + s];
    int K = op->mra->K;
    return &op->blocks[(size_t)(op->off[t * op->nscales + s] + l + L) * 4 * K * K];
}

/* contribution bound of one item; fixed summation order */
double orc_item_bound(const double *nx, const double *ny, const double *nz, const double *cn, int root) {
    double b = 0.0;
    for (int ft = 0; ft < 8; ft++) {
        if (cn[ft] == 0.0) continue;
        int fx = ft & 1, fy = (ft >> 1) & 1, fz = (ft >> 2) & 1;
        double s = 0.0;
        for (int gt = 0; gt < 8; gt++) {
            if (!root && ft == 0 && gt == 0) continue;
            int gx = gt & 1, gy = (gt >> 1) & 1, gz = (gt >> 2) & 1;
            s += nx[2 * gx + fx] * ny[2 * gy + fy] * nz[2 * gz + fz];
        }
        b += cn[ft] * s;
    }
    return b;
}

/* out += c (Az (x) Ay (x) Ax) in, all K^3, A row-major K x K with row stride lda */
static void contract3(int K, double c, const double *Ax, const double *Ay, const double *Az, int lda, const double *in,
                      double *out, double *t1, double *t2) {
    int KK = K * K;
    for (int z = 0; z < K; z++)
        for (int y = 0; y < K; y++)
            for (int x = 0; x < K; x++) {
                double v = 0.0;
                for (int i = 0; i < K; i++) v += Ax[x * lda + i] * in[z * KK + y * K + i];
                t1[z * KK + y * K + x] = v;
            }
    for (int z = 0; z < K; z++)
        for (int y = 0; y < K; y++)
            for (int x = 0; x < K; x++) {
                double v = 0.0;
                for (int i = 0; i < K; i++) v += Ay[y * lda + i] * t1[z * KK + i * K + x];
                t2[z * KK + y * K + x] = v;
            }
    for (int z = 0; z < K; z++)
        for (int y = 0; y < K; y++)
            for (int x = 0; x < K; x++) {
                double v = 0.0;
                for (int i = 0; i < K; i++) v += Az[z * lda + i] * t2[i * KK + y * K + x];
                out[z * KK + y * K + x] += c * v;
            }
}

/* RMS-value weight of the precision-steering trees on box (n,l) */
static double prec_weight(int np, orc_tree *const *pt, int n, const int l[3]) {
    double w = 0.0;
    for (int p = 0; p < np; p++) {
        const orc_tree *t = pt[p];
        int idx = orc_hmap_get(&t->map, n, l);
        int an = n, al[3] = {l[0], l[1], l[2]};
        while (idx < 0) {
            an--;
            if (an < t->mra->n0) break;
            for (int d = 0; d < 3; d++) al[d] = orc_floordiv2(al[d]);
            idx = orc_hmap_get(&t->map, an, al);
        }
        if (idx < 0) continue;
        w += orc_block_norm(t->nodes[idx].cn) * pow(2.0, 1.5 * an);
    }
    return w;
}

int orc_apply(double prec, orc_tree *out, const orc_oper *op, orc_tree *inp, int max_iter, int abs_prec,
              int nprec_trees, orc_tree *const *prec_trees, orc_stats *stats) {
    const orc_mra *m = out->mra;
    if (inp->mra != m || op->mra != m) return -1;
    int K = m->K, K3 = K * K * K, bs = m->bs, K2 = 2 * K;
    int maxn = m->n0 + m->max_depth - 1;
#ifdef _OPENMP
    double t_start = omp_get_wtime();
#endif
    orc_clear(out);
    orc_stats st;
    memset(&st, 0, sizeof(st));

    /* largest input block norm (bounds generated blocks too) */
    double fmax = 0.0;
    for (int i = 0; i < inp->nn; i++) {
        double b = orc_block_norm(inp->nodes[i].cn);
        if (b > fmax) fmax = b;
    }
    /* per (t, s): max over l of all / non-ss sub-block norms */
    int T = op->T, S = op->nscales;
    double *amax = (double *)calloc((size_t)T * S, sizeof(double));
    double *xmax = (double *)calloc((size_t)T * S, sizeof(double));
    for (int t = 0; t < T; t++)
        for (int s = 0; s < S; s++) {
            int L = op->band[t * S + s];
            for (int l = -L; l <= L && L >= 0; l++) {
                const double *nr = op_norm(op, t, s, l);
                for (int q = 0; q < 4; q++) {
                    if (nr[q] > amax[t * S + s]) amax[t * S + s] = nr[q];
                    if (q > 0 && nr[q] > xmax[t * S + s]) xmax[t * S + s] = nr[q];
                }
            }
        }

    double R = 1.0;
    int nwork = out->nn;
    int *work = (int *)malloc(sizeof(int) * nwork);
    for (int i = 0; i < nwork; i++) work[i] = i;
    int iter = 0;
    while (nwork > 0) {
        int n = out->nodes[work[0]].n, s = n - m->n0;
        int root = (n == m->n0);
        double thr_split = orc_split_thr(prec, R, n);
        double thr_screen = ORC_SCREEN_FAC * thr_split;
        double *wgt = (double *)malloc(sizeof(double) * nwork);
        for (int w = 0; w < nwork; w++)
            wgt[w] = nprec_trees > 0 ? prec_weight(nprec_trees, prec_trees, n, out->nodes[work[w]].l) : 1.0;

        /* phase A: candidate items (bounds use ancestor norms for missing inputs) */
        itemvec *cand = (itemvec *)calloc(nwork, sizeof(itemvec));
        orc_hmap genmap;
        orc_hmap_init(&genmap, 1024);
        int ngen = 0, gcap = 0;
        int *genkeys = NULL;
#pragma omp parallel for schedule(dynamic, 1)
        for (int w = 0; w < nwork; w++) {
            const orc_node *o = &out->nodes[work[w]];
            if (!root && wgt[w] <= 0.0) continue;
            double thr = root ? 0.0 : thr_screen / wgt[w];
            for (int t = 0; t < T; t++) {
                int L = op->band[t * S + s];
                if (L < 0) continue;
                double A = amax[t * S + s], X = xmax[t * S + s];
                if (!root && 8.0 * 2.8285 * fmax * 3.0 * X * A * A < thr) continue;
                for (int lz = -L; lz <= L; lz++) {
                    const double *nz = op_norm(op, t, s, lz);
                    double az = fmax2(fmax2(nz[0], nz[1]), fmax2(nz[2], nz[3]));
                    double xz = fmax2(nz[1], fmax2(nz[2], nz[3]));
                    if (!root && 8.0 * 2.8285 * fmax * (xz * A * A + 2.0 * az * X * A) < thr) continue;
                    for (int ly = -L; ly <= L; ly++) {
                        const double *ny = op_norm(op, t, s, ly);
                        double ay = fmax2(fmax2(ny[0], ny[1]), fmax2(ny[2], ny[3]));
                        double xy = fmax2(ny[1], fmax2(ny[2], ny[3]));
                        if (!root && 8.0 * 2.8285 * fmax * (xz * ay * A + az * xy * A + az * ay * X) < thr) continue;
                        for (int lx = -L; lx <= L; lx++) {
                            int p[3] = {o->l[0] - lx, o->l[1] - ly, o->l[2] - lz};
                            if (!orc_in_world(m, n, p)) continue;
                            const double *nx = op_norm(op, t, s, lx);
                            int idx = orc_hmap_get(&inp->map, n, p);
                            double cn[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                            if (idx >= 0) {
                                memcpy(cn, inp->nodes[idx].cn, sizeof(cn));
                            } else {
                                int an = n, al[3] = {p[0], p[1], p[2]}, a = -1;
                                while (a < 0) {
                                    an--;
                                    for (int d = 0; d < 3; d++) al[d] = orc_floordiv2(al[d]);
                                    a = orc_hmap_get(&inp->map, an, al);
                                }
                                cn[0] = orc_block_norm(inp->nodes[a].cn);
                            }
                            double b = orc_item_bound(nx, ny, nz, cn, root);
                            if (!root && b < thr) continue;
                            item it = {t, {lx, ly, lz}, idx, idx < 0};
                            iv_push(&cand[w], it);
                        }
                    }
                }
            }
        }
        /* phase B: generated input nodes (serial dedupe, parallel generation) */
        for (int w = 0; w < nwork; w++) {
            const orc_node *o = &out->nodes[work[w]];
            for (int k = 0; k < cand[w].n; k++) {
                item *it = &cand[w].v[k];
                if (!it->gen) continue;
                int p[3] = {o->l[0] - it->l[0], o->l[1] - it->l[1], o->l[2] - it->l[2]};
                int g = orc_hmap_get(&genmap, n, p);
                if (g < 0) {
                    g = ngen++;
                    if (ngen > gcap) {
                        gcap = gcap ? 2 * gcap : 1024;
                        genkeys = (int *)realloc(genkeys, sizeof(int) * 3 * gcap);
                    }
                    memcpy(&genkeys[3 * g], p, sizeof(p));
                    orc_hmap_put(&genmap, n, p, g);
                }
                it->src = g;
            }
        }
        double *gblk = (double *)malloc(sizeof(double) * (size_t)(ngen > 0 ? ngen : 1) * bs);
        double *gcn = (double *)malloc(sizeof(double) * 8 * (ngen > 0 ? ngen : 1));
#pragma omp parallel for schedule(dynamic, 4)
        for (int g = 0; g < ngen; g++) {
            orc_tree_block(inp, n, &genkeys[3 * g], &gblk[(size_t)g * bs], NULL);
            orc_comp_norms(m, &gblk[(size_t)g * bs], &gcn[8 * g]);
        }
        st.generated += ngen;

        /* phase C: exact screening and contraction */
        long long items = 0, pairs = 0;
#pragma omp parallel reduction(+ : items, pairs)
        {
            double *t1 = (double *)malloc(sizeof(double) * K3), *t2 = (double *)malloc(sizeof(double) * K3);
#pragma omp for schedule(dynamic, 1)
            for (int w = 0; w < nwork; w++) {
                double *ob = &out->coefs[(size_t)work[w] * bs];
                memset(ob, 0, sizeof(double) * bs);
                double thr = root ? 0.0 : thr_screen / wgt[w];
                for (int k = 0; k < cand[w].n; k++) {
                    const item *it = &cand[w].v[k];
                    const double *cn = it->gen ? &gcn[8 * it->src] : inp->nodes[it->src].cn;
                    const double *in = it->gen ? &gblk[(size_t)it->src * bs] : &inp->coefs[(size_t)it->src * bs];
                    const double *nx = op_norm(op, it->t, s, it->l[0]);
                    const double *ny = op_norm(op, it->t, s, it->l[1]);
                    const double *nz = op_norm(op, it->t, s, it->l[2]);
                    if (it->gen && !root && orc_item_bound(nx, ny, nz, cn, root) < thr) continue;
                    items++;
                    if (!root) {
                        double r = orc_item_bound(nx, ny, nz, cn, root) / thr;
                        int bin = r >= 1.0 ? (int)floor(log10(r)) : 0;
                        if (bin > 15) bin = 15;
                        int near = abs(it->l[0]) <= 1 && abs(it->l[1]) <= 1 && abs(it->l[2]) <= 1;
#pragma omp atomic
                        st.bound_hist[bin]++;
                        if (near) {
#pragma omp atomic
                            st.bound_hist[16 + bin]++;
                        }
                    }
                    const double *bx = op_block(op, it->t, s, it->l[0]);
                    const double *by = op_block(op, it->t, s, it->l[1]);
                    const double *bz = op_block(op, it->t, s, it->l[2]);
                    double c = op->c[it->t];
                    for (int ft = 0; ft < 8; ft++) {
                        if (cn[ft] == 0.0) continue;
                        int fx = ft & 1, fy = (ft >> 1) & 1, fz = (ft >> 2) & 1;
                        for (int gt = 0; gt < 8; gt++) {
                            if (!root && ft == 0 && gt == 0) continue;
                            int gx = gt & 1, gy = (gt >> 1) & 1, gz = (gt >> 2) & 1;
                            if (nx[2 * gx + fx] == 0.0 || ny[2 * gy + fy] == 0.0 || nz[2 * gz + fz] == 0.0) continue;
                            pairs++;
                            contract3(K, c, &bx[gx * K * K2 + fx * K], &by[gy * K * K2 + fy * K],
                                      &bz[gz * K * K2 + fz * K], K2, &in[ft * K3], &ob[gt * K3], t1, t2);
                        }
                    }
                }
                orc_comp_norms(m, ob, out->nodes[work[w]].cn);
            }
            free(t1);
            free(t2);
        }
        st.items += items;
        st.pairs += pairs;
        st.out_nodes += nwork;
        for (int w = 0; w < nwork; w++) free(cand[w].v);
        free(cand);
        free(gblk);
        free(gcn);
        free(genkeys);
        orc_hmap_free(&genmap);

        if (root && !abs_prec) {
            double r2 = 0.0;
            for (int w = 0; w < nwork; w++) {
                double b = orc_block_norm(out->nodes[work[w]].cn);
                r2 += b * b;
            }
            R = sqrt(r2);
            if (R <= 0.0) R = 1.0;
            thr_split = orc_split_thr(prec, R, n);
        }
        /* split decisions */
        int *next = NULL, nnext = 0;
        if ((max_iter < 0 || iter < max_iter) && n < maxn) {
            for (int w = 0; w < nwork; w++) {
                int i = work[w];
                double wn = orc_wavelet_norm(out->nodes[i].cn) * wgt[w];
                if (wn > thr_split) {
                    int c0 = orc_tree_split(out, i);
                    next = (int *)realloc(next, sizeof(int) * (nnext + 8));
                    for (int c = 0; c < 8; c++) next[nnext++] = c0 + c;
                }
            }
        }
        free(wgt);
        free(work);
        work = next;
        nwork = nnext;
        iter++;
    }
    free(work);
    free(amax);
    free(xmax);

    /* post-processing: top-down sum over scales, bottom-up compression */
    int maxs = m->n0;
    for (int i = 0; i < out->nn; i++)
        if (out->nodes[i].n > maxs) maxs = out->nodes[i].n;
    for (int n = m->n0; n < maxs; n++) {
#pragma omp parallel
        {
            double *ch = (double *)malloc(sizeof(double) * bs);
#pragma omp for schedule(dynamic, 16)
            for (int i = 0; i < out->nn; i++) {
                orc_node *nd = &out->nodes[i];
                if (nd->n != n || nd->child0 < 0) continue;
                orc_reconstruct(m, &out->coefs[(size_t)i * bs], ch);
                for (int c = 0; c < 8; c++) {
                    double *cb = &out->coefs[(size_t)(nd->child0 + c) * bs];
                    for (int q = 0; q < K3; q++) cb[q] += ch[c * K3 + q];
                }
            }
            free(ch);
        }
    }
    orc_tree_update_norms(out);
    orc_tree_compress(out);
    st.flops = (double)st.pairs * 6.0 * K * K * K * K;
#ifdef _OPENMP
    st.seconds = omp_get_wtime() - t_start;
#endif
    if (stats) *stats = st;
    return 0;
}
