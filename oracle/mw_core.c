/*
 * mw_core.c -- oracle: scaling bases, two-scale filters, function trees,
 * projection, multiwavelet transforms, norms, dot, integrate, evaluation.
 *
 * TEST INFRASTRUCTURE ONLY (see mworacle.h).  Plain C11 + OpenMP, FP64.
 *
 * Reference-side definitions followed here:
 *   - MRA / world box (root scale, corner, boxes, order, max depth):
 *     src/mrenv.cpp:99-127, tests/unit_tests.cpp:66-84.
 *   - Interpolating scaling functions
 *     phi^I_j(x) = sqrt(w_j) sum_i phi^L_i(x_j) phi^L_i(x) on Gauss-Legendre
 *     roots: tools/legendre_to_interpolating_basis/legendre_to_interpolating.py:17-31.
 *   - Hydrogen orbitals (radial Laguerre form, real solid harmonics with
 *     m=0,1,2 -> x,y,z): src/analyticfunctions/HydrogenFunction.cpp:35-198.
 */
#include "mw_internal.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* quadrature and polynomials                                          */
/* ------------------------------------------------------------------ */

void orc_gauss_legendre(int n, double *x, double *w) {
    /* Newton iteration on P_n, mapped to [0,1]; ascending nodes */
    for (int i = 0; i < n; i++) {
        double t = cos(M_PI * (i + 0.75) / (n + 0.5));
        double dp = 1.0;
        for (int it = 0; it < 100; it++) {
            double pm = 1.0, p = t;
            for (int j = 2; j <= n; j++) {
                double pn = ((2.0 * j - 1.0) * t * p - (j - 1.0) * pm) / j;
                pm = p;
                p = pn;
            }
            dp = n * (t * p - pm) / (t * t - 1.0);
            double dt = p / dp;
            t -= dt;
            if (fabs(dt) < 1e-16) break;
        }
        double pm = 1.0, p = t;
        for (int j = 2; j <= n; j++) {
            double pn = ((2.0 * j - 1.0) * t * p - (j - 1.0) * pm) / j;
            pm = p;
            p = pn;
        }
        dp = n * (t * p - pm) / (t * t - 1.0);
        x[i] = 0.5 * (1.0 - t);
        w[i] = 1.0 / ((1.0 - t * t) * dp * dp);
    }
}

/* shifted Legendre P_j(2x-1), j = 0..n-1 */
void orc_legendre_all(int n, double x, double *p) {
    double t = 2.0 * x - 1.0;
    if (n > 0) p[0] = 1.0;
    if (n > 1) p[1] = t;
    for (int j = 1; j + 1 < n; j++) p[j + 1] = ((2.0 * j + 1.0) * t * p[j] - j * p[j - 1]) / (j + 1.0);
}

static void legendre_scaling_all(int K, double x, double *out) {
    orc_legendre_all(K, x, out);
    for (int j = 0; j < K; j++) out[j] *= sqrt(2.0 * j + 1.0);
}

/* all K scaling functions of the MRA's basis at x in [0,1] */
void orc_basis_eval(const orc_mra *m, double x, double *out) {
    int K = m->K;
    if (m->basis == ORC_LEGENDRE) {
        legendre_scaling_all(K, x, out);
        return;
    }
    double pl[ORC_KMAX];
    legendre_scaling_all(K, x, pl);
    for (int j = 0; j < K; j++) {
        double s = 0.0;
        for (int i = 0; i < K; i++) s += m->legq[j * K + i] * pl[i];
        out[j] = sqrt(m->qw[j]) * s;
    }
}

/* ------------------------------------------------------------------ */
/* MRA                                                                 */
/* ------------------------------------------------------------------ */

orc_mra *orc_mra_create(int root_scale, const int corner[3], const int boxes[3], int order, int basis_type,
                        int max_depth) {
    int K = order + 1;
    if (K < 2 || K > ORC_KMAX || max_depth < 1) return NULL;
    orc_mra *m = (orc_mra *)calloc(1, sizeof(orc_mra));
    m->n0 = root_scale;
    for (int d = 0; d < 3; d++) {
        m->corner[d] = corner[d];
        m->boxes[d] = boxes[d];
    }
    m->k = order;
    m->K = K;
    m->basis = basis_type;
    m->max_depth = max_depth;
    m->bs = 8 * K * K * K;
    orc_gauss_legendre(K, m->qx, m->qw);
    /* Legendre scaling functions at the roots (used by the interpolating basis) */
    for (int j = 0; j < K; j++) legendre_scaling_all(K, m->qx[j], &m->legq[j * K]);
    /* coefficient <-> value maps at the K quadrature points */
    for (int q = 0; q < K; q++) {
        double ph[ORC_KMAX];
        orc_basis_eval(m, m->qx[q], ph);
        for (int j = 0; j < K; j++) {
            m->c2v[q * K + j] = ph[j];
            m->v2c[j * K + q] = m->qw[q] * ph[j];
        }
    }
    /* integrals of the scaling functions on [0,1] */
    for (int j = 0; j < K; j++) {
        double s = 0.0;
        for (int q = 0; q < K; q++) s += m->qw[q] * m->c2v[q * K + j];
        m->integ[j] = s;
    }
    /* two-scale filters: H0_ij = 2^-1/2 int phi_i(y/2) phi_j(y) dy, H1 with (y+1)/2 */
    int K2 = 2 * K;
    double *W = m->W;
    memset(W, 0, sizeof(double) * K2 * K2);
    for (int q = 0; q < K; q++) {
        double a0[ORC_KMAX], a1[ORC_KMAX], b[ORC_KMAX];
        orc_basis_eval(m, 0.5 * m->qx[q], a0);
        orc_basis_eval(m, 0.5 * (m->qx[q] + 1.0), a1);
        orc_basis_eval(m, m->qx[q], b);
        for (int i = 0; i < K; i++)
            for (int j = 0; j < K; j++) {
                W[i * K2 + j] += M_SQRT1_2 * m->qw[q] * a0[i] * b[j];
                W[i * K2 + K + j] += M_SQRT1_2 * m->qw[q] * a1[i] * b[j];
            }
    }
    /* wavelet rows: Gram-Schmidt (two passes) of the candidates (e_j, -e_j)/sqrt2
     * against the scaling rows and the previous wavelet rows */
    for (int j = 0; j < K; j++) {
        double v[2 * ORC_KMAX];
        memset(v, 0, sizeof(v));
        v[j] = M_SQRT1_2;
        v[K + j] = -M_SQRT1_2;
        for (int pass = 0; pass < 2; pass++) {
            for (int r = 0; r < K + j; r++) {
                double dot = 0.0;
                for (int c = 0; c < K2; c++) dot += W[r * K2 + c] * v[c];
                for (int c = 0; c < K2; c++) v[c] -= dot * W[r * K2 + c];
            }
            double nrm = 0.0;
            for (int c = 0; c < K2; c++) nrm += v[c] * v[c];
            nrm = sqrt(nrm);
            for (int c = 0; c < K2; c++) v[c] /= nrm;
        }
        for (int c = 0; c < K2; c++) W[(K + j) * K2 + c] = v[c];
    }
    for (int r = 0; r < K2; r++)
        for (int c = 0; c < K2; c++) m->WT[c * K2 + r] = W[r * K2 + c];
    /* permutation between component-major blocks and the (2K)^3 cube */
    int K3 = K * K * K;
    m->perm = (int *)malloc(sizeof(int) * 8 * K3);
    for (int Z = 0; Z < K2; Z++)
        for (int Y = 0; Y < K2; Y++)
            for (int X = 0; X < K2; X++) {
                int c = (X / K) | ((Y / K) << 1) | ((Z / K) << 2);
                int bi = c * K3 + (X % K) + K * (Y % K) + K * K * (Z % K);
                m->perm[(Z * K2 + Y) * K2 + X] = bi;
            }
    return m;
}

void orc_mra_free(orc_mra *m) {
    if (!m) return;
    free(m->perm);
    free(m);
}

int orc_mra_order(const orc_mra *m) { return m->k; }

void orc_mra_basis(const orc_mra *m, double *qx, double *qw, double *W, double *c2v, double *v2c) {
    int K = m->K;
    if (qx) memcpy(qx, m->qx, sizeof(double) * K);
    if (qw) memcpy(qw, m->qw, sizeof(double) * K);
    if (W) memcpy(W, m->W, sizeof(double) * 4 * K * K);
    if (c2v) memcpy(c2v, m->c2v, sizeof(double) * K * K);
    if (v2c) memcpy(v2c, m->v2c, sizeof(double) * K * K);
}

int orc_in_world(const orc_mra *m, int n, const int l[3]) {
    int sh = n - m->n0;
    for (int d = 0; d < 3; d++) {
        long lo = (long)m->corner[d] * (1L << sh);
        long hi = (long)(m->corner[d] + m->boxes[d]) * (1L << sh);
        if (l[d] < lo || l[d] >= hi) return 0;
    }
    return 1;
}

/* ------------------------------------------------------------------ */
/* 3-D transforms on blocks                                            */
/* ------------------------------------------------------------------ */

/* out = (M (x) M (x) M) in, with blocks in component-major layout and M 2K x 2K */
void orc_transform3(const orc_mra *m, const double *M, const double *in, double *out) {
    int K = m->K, K2 = 2 * K, N = K2 * K2 * K2;
    double *a = (double *)malloc(sizeof(double) * N), *b = (double *)malloc(sizeof(double) * N);
    for (int i = 0; i < N; i++) a[i] = in[m->perm[i]];
    /* x */
    for (int Z = 0; Z < K2; Z++)
        for (int Y = 0; Y < K2; Y++)
            for (int X = 0; X < K2; X++) {
                double s = 0.0;
                const double *row = &M[X * K2];
                const double *src = &a[(Z * K2 + Y) * K2];
                for (int i = 0; i < K2; i++) s += row[i] * src[i];
                b[(Z * K2 + Y) * K2 + X] = s;
            }
    /* y */
    for (int Z = 0; Z < K2; Z++)
        for (int Y = 0; Y < K2; Y++)
            for (int X = 0; X < K2; X++) {
                double s = 0.0;
                for (int i = 0; i < K2; i++) s += M[Y * K2 + i] * b[(Z * K2 + i) * K2 + X];
                a[(Z * K2 + Y) * K2 + X] = s;
            }
    /* z */
    for (int Z = 0; Z < K2; Z++)
        for (int Y = 0; Y < K2; Y++)
            for (int X = 0; X < K2; X++) {
                double s = 0.0;
                for (int i = 0; i < K2; i++) s += M[Z * K2 + i] * a[(i * K2 + Y) * K2 + X];
                b[(Z * K2 + Y) * K2 + X] = s;
            }
    for (int i = 0; i < N; i++) out[m->perm[i]] = b[i];
    free(a);
    free(b);
}

/* children scaling coefficients (component-major "child" layout) -> node (s,d) block */
void orc_compress(const orc_mra *m, const double *children, double *block) {
    orc_transform3(m, m->W, children, block);
}

void orc_reconstruct(const orc_mra *m, const double *block, double *children) {
    orc_transform3(m, m->WT, block, children);
}

/* per-dimension K x K map applied to each of the 8 sub-blocks */
void orc_map_children(const orc_mra *m, const double *A, const double *in, double *out) {
    int K = m->K, K3 = K * K * K;
    double *t1 = (double *)malloc(sizeof(double) * K3), *t2 = (double *)malloc(sizeof(double) * K3);
    for (int c = 0; c < 8; c++) {
        const double *s = in + c * K3;
        for (int z = 0; z < K; z++)
            for (int y = 0; y < K; y++)
                for (int x = 0; x < K; x++) {
                    double v = 0.0;
                    for (int i = 0; i < K; i++) v += A[x * K + i] * s[z * K * K + y * K + i];
                    t1[z * K * K + y * K + x] = v;
                }
        for (int z = 0; z < K; z++)
            for (int y = 0; y < K; y++)
                for (int x = 0; x < K; x++) {
                    double v = 0.0;
                    for (int i = 0; i < K; i++) v += A[y * K + i] * t1[z * K * K + i * K + x];
                    t2[z * K * K + y * K + x] = v;
                }
        for (int z = 0; z < K; z++)
            for (int y = 0; y < K; y++)
                for (int x = 0; x < K; x++) {
                    double v = 0.0;
                    for (int i = 0; i < K; i++) v += A[z * K + i] * t2[i * K * K + y * K + x];
                    out[c * K3 + z * K * K + y * K + x] = v;
                }
    }
    free(t1);
    free(t2);
}

void orc_comp_norms(const orc_mra *m, const double *block, double *cn) {
    int K3 = m->K * m->K * m->K;
    for (int c = 0; c < 8; c++) {
        double s = 0.0;
        for (int i = 0; i < K3; i++) s += block[c * K3 + i] * block[c * K3 + i];
        cn[c] = sqrt(s);
    }
}

double orc_wavelet_norm(const double *cn) {
    double s = 0.0;
    for (int c = 1; c < 8; c++) s += cn[c] * cn[c];
    return sqrt(s);
}

double orc_block_norm(const double *cn) {
    double s = 0.0;
    for (int c = 0; c < 8; c++) s += cn[c] * cn[c];
    return sqrt(s);
}

/* ------------------------------------------------------------------ */
/* hash map on node keys                                               */
/* ------------------------------------------------------------------ */

static unsigned long long key_hash(int n, const int l[3]) {
    unsigned long long h = (unsigned long long)(unsigned)n * 0x9E3779B97F4A7C15ULL;
    h ^= (unsigned long long)(unsigned)l[0] + 0x632BE59BD9B4E019ULL + (h << 6) + (h >> 2);
    h ^= (unsigned long long)(unsigned)l[1] * 0xC2B2AE3D27D4EB4FULL + (h << 6) + (h >> 2);
    h ^= (unsigned long long)(unsigned)l[2] * 0x165667B19E3779F9ULL + (h << 6) + (h >> 2);
    h ^= h >> 29;
    h *= 0xBF58476D1CE4E5B9ULL;
    h ^= h >> 32;
    return h;
}

void orc_hmap_init(orc_hmap *h, int cap) {
    int c = 16;
    while (c < 2 * cap) c <<= 1;
    h->cap = c;
    h->n = 0;
    h->keys = (int *)malloc(sizeof(int) * 4 * c);
    h->vals = (int *)malloc(sizeof(int) * c);
    for (int i = 0; i < c; i++) h->vals[i] = -1;
}

void orc_hmap_free(orc_hmap *h) {
    free(h->keys);
    free(h->vals);
    h->keys = NULL;
    h->vals = NULL;
}

static void hmap_grow(orc_hmap *h) {
    orc_hmap nh;
    orc_hmap_init(&nh, h->cap);
    for (int i = 0; i < h->cap; i++)
        if (h->vals[i] >= 0) orc_hmap_put(&nh, h->keys[4 * i], &h->keys[4 * i + 1], h->vals[i]);
    orc_hmap_free(h);
    *h = nh;
}

void orc_hmap_put(orc_hmap *h, int n, const int l[3], int v) {
    if (2 * (h->n + 1) > h->cap) hmap_grow(h);
    unsigned long long i = key_hash(n, l) & (unsigned long long)(h->cap - 1);
    while (h->vals[i] >= 0) {
        int *k = &h->keys[4 * i];
        if (k[0] == n && k[1] == l[0] && k[2] == l[1] && k[3] == l[2]) {
            h->vals[i] = v;
            return;
        }
        i = (i + 1) & (unsigned long long)(h->cap - 1);
    }
    h->keys[4 * i] = n;
    h->keys[4 * i + 1] = l[0];
    h->keys[4 * i + 2] = l[1];
    h->keys[4 * i + 3] = l[2];
    h->vals[i] = v;
    h->n++;
}

int orc_hmap_get(const orc_hmap *h, int n, const int l[3]) {
    unsigned long long i = key_hash(n, l) & (unsigned long long)(h->cap - 1);
    while (h->vals[i] >= 0) {
        const int *k = &h->keys[4 * i];
        if (k[0] == n && k[1] == l[0] && k[2] == l[1] && k[3] == l[2]) return h->vals[i];
        i = (i + 1) & (unsigned long long)(h->cap - 1);
    }
    return -1;
}

/* ------------------------------------------------------------------ */
/* trees                                                               */
/* ------------------------------------------------------------------ */

static void tree_reserve(orc_tree *t, int cap) {
    if (cap <= t->cap) return;
    int nc = t->cap ? t->cap : 64;
    while (nc < cap) nc *= 2;
    t->nodes = (orc_node *)realloc(t->nodes, sizeof(orc_node) * nc);
    t->coefs = (double *)realloc(t->coefs, sizeof(double) * (size_t)nc * t->mra->bs);
    t->cap = nc;
}

int orc_tree_add(orc_tree *t, int n, const int l[3], int parent) {
    tree_reserve(t, t->nn + 1);
    int i = t->nn++;
    orc_node *nd = &t->nodes[i];
    nd->n = n;
    nd->l[0] = l[0];
    nd->l[1] = l[1];
    nd->l[2] = l[2];
    nd->parent = parent;
    nd->child0 = -1;
    for (int c = 0; c < 8; c++) nd->cn[c] = 0.0;
    nd->aux = 0.0;
    memset(&t->coefs[(size_t)i * t->mra->bs], 0, sizeof(double) * t->mra->bs);
    orc_hmap_put(&t->map, n, l, i);
    return i;
}

/* creates the 8 children of node i (contiguous); returns index of child 0 */
int orc_tree_split(orc_tree *t, int i) {
    if (t->nodes[i].child0 >= 0) return t->nodes[i].child0;
    tree_reserve(t, t->nn + 8);
    int n = t->nodes[i].n, l[3] = {t->nodes[i].l[0], t->nodes[i].l[1], t->nodes[i].l[2]};
    int first = t->nn;
    for (int c = 0; c < 8; c++) {
        int cl[3] = {2 * l[0] + (c & 1), 2 * l[1] + ((c >> 1) & 1), 2 * l[2] + ((c >> 2) & 1)};
        orc_tree_add(t, n + 1, cl, i);
    }
    t->nodes[i].child0 = first;
    return first;
}

orc_tree *orc_tree_create(const orc_mra *m) {
    orc_tree *t = (orc_tree *)calloc(1, sizeof(orc_tree));
    t->mra = m;
    orc_hmap_init(&t->map, 64);
    for (int bz = 0; bz < m->boxes[2]; bz++)
        for (int by = 0; by < m->boxes[1]; by++)
            for (int bx = 0; bx < m->boxes[0]; bx++) {
                int l[3] = {m->corner[0] + bx, m->corner[1] + by, m->corner[2] + bz};
                orc_tree_add(t, m->n0, l, -1);
            }
    t->nroots = t->nn;
    return t;
}

void orc_tree_free(orc_tree *t) {
    if (!t) return;
    free(t->nodes);
    free(t->coefs);
    orc_hmap_free(&t->map);
    free(t);
}

void orc_clear(orc_tree *t) {
    const orc_mra *m = t->mra;
    t->nn = 0;
    orc_hmap_free(&t->map);
    orc_hmap_init(&t->map, 64);
    for (int bz = 0; bz < m->boxes[2]; bz++)
        for (int by = 0; by < m->boxes[1]; by++)
            for (int bx = 0; bx < m->boxes[0]; bx++) {
                int l[3] = {m->corner[0] + bx, m->corner[1] + by, m->corner[2] + bz};
                orc_tree_add(t, m->n0, l, -1);
            }
    t->nroots = t->nn;
}

int orc_tree_nnodes(const orc_tree *t) { return t->nn; }

int orc_tree_nleaves(const orc_tree *t) {
    int c = 0;
    for (int i = 0; i < t->nn; i++) c += (t->nodes[i].child0 < 0);
    return c;
}

int orc_tree_depth(const orc_tree *t) {
    int mx = t->mra->n0;
    for (int i = 0; i < t->nn; i++)
        if (t->nodes[i].n > mx) mx = t->nodes[i].n;
    return mx - t->mra->n0 + 1;
}

void orc_tree_update_norms(orc_tree *t) {
    int bs = t->mra->bs;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < t->nn; i++) orc_comp_norms(t->mra, &t->coefs[(size_t)i * bs], t->nodes[i].cn);
}

/* sum of squared leaf-block norms, in node order */
double orc_tree_sqnorm(const orc_tree *t) {
    double s = 0.0;
    for (int i = 0; i < t->nn; i++) {
        if (t->nodes[i].child0 >= 0) continue;
        const double *cn = t->nodes[i].cn;
        for (int c = 0; c < 8; c++) s += cn[c] * cn[c];
    }
    return s;
}

double orc_tree_norm(const orc_tree *t) { return sqrt(orc_tree_sqnorm(t)); }

/* Morton "less than" on translations shifted to non-negative values, z most significant */
static int less_msb(unsigned a, unsigned b) { return a < b && a < (a ^ b); }

static const orc_mra *g_sort_mra;
static const orc_node *g_sort_nodes;

int orc_key_cmp(const orc_mra *m, int na, const int *la, int nb, const int *lb) {
    if (na != nb) return na < nb ? -1 : 1;
    int sh = na - m->n0;
    unsigned ua[3], ub[3];
    for (int d = 0; d < 3; d++) {
        ua[d] = (unsigned)(la[d] - m->corner[d] * (1 << sh));
        ub[d] = (unsigned)(lb[d] - m->corner[d] * (1 << sh));
    }
    int dim = 2;
    unsigned xm = ua[2] ^ ub[2];
    for (int d = 1; d >= 0; d--) {
        unsigned x = ua[d] ^ ub[d];
        if (less_msb(xm, x)) {
            dim = d;
            xm = x;
        }
    }
    if (ua[dim] == ub[dim]) return 0;
    return ua[dim] < ub[dim] ? -1 : 1;
}

static int node_cmp(const void *a, const void *b) {
    const orc_node *x = &g_sort_nodes[*(const int *)a], *y = &g_sort_nodes[*(const int *)b];
    return orc_key_cmp(g_sort_mra, x->n, x->l, y->n, y->l);
}

int *orc_tree_canonical_order(const orc_tree *t) {
    int *idx = (int *)malloc(sizeof(int) * t->nn);
    for (int i = 0; i < t->nn; i++) idx[i] = i;
#pragma omp critical(orc_sort)
    {
        g_sort_mra = t->mra;
        g_sort_nodes = t->nodes;
        qsort(idx, t->nn, sizeof(int), node_cmp);
    }
    return idx;
}

void orc_tree_export(const orc_tree *t, int *keys, double *coefs, unsigned char *is_leaf) {
    int *idx = orc_tree_canonical_order(t);
    int bs = t->mra->bs;
    for (int j = 0; j < t->nn; j++) {
        const orc_node *nd = &t->nodes[idx[j]];
        if (keys) {
            keys[4 * j] = nd->n;
            keys[4 * j + 1] = nd->l[0];
            keys[4 * j + 2] = nd->l[1];
            keys[4 * j + 3] = nd->l[2];
        }
        if (coefs) memcpy(&coefs[(size_t)j * bs], &t->coefs[(size_t)idx[j] * bs], sizeof(double) * bs);
        if (is_leaf) is_leaf[j] = (nd->child0 < 0);
    }
    free(idx);
}

/* rebuild a tree from (key, block) pairs given in any order */
orc_tree *orc_tree_import(const orc_mra *m, int nnodes, const int *keys, const double *coefs) {
    orc_hmap tmp;
    orc_hmap_init(&tmp, nnodes);
    for (int i = 0; i < nnodes; i++) orc_hmap_put(&tmp, keys[4 * i], &keys[4 * i + 1], i);
    orc_tree *t = orc_tree_create(m);
    int bs = m->bs;
    /* breadth-first: split every node whose children are present */
    for (int i = 0; i < t->nn; i++) {
        orc_node *nd = &t->nodes[i];
        int src = orc_hmap_get(&tmp, nd->n, nd->l);
        if (src < 0) {
            orc_hmap_free(&tmp);
            orc_tree_free(t);
            return NULL;
        }
        memcpy(&t->coefs[(size_t)i * bs], &coefs[(size_t)src * bs], sizeof(double) * bs);
        int cl[3] = {2 * nd->l[0], 2 * nd->l[1], 2 * nd->l[2]};
        if (orc_hmap_get(&tmp, nd->n + 1, cl) >= 0) orc_tree_split(t, i);
    }
    orc_hmap_free(&tmp);
    if (t->nn != nnodes) {
        orc_tree_free(t);
        return NULL;
    }
    orc_tree_update_norms(t);
    return t;
}

/* bottom-up: every branch node's block <- compress(children scaling parts) */
void orc_tree_compress(orc_tree *t) {
    const orc_mra *m = t->mra;
    int bs = m->bs, K3 = m->K * m->K * m->K;
    int maxn = m->n0;
    for (int i = 0; i < t->nn; i++)
        if (t->nodes[i].n > maxn) maxn = t->nodes[i].n;
    for (int n = maxn - 1; n >= m->n0; n--) {
#pragma omp parallel
        {
            double *ch = (double *)malloc(sizeof(double) * bs);
#pragma omp for schedule(dynamic, 16)
            for (int i = 0; i < t->nn; i++) {
                orc_node *nd = &t->nodes[i];
                if (nd->n != n || nd->child0 < 0) continue;
                for (int c = 0; c < 8; c++)
                    memcpy(&ch[c * K3], &t->coefs[(size_t)(nd->child0 + c) * bs], sizeof(double) * K3);
                orc_compress(m, ch, &t->coefs[(size_t)i * bs]);
                orc_comp_norms(m, &t->coefs[(size_t)i * bs], nd->cn);
            }
            free(ch);
        }
    }
}

/*
 * Block of the function at node (n,l): the stored block if the node exists,
 * else a generated block (scaling part reconstructed from the deepest existing
 * ancestor, wavelet part zero).  Returns the node index (>= 0), -1 for a
 * generated block written to buf, -2 if (n,l) lies outside the world box.
 * *anc receives the ancestor's index for generated blocks.
 */
int orc_tree_block(const orc_tree *t, int n, const int l[3], double *buf, int *anc) {
    const orc_mra *m = t->mra;
    int idx = orc_hmap_get(&t->map, n, l);
    if (idx >= 0) return idx;
    if (!orc_in_world(m, n, l)) return -2;
    int an = n, al[3] = {l[0], l[1], l[2]};
    int a = -1;
    while (a < 0) {
        an--;
        for (int d = 0; d < 3; d++) al[d] = orc_floordiv2(al[d]);
        a = orc_hmap_get(&t->map, an, al);
    }
    if (anc) *anc = a;
    int bs = m->bs, K3 = m->K * m->K * m->K;
    double *cur = (double *)malloc(sizeof(double) * bs), *ch = (double *)malloc(sizeof(double) * bs);
    memcpy(cur, &t->coefs[(size_t)a * bs], sizeof(double) * bs);
    for (int s = an; s < n; s++) {
        int sh = n - (s + 1);
        int c = 0;
        for (int d = 0; d < 3; d++) c |= ((l[d] >> sh) & 1) << d;
        orc_reconstruct(m, cur, ch);
        memset(cur, 0, sizeof(double) * bs);
        memcpy(cur, &ch[c * K3], sizeof(double) * K3);
    }
    memcpy(buf, cur, sizeof(double) * bs);
    free(cur);
    free(ch);
    return -1;
}

/* ------------------------------------------------------------------ */
/* analytic functions and projection                                   */
/* ------------------------------------------------------------------ */

typedef struct {
    int kind; /* 0 gaussian sum, 1 hydrogen */
    int nterms;
    const orc_gterm *terms;
    int hn, hl, hm;
    double Z, origin[3];
    double hnorm;
} afunc;

static double factorial(int n) {
    double f = 1.0;
    for (int i = 2; i <= n; i++) f *= i;
    return f;
}

/* generalized Laguerre L^a_k(x) by the three-term recurrence */
static double laguerre(int k, int a, double x) {
    if (k == 0) return 1.0;
    double l0 = 1.0, l1 = 1.0 + a - x;
    for (int j = 1; j < k; j++) {
        double l2 = ((2.0 * j + 1.0 + a - x) * l1 - (j + a) * l0) / (j + 1.0);
        l0 = l1;
        l1 = l2;
    }
    return l1;
}

static double afunc_eval(const afunc *f, const double r[3]) {
    if (f->kind == 0) {
        double v = 0.0;
        for (int t = 0; t < f->nterms; t++) {
            const orc_gterm *g = &f->terms[t];
            double dx = r[0] - g->pos[0], dy = r[1] - g->pos[1], dz = r[2] - g->pos[2];
            double r2 = dx * dx + dy * dy + dz * dz;
            double e = g->alpha * r2;
            if (e > 700.0) continue;
            double p = g->coef;
            for (int i = 0; i < g->pw[0]; i++) p *= dx;
            for (int i = 0; i < g->pw[1]; i++) p *= dy;
            for (int i = 0; i < g->pw[2]; i++) p *= dz;
            v += p * exp(-e);
        }
        return v;
    }
    double q[3] = {r[0] - f->origin[0], r[1] - f->origin[1], r[2] - f->origin[2]};
    double rr = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
    double rho = 2.0 * f->Z * rr / f->hn;
    double rad = f->hnorm * pow(rho, f->hl) * laguerre(f->hn - f->hl - 1, 2 * f->hl + 1, rho) * exp(-0.5 * rho);
    double ang = 0.5 / sqrt(M_PI);
    if (f->hl == 1) ang *= sqrt(3.0) * (rr > 0.0 ? q[f->hm] / rr : 0.0);
    return rad * ang;
}

/* distance from point p to box [lo,hi] */
static double box_dist(const double lo[3], const double hi[3], const double p[3]) {
    double s = 0.0;
    for (int d = 0; d < 3; d++) {
        double e = 0.0;
        if (p[d] < lo[d]) e = lo[d] - p[d];
        if (p[d] > hi[d]) e = p[d] - hi[d];
        s += e * e;
    }
    return sqrt(s);
}

/* zero: every term is negligible on the box; forced: a term's width is not
 * resolved by the K points of the children */
static void afunc_box_flags(const afunc *f, int K, int n, const int l[3], int *zero, int *forced) {
    double h = ldexp(1.0, -n), lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
        lo[d] = h * l[d];
        hi[d] = h * (l[d] + 1);
    }
    *zero = 1;
    *forced = 0;
    if (f->kind == 0) {
        for (int t = 0; t < f->nterms; t++) {
            const orc_gterm *g = &f->terms[t];
            double dist = box_dist(lo, hi, g->pos);
            if (g->alpha * dist * dist > ORC_ZERO_EXP) continue;
            *zero = 0;
            double sigma = 1.0 / sqrt(2.0 * g->alpha);
            if (0.5 * h > 0.5 * K * sigma) *forced = 1;
        }
    } else {
        double dist = box_dist(lo, hi, f->origin);
        double decay = f->Z / f->hn;
        if (decay * dist < ORC_ZERO_EXP) {
            *zero = 0;
            double sigma = 1.0 / decay;
            if (0.5 * h > 0.5 * K * sigma) *forced = 1;
        }
    }
}

/* node block by K-point quadrature on each child, then compression */
static void project_node(const orc_mra *m, const afunc *f, int n, const int l[3], double *block, double *work) {
    int K = m->K, K3 = K * K * K;
    double *vals = work, *ch = work + 8 * K3;
    double h = ldexp(1.0, -(n + 1));
    for (int c = 0; c < 8; c++) {
        int cl[3] = {2 * l[0] + (c & 1), 2 * l[1] + ((c >> 1) & 1), 2 * l[2] + ((c >> 2) & 1)};
        for (int iz = 0; iz < K; iz++)
            for (int iy = 0; iy < K; iy++)
                for (int ix = 0; ix < K; ix++) {
                    double r[3] = {h * (cl[0] + m->qx[ix]), h * (cl[1] + m->qx[iy]), h * (cl[2] + m->qx[iz])};
                    vals[c * K3 + ix + K * iy + K * K * iz] = afunc_eval(f, r);
                }
    }
    /* values -> child scaling coefficients: 2^{-3(n+1)/2} (V2C (x) V2C (x) V2C) */
    orc_map_children(m, m->v2c, vals, ch);
    double sc = pow(2.0, -1.5 * (n + 1));
    for (int i = 0; i < 8 * K3; i++) ch[i] *= sc;
    orc_compress(m, ch, block);
}

double orc_split_thr(double prec, double R, int n) { return prec * R * pow(2.0, -0.5 * (n + 1)); }

static int project_generic(double prec, orc_tree *t, const afunc *f, int abs_prec) {
    const orc_mra *m = t->mra;
    orc_clear(t);
    int bs = m->bs;
    int maxn = m->n0 + m->max_depth - 1;
    int nwork = t->nn;
    int *work = (int *)malloc(sizeof(int) * nwork);
    for (int i = 0; i < nwork; i++) work[i] = i;
    unsigned char *forced = NULL;
    while (nwork > 0) {
        forced = (unsigned char *)realloc(forced, nwork);
#pragma omp parallel
        {
            double *wk = (double *)malloc(sizeof(double) * 2 * bs);
#pragma omp for schedule(dynamic, 4)
            for (int w = 0; w < nwork; w++) {
                orc_node *nd = &t->nodes[work[w]];
                int zero, frc;
                afunc_box_flags(f, m->K, nd->n, nd->l, &zero, &frc);
                forced[w] = (unsigned char)(frc && !zero);
                double *blk = &t->coefs[(size_t)work[w] * bs];
                if (zero)
                    memset(blk, 0, sizeof(double) * bs);
                else
                    project_node(m, f, nd->n, nd->l, blk, wk);
                orc_comp_norms(m, blk, nd->cn);
            }
            free(wk);
        }
        double R = abs_prec ? 1.0 : orc_tree_norm(t);
        int *next = NULL, nnext = 0;
        for (int w = 0; w < nwork; w++) {
            int i = work[w];
            int n = t->nodes[i].n;
            if (n >= maxn) continue;
            double wn = orc_wavelet_norm(t->nodes[i].cn);
            if (forced[w] || wn > orc_split_thr(prec, R, n)) {
                int c0 = orc_tree_split(t, i);
                next = (int *)realloc(next, sizeof(int) * (nnext + 8));
                for (int c = 0; c < 8; c++) next[nnext++] = c0 + c;
            }
        }
        free(work);
        work = next;
        nwork = nnext;
    }
    free(work);
    free(forced);
    orc_tree_compress(t);
    return 0;
}

int orc_project_gauss(double prec, orc_tree *out, int nterms, const orc_gterm *terms, int abs_prec) {
    afunc f;
    memset(&f, 0, sizeof(f));
    f.kind = 0;
    f.nterms = nterms;
    f.terms = terms;
    return project_generic(prec, out, &f, abs_prec);
}

int orc_project_hydrogen(double prec, orc_tree *out, int n, int l, int m, double Z, const double origin[3],
                         int abs_prec) {
    if (n < 1 || l < 0 || l > 1 || l >= n || m < 0 || m > 2 * l) return -1;
    afunc f;
    memset(&f, 0, sizeof(f));
    f.kind = 1;
    f.hn = n;
    f.hl = l;
    f.hm = m;
    f.Z = Z;
    for (int d = 0; d < 3; d++) f.origin[d] = origin[d];
    f.hnorm = sqrt(pow(2.0 * Z / n, 3) * factorial(n - l - 1) / (2.0 * n * factorial(n + l)));
    return project_generic(prec, out, &f, abs_prec);
}

/* ------------------------------------------------------------------ */
/* grids, dot, integrate, evaluate                                     */
/* ------------------------------------------------------------------ */

void orc_copy_grid(orc_tree *out, const orc_tree *inp) {
    orc_clear(out);
    for (int i = 0; i < out->nn; i++) {
        orc_node *nd = &out->nodes[i];
        int j = orc_hmap_get(&inp->map, nd->n, nd->l);
        if (j >= 0 && inp->nodes[j].child0 >= 0) orc_tree_split(out, i);
    }
}

/* extends out's grid by the union of the given trees' grids (coefficients untouched
 * for existing nodes, zero for new ones) */
void orc_build_grid(orc_tree *out, int ntrees, orc_tree *const *trees) {
    for (int i = 0; i < out->nn; i++) {
        orc_node *nd = &out->nodes[i];
        if (nd->child0 >= 0) continue;
        for (int k = 0; k < ntrees; k++) {
            int j = orc_hmap_get(&trees[k]->map, nd->n, nd->l);
            if (j >= 0 && trees[k]->nodes[j].child0 >= 0) {
                orc_tree_split(out, i);
                break;
            }
        }
    }
}

double orc_dot(const orc_tree *a, const orc_tree *b) {
    const orc_mra *m = a->mra;
    int bs = m->bs, K3 = m->K * m->K * m->K;
    double s = 0.0;
    for (int i = 0; i < a->nn; i++) {
        const orc_node *nd = &a->nodes[i];
        int j = orc_hmap_get(&b->map, nd->n, nd->l);
        if (j < 0) continue;
        const double *x = &a->coefs[(size_t)i * bs], *y = &b->coefs[(size_t)j * bs];
        int start = (nd->n == m->n0) ? 0 : K3;
        for (int q = start; q < bs; q++) s += x[q] * y[q];
    }
    return s;
}

double orc_tree_integrate(const orc_tree *t) {
    const orc_mra *m = t->mra;
    int K = m->K, bs = m->bs;
    double s = 0.0;
    for (int i = 0; i < t->nroots; i++) {
        const double *x = &t->coefs[(size_t)i * bs];
        for (int iz = 0; iz < K; iz++)
            for (int iy = 0; iy < K; iy++)
                for (int ix = 0; ix < K; ix++)
                    s += x[ix + K * iy + K * K * iz] * m->integ[ix] * m->integ[iy] * m->integ[iz];
    }
    return s * pow(2.0, -1.5 * m->n0);
}

double orc_tree_eval(const orc_tree *t, const double r[3]) {
    const orc_mra *m = t->mra;
    int K = m->K, bs = m->bs, K3 = K * K * K;
    /* locate the root box */
    double hr = ldexp(1.0, -m->n0);
    int l[3];
    for (int d = 0; d < 3; d++) {
        l[d] = (int)floor(r[d] / hr);
        if (l[d] < m->corner[d] || l[d] >= m->corner[d] + m->boxes[d]) return 0.0;
    }
    int idx = orc_hmap_get(&t->map, m->n0, l);
    while (t->nodes[idx].child0 >= 0) {
        int n = t->nodes[idx].n;
        double h = ldexp(1.0, -(n + 1));
        int c = 0;
        for (int d = 0; d < 3; d++) {
            int cl = (int)floor(r[d] / h);
            if (cl < 2 * t->nodes[idx].l[d]) cl = 2 * t->nodes[idx].l[d];
            if (cl > 2 * t->nodes[idx].l[d] + 1) cl = 2 * t->nodes[idx].l[d] + 1;
            c |= (cl - 2 * t->nodes[idx].l[d]) << d;
        }
        idx = t->nodes[idx].child0 + c;
    }
    const orc_node *nd = &t->nodes[idx];
    double *ch = (double *)malloc(sizeof(double) * bs);
    orc_reconstruct(m, &t->coefs[(size_t)idx * bs], ch);
    double h = ldexp(1.0, -(nd->n + 1));
    int c = 0;
    double ph[3][ORC_KMAX];
    for (int d = 0; d < 3; d++) {
        int cl = (int)floor(r[d] / h);
        if (cl < 2 * nd->l[d]) cl = 2 * nd->l[d];
        if (cl > 2 * nd->l[d] + 1) cl = 2 * nd->l[d] + 1;
        c |= (cl - 2 * nd->l[d]) << d;
        double y = r[d] / h - cl;
        orc_basis_eval(m, y, ph[d]);
    }
    double v = 0.0;
    const double *s = &ch[c * K3];
    for (int iz = 0; iz < K; iz++)
        for (int iy = 0; iy < K; iy++)
            for (int ix = 0; ix < K; ix++) v += s[ix + K * iy + K * K * iz] * ph[0][ix] * ph[1][iy] * ph[2][iz];
    free(ch);
    return v * pow(2.0, 1.5 * (nd->n + 1));
}

void orc_tree_rescale(orc_tree *t, double c) {
    size_t N = (size_t)t->nn * t->mra->bs;
    for (size_t i = 0; i < N; i++) t->coefs[i] *= c;
    for (int i = 0; i < t->nn; i++)
        for (int k = 0; k < 8; k++) t->nodes[i].cn[k] *= fabs(c);
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
