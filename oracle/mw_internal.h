/*
 * mw_internal.h -- oracle internals (TEST INFRASTRUCTURE ONLY, see mworacle.h).
 */
#ifndef MW_ORACLE_INTERNAL_H
#define MW_ORACLE_INTERNAL_H

#include "mworacle.h"

#define ORC_KMAX 12
#define ORC_LEGENDRE 0
#define ORC_INTERPOLATING 1
/* exp(-ORC_ZERO_EXP) below which an analytic term is treated as zero on a box */
#define ORC_ZERO_EXP 45.0
/* apply screening: a (output node, input node, term) item is skipped when its
 * contribution bound is below ORC_SCREEN_FAC times the output split threshold */
#define ORC_SCREEN_FAC 0.01

struct orc_mra {
    int n0, corner[3], boxes[3], k, K, basis, max_depth, bs;
    double qx[ORC_KMAX], qw[ORC_KMAX];
    double legq[ORC_KMAX * ORC_KMAX];
    double c2v[ORC_KMAX * ORC_KMAX]; /* c2v[q*K+j] = phi_j(x_q) */
    double v2c[ORC_KMAX * ORC_KMAX]; /* v2c[j*K+q] = w_q phi_j(x_q) */
    double integ[ORC_KMAX];
    double W[4 * ORC_KMAX * ORC_KMAX];  /* [s;d] = W [child0; child1] */
    double WT[4 * ORC_KMAX * ORC_KMAX];
    int *perm; /* cube index -> block index */
};

typedef struct {
    int cap, n;
    int *keys; /* 4 per slot */
    int *vals; /* -1 = empty */
} orc_hmap;

typedef struct {
    int n, l[3];
    int parent, child0;
    double cn[8]; /* component norms */
    double aux;
} orc_node;

struct orc_tree {
    const orc_mra *mra;
    int nn, cap, nroots;
    orc_node *nodes;
    double *coefs;
    orc_hmap map;
};

struct orc_oper {
    const orc_mra *mra;
    int kind; /* 0 poisson, 1 helmholtz */
    double mu, prec, eps, rmin, rmax;
    int T, nscales;
    double *c, *a;
    int *band;        /* [T][nscales] */
    long *off;        /* [T][nscales] block index of l = -band */
    double *blocks;   /* (2K)^2 per block */
    double *norms;    /* 4 per block: [g][f] = ss, sw, ws, ww */
    long nblocks;
};

static inline int orc_floordiv2(int l) { return (l - (l & 1)) / 2; }
static inline double fmax2(double a, double b) { return a > b ? a : b; }

void orc_gauss_legendre(int n, double *x, double *w);
void orc_legendre_all(int n, double x, double *p);
void orc_basis_eval(const orc_mra *m, double x, double *out);
int orc_in_world(const orc_mra *m, int n, const int l[3]);
void orc_transform3(const orc_mra *m, const double *M, const double *in, double *out);
void orc_compress(const orc_mra *m, const double *children, double *block);
void orc_reconstruct(const orc_mra *m, const double *block, double *children);
void orc_map_children(const orc_mra *m, const double *A, const double *in, double *out);
void orc_comp_norms(const orc_mra *m, const double *block, double *cn);
double orc_wavelet_norm(const double *cn);
double orc_block_norm(const double *cn);
double orc_split_thr(double prec, double R, int n);
double orc_item_bound(const double *nx, const double *ny, const double *nz, const double *cn, int root);
void orc_product_block(const orc_mra *m, double coef, int n, const double *ba, const double *bb, double *out, double *work);

void orc_hmap_init(orc_hmap *h, int cap);
void orc_hmap_free(orc_hmap *h);
void orc_hmap_put(orc_hmap *h, int n, const int l[3], int v);
int orc_hmap_get(const orc_hmap *h, int n, const int l[3]);

int orc_tree_add(orc_tree *t, int n, const int l[3], int parent);
int orc_tree_split(orc_tree *t, int i);
void orc_tree_update_norms(orc_tree *t);
void orc_tree_compress(orc_tree *t);
int orc_tree_block(const orc_tree *t, int n, const int l[3], double *buf, int *anc);
int *orc_tree_canonical_order(const orc_tree *t);
int orc_key_cmp(const orc_mra *m, int na, const int *la, int nb, const int *lb);

#endif
