/*
 * mworacle.h -- CPU oracle for the multiwavelet apply / multiply / add path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C (C11 + OpenMP), FP64
 * restatement of the published adaptive multiwavelet algorithms that MRChem
 * reaches through MRCPP (commit 0e5b32003eed8e1abb22a44ba4e1a2ce9fd9ddb1,
 * fetched by external/upstream/fetch_mrcpp.cmake:39-42; MRCPP itself is not
 * vendored in the reference tree).  It is used by the tests, by the smoke
 * check and by bench.py's CPU-baseline leg, as the CPU result the GPU path is
 * compared with; the product (mrchem_gb300) never links or calls it.
 *
 * Published methods restated here:
 *   - Alpert multiwavelets (SIAM J. Math. Anal. 24 (1993) 246) with the
 *     Legendre and interpolating scaling bases; the interpolating basis follows
 *     tools/legendre_to_interpolating_basis/legendre_to_interpolating.py:17-31.
 *   - Non-standard-form separated convolution, Beylkin-Coifman-Rokhlin and
 *     Frediani et al., Mol. Phys. 111 (2013) 1143.
 *   - Gaussian-sum kernels from the trapezoidal rule of
 *     1/r = 2/sqrt(pi) int exp(-r^2 e^{2s} + s) ds (Harrison et al.,
 *     J. Chem. Phys. 121 (2004) 11587), and its Helmholtz variant.
 *
 * Parity with MRCPP's own discretisation is unpinned (MRCPP cannot be built
 * here); the oracle is pinned against analytic potentials and integrals.
 *
 * Conventions shared with the product (must stay identical):
 *   node key   (n, lx, ly, lz): box [2^-n l, 2^-n (l+1)] per dimension
 *   block      8 components x K^3 doubles, component c = cx | cy<<1 | cz<<2
 *              (bit set = wavelet in that dimension), inner index
 *              ix + K*iy + K*K*iz
 *   children   child c = bx | by<<1 | bz<<2, translation 2l + b
 */
#ifndef MWORACLE_H
#define MWORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_mra orc_mra;
typedef struct orc_tree orc_tree;
typedef struct orc_oper orc_oper;

/* one analytic term: coef * (x-X)^px (y-Y)^py (z-Z)^pz * exp(-alpha |r-R|^2) */
typedef struct {
    double coef;
    double alpha;
    double pos[3];
    int pw[3];
    int pad;
} orc_gterm;

typedef struct {
    long long out_nodes;      /* output nodes computed */
    long long items;          /* surviving (output node, input node, term) items */
    long long pairs;          /* surviving (item, component pair) contractions */
    long long generated;      /* generated input nodes */
    double flops;             /* 6K^4 per surviving component pair */
    double seconds;
    /* surviving items by floor(log10(bound / screening threshold)), 0..15;
     * [0..15] all items, [16..31] items with |l|_inf <= 1 */
    long long bound_hist[32];
} orc_stats;

/* ---- MRA ---- */
orc_mra *orc_mra_create(int root_scale, const int corner[3], const int boxes[3], int order, int basis_type,
                        int max_depth);
void orc_mra_free(orc_mra *mra);
int orc_mra_order(const orc_mra *mra);
/* quadrature points/weights on [0,1], filters W (2K x 2K, row-major), c2v, v2c */
void orc_mra_basis(const orc_mra *mra, double *qx, double *qw, double *W, double *c2v, double *v2c);

/* ---- trees ---- */
orc_tree *orc_tree_create(const orc_mra *mra);
void orc_tree_free(orc_tree *t);
int orc_tree_nnodes(const orc_tree *t);
int orc_tree_nleaves(const orc_tree *t);
int orc_tree_depth(const orc_tree *t);
/* canonical order: by scale, then Morton order of translation */
void orc_tree_export(const orc_tree *t, int *keys, double *coefs, unsigned char *is_leaf);
orc_tree *orc_tree_import(const orc_mra *mra, int nnodes, const int *keys, const double *coefs);
double orc_tree_norm(const orc_tree *t);
double orc_tree_sqnorm(const orc_tree *t);
double orc_tree_integrate(const orc_tree *t);
double orc_tree_eval(const orc_tree *t, const double r[3]);
void orc_tree_rescale(orc_tree *t, double c);
double orc_dot(const orc_tree *a, const orc_tree *b);

/* projection of analytic functions */
int orc_project_gauss(double prec, orc_tree *out, int nterms, const orc_gterm *terms, int abs_prec);
int orc_project_hydrogen(double prec, orc_tree *out, int n, int l, int m, double Z, const double origin[3],
                         int abs_prec);

/* grids */
void orc_copy_grid(orc_tree *out, const orc_tree *inp);
void orc_build_grid(orc_tree *out, int ntrees, orc_tree *const *trees);
void orc_clear(orc_tree *t);

/* ---- operators ---- */
orc_oper *orc_oper_poisson(const orc_mra *mra, double prec);
orc_oper *orc_oper_helmholtz(const orc_mra *mra, double mu, double prec);
void orc_oper_free(orc_oper *op);
int orc_oper_nterms(const orc_oper *op);
void orc_oper_terms(const orc_oper *op, double *coefs, double *exps);
/* band of term t at scale n (-1 = inactive); block l in [-band, band]: 2K x 2K row-major */
int orc_oper_band(const orc_oper *op, int t, int n);
int orc_oper_block(const orc_oper *op, int t, int n, int l, double *blk, double *norms4);
double orc_oper_kernel_eval(const orc_oper *op, double r);

/* ---- the hot path ---- */
int orc_apply(double prec, orc_tree *out, const orc_oper *op, orc_tree *inp, int max_iter, int abs_prec,
              int nprec_trees, orc_tree *const *prec_trees, orc_stats *stats);
int orc_multiply(double prec, orc_tree *out, double coef, orc_tree *a, orc_tree *b, int max_iter, int abs_prec,
                 int use_max_norms);
int orc_add(double prec, orc_tree *out, int n, const double *coefs, orc_tree *const *trees, int max_iter);
void orc_crop(orc_tree *t, double prec, int abs_prec);

void orc_set_threads(int n);
int orc_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
