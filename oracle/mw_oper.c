/*
 * mw_oper.c -- oracle: separated Gaussian-sum convolution operators.
 *
 * TEST INFRASTRUCTURE ONLY (see mworacle.h).
 *
 * Kernel expansion (published method, Harrison et al. JCP 121 (2004) 11587;
 * Beylkin & Monzon): trapezoidal rule with step h on
 *     1/r         = 2/sqrt(pi) int exp(-r^2 e^{2s} + s) ds
 *     e^{-mu r}/r = 2/sqrt(pi) int exp(-r^2 e^{2s} - mu^2 e^{-2s}/4 + s) ds
 * giving K(r) ~ sum_t c_t exp(-a_t r^2).  The step is shrunk until the
 * sampled relative error (relative to 1/r) on [r_min, r_max] is below eps.
 * Reference call sites: PoissonOperator(MRA, prec) src/driver.cpp:1131,1283;
 * HelmholtzOperator(MRA, mu, prec) src/scf_solver/HelmholtzVector.cpp:144.
 *
 * 1-D operator blocks (non-standard form): for term t at scale n the 2K x 2K
 * block coupling output node l_o to input node l_i (l = l_o - l_i) is
 *     NS_n(l) = W [[tau(2l), tau(2l-1)], [tau(2l+1), tau(2l)]] W^T
 * with tau(m)_{ij} = 2^{-(n+1)} int int phi_i(u) phi_j(v)
 *                    exp(-a 4^{-(n+1)} (u - v + m)^2) du dv,
 * evaluated through the Legendre expansion of the scaling-function
 * cross-correlations (exact polynomials of degree 2K-1) against Gaussian
 * moments computed by composite Gauss-Legendre quadrature.
 */
#include "mw_internal.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NS_CLEAN 1e-13
#define BAND_CAP 1024
#define QPTS 16

/* ---------------- kernel expansion ---------------- */

static double erfc_inv_small(double y) {
    /* x with erfc(x) = y for small y, by bisection */
    double lo = 0.0, hi = 30.0;
    for (int i = 0; i < 200; i++) {
        double mid = 0.5 * (lo + hi);
        if (erfc(mid) > y)
            lo = mid;
        else
            hi = mid;
    }
    return 0.5 * (lo + hi);
}

static void make_terms(int kind, double mu, double eps, double rmin, double rmax, double h, int *T, double **c,
                       double **a) {
    double s_lo = log(eps * sqrt(M_PI) / (8.0 * rmax));
    double s_hi = log(erfc_inv_small(0.25 * eps) / rmin);
    int n = (int)ceil((s_hi - s_lo) / h) + 1;
    double *cc = (double *)malloc(sizeof(double) * n), *aa = (double *)malloc(sizeof(double) * n);
    int m = 0;
    for (int j = 0; j < n; j++) {
        double s = s_lo + h * j;
        double cj = 2.0 * h / sqrt(M_PI) * exp(s);
        if (kind == 1) cj *= exp(-0.25 * mu * mu * exp(-2.0 * s));
        double aj = exp(2.0 * s);
        /* largest relative (to 1/r) contribution of this term: c/sqrt(2 e a) */
        if (cj / sqrt(2.0 * M_E * aj) < 0.01 * eps / n) continue;
        cc[m] = cj;
        aa[m] = aj;
        m++;
    }
    *T = m;
    *c = cc;
    *a = aa;
}

static double kernel_exact(int kind, double mu, double r) { return kind == 1 ? exp(-mu * r) / r : 1.0 / r; }

static double terms_max_relerr(int kind, double mu, int T, const double *c, const double *a, double rmin,
                               double rmax) {
    double err = 0.0;
    int N = 4000;
    for (int i = 0; i <= N; i++) {
        double r = rmin * pow(rmax / rmin, (double)i / N);
        double v = 0.0;
        for (int t = 0; t < T; t++) v += c[t] * exp(-a[t] * r * r);
        double e = fabs(v - kernel_exact(kind, mu, r)) * r;
        if (e > err) err = e;
    }
    return err;
}

double orc_oper_kernel_eval(const orc_oper *op, double r) {
    double v = 0.0;
    for (int t = 0; t < op->T; t++) v += op->c[t] * exp(-op->a[t] * r * r);
    return v;
}

/* ---------------- 1-D blocks ---------------- */

typedef struct {
    int K;
    double *acc;          /* a[(i*K + j)*2K + p] */
    double gx[QPTS], gw[QPTS];
} ccorr;

static void ccorr_init(const orc_mra *m, ccorr *cc) {
    int K = m->K, K2 = 2 * K;
    cc->K = K;
    cc->acc = (double *)calloc((size_t)K * K * K2, sizeof(double));
    orc_gauss_legendre(QPTS, cc->gx, cc->gw);
    double zx[2 * ORC_KMAX], zw[2 * ORC_KMAX];
    orc_gauss_legendre(K2, zx, zw);
    for (int q = 0; q < K2; q++) {
        double z = zx[q];
        double C[ORC_KMAX * ORC_KMAX];
        memset(C, 0, sizeof(C));
        for (int r = 0; r < K; r++) {
            double u = z + (1.0 - z) * m->qx[r];
            double pu[ORC_KMAX], pv[ORC_KMAX];
            orc_basis_eval(m, u, pu);
            orc_basis_eval(m, u - z, pv);
            double wr = m->qw[r] * (1.0 - z);
            for (int i = 0; i < K; i++)
                for (int j = 0; j < K; j++) C[i * K + j] += wr * pu[i] * pv[j];
        }
        double P[2 * ORC_KMAX];
        orc_legendre_all(K2, z, P);
        for (int i = 0; i < K; i++)
            for (int j = 0; j < K; j++)
                for (int p = 0; p < K2; p++) cc->acc[(i * K + j) * K2 + p] += (2.0 * p + 1.0) * zw[q] * C[i * K + j] * P[p];
    }
}

/* G[p] = int_0^1 P_p(2z-1) exp(-beta (z+l)^2) dz, p < np */
static void gauss_moments(const ccorr *cc, double beta, double l, int np, double *G) {
    for (int p = 0; p < np; p++) G[p] = 0.0;
    double c = -l, w = 1.0 / sqrt(beta);
    double lo = c - 12.0 * w, hi = c + 12.0 * w;
    if (lo < 0.0) lo = 0.0;
    if (hi > 1.0) hi = 1.0;
    if (lo >= hi) return;
    double pw = 0.5 * w;
    if (pw > 0.125) pw = 0.125;
    int np_ = (int)ceil((hi - lo) / pw);
    double step = (hi - lo) / np_;
    double P[2 * ORC_KMAX];
    for (int k = 0; k < np_; k++) {
        double a0 = lo + k * step;
        for (int q = 0; q < QPTS; q++) {
            double z = a0 + step * cc->gx[q];
            double e = beta * (z + l) * (z + l);
            if (e > 745.0) continue;
            double g = step * cc->gw[q] * exp(-e);
            orc_legendre_all(np, z, P);
            for (int p = 0; p < np; p++) G[p] += g * P[p];
        }
    }
}

/* tau(m) at scale s (m = translation) for exponent a */
static void make_tau(const ccorr *cc, double a, int s, int m, double *tau) {
    int K = cc->K, K2 = 2 * K;
    double beta = a * pow(4.0, -s), pref = pow(2.0, -s);
    double Gp[2 * ORC_KMAX], Gm[2 * ORC_KMAX];
    gauss_moments(cc, beta, (double)m, K2, Gp);
    gauss_moments(cc, beta, (double)(-m), K2, Gm);
    for (int i = 0; i < K; i++)
        for (int j = 0; j < K; j++) {
            double v = 0.0;
            const double *aij = &cc->acc[(i * K + j) * K2], *aji = &cc->acc[(j * K + i) * K2];
            for (int p = 0; p < K2; p++) v += aij[p] * Gp[p] + aji[p] * Gm[p];
            tau[i * K + j] = pref * v;
        }
}

static void make_ns(const orc_mra *mra, const double *tm1, const double *t0, const double *tp1, double *ns) {
    int K = mra->K, K2 = 2 * K;
    double M[4 * ORC_KMAX * ORC_KMAX], T1[4 * ORC_KMAX * ORC_KMAX];
    for (int i = 0; i < K; i++)
        for (int j = 0; j < K; j++) {
            M[i * K2 + j] = t0[i * K + j];
            M[i * K2 + K + j] = tm1[i * K + j];
            M[(K + i) * K2 + j] = tp1[i * K + j];
            M[(K + i) * K2 + K + j] = t0[i * K + j];
        }
    /* T1 = W M ; ns = T1 W^T */
    for (int r = 0; r < K2; r++)
        for (int c = 0; c < K2; c++) {
            double v = 0.0;
            for (int k = 0; k < K2; k++) v += mra->W[r * K2 + k] * M[k * K2 + c];
            T1[r * K2 + c] = v;
        }
    for (int r = 0; r < K2; r++)
        for (int c = 0; c < K2; c++) {
            double v = 0.0;
            for (int k = 0; k < K2; k++) v += T1[r * K2 + k] * mra->W[c * K2 + k];
            ns[r * K2 + c] = v;
        }
}

static void sub_norms(int K, const double *ns, double *nr) {
    int K2 = 2 * K;
    for (int g = 0; g < 2; g++)
        for (int f = 0; f < 2; f++) {
            double s = 0.0;
            for (int i = 0; i < K; i++)
                for (int j = 0; j < K; j++) {
                    double v = ns[(g * K + i) * K2 + f * K + j];
                    s += v * v;
                }
            nr[2 * g + f] = sqrt(s);
        }
}

static void transpose_block(int K2, const double *in, double *out) {
    for (int r = 0; r < K2; r++)
        for (int c = 0; c < K2; c++) out[c * K2 + r] = in[r * K2 + c];
}

typedef struct {
    int band;
    double *blk; /* (2*band+1) blocks */
    double *nrm;
} tn_data;

static void build_tn(const orc_mra *mra, const ccorr *cc, double a, int n, tn_data *out) {
    int K = mra->K, K2 = 2 * K, bsz = K2 * K2;
    int s = n + 1;
    int root = (n == mra->n0);
    int maxbox = mra->boxes[0];
    for (int d = 1; d < 3; d++)
        if (mra->boxes[d] > maxbox) maxbox = mra->boxes[d];
    long world = (long)maxbox << (n - mra->n0);
    int cap = BAND_CAP;
    if (world - 1 < cap) cap = (int)(world - 1);
    double *pos = NULL, *pnr = NULL; /* blocks for l = 0..L */
    int L = -1;
    double tm1[ORC_KMAX * ORC_KMAX], t0[ORC_KMAX * ORC_KMAX], tp1[ORC_KMAX * ORC_KMAX];
    double peak = 0.0;
    for (int l = 0; l <= cap; l++) {
        make_tau(cc, a, s, 2 * l - 1, tm1);
        make_tau(cc, a, s, 2 * l, t0);
        make_tau(cc, a, s, 2 * l + 1, tp1);
        pos = (double *)realloc(pos, sizeof(double) * bsz * (l + 1));
        pnr = (double *)realloc(pnr, sizeof(double) * 4 * (l + 1));
        make_ns(mra, tm1, t0, tp1, &pos[(size_t)l * bsz]);
        sub_norms(K, &pos[(size_t)l * bsz], &pnr[4 * l]);
        L = l;
        if (root) continue;
        double mx = 0.0, ns = 0.0;
        for (int q = 0; q < 4; q++)
            if (pnr[4 * l + q] > mx) mx = pnr[4 * l + q];
        for (int q = 1; q < 4; q++)
            if (pnr[4 * l + q] > ns) ns = pnr[4 * l + q];
        if (l <= 1 && mx > peak) peak = mx;
        if (l >= 2 && ns < NS_CLEAN * peak) {
            L = l - 1;
            break;
        }
    }
    if (!root) {
        /* clean rounding-level sub-blocks */
        int active = 0;
        for (int l = 0; l <= L; l++)
            for (int g = 0; g < 2; g++)
                for (int f = 0; f < 2; f++) {
                    if (pnr[4 * l + 2 * g + f] < NS_CLEAN * peak) {
                        pnr[4 * l + 2 * g + f] = 0.0;
                        for (int i = 0; i < K; i++)
                            for (int j = 0; j < K; j++) pos[(size_t)l * bsz + (g * K + i) * K2 + f * K + j] = 0.0;
                    } else if (g + f > 0) {
                        active = 1;
                    }
                }
        if (!active) L = -1;
    }
    out->band = L;
    if (L < 0) {
        out->blk = NULL;
        out->nrm = NULL;
        free(pos);
        free(pnr);
        return;
    }
    out->blk = (double *)malloc(sizeof(double) * bsz * (2 * L + 1));
    out->nrm = (double *)malloc(sizeof(double) * 4 * (2 * L + 1));
    for (int l = -L; l <= L; l++) {
        double *dst = &out->blk[(size_t)(l + L) * bsz];
        double *dn = &out->nrm[4 * (l + L)];
        if (l >= 0) {
            memcpy(dst, &pos[(size_t)l * bsz], sizeof(double) * bsz);
            memcpy(dn, &pnr[4 * l], sizeof(double) * 4);
        } else {
            transpose_block(K2, &pos[(size_t)(-l) * bsz], dst);
            /* transposition swaps the (g,f) = (0,1) and (1,0) sub-blocks */
            dn[0] = pnr[4 * (-l) + 0];
            dn[1] = pnr[4 * (-l) + 2];
            dn[2] = pnr[4 * (-l) + 1];
            dn[3] = pnr[4 * (-l) + 3];
        }
    }
    free(pos);
    free(pnr);
}

static orc_oper *oper_create(const orc_mra *mra, int kind, double mu, double prec) {
    orc_oper *op = (orc_oper *)calloc(1, sizeof(orc_oper));
    op->mra = mra;
    op->kind = kind;
    op->mu = mu;
    op->prec = prec;
    op->eps = 0.1 * prec;
    int maxbox = mra->boxes[0];
    for (int d = 1; d < 3; d++)
        if (mra->boxes[d] > maxbox) maxbox = mra->boxes[d];
    op->rmax = sqrt(3.0) * maxbox * ldexp(1.0, -mra->n0);
    op->rmin = ldexp(1.0, -(mra->n0 + mra->max_depth));
    /* trapezoid step: start from the strip-width estimate, shrink until sampled error < eps */
    double h = M_PI * M_PI / (2.0 * log(1.0 / op->eps));
    for (int it = 0; it < 60; it++) {
        make_terms(kind, mu, op->eps, op->rmin, op->rmax, h, &op->T, &op->c, &op->a);
        double err = terms_max_relerr(kind, mu, op->T, op->c, op->a, op->rmin, op->rmax);
        if (err <= op->eps) break;
        free(op->c);
        free(op->a);
        h *= 0.93;
    }
    int K = mra->K, bsz = 4 * K * K;
    op->nscales = mra->max_depth;
    int T = op->T, S = op->nscales;
    ccorr cc;
    ccorr_init(mra, &cc);
    tn_data *tn = (tn_data *)calloc((size_t)T * S, sizeof(tn_data));
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
    for (int t = 0; t < T; t++)
        for (int s = 0; s < S; s++) build_tn(mra, &cc, op->a[t], mra->n0 + s, &tn[t * S + s]);
    op->band = (int *)malloc(sizeof(int) * T * S);
    op->off = (long *)malloc(sizeof(long) * T * S);
    long nb = 0;
    for (int i = 0; i < T * S; i++) {
        op->band[i] = tn[i].band;
        op->off[i] = nb;
        if (tn[i].band >= 0) nb += 2 * tn[i].band + 1;
    }
    op->nblocks = nb;
    op->blocks = (double *)malloc(sizeof(double) * bsz * (nb > 0 ? nb : 1));
    op->norms = (double *)malloc(sizeof(double) * 4 * (nb > 0 ? nb : 1));
    for (int i = 0; i < T * S; i++) {
        if (tn[i].band < 0) continue;
        int cnt = 2 * tn[i].band + 1;
        memcpy(&op->blocks[(size_t)op->off[i] * bsz], tn[i].blk, sizeof(double) * bsz * cnt);
        memcpy(&op->norms[(size_t)op->off[i] * 4], tn[i].nrm, sizeof(double) * 4 * cnt);
        free(tn[i].blk);
        free(tn[i].nrm);
    }
    free(tn);
    free(cc.acc);
    return op;
}

orc_oper *orc_oper_poisson(const orc_mra *mra, double prec) { return oper_create(mra, 0, 0.0, prec); }

orc_oper *orc_oper_helmholtz(const orc_mra *mra, double mu, double prec) {
    if (!(mu > 0.0)) return NULL;
    return oper_create(mra, 1, mu, prec);
}

void orc_oper_free(orc_oper *op) {
    if (!op) return;
    free(op->c);
    free(op->a);
    free(op->band);
    free(op->off);
    free(op->blocks);
    free(op->norms);
    free(op);
}

int orc_oper_nterms(const orc_oper *op) { return op->T; }

void orc_oper_terms(const orc_oper *op, double *coefs, double *exps) {
    for (int t = 0; t < op->T; t++) {
        if (coefs) coefs[t] = op->c[t];
        if (exps) exps[t] = op->a[t];
    }
}

int orc_oper_band(const orc_oper *op, int t, int n) {
    int s = n - op->mra->n0;
    if (t < 0 || t >= op->T || s < 0 || s >= op->nscales) return -1;
    return op->band[t * op->nscales + s];
}

int orc_oper_block(const orc_oper *op, int t, int n, int l, double *blk, double *norms4) {
    int L = orc_oper_band(op, t, n);
    if (L < 0 || l < -L || l > L) return -1;
    int K = op->mra->K, bsz = 4 * K * K;
    long b = op->off[t * op->nscales + (n - op->mra->n0)] + (l + L);
    if (blk) memcpy(blk, &op->blocks[(size_t)b * bsz], sizeof(double) * bsz);
    if (norms4) memcpy(norms4, &op->norms[(size_t)b * 4], sizeof(double) * 4);
    return 0;
}
