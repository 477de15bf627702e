// mw_basis.cpp -- scaling bases, two-scale filters and Gaussian-sum
// convolution operators (host-side set-up, FP64).
//
// Reference-side definitions:
//   MRA parameters            src/mrenv.cpp:99-127, tests/unit_tests.cpp:66-84
//   interpolating basis       tools/legendre_to_interpolating_basis/legendre_to_interpolating.py:17-31
//   PoissonOperator(MRA,prec) src/driver.cpp:1131,1283
//   HelmholtzOperator(MRA,mu,prec) src/scf_solver/HelmholtzVector.cpp:144
// MRCPP (which implements them) is not vendored; the operators follow the
// published trapezoidal Gaussian-sum construction (Harrison et al., JCP 121
// (2004) 11587) and the non-standard form of Beylkin, Coifman & Rokhlin.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mw_host.h"
#include "mw_tc05_layout.h"

namespace mwg {

void gauss_legendre(int n, double *x, double *w) {
    for (int i = 0; i < n; i++) {
        double t = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 1.0;
        auto legendre_pair = [&](double tt, double &p, double &pm) {
            pm = 1.0;
            p = tt;
            for (int j = 2; j <= n; j++) {
                double pn = ((2.0 * j - 1.0) * tt * p - (j - 1.0) * pm) / j;
                pm = p;
                p = pn;
            }
        };
        for (int it = 0; it < 100; it++) {
            double p, pm;
            legendre_pair(t, p, pm);
            dp = n * (t * p - pm) / (t * t - 1.0);
            double dt = p / dp;
            t -= dt;
            if (std::fabs(dt) < 1e-16) break;
        }
        double p, pm;
        legendre_pair(t, p, pm);
        dp = n * (t * p - pm) / (t * t - 1.0);
        x[i] = 0.5 * (1.0 - t);
        w[i] = 1.0 / ((1.0 - t * t) * dp * dp);
    }
}

void legendre_shifted(int n, double x, double *p) {
    double t = 2.0 * x - 1.0;
    if (n > 0) p[0] = 1.0;
    if (n > 1) p[1] = t;
    for (int j = 1; j + 1 < n; j++) p[j + 1] = ((2.0 * j + 1.0) * t * p[j] - j * p[j - 1]) / (j + 1.0);
}

static void legendre_scaling(int K, double x, double *out) {
    legendre_shifted(K, x, out);
    for (int j = 0; j < K; j++) out[j] *= std::sqrt(2.0 * j + 1.0);
}

void Basis::eval(double x, double *out) const {
    if (type == MW_BASIS_LEGENDRE) {
        legendre_scaling(K, x, out);
        return;
    }
    double pl[KMAX + 2];
    legendre_scaling(K, x, pl);
    for (int j = 0; j < K; j++) {
        double s = 0.0;
        for (int i = 0; i < K; i++) s += legq[j * K + i] * pl[i];
        out[j] = std::sqrt(qw[j]) * s;
    }
}

bool Basis::in_world(int n, const int *l) const {
    int sh = n - n0;
    for (int d = 0; d < 3; d++) {
        long lo = (long)corner[d] * (1L << sh), hi = (long)(corner[d] + boxes[d]) * (1L << sh);
        if (l[d] < lo || l[d] >= hi) return false;
    }
    return true;
}

void Basis::init(int root_scale, const int *c, const int *b, int order, int tp, int md) {
    n0 = root_scale;
    for (int d = 0; d < 3; d++) {
        corner[d] = c[d];
        boxes[d] = b[d];
    }
    k = order;
    K = order + 1;
    type = tp;
    max_depth = md;
    bs = 8 * K * K * K;
    qx.assign(K, 0.0);
    qw.assign(K, 0.0);
    gauss_legendre(K, qx.data(), qw.data());
    legq.assign(K * K, 0.0);
    for (int j = 0; j < K; j++) legendre_scaling(K, qx[j], &legq[j * K]);
    c2v.assign(K * K, 0.0);
    v2c.assign(K * K, 0.0);
    for (int q = 0; q < K; q++) {
        double ph[KMAX + 2];
        eval(qx[q], ph);
        for (int j = 0; j < K; j++) {
            c2v[q * K + j] = ph[j];
            v2c[j * K + q] = qw[q] * ph[j];
        }
    }
    integ.assign(K, 0.0);
    for (int j = 0; j < K; j++)
        for (int q = 0; q < K; q++) integ[j] += qw[q] * c2v[q * K + j];
    // filter W: rows 0..K-1 scaling (H0 | H1), rows K..2K-1 wavelets (G0 | G1)
    int K2 = 2 * K;
    W.assign(K2 * K2, 0.0);
    for (int q = 0; q < K; q++) {
        double a0[KMAX + 2], a1[KMAX + 2], bq[KMAX + 2];
        eval(0.5 * qx[q], a0);
        eval(0.5 * (qx[q] + 1.0), a1);
        eval(qx[q], bq);
        for (int i = 0; i < K; i++)
            for (int j = 0; j < K; j++) {
                W[i * K2 + j] += M_SQRT1_2 * qw[q] * a0[i] * bq[j];
                W[i * K2 + K + j] += M_SQRT1_2 * qw[q] * a1[i] * bq[j];
            }
    }
    // wavelet rows: two-pass Gram-Schmidt of (e_j, -e_j)/sqrt2 against all earlier rows
    for (int j = 0; j < K; j++) {
        std::vector<double> v(K2, 0.0);
        v[j] = M_SQRT1_2;
        v[K + j] = -M_SQRT1_2;
        for (int pass = 0; pass < 2; pass++) {
            for (int r = 0; r < K + j; r++) {
                double dot = 0.0;
                for (int cc = 0; cc < K2; cc++) dot += W[r * K2 + cc] * v[cc];
                for (int cc = 0; cc < K2; cc++) v[cc] -= dot * W[r * K2 + cc];
            }
            double nrm = 0.0;
            for (double e : v) nrm += e * e;
            nrm = std::sqrt(nrm);
            for (double &e : v) e /= nrm;
        }
        for (int cc = 0; cc < K2; cc++) W[(K + j) * K2 + cc] = v[cc];
    }
    WT.assign(K2 * K2, 0.0);
    for (int r = 0; r < K2; r++)
        for (int cc = 0; cc < K2; cc++) WT[cc * K2 + r] = W[r * K2 + cc];
}

// ------------------------------------------------------------------ operators

namespace {

constexpr int QPTS = 16;

double erfc_inverse(double y) {
    double lo = 0.0, hi = 30.0;
    for (int i = 0; i < 200; i++) {
        double mid = 0.5 * (lo + hi);
        (std::erfc(mid) > y ? lo : hi) = mid;
    }
    return 0.5 * (lo + hi);
}

void expansion(int kind, double mu, double eps, double rmin, double rmax, double h, std::vector<double> &c,
               std::vector<double> &a) {
    double s_lo = std::log(eps * std::sqrt(M_PI) / (8.0 * rmax));
    double s_hi = std::log(erfc_inverse(0.25 * eps) / rmin);
    int n = (int)std::ceil((s_hi - s_lo) / h) + 1;
    c.clear();
    a.clear();
    for (int j = 0; j < n; j++) {
        double s = s_lo + h * j;
        double cj = 2.0 * h / std::sqrt(M_PI) * std::exp(s);
        if (kind == 1) cj *= std::exp(-0.25 * mu * mu * std::exp(-2.0 * s));
        double aj = std::exp(2.0 * s);
        if (cj / std::sqrt(2.0 * M_E * aj) < 0.01 * eps / n) continue;
        c.push_back(cj);
        a.push_back(aj);
    }
}

double expansion_error(int kind, double mu, const std::vector<double> &c, const std::vector<double> &a, double rmin,
                       double rmax) {
    double err = 0.0;
    const int N = 4000;
    for (int i = 0; i <= N; i++) {
        double r = rmin * std::pow(rmax / rmin, (double)i / N), v = 0.0;
        for (size_t t = 0; t < c.size(); t++) v += c[t] * std::exp(-a[t] * r * r);
        double ex = kind == 1 ? std::exp(-mu * r) / r : 1.0 / r;
        err = std::max(err, std::fabs(v - ex) * r);
    }
    return err;
}

// Legendre expansion of the scaling-function cross-correlations
//   C_ij(z) = int phi_i(u) phi_j(u - z) du,  z in [0,1]
struct CrossCorr {
    int K = 0;
    std::vector<double> coef;  // [(i*K + j)*2K + p]
    double gx[QPTS], gw[QPTS];

    void init(const Basis &b) {
        K = b.K;
        int K2 = 2 * K;
        coef.assign((size_t)K * K * K2, 0.0);
        gauss_legendre(QPTS, gx, gw);
        std::vector<double> zx(K2), zw(K2);
        gauss_legendre(K2, zx.data(), zw.data());
        for (int q = 0; q < K2; q++) {
            double z = zx[q];
            std::vector<double> Cz(K * K, 0.0);
            for (int r = 0; r < K; r++) {
                double u = z + (1.0 - z) * b.qx[r], pu[KMAX + 2], pv[KMAX + 2];
                b.eval(u, pu);
                b.eval(u - z, pv);
                double wr = b.qw[r] * (1.0 - z);
                for (int i = 0; i < K; i++)
                    for (int j = 0; j < K; j++) Cz[i * K + j] += wr * pu[i] * pv[j];
            }
            double P[2 * KMAX + 2];
            legendre_shifted(K2, z, P);
            for (int i = 0; i < K; i++)
                for (int j = 0; j < K; j++)
                    for (int p = 0; p < K2; p++) coef[(i * K + j) * K2 + p] += (2.0 * p + 1.0) * zw[q] * Cz[i * K + j] * P[p];
        }
    }

    // G[p] = int_0^1 P_p(2z-1) exp(-beta (z + l)^2) dz
    void moments(double beta, double l, int np, double *G) const {
        std::fill(G, G + np, 0.0);
        double c0 = -l, w = 1.0 / std::sqrt(beta);
        double lo = std::max(0.0, c0 - 12.0 * w), hi = std::min(1.0, c0 + 12.0 * w);
        if (lo >= hi) return;
        double pw = std::min(0.125, 0.5 * w);
        int npc = (int)std::ceil((hi - lo) / pw);
        double step = (hi - lo) / npc;
        double P[2 * KMAX + 2];
        for (int k = 0; k < npc; k++) {
            double a0 = lo + k * step;
            for (int q = 0; q < QPTS; q++) {
                double z = a0 + step * gx[q], e = beta * (z + l) * (z + l);
                if (e > 745.0) continue;
                double g = step * gw[q] * std::exp(-e);
                legendre_shifted(np, z, P);
                for (int p = 0; p < np; p++) G[p] += g * P[p];
            }
        }
    }

    // tau(m)_{ij} = 2^{-s} int int phi_i(u) phi_j(v) exp(-a 4^{-s} (u - v + m)^2)
    void tau(double a, int s, int m, double *out) const {
        int K2 = 2 * K;
        double beta = a * std::pow(4.0, -s), pref = std::pow(2.0, -s);
        double Gp[2 * KMAX + 2], Gm[2 * KMAX + 2];
        moments(beta, (double)m, K2, Gp);
        moments(beta, (double)(-m), K2, Gm);
        for (int i = 0; i < K; i++)
            for (int j = 0; j < K; j++) {
                const double *aij = &coef[(i * K + j) * K2], *aji = &coef[(j * K + i) * K2];
                double v = 0.0;
                for (int p = 0; p < K2; p++) v += aij[p] * Gp[p] + aji[p] * Gm[p];
                out[i * K + j] = pref * v;
            }
    }
};

struct TermScale {
    int band = -1;
    std::vector<double> blk, nrm;
};

void ns_block(const Basis &b, const double *tm1, const double *t0, const double *tp1, double *ns) {
    int K = b.K, K2 = 2 * K;
    std::vector<double> M(K2 * K2), T1(K2 * K2);
    for (int i = 0; i < K; i++)
        for (int j = 0; j < K; j++) {
            M[i * K2 + j] = t0[i * K + j];
            M[i * K2 + K + j] = tm1[i * K + j];
            M[(K + i) * K2 + j] = tp1[i * K + j];
            M[(K + i) * K2 + K + j] = t0[i * K + j];
        }
    for (int r = 0; r < K2; r++)
        for (int c = 0; c < K2; c++) {
            double v = 0.0;
            for (int k = 0; k < K2; k++) v += b.W[r * K2 + k] * M[k * K2 + c];
            T1[r * K2 + c] = v;
        }
    for (int r = 0; r < K2; r++)
        for (int c = 0; c < K2; c++) {
            double v = 0.0;
            for (int k = 0; k < K2; k++) v += T1[r * K2 + k] * b.W[c * K2 + k];
            ns[r * K2 + c] = v;
        }
}

void sub_norms(int K, const double *ns, double *nr) {
    int K2 = 2 * K;
    for (int g = 0; g < 2; g++)
        for (int f = 0; f < 2; f++) {
            double s = 0.0;
            for (int i = 0; i < K; i++)
                for (int j = 0; j < K; j++) {
                    double v = ns[(g * K + i) * K2 + f * K + j];
                    s += v * v;
                }
            nr[2 * g + f] = std::sqrt(s);
        }
}

void term_scale(const Basis &b, const CrossCorr &cc, double a, int n, TermScale &out) {
    int K = b.K, K2 = 2 * K, bsz = K2 * K2, s = n + 1;
    bool root = (n == b.n0);
    int maxbox = std::max(b.boxes[0], std::max(b.boxes[1], b.boxes[2]));
    long world = (long)maxbox << (n - b.n0);
    int cap = (int)std::min<long>(1024, world - 1);
    std::vector<double> pos, pnr;
    std::vector<double> tm1(K * K), t0(K * K), tp1(K * K);
    int L = -1;
    double peak = 0.0;
    for (int l = 0; l <= cap; l++) {
        cc.tau(a, s, 2 * l - 1, tm1.data());
        cc.tau(a, s, 2 * l, t0.data());
        cc.tau(a, s, 2 * l + 1, tp1.data());
        pos.resize((size_t)bsz * (l + 1));
        pnr.resize(4 * (l + 1));
        ns_block(b, tm1.data(), t0.data(), tp1.data(), &pos[(size_t)l * bsz]);
        sub_norms(K, &pos[(size_t)l * bsz], &pnr[4 * l]);
        L = l;
        if (root) continue;
        double mx = *std::max_element(&pnr[4 * l], &pnr[4 * l] + 4);
        double nsn = std::max(pnr[4 * l + 1], std::max(pnr[4 * l + 2], pnr[4 * l + 3]));
        if (l <= 1) peak = std::max(peak, mx);
        if (l >= 2 && nsn < NS_CLEAN * peak) {
            L = l - 1;
            break;
        }
    }
    if (!root) {
        bool active = false;
        for (int l = 0; l <= L; l++)
            for (int g = 0; g < 2; g++)
                for (int f = 0; f < 2; f++) {
                    if (pnr[4 * l + 2 * g + f] < NS_CLEAN * peak) {
                        pnr[4 * l + 2 * g + f] = 0.0;
                        for (int i = 0; i < K; i++)
                            for (int j = 0; j < K; j++) pos[(size_t)l * bsz + (g * K + i) * K2 + f * K + j] = 0.0;
                    } else if (g + f > 0) {
                        active = true;
                    }
                }
        if (!active) L = -1;
    }
    out.band = L;
    if (L < 0) return;
    out.blk.assign((size_t)bsz * (2 * L + 1), 0.0);
    out.nrm.assign(4 * (2 * L + 1), 0.0);
    for (int l = -L; l <= L; l++) {
        double *dst = &out.blk[(size_t)(l + L) * bsz];
        double *dn = &out.nrm[4 * (l + L)];
        if (l >= 0) {
            std::memcpy(dst, &pos[(size_t)l * bsz], sizeof(double) * bsz);
            std::memcpy(dn, &pnr[4 * l], sizeof(double) * 4);
        } else {
            // NS(-l) = NS(l)^T; transposition swaps the (0,1) and (1,0) sub-blocks
            const double *src = &pos[(size_t)(-l) * bsz];
            for (int r = 0; r < K2; r++)
                for (int c = 0; c < K2; c++) dst[c * K2 + r] = src[r * K2 + c];
            dn[0] = pnr[4 * (-l) + 0];
            dn[1] = pnr[4 * (-l) + 2];
            dn[2] = pnr[4 * (-l) + 1];
            dn[3] = pnr[4 * (-l) + 3];
        }
    }
}

}  // namespace

void Oper::build(const Basis &b) {
    eps = 0.1 * prec;
    int maxbox = std::max(b.boxes[0], std::max(b.boxes[1], b.boxes[2]));
    rmax = std::sqrt(3.0) * maxbox * std::ldexp(1.0, -b.n0);
    rmin = std::ldexp(1.0, -(b.n0 + b.max_depth));
    double h = M_PI * M_PI / (2.0 * std::log(1.0 / eps));
    for (int it = 0; it < 60; it++) {
        expansion(kind, mu, eps, rmin, rmax, h, c, a);
        if (expansion_error(kind, mu, c, a, rmin, rmax) <= eps) break;
        h *= 0.93;
    }
    T = (int)c.size();
    S = b.max_depth;
    CrossCorr cc;
    cc.init(b);
    std::vector<TermScale> ts((size_t)T * S);
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
    for (int t = 0; t < T; t++)
        for (int s = 0; s < S; s++) term_scale(b, cc, a[t], b.n0 + s, ts[(size_t)t * S + s]);
    band.assign(T * S, -1);
    off.assign(T * S, 0);
    nblocks = 0;
    for (int i = 0; i < T * S; i++) {
        band[i] = ts[i].band;
        off[i] = nblocks;
        if (ts[i].band >= 0) nblocks += 2 * ts[i].band + 1;
    }
    int K = b.K, bsz = 4 * K * K;
    std::vector<double> blocks((size_t)std::max<long>(nblocks, 1) * bsz, 0.0);
    norms.assign((size_t)std::max<long>(nblocks, 1) * 4, 0.0);
    amax.assign(T * S, 0.0);
    xmax.assign(T * S, 0.0);
    for (int i = 0; i < T * S; i++) {
        if (ts[i].band < 0) continue;
        int cnt = 2 * ts[i].band + 1;
        std::memcpy(&blocks[(size_t)off[i] * bsz], ts[i].blk.data(), sizeof(double) * bsz * cnt);
        std::memcpy(&norms[(size_t)off[i] * 4], ts[i].nrm.data(), sizeof(double) * 4 * cnt);
        for (int q = 0; q < 4 * cnt; q++) {
            amax[i] = std::max(amax[i], ts[i].nrm[q]);
            if (q % 4 > 0) xmax[i] = std::max(xmax[i], ts[i].nrm[q]);
        }
    }
    // device copies: FP64, and FP32 for the reduced tiers.  Each FP32 block is its high part (the
    // value rounded to FP32, read by the FP32 and TF32 tiers) followed by its low part (the
    // rounded remainder, read with the high part by the double-FP32 tier).
    size_t nel = blocks.size();
    std::vector<float> b32(2 * nel);
    for (size_t i = 0; i < nel; i++) {
        const size_t blk = i / (size_t)bsz, r = i - blk * (size_t)bsz;
        const float h = (float)blocks[i];
        b32[2 * blk * bsz + r] = h;
        b32[2 * blk * bsz + bsz + r] = (float)(blocks[i] - (double)h);
    }
    MWG_CUDA(cudaMalloc(&d_blocks, sizeof(double) * nel));
    MWG_CUDA(cudaMalloc(&d_blocks32, sizeof(float) * 2 * nel));
    MWG_CUDA(cudaMemcpy(d_blocks, blocks.data(), sizeof(double) * nel, cudaMemcpyHostToDevice));
    MWG_CUDA(cudaMemcpy(d_blocks32, b32.data(), sizeof(float) * 2 * nel, cudaMemcpyHostToDevice));
    // the tensor-core tier's B operand of every block (mw_tc05_layout.h): k-groups of 4 columns,
    // rows n < 2K = A[n][k], rows 2K + i (i < K) = A[i][k] for k >= K (zero for k < K), TF32
    if (K >= 4 && K <= KMAX) {
        const int N2 = 2 * K, NB = tc5_n(K);
        const size_t per = tc5_b_floats(K), nb = nel / (size_t)bsz;
        std::vector<float> tc(per * nb, 0.0f);
        for (size_t blk = 0; blk < nb; blk++) {
            const float *h = &b32[2 * blk * bsz];
            float *o = &tc[blk * per];
            for (int n = 0; n < NB; n++)
                for (int k = 0; k < N2; k++) {
                    float v = 0.0f;
                    if (n < N2)
                        v = h[n * N2 + k];
                    else if (n < N2 + K && k >= K)
                        v = h[(n - N2) * N2 + k];
                    o[((size_t)(k / 4) * NB + n) * 4 + (k % 4)] = tf32_round_host(v);
                }
        }
        MWG_CUDA(cudaMalloc(&d_blocks_tc, sizeof(float) * tc.size()));
        MWG_CUDA(cudaMemcpy(d_blocks_tc, tc.data(), sizeof(float) * tc.size(), cudaMemcpyHostToDevice));
    }
}

}  // namespace mwg
