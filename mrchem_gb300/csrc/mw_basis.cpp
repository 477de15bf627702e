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
#pragma omp parallel for reduction(max : err) schedule(static)
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

};

}  // namespace

void Oper::build(const Basis &b) { build_operators({this}, b); }

// Builds several operators of one context together: the Gaussian-sum fits on the host, then
// one band walk (phase 1) over every (operator, term, scale), one copy of its results, the
// band cuts on the host, and one launch (phase 2) for all the kept blocks.
void build_operators(const std::vector<Oper *> &ops, const Basis &b) {
    if (ops.empty()) return;
    Ctx &cx = *ops[0]->ctx;
    const int K = b.K, K2 = 2 * K, bsz = K2 * K2;
    const int maxbox = std::max(b.boxes[0], std::max(b.boxes[1], b.boxes[2]));
    // the fits, one operator per host thread (a single operator's error sampling is itself parallel)
#pragma omp parallel for schedule(dynamic, 1) if (ops.size() > 1)
    for (size_t o = 0; o < ops.size(); o++) {
        Oper *op = ops[o];
        op->eps = 0.1 * op->prec;
        op->rmax = std::sqrt(3.0) * maxbox * std::ldexp(1.0, -b.n0);
        op->rmin = std::ldexp(1.0, -(b.n0 + b.max_depth));
        double h = M_PI * M_PI / (2.0 * std::log(1.0 / op->eps));
        for (int it = 0; it < 60; it++) {
            expansion(op->kind, op->mu, op->eps, op->rmin, op->rmax, h, op->c, op->a);
            if (expansion_error(op->kind, op->mu, op->c, op->a, op->rmin, op->rmax) <= op->eps) break;
            h *= 0.93;
        }
        op->T = (int)op->c.size();
        op->S = b.max_depth;
    }
    // phase 1 tasks of all operators, operator after operator
    CrossCorr cc;
    cc.init(b);
    std::vector<int> base(ops.size() + 1, 0);
    for (size_t o = 0; o < ops.size(); o++) base[o + 1] = base[o] + ops[o]->T * ops[o]->S;
    const int ntask = base.back();
    std::vector<OpBuildTask> tasks(ntask);
    long nrm_total = 0;
    for (size_t o = 0; o < ops.size(); o++) {
        const Oper &op = *ops[o];
        for (int t = 0; t < op.T; t++)
            for (int si = 0; si < op.S; si++) {
                const int n = b.n0 + si, sc = n + 1;
                const long world = (long)maxbox << (n - b.n0);
                OpBuildTask &tk = tasks[(size_t)base[o] + (size_t)t * op.S + si];
                tk.beta = op.a[t] * std::pow(4.0, -sc);
                tk.pref = std::pow(2.0, -sc);
                tk.root = n == b.n0 ? 1 : 0;
                tk.cap = (int)std::min<long>(1024, world - 1);
                tk.nrm_off = nrm_total;
                nrm_total += 4L * (tk.cap + 1);
            }
    }
    cudaStream_t st = cx.stream;
    double *d_cc = nullptr, *d_q = nullptr, *d_nrm = nullptr, *d_peak = nullptr, *d_head = nullptr;
    int *d_band = nullptr;
    OpBuildTask *d_tasks = nullptr;
    OpBlockJob *d_jobs = nullptr;
    MWG_CUDA(cudaMalloc(&d_cc, sizeof(double) * cc.coef.size()));
    MWG_CUDA(cudaMalloc(&d_q, sizeof(double) * 2 * 16));
    MWG_CUDA(cudaMalloc(&d_tasks, sizeof(OpBuildTask) * ntask));
    MWG_CUDA(cudaMalloc(&d_nrm, sizeof(double) * nrm_total));
    MWG_CUDA(cudaMalloc(&d_band, sizeof(int) * ntask));
    MWG_CUDA(cudaMalloc(&d_peak, sizeof(double) * ntask));
    MWG_CUDA(cudaMalloc(&d_head, sizeof(double) * ntask * 4 * OP_NRM_HEAD));
    double q[32];
    std::copy(cc.gx, cc.gx + 16, q);
    std::copy(cc.gw, cc.gw + 16, q + 16);
    MWG_CUDA(cudaMemcpyAsync(d_cc, cc.coef.data(), sizeof(double) * cc.coef.size(), cudaMemcpyHostToDevice, st));
    MWG_CUDA(cudaMemcpyAsync(d_q, q, sizeof(q), cudaMemcpyHostToDevice, st));
    MWG_CUDA(cudaMemcpyAsync(d_tasks, tasks.data(), sizeof(OpBuildTask) * ntask, cudaMemcpyHostToDevice, st));
    k_op_band(K, cx.dbasis.W, d_cc, d_q, d_q + 16, d_tasks, ntask, d_nrm, d_head, d_band, d_peak, st);
    std::vector<int> walked(ntask);
    std::vector<double> peak(ntask), head((size_t)ntask * 4 * OP_NRM_HEAD);
    MWG_CUDA(cudaMemcpyAsync(walked.data(), d_band, sizeof(int) * ntask, cudaMemcpyDeviceToHost, st));
    MWG_CUDA(cudaMemcpyAsync(peak.data(), d_peak, sizeof(double) * ntask, cudaMemcpyDeviceToHost, st));
    MWG_CUDA(cudaMemcpyAsync(head.data(), d_head, sizeof(double) * head.size(), cudaMemcpyDeviceToHost, st));
    MWG_CUDA(cudaStreamSynchronize(st));
    // the walked norms: the first OP_NRM_HEAD translations of every task came in one copy, longer
    // walks are fetched one by one
    std::vector<std::vector<double>> pnr(ntask);
    bool fetch = false;
    for (int i = 0; i < ntask; i++) {
        pnr[i].resize(4 * (size_t)(walked[i] + 1));
        if (walked[i] < OP_NRM_HEAD) {
            std::copy(&head[(size_t)i * 4 * OP_NRM_HEAD], &head[(size_t)i * 4 * OP_NRM_HEAD] + pnr[i].size(),
                      pnr[i].begin());
        } else {
            MWG_CUDA(cudaMemcpyAsync(pnr[i].data(), d_nrm + tasks[i].nrm_off, sizeof(double) * pnr[i].size(),
                                     cudaMemcpyDeviceToHost, st));
            fetch = true;
        }
    }
    if (fetch) MWG_CUDA(cudaStreamSynchronize(st));
    // per operator: band cut (sub-blocks below NS_CLEAN x the (t, n) peak are zeroed, and a term
    // with no scaling-wavelet, wavelet-scaling or wavelet-wavelet sub-block left is inactive at
    // n), block offsets, host norm tables, device allocations and phase 2 jobs
    std::vector<OpBlockJob> jobs;
    for (size_t o = 0; o < ops.size(); o++) {
        Oper &op = *ops[o];
        const int nt = op.T * op.S;
        op.band.assign(nt, -1);
        op.off.assign(nt, 0);
        std::vector<std::vector<int>> zero(nt);
        for (int i = 0; i < nt; i++) {
            const int g0 = base[o] + i;
            int L = walked[g0];
            zero[i].assign(L + 1, 0);
            if (!tasks[g0].root) {
                bool active = false;
                for (int l = 0; l <= L; l++)
                    for (int g = 0; g < 2; g++)
                        for (int f = 0; f < 2; f++) {
                            double &v = pnr[g0][4 * l + 2 * g + f];
                            if (v < NS_CLEAN * peak[g0]) {
                                v = 0.0;
                                zero[i][l] |= 1 << (2 * g + f);
                            } else if (g + f > 0) {
                                active = true;
                            }
                        }
                if (!active) L = -1;
            }
            op.band[i] = L;
        }
        op.nblocks = 0;
        for (int i = 0; i < nt; i++) {
            op.off[i] = op.nblocks;
            if (op.band[i] >= 0) op.nblocks += 2 * op.band[i] + 1;
        }
        op.norms.assign((size_t)std::max<long>(op.nblocks, 1) * 4, 0.0);
        op.amax.assign(nt, 0.0);
        op.xmax.assign(nt, 0.0);
        const size_t nel = (size_t)std::max<long>(op.nblocks, 1) * bsz;
        MWG_CUDA(cudaMalloc(&op.d_blocks, sizeof(double) * nel));
        MWG_CUDA(cudaMemsetAsync(op.d_blocks, 0, sizeof(double) * nel, st));
        for (int i = 0; i < nt; i++) {
            const int L = op.band[i];
            if (L < 0) continue;
            const int g0 = base[o] + i;
            for (int l = -L; l <= L; l++) {
                double *dn = &op.norms[(size_t)(op.off[i] + l + L) * 4];
                const double *src = &pnr[g0][4 * std::abs(l)];
                if (l >= 0) {
                    for (int k = 0; k < 4; k++) dn[k] = src[k];
                } else {  // NS(-l) = NS(l)^T swaps the (0,1) and (1,0) sub-blocks
                    dn[0] = src[0];
                    dn[1] = src[2];
                    dn[2] = src[1];
                    dn[3] = src[3];
                }
                for (int k = 0; k < 4; k++) {
                    op.amax[i] = std::max(op.amax[i], dn[k]);
                    if (k > 0) op.xmax[i] = std::max(op.xmax[i], dn[k]);
                }
            }
            for (int l = 0; l <= L; l++) jobs.push_back(OpBlockJob{g0, l, L, zero[i][l], op.off[i], op.d_blocks});
        }
    }
    if (!jobs.empty()) {
        MWG_CUDA(cudaMalloc(&d_jobs, sizeof(OpBlockJob) * jobs.size()));
        MWG_CUDA(cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(OpBlockJob) * jobs.size(), cudaMemcpyHostToDevice, st));
        k_op_blocks(K, cx.dbasis.W, d_cc, d_q, d_q + 16, d_tasks, d_jobs, (int)jobs.size(), st);
    }
    // device copies for the reduced tiers: FP32 high part then low part per block (FP32 and
    // double-FP32 tiers), and the tensor-core tier's B operand (mw_tc05_layout.h)
    const bool tc = K >= 4 && K <= KMAX;
    for (Oper *op : ops) {
        const long nb = std::max<long>(op->nblocks, 1);
        MWG_CUDA(cudaMalloc(&op->d_blocks32, sizeof(float) * 2 * (size_t)nb * bsz));
        if (tc) {
            MWG_CUDA(cudaMalloc(&op->d_blocks_tc, sizeof(float) * tc5_b_stride(K) * (size_t)nb));
            if (tc5_split_wide(K)) MWG_CUDA(cudaMalloc(&op->d_blocks_tc2, sizeof(float) * tc5_b_stride(K) * (size_t)nb));
        }
        k_op_convert(op->d_blocks, op->d_blocks32, tc ? op->d_blocks_tc : nullptr, op->d_blocks_tc2, nb,
                     K, tc5_n(K), 2 * tc5_ks(K), st);
    }
    MWG_CUDA(cudaStreamSynchronize(st));
    for (void *pp : {(void *)d_cc, (void *)d_q, (void *)d_tasks, (void *)d_nrm, (void *)d_band, (void *)d_peak,
                     (void *)d_jobs, (void *)d_head})
        if (pp) cudaFree(pp);
}

void Oper::free_device() {
    if (d_blocks) cudaFree(d_blocks);
    if (d_blocks32) cudaFree(d_blocks32);
    if (d_blocks_tc) cudaFree(d_blocks_tc);
    if (d_blocks_tc2) cudaFree(d_blocks_tc2);
    if (d_screen) cudaFree(d_screen);
    d_blocks = nullptr;
    d_blocks32 = nullptr;
    d_blocks_tc = nullptr;
    d_blocks_tc2 = nullptr;
    d_screen = nullptr;
}

}  // namespace mwg
