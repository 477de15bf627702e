// mw_opbuild.cu -- the non-standard-form blocks of a separated-Gaussian operator, built on the GPU.
//
// For term t (exponent a) at scale n (s = n + 1) the 1-D NS block of translation l is
//   NS_n(l) = W [[tau(2l), tau(2l-1)], [tau(2l+1), tau(2l)]] W^T,
//   tau(m)_ij = 2^-s int int phi_i(u) phi_j(v) exp(-a 4^-s (u - v + m)^2) du dv,
// evaluated through the Legendre expansion of the scaling functions' cross-correlation (degree
// 2K-1, coefficients prepared on the host) against Gaussian moments
//   G[p] = int_0^1 P_p(2z-1) exp(-beta (z + m)^2) dz
// by composite 16-point Gauss-Legendre quadrature, as the host construction does (mw_basis.cpp).
//
// Phase 1 (one CTA per (term, scale)) walks l = 0, 1, ... and keeps only the four sub-block
// norms of each NS(l), stopping where the host construction stops: the band follows from them.
// Phase 2 (one CTA per (term, scale, l) inside the band) recomputes the block, zeroes the
// sub-blocks the host marked, and writes NS(l) and NS(-l) = NS(l)^T at their final places.
// All arithmetic is FP64; the quadrature points of a moment are spread over the CTA's threads
// and their partial sums added in a fixed order, so the blocks are reproducible.
#include "mw_host.h"

namespace mwg {

namespace {

constexpr int OB_THREADS = 128;
constexpr int OB_QPTS = 16;

struct ObShared {
    double G[2][2 * KMAX + 2];              // moments of +m and -m
    double red[OB_THREADS][2 * KMAX + 2];   // partial sums of the threads
    double tm1[KMAX * KMAX], t0[KMAX * KMAX], tp1[KMAX * KMAX];
    double M[4 * KMAX * KMAX], T1[4 * KMAX * KMAX], ns[4 * KMAX * KMAX];
    double nrm[4];
    double gx[OB_QPTS], gw[OB_QPTS];
};

// G[p] = int_0^1 P_p(2z-1) exp(-beta (z + l)^2) dz, p < np, into S.G[slot] (all threads call)
__device__ void ob_moments(double beta, double l, int np, int slot, ObShared &S) {
    const int tid = threadIdx.x;
    double acc[2 * KMAX + 2];
#pragma unroll
    for (int p = 0; p < 2 * KMAX + 2; p++) acc[p] = 0.0;
    const double c0 = -l, w = 1.0 / sqrt(beta);
    const double lo = fmax(0.0, c0 - 12.0 * w), hi = fmin(1.0, c0 + 12.0 * w);
    if (lo < hi) {
        const double pw = fmin(0.125, 0.5 * w);
        const int npc = (int)ceil((hi - lo) / pw);
        const double step = (hi - lo) / npc;
        for (int i = tid; i < npc * OB_QPTS; i += blockDim.x) {
            const int k = i / OB_QPTS, q = i - k * OB_QPTS;
            const double z = (lo + k * step) + step * S.gx[q], e = beta * (z + l) * (z + l);
            if (e > 745.0) continue;
            const double g = step * S.gw[q] * exp(-e);
            const double t = 2.0 * z - 1.0;
            double pm = 1.0, pc = t;
            acc[0] += g;
            acc[1] += g * t;
#pragma unroll
            for (int j = 1; j + 1 < 2 * KMAX + 2; j++) {  // P_{j+1} by the three-term recurrence
                if (j + 1 >= np) break;
                const double pn = ((2.0 * j + 1.0) * t * pc - j * pm) / (j + 1.0);
                acc[j + 1] += g * pn;
                pm = pc;
                pc = pn;
            }
        }
    }
#pragma unroll
    for (int p = 0; p < 2 * KMAX + 2; p++)
        if (p < np) S.red[tid][p] = acc[p];
    __syncthreads();
    if (tid < np) {
        double s = 0.0;
        for (int r = 0; r < (int)blockDim.x; r++) s += S.red[r][tid];
        S.G[slot][tid] = s;
    }
    __syncthreads();
}

// out = tau(m) (K x K), all threads call
__device__ void ob_tau(int K, double beta, double pref, int m, const double *cc, ObShared &S, double *out) {
    const int K2 = 2 * K;
    ob_moments(beta, (double)m, K2, 0, S);
    ob_moments(beta, (double)(-m), K2, 1, S);
    for (int e = threadIdx.x; e < K * K; e += blockDim.x) {
        const int i = e / K, j = e - i * K;
        const double *aij = cc + (size_t)(i * K + j) * K2, *aji = cc + (size_t)(j * K + i) * K2;
        double v = 0.0;
        for (int p = 0; p < K2; p++) v += aij[p] * S.G[0][p] + aji[p] * S.G[1][p];
        out[e] = pref * v;
    }
    __syncthreads();
}

// S.ns = W [[t0, tm1], [tp1, t0]] W^T and its four sub-block norms, all threads call
__device__ void ob_ns(int K, const double *W, ObShared &S) {
    const int K2 = 2 * K, KK2 = K2 * K2;
    for (int e = threadIdx.x; e < KK2; e += blockDim.x) {
        const int r = e / K2, c = e - r * K2, i = r % K, j = c % K;
        const double *src = r < K ? (c < K ? S.t0 : S.tm1) : (c < K ? S.tp1 : S.t0);
        S.M[e] = src[i * K + j];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < KK2; e += blockDim.x) {
        const int r = e / K2, c = e - r * K2;
        double v = 0.0;
        for (int k = 0; k < K2; k++) v += W[r * K2 + k] * S.M[k * K2 + c];
        S.T1[e] = v;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < KK2; e += blockDim.x) {
        const int r = e / K2, c = e - r * K2;
        double v = 0.0;
        for (int k = 0; k < K2; k++) v += S.T1[r * K2 + k] * W[c * K2 + k];
        S.ns[e] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        const int g = threadIdx.x >> 1, f = threadIdx.x & 1;
        double s = 0.0;
        for (int i = 0; i < K; i++)
            for (int j = 0; j < K; j++) {
                const double v = S.ns[(g * K + i) * K2 + f * K + j];
                s += v * v;
            }
        S.nrm[threadIdx.x] = sqrt(s);
    }
    __syncthreads();
}

__device__ void ob_setup(const double *gx, const double *gw, ObShared &S) {
    if (threadIdx.x < OB_QPTS) {
        S.gx[threadIdx.x] = gx[threadIdx.x];
        S.gw[threadIdx.x] = gw[threadIdx.x];
    }
    __syncthreads();
}

// phase 1: per task the sub-block norms of NS(0..L) and L, where the walk stops
__global__ void __launch_bounds__(OB_THREADS) op_band_kernel(int K, const double *W, const double *cc, const double *gx,
                                                             const double *gw, const OpBuildTask *tasks, int ntask,
                                                             double *nrm, double *head, int *band, double *peak) {
    extern __shared__ __align__(16) unsigned char ob_smem[];
    ObShared &S = *reinterpret_cast<ObShared *>(ob_smem);
    ob_setup(gx, gw, S);
    for (int t = blockIdx.x; t < ntask; t += gridDim.x) {
        const OpBuildTask T = tasks[t];
        double *tn = nrm + T.nrm_off;
        double pk = 0.0;
        int L = -1;
        for (int l = 0; l <= T.cap; l++) {
            if (l == 0) {
                ob_tau(K, T.beta, T.pref, -1, cc, S, S.tm1);
                ob_tau(K, T.beta, T.pref, 0, cc, S, S.t0);
            } else {
                // tau(2l-1) is the previous step's tau(2l+1)
                for (int e = threadIdx.x; e < K * K; e += blockDim.x) S.tm1[e] = S.tp1[e];
                __syncthreads();
                ob_tau(K, T.beta, T.pref, 2 * l, cc, S, S.t0);
            }
            ob_tau(K, T.beta, T.pref, 2 * l + 1, cc, S, S.tp1);
            ob_ns(K, W, S);
            if (threadIdx.x < 4) {
                tn[4 * l + threadIdx.x] = S.nrm[threadIdx.x];
                if (l < OP_NRM_HEAD) head[((size_t)t * OP_NRM_HEAD + l) * 4 + threadIdx.x] = S.nrm[threadIdx.x];
            }
            L = l;
            bool stop = false;
            if (!T.root) {
                const double mx = fmax(fmax(S.nrm[0], S.nrm[1]), fmax(S.nrm[2], S.nrm[3]));
                const double nsn = fmax(S.nrm[1], fmax(S.nrm[2], S.nrm[3]));
                if (l <= 1) pk = fmax(pk, mx);
                if (l >= 2 && nsn < NS_CLEAN * pk) {
                    L = l - 1;
                    stop = true;
                }
            }
            __syncthreads();
            if (stop) break;
        }
        if (threadIdx.x == 0) {
            band[t] = L;
            peak[t] = pk;
        }
    }
}

// phase 2: block l of task `task` (one CTA per (task, l) pair); zero: 4 bits, sub-blocks to zero
__global__ void __launch_bounds__(OB_THREADS) op_block_kernel(int K, const double *W, const double *cc, const double *gx,
                                                              const double *gw, const OpBuildTask *tasks,
                                                              const OpBlockJob *jobs, int njob) {
    extern __shared__ __align__(16) unsigned char ob_smem[];
    ObShared &S = *reinterpret_cast<ObShared *>(ob_smem);
    ob_setup(gx, gw, S);
    const int K2 = 2 * K, bsz = K2 * K2;
    for (int q = blockIdx.x; q < njob; q += gridDim.x) {
        const OpBlockJob J = jobs[q];
        const OpBuildTask T = tasks[J.task];
        const int l = J.l;
        ob_tau(K, T.beta, T.pref, 2 * l - 1, cc, S, S.tm1);
        ob_tau(K, T.beta, T.pref, 2 * l, cc, S, S.t0);
        ob_tau(K, T.beta, T.pref, 2 * l + 1, cc, S, S.tp1);
        ob_ns(K, W, S);
        double *pos = J.blocks + (size_t)(J.off + J.band + l) * bsz;
        double *neg = J.blocks + (size_t)(J.off + J.band - l) * bsz;
        for (int e = threadIdx.x; e < bsz; e += blockDim.x) {
            const int r = e / K2, c = e - r * K2;
            const int g = r / K, f = c / K;
            const double v = (J.zero >> (2 * g + f)) & 1 ? 0.0 : S.ns[e];
            pos[e] = v;
            if (l > 0) neg[c * K2 + r] = v;  // NS(-l) = NS(l)^T
        }
        __syncthreads();
    }
}

// FP32 high and low parts of every block, and the tensor-core tier's B operand (mw_tc05_layout.h)
// round to TF32: nearest, ties away from zero (infinities and NaNs unchanged)
__device__ __forceinline__ float tf32_round(float v) {
    uint32_t u = __float_as_uint(v);
    if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0x1000u) & ~0x1fffu;
    return __uint_as_float(u);
}

__global__ void op_convert_kernel(const double *blocks, float *b32, float *btc, float *btc2, long nblocks, int K,
                                  int NB, int groups) {
    const int N2 = 2 * K, bsz = N2 * N2;
    const size_t total = (size_t)nblocks * bsz;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t blk = i / bsz;
        const int r = (int)(i - blk * bsz);
        const double d = blocks[i];
        const float h = __double2float_rn(d);
        b32[2 * blk * bsz + r] = h;
        b32[2 * blk * bsz + bsz + r] = __double2float_rn(d - (double)h);
    }
    if (!btc) return;
    // per block: the B operand rounded to TF32 (hi), then the remainder rounded to TF32 (lo)
    const size_t per = (size_t)groups * NB * 4, ttot = (size_t)nblocks * per;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ttot; i += (size_t)gridDim.x * blockDim.x) {
        const size_t blk = i / per;
        const int rem = (int)(i - blk * per), g = rem / (NB * 4), n = (rem / 4) % NB, c = rem % 4, k = 4 * g + c;
        double d = 0.0;
        if (k < N2) {
            const size_t base = blk * bsz;
            if (n < N2)
                d = blocks[base + (size_t)n * N2 + k];
            else if (n < N2 + K && k >= K)
                d = blocks[base + (size_t)(n - N2) * N2 + k];
        }
        const float h = tf32_round(__double2float_rn(d));
        const float l = tf32_round(__double2float_rn(d - (double)h));
        btc[2 * blk * per + rem] = h;
        btc[2 * blk * per + per + rem] = l;
        if (btc2) {  // the split tier's layout: per k-group its NB hi rows, then its NB lo rows
            const size_t gb = 2 * blk * per + (size_t)g * 2 * NB * 4 + (size_t)(rem % (NB * 4));
            btc2[gb] = h;
            btc2[gb + NB * 4] = l;
        }
    }
}

}  // namespace

size_t op_build_smem() { return sizeof(ObShared); }

void k_op_band(int K, const double *W, const double *cc, const double *gx, const double *gw, const OpBuildTask *tasks,
               int ntask, double *nrm, double *head, int *band, double *peak, cudaStream_t s) {
    if (ntask <= 0) return;
    const int smem = (int)sizeof(ObShared);
    MWG_CUDA(cudaFuncSetAttribute(op_band_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    op_band_kernel<<<ntask, OB_THREADS, smem, s>>>(K, W, cc, gx, gw, tasks, ntask, nrm, head, band, peak);
    MWG_CUDA(cudaGetLastError());
}

void k_op_blocks(int K, const double *W, const double *cc, const double *gx, const double *gw, const OpBuildTask *tasks,
                 const OpBlockJob *jobs, int njob, cudaStream_t s) {
    if (njob <= 0) return;
    const int smem = (int)sizeof(ObShared);
    MWG_CUDA(cudaFuncSetAttribute(op_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    op_block_kernel<<<njob < 65535 ? njob : 65535, OB_THREADS, smem, s>>>(K, W, cc, gx, gw, tasks, jobs, njob);
    MWG_CUDA(cudaGetLastError());
}

void k_op_convert(const double *blocks, float *b32, float *btc, float *btc2, long nblocks, int K, int NB, int groups,
                  cudaStream_t s) {
    if (nblocks <= 0) return;
    op_convert_kernel<<<1024, 256, 0, s>>>(blocks, b32, btc, btc2, nblocks, K, NB, groups);
    MWG_CUDA(cudaGetLastError());
}

}  // namespace mwg
