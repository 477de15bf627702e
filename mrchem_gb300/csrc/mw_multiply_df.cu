// mw_multiply_df.cu -- the tree multiply's node kernels in double-FP32 arithmetic.
//
// mrcpp::multiply (QMPotential.cpp:147, ExchangePotential.cpp:175) computes every end node of the
// output grid from the two input blocks at that node:
//   values   each input block is reconstructed to the children's scaling coefficients (W^T along
//            each dimension) and mapped to function values at the children's Gauss-Legendre points
//            (the K x K map c2v on each half of each dimension);
//   product  the values are multiplied pointwise, times coef * 2^{3(n+1)/2};
//   back     the product values are mapped back to coefficients (v2c on each half) and compressed
//            into the node's block (W along each dimension), with its 8 component norms.
// Per dimension the two forward steps are one 2K x 2K matrix, M_in = diag(c2v, c2v) W^T, and the
// two backward steps another, M_out = W diag(v2c, v2c), both formed in FP64 in each CTA's prologue.
// values_df_kernel maps blocks to value cubes (three line passes with M_in); a value cube depends
// only on its block, so an input tree that feeds several products (the exchange-like 528 pair
// products share 32 orbitals) has each node's cube computed once per batch.
// multiply_values_df_kernel forms a node from two value cubes: the product, then three line passes
// with M_out, the last writing the FP64 block and its norms.
//
// Arithmetic: every value is an unevaluated FP32 pair (hi + lo) and every multiply-add is the
// error-free double-FP32 update of the apply's double-FP32 tier, as in the post-processing
// transforms (mw_post_df.cu): about (2K + 4) 2^-48 of sum |M| |x| per pass, 1e-14 relative, at
// about 8x GB300's FP64 rate.  Blocks in global memory stay FP64; norms are summed in FP64.  The
// FP64 blocks are split into FP32 pairs and joined back with integer operations (mw_dfconv.cuh),
// which keeps the conversions off GB300's slow FP64 pipe.
//
// Layout: one CTA per node, one thread per line of the cube, the cube in shared memory (rows padded
// to 2K + 1 pairs, conflict-free row stores); every pass transforms a line in place (the thread
// reads all of it first).  Value cubes in global memory are (hi, lo) pairs in cube order [Z][Y][X].
#include "mw_dfconv.cuh"
#include "mw_host.h"

namespace mwg {

namespace {

// (sh, sl) += (ah + al) * (bh + bl), every step explicitly rounded
__device__ __forceinline__ void mdf_fma(float &sh, float &sl, float ah, float al, float bh, float bl) {
    const float p = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    const float t = __fadd_rn(sh, p);
    const float bp = __fsub_rn(t, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    sl = __fadd_rn(sl, __fadd_rn(err, e));
    sh = t;
}

// (ah + al) * (bh + bl) as a renormalised pair
__device__ __forceinline__ float2 mdf_mul(float ah, float al, float bh, float bl) {
    const float p = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    const float t = __fadd_rn(p, e);
    return make_float2(t, __fsub_rn(e, __fsub_rn(t, p)));
}

__device__ __forceinline__ void mdf_split(double d, float &h, float &l) {
    h = __double2float_rn(d);
    l = __double2float_rn(d - (double)h);
}


// out = M v for one line of 2K values held in shared memory (element i at line[i * stride]), M^T
// in shared memory as hi / lo rows (M^T[k][j] = M[j][k]); every output is formed before the first
// is handed to store(j, hi, lo) (renormalised), so a pass may write back into the line it read.
// The k loop is rolled: a few hundred instructions, where a fully unrolled transform (thousands)
// stalled the warps on instruction fetch.
template <int K, class Store>
__device__ __forceinline__ void mdf_line(const float2 *line, int stride, const float *mth, const float *mtl,
                                         Store store) {
    constexpr int N2 = 2 * K;
    float oh[N2], ol[N2];
#pragma unroll
    for (int j = 0; j < N2; j++) oh[j] = ol[j] = 0.0f;
#pragma unroll 1
    for (int k = 0; k < N2; k++) {
        const float2 v = line[k * stride];
#pragma unroll
        for (int j = 0; j < N2; j++) mdf_fma(oh[j], ol[j], mth[k * N2 + j], mtl[k * N2 + j], v.x, v.y);
    }
#pragma unroll
    for (int j = 0; j < N2; j++) {
        const float t = __fadd_rn(oh[j], ol[j]);
        store(j, t, __fsub_rn(ol[j], __fsub_rn(t, oh[j])));
    }
}

// Geometry of both kernels.
template <int K>
struct ValGeo {
    static constexpr int N2 = 2 * K, NC = N2 * N2, K3 = K * K * K, RS = N2 + 1;
    static constexpr int THREADS = ((NC + 31) / 32) * 32;
    static constexpr int VALS = N2 * N2 * N2;  // float2 per value cube, cube order [Z][Y][X]
    // one cube (N2 x N2 rows of RS pairs), one matrix transposed (hi and lo), 8 K^2 norm partials
    static constexpr size_t SMEM = sizeof(float2) * (size_t)NC * RS + sizeof(float) * 2 * (size_t)NC + sizeof(double) * 8 * K * K;
};

// M^T[k][j] of M_in (in = true) or M_out, formed in FP64 and split into hi / lo:
//   M_in^T[k][j] = sum_x' c2v[j % K][x'] W^T[h(j) + x'][k],  M_out^T[k][j] = sum_m W[j][h(k) + m] v2c[m][k % K]
// (h(i) = K * (i >= K))
template <int K>
__device__ void mul_matrix(const DevBasis &bas, bool in, float *mh, float *ml) {
    constexpr int N2 = 2 * K, NC = N2 * N2;
    for (int i = threadIdx.x; i < NC; i += blockDim.x) {
        const int k = i / N2, j = i - k * N2;
        const int hj = j >= K ? K : 0, hk = k >= K ? K : 0;
        double m = 0.0;
        for (int q = 0; q < K; q++)
            m = in ? fma(bas.c2v[(j - hj) * K + q], bas.WT[(hj + q) * N2 + k], m)
                   : fma(bas.W[j * N2 + hk + q], bas.v2c[q * K + (k - hk)], m);
        mdf_split(m, mh[i], ml[i]);
    }
}

template <int K>
__global__ void __launch_bounds__(ValGeo<K>::THREADS) values_df_kernel(DevBasis bas, const double *const *blocks,
                                                                       float2 *const *vals, int n) {
    using G = ValGeo<K>;
    constexpr int N2 = G::N2, NC = G::NC, K3 = G::K3, RS = G::RS;
    extern __shared__ __align__(16) float2 smem_val[];
    float2 *s_a = smem_val;
    float *s_mh = reinterpret_cast<float *>(s_a + (size_t)NC * RS), *s_ml = s_mh + NC;
    const int tid = threadIdx.x;
    const bool active = tid < NC;
    const int p = tid % N2, q = tid / N2;
    mul_matrix<K>(bas, true, s_mh, s_ml);
    for (int t = blockIdx.x; t < n; t += gridDim.x) {
        const double *blk = blocks[t];
        __syncthreads();
        for (int gi = tid; gi < 8 * K3; gi += blockDim.x) {
            const int c = gi / K3, r = gi - c * K3;
            const int ix = r % K, iy = (r / K) % K, iz = r / (K * K);
            const int X = (c & 1) * K + ix, Y = ((c >> 1) & 1) * K + iy, Z = (c >> 2) * K + iz;
            float h, l;
            df_split(blk[gi], h, l);
            s_a[(Z * N2 + Y) * RS + X] = make_float2(h, l);
        }
#pragma unroll 1
        for (int dim = 0; dim < 3; dim++) {
            __syncthreads();
            if (!active) continue;
            const int base = dim == 0 ? (q * N2 + p) * RS : (dim == 1 ? q * N2 * RS + p : p + q * RS);
            const int stride = dim == 0 ? 1 : (dim == 1 ? RS : N2 * RS);
            mdf_line<K>(s_a + base, stride, s_mh, s_ml,
                        [&](int j, float h, float l) { s_a[base + j * stride] = make_float2(h, l); });
        }
        __syncthreads();
        float2 *out = vals[t];
        for (int i = tid; i < G::VALS; i += blockDim.x) {
            const int X = i % N2, YZ = i / N2;
            out[i] = s_a[YZ * RS + X];
        }
    }
}

template <int K>
__global__ void __launch_bounds__(ValGeo<K>::THREADS) multiply_values_df_kernel(DevBasis bas, const MulVTask *tasks,
                                                                                int n) {
    using G = ValGeo<K>;
    constexpr int N2 = G::N2, NC = G::NC, K3 = G::K3, RS = G::RS;
    extern __shared__ __align__(16) float2 smem_mv[];
    float2 *s_a = smem_mv;  // the product's cube, then the output
    float *s_mh = reinterpret_cast<float *>(s_a + (size_t)NC * RS), *s_ml = s_mh + NC;
    double *s_red = reinterpret_cast<double *>(s_ml + NC);  // [component][K^2]
    const int tid = threadIdx.x;
    const bool active = tid < NC;
    const int p = tid % N2, q = tid / N2;
    mul_matrix<K>(bas, false, s_mh, s_ml);
    for (int t = blockIdx.x; t < n; t += gridDim.x) {
        const MulVTask task = tasks[t];
        float sh, sl;
        mdf_split(task.scale, sh, sl);
        double s0 = 0.0, s1 = 0.0;
        __syncthreads();
        // the product: a * scale * b, element by element
        for (int i = tid; i < G::VALS; i += blockDim.x) {
            const float2 av = task.a[i], bv = task.b[i];
            const float2 as = mdf_mul(av.x, av.y, sh, sl);
            const int X = i % N2, YZ = i / N2;
            s_a[YZ * RS + X] = mdf_mul(as.x, as.y, bv.x, bv.y);
        }
#pragma unroll 1
        for (int dim = 0; dim < 3; dim++) {
            __syncthreads();
            if (!active) continue;
            const int base = dim == 0 ? (q * N2 + p) * RS : (dim == 1 ? q * N2 * RS + p : p + q * RS);
            const int stride = dim == 0 ? 1 : (dim == 1 ? RS : N2 * RS);
            const int cxy = (p >= K ? 1 : 0) | (q >= K ? 2 : 0);
            const int r8 = (q % K) * K + p % K;
            mdf_line<K>(s_a + base, stride, s_mh, s_ml, [&](int j, float h, float l) {
                if (dim == 2) {
                    const int c = cxy | (j >= K ? 4 : 0);
                    const double v = df_widen(h) + df_widen(l);
                    task.out[(size_t)c * K3 + (size_t)(j % K) * K * K + r8] = v;
                    if (j < K)
                        s0 = fma(v, v, s0);
                    else
                        s1 = fma(v, v, s1);
                } else {
                    s_a[base + j * stride] = make_float2(h, l);
                }
            });
            if (dim == 2) {
                s_red[cxy * K * K + r8] = s0;
                s_red[(cxy | 4) * K * K + r8] = s1;
            }
        }
        __syncthreads();
        const int warp = tid >> 5, lane = tid & 31, nw = blockDim.x >> 5;
        for (int c = warp; c < 8; c += nw) {
            double s = 0.0;
            for (int j = lane; j < K * K; j += 32) s += s_red[c * K * K + j];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) task.cn[c] = sqrt(s);
        }
        __syncthreads();
    }
}

template <int K, class Fn>
int persistent_grid(Fn fn, int n, int nsm) {
    using G = ValGeo<K>;
    kernel_smem((const void *)fn, (int)G::SMEM);
    int per_sm = kernel_ctas_per_sm((const void *)fn, G::THREADS, (int)G::SMEM);
    if (per_sm < 1) per_sm = 1;
    const int slots = per_sm * (nsm > 0 ? nsm : 1);
    return n < slots ? n : slots;
}

template <int K>
void launch_values_df(const DevBasis &b, const double *const *blocks, float2 *const *vals, int n, int nsm,
                      cudaStream_t s) {
    const int grid = persistent_grid<K>(values_df_kernel<K>, n, nsm);
    values_df_kernel<K><<<grid, ValGeo<K>::THREADS, ValGeo<K>::SMEM, s>>>(b, blocks, vals, n);
    MWG_CUDA(cudaGetLastError());
}

template <int K>
void launch_multiply_values_df(const DevBasis &b, const MulVTask *tasks, int n, int nsm, cudaStream_t s) {
    const int grid = persistent_grid<K>(multiply_values_df_kernel<K>, n, nsm);
    multiply_values_df_kernel<K><<<grid, ValGeo<K>::THREADS, ValGeo<K>::SMEM, s>>>(b, tasks, n);
    MWG_CUDA(cudaGetLastError());
}

}  // namespace

size_t mul_value_floats(int K) { return (size_t)2 * (2 * K) * (2 * K) * (2 * K); }

void k_values_df(const DevBasis &b, const double *const *blocks, float2 *const *vals, int n, int nsm, cudaStream_t s) {
    if (n <= 0) return;
    switch (b.K) {
        case 4: launch_values_df<4>(b, blocks, vals, n, nsm, s); break;
        case 5: launch_values_df<5>(b, blocks, vals, n, nsm, s); break;
        case 6: launch_values_df<6>(b, blocks, vals, n, nsm, s); break;
        case 7: launch_values_df<7>(b, blocks, vals, n, nsm, s); break;
        case 8: launch_values_df<8>(b, blocks, vals, n, nsm, s); break;
        case 9: launch_values_df<9>(b, blocks, vals, n, nsm, s); break;
        case 10: launch_values_df<10>(b, blocks, vals, n, nsm, s); break;
        default: throw Error(MW_ERR_ARG, "no multiply kernel for this order");
    }
}

void k_multiply_values_df(const DevBasis &b, const MulVTask *tasks, int n, int nsm, cudaStream_t s) {
    if (n <= 0) return;
    switch (b.K) {
        case 4: launch_multiply_values_df<4>(b, tasks, n, nsm, s); break;
        case 5: launch_multiply_values_df<5>(b, tasks, n, nsm, s); break;
        case 6: launch_multiply_values_df<6>(b, tasks, n, nsm, s); break;
        case 7: launch_multiply_values_df<7>(b, tasks, n, nsm, s); break;
        case 8: launch_multiply_values_df<8>(b, tasks, n, nsm, s); break;
        case 9: launch_multiply_values_df<9>(b, tasks, n, nsm, s); break;
        case 10: launch_multiply_values_df<10>(b, tasks, n, nsm, s); break;
        default: throw Error(MW_ERR_ARG, "no multiply kernel for this order");
    }
}

}  // namespace mwg
