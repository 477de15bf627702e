// mw_multiply_df.cu -- the tree multiply's node kernel in double-FP32 arithmetic.
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
// two backward steps another, M_out = W diag(v2c, v2c), both formed in FP64 in the CTA's prologue.
// A node is then nine line passes (three per cube) of 2K x 2K multiply-adds.
//
// Arithmetic: every value is an unevaluated FP32 pair (hi + lo) and every multiply-add is the
// error-free double-FP32 update of the apply's double-FP32 tier, as in the post-processing
// transforms (mw_post_df.cu): about (2K + 4) 2^-48 of sum |M| |x| per pass, 1e-14 relative, at
// about 8x GB300's FP64 rate.  Blocks in global memory stay FP64; norms are summed in FP64.  The
// FP64 blocks are split into FP32 pairs and joined back with integer operations (mw_dfconv.cuh),
// which keeps the conversions off GB300's slow FP64 pipe.
//
// Layout: one CTA per node, one thread per line of the cube, the two cubes in shared memory
// (rows padded to 2K + 1 pairs, conflict-free row stores).  The two input blocks are staged as
// cubes by coalesced loads; every pass transforms a line in place (the thread reads all of it
// first); the product is formed in b's z pass by the thread that owns the same line of a's cube;
// the last (z) pass of the backward transform writes the FP64 block.
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

template <int K>
struct MulGeo {
    static constexpr int N2 = 2 * K, NC = N2 * N2, K3 = K * K * K, RS = N2 + 1;
    static constexpr int THREADS = ((NC + 31) / 32) * 32;
    // two cubes (N2 x N2 rows of RS pairs), M_in^T and M_out^T (hi and lo, NC floats each),
    // 8 K^2 norm partials
    static constexpr size_t SMEM =
        sizeof(float2) * 2 * (size_t)NC * RS + sizeof(float) * 4 * (size_t)NC + sizeof(double) * 8 * K * K;
};

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

// The two FP64 input blocks are first staged as cubes of FP32 pairs (coalesced loads); then the
// nine line passes of a node, in order, each in place on its cube; passes of one group run between
// the same two barriers:
//   0, 1  x passes of a and b                                          (group 0)
//   2, 3  y passes of a and b                                          (group 1)
//   4, 5  z passes of a (into its cube) and b (product into a's cube)  (group 2)
//   6     x pass of the product, 7 its y pass                         (groups 3, 4)
//   8     z pass of the product, written to the FP64 block with norms  (group 5)
// Thread mapping per pass: x passes (Y, Z) = (p, q), y passes (X, Z) = (p, q), z passes (X, Y) = (p, q).
template <int K>
__global__ void __launch_bounds__(MulGeo<K>::THREADS) multiply_df_kernel(DevBasis bas, const MulTask *tasks, int n) {
    using G = MulGeo<K>;
    constexpr int N2 = G::N2, NC = G::NC, K3 = G::K3, RS = G::RS;
    extern __shared__ __align__(16) float2 smem_mul[];
    float2 *s_a = smem_mul;                 // a's cube, then the product, then the output
    float2 *s_b = s_a + (size_t)NC * RS;     // b's cube
    float *s_inh = reinterpret_cast<float *>(s_b + (size_t)NC * RS);
    float *s_inl = s_inh + NC, *s_outh = s_inl + NC, *s_outl = s_outh + NC;
    double *s_red = reinterpret_cast<double *>(s_outl + NC);  // [component][K^2]
    const int tid = threadIdx.x;
    const bool active = tid < NC;
    const int p = tid % N2, q = tid / N2;  // the line's two fixed coordinates

    // M_in^T[k][j] = M_in[j][k] = sum_x' c2v[j % K][x'] W^T[h(j) + x'][k];
    // M_out^T[k][j] = M_out[j][k] = sum_m W[j][h(k) + m] v2c[m][k % K]   (h(i) = K * (i >= K))
    for (int i = tid; i < NC; i += blockDim.x) {
        const int k = i / N2, j = i - k * N2;
        const int hj = j >= K ? K : 0, hk = k >= K ? K : 0;
        double mi = 0.0, mo = 0.0;
        for (int m = 0; m < K; m++) {
            mi = fma(bas.c2v[(j - hj) * K + m], bas.WT[(hj + m) * N2 + k], mi);
            mo = fma(bas.W[j * N2 + hk + m], bas.v2c[m * K + (k - hk)], mo);
        }
        mdf_split(mi, s_inh[i], s_inl[i]);
        mdf_split(mo, s_outh[i], s_outl[i]);
    }

    for (int t = blockIdx.x; t < n; t += gridDim.x) {
        const MulTask task = tasks[t];
        float sh, sl;
        mdf_split(task.scale, sh, sl);
        double s0 = 0.0, s1 = 0.0;  // pass 8: this line's squared norms (Z < K, Z >= K)
        __syncthreads();  // the matrices are ready; the previous node's cubes are no longer read
        for (int gi = tid; gi < 8 * K3; gi += blockDim.x) {
            const int c = gi / K3, r = gi - c * K3;
            const int ix = r % K, iy = (r / K) % K, iz = r / (K * K);
            const int X = (c & 1) * K + ix, Y = ((c >> 1) & 1) * K + iy, Z = (c >> 2) * K + iz;
            const int at = (Z * N2 + Y) * RS + X;
            float h, l;
            df_split(task.a[gi], h, l);
            s_a[at] = make_float2(h, l);
            df_split(task.b[gi], h, l);
            s_b[at] = make_float2(h, l);
        }
#pragma unroll 1
        for (int pass = 0; pass < 9; pass++) {
            if (pass == 0 || pass == 2 || pass == 4 || pass >= 6) __syncthreads();
            if (!active) continue;
            const int dim = pass == 6 ? 0 : (pass == 7 ? 1 : (pass == 8 ? 2 : pass >> 1));  // 0 x, 1 y, 2 z
            const bool on_b = pass < 6 && (pass & 1);
            float2 *cube = on_b ? s_b : s_a;
            // line start and element stride in the cube
            const int base = dim == 0 ? (q * N2 + p) * RS : (dim == 1 ? q * N2 * RS + p : p + q * RS);
            const int stride = dim == 0 ? 1 : (dim == 1 ? RS : N2 * RS);
            const float *mth = pass < 6 ? s_inh : s_outh, *mtl = pass < 6 ? s_inl : s_outl;
            const int cxy = (p >= K ? 1 : 0) | (q >= K ? 2 : 0);  // pass 8: (X, Y) = (p, q)
            const int r8 = (q % K) * K + p % K;
            mdf_line<K>(cube + base, stride, mth, mtl, [&](int j, float h, float l) {
                if (pass == 5) {  // product on a's z line: a * scale * b
                    const float2 av = s_a[base + j * stride];
                    const float2 as = mdf_mul(av.x, av.y, sh, sl);
                    s_a[base + j * stride] = mdf_mul(as.x, as.y, h, l);
                } else if (pass == 8) {
                    const int c = cxy | (j >= K ? 4 : 0);
                    const double v = df_widen(h) + df_widen(l);
                    task.out[(size_t)c * K3 + (size_t)(j % K) * K * K + r8] = v;
                    if (j < K)
                        s0 = fma(v, v, s0);
                    else
                        s1 = fma(v, v, s1);
                } else {
                    cube[base + j * stride] = make_float2(h, l);
                }
            });
            if (pass == 8) {
                s_red[cxy * K * K + r8] = s0;
                s_red[(cxy | 4) * K * K + r8] = s1;
            }
        }
        __syncthreads();
        // component c summed by one warp: lane-strided, then a fixed butterfly (deterministic)
        const int warp = tid >> 5, lane = tid & 31, nw = blockDim.x >> 5;
        for (int c = warp; c < 8; c += nw) {
            double s = 0.0;
            for (int j = lane; j < K * K; j += 32) s += s_red[c * K * K + j];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) task.cn[c] = sqrt(s);
        }
        __syncthreads();  // s_red is rewritten by the next node
    }
}

template <int K>
void launch_multiply_df(const DevBasis &b, const MulTask *tasks, int n, int nsm, cudaStream_t s) {
    using G = MulGeo<K>;
    auto fn = multiply_df_kernel<K>;
    MWG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM));
    int per_sm = 0;
    MWG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, G::THREADS, G::SMEM));
    if (per_sm < 1) per_sm = 1;
    // persistent CTAs (the matrices are formed once per CTA), as many as fit on the GPU
    const int slots = per_sm * (nsm > 0 ? nsm : 1);
    const int grid = n < slots ? n : slots;
    fn<<<grid, G::THREADS, G::SMEM, s>>>(b, tasks, n);
    MWG_CUDA(cudaGetLastError());
}

}  // namespace

void k_multiply_df(const DevBasis &b, const MulTask *tasks, int n, int nsm, cudaStream_t s) {
    if (n <= 0) return;
    switch (b.K) {
        case 4: launch_multiply_df<4>(b, tasks, n, nsm, s); break;
        case 5: launch_multiply_df<5>(b, tasks, n, nsm, s); break;
        case 6: launch_multiply_df<6>(b, tasks, n, nsm, s); break;
        case 7: launch_multiply_df<7>(b, tasks, n, nsm, s); break;
        case 8: launch_multiply_df<8>(b, tasks, n, nsm, s); break;
        case 9: launch_multiply_df<9>(b, tasks, n, nsm, s); break;
        case 10: launch_multiply_df<10>(b, tasks, n, nsm, s); break;
        default: throw Error(MW_ERR_ARG, "no multiply kernel for this order");
    }
}

}  // namespace mwg
