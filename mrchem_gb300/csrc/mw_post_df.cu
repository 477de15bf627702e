// mw_post_df.cu -- double-FP32 two-scale transforms of the NS-form post-processing.
//
// After the levels of a mixed-precision apply, the output trees go through the
// same two passes as in FP64 (mw_kernels.cu, topdown_kernel / compress_kernel):
//   top-down   every parent's block, reconstructed (W^T along each dimension),
//              is added to its children's scaling parts, scale by scale from
//              the roots;
//   bottom-up  every parent's block is recomputed from its children's scaling
//              parts (W along each dimension) with its 8 component norms.
// Each node costs 3 (2K)^4 multiply-adds, which GB300's FP64 pipe (about
// 1.7 FMA per clock per SM) turns into ~140 us per node and SM.  Here every
// value is an unevaluated FP32 pair (hi + lo) and every multiply-add is the
// error-free double-FP32 update of the double-FP32 apply tier, so a pass is
// accurate to about (2K + 4) 2^-48 of sum |W| |x| -- 1e-14 relative, far below
// any precision an apply is asked for -- at ~8x the FP64 rate.  The blocks in
// global memory stay FP64; the norms are summed in FP64.  The FP64 values are split into FP32
// pairs with integer operations (mw_dfconv.cuh), off GB300's slow FP64 pipe.
//
// One CTA per node, one thread per line of the cube: the x pass reads its row
// straight from the FP64 block(s) in global memory into registers and writes
// the transformed row to the shared cube, the y and z passes read a column into
// registers and write it back (y) or out to global memory (z).  The shared cube
// rows are padded to 2K + 1 pairs, which makes the row-wise x-pass stores free
// of bank conflicts.
#include "mw_dfconv.cuh"
#include "mw_host.h"

namespace mwg {

namespace {

// (sh, sl) += (ah + al) * (bh + bl), every step explicitly rounded
__device__ __forceinline__ void pdf_fma(float &sh, float &sl, float ah, float al, float bh, float bl) {
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

__device__ __forceinline__ void pdf_split(double d, float &h, float &l) {
    h = __double2float_rn(d);
    l = __double2float_rn(d - (double)h);
}

template <int K>
struct PostGeo {
    static constexpr int N2 = 2 * K, NC = N2 * N2, K3 = K * K * K, RS = N2 + 1;
    static constexpr int THREADS = ((NC + 31) / 32) * 32;
    // cube (N2 x N2 rows of RS pairs), M^T hi and lo (NC floats each), 8 K^2 norm partials
    static constexpr size_t SMEM =
        sizeof(float2) * (size_t)NC * RS + sizeof(float) * 2 * (size_t)NC + sizeof(double) * 8 * K * K;
};

// out = M v for one line of 2K values, M^T in shared memory as hi / lo rows (M^T[k][j] = M[j][k]);
// the outputs are made in two halves of K and handed to store(j, hi, lo) renormalised
// (|lo| <= ulp(hi) / 2), so that only K accumulator pairs are live beside the line
template <int K, class Store>
__device__ __forceinline__ void pdf_line(const float (&vh)[2 * K], const float (&vl)[2 * K], const float *mth,
                                         const float *mtl, Store store) {
    constexpr int N2 = 2 * K;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        float oh[K], ol[K];
#pragma unroll
        for (int j = 0; j < K; j++) oh[j] = ol[j] = 0.0f;
#pragma unroll
        for (int k = 0; k < N2; k++) {
#pragma unroll
            for (int j = 0; j < K; j++)
                pdf_fma(oh[j], ol[j], mth[k * N2 + h * K + j], mtl[k * N2 + h * K + j], vh[k], vl[k]);
        }
#pragma unroll
        for (int j = 0; j < K; j++) {
            const float t = __fadd_rn(oh[j], ol[j]);
            store(h * K + j, t, __fsub_rn(ol[j], __fsub_rn(t, oh[j])));
        }
    }
}

// MODE 0: top-down (M = W^T, input = the parent's block, children's scaling parts +=)
// MODE 1: bottom-up (M = W, input = the children's scaling parts, parent's block = and its norms)
template <int K, int MODE>
__global__ void __launch_bounds__(PostGeo<K>::THREADS, 1)
    post_df_kernel(const double *M, const PairTask *tasks, double *const *cn, int n) {
    using G = PostGeo<K>;
    constexpr int N2 = G::N2, NC = G::NC, K3 = G::K3, RS = G::RS;
    extern __shared__ __align__(16) float2 smem_post[];
    float2 *s_cube = smem_post;  // cube[Z][Y][X] at (Z * N2 + Y) * RS + X
    float *s_mth = reinterpret_cast<float *>(s_cube + (size_t)NC * RS);
    float *s_mtl = s_mth + NC;
    double *s_red = reinterpret_cast<double *>(s_mtl + NC);  // [component][K^2]
    const int tid = threadIdx.x;
    const bool active = tid < NC;
    const int a = tid % N2, bq = tid / N2;  // the line's two fixed coordinates

    for (int i = tid; i < NC; i += blockDim.x) {
        const int k = i / N2, j = i - k * N2;  // M^T[k][j] = M[j][k]
        float h, l;
        pdf_split(M[j * N2 + k], h, l);
        s_mth[i] = h;
        s_mtl[i] = l;
    }

    for (int t = blockIdx.x; t < n; t += gridDim.x) {
        const PairTask task = tasks[t];
        double s0 = 0.0, s1 = 0.0;  // MODE 1, z pass: this line's squared norms (Z < K, Z >= K)
        // The three passes run through one instance of the line transform (an instance per pass
        // overflowed the instruction cache): x reads the thread's row from the FP64 block(s), y and
        // z read a line of the shared cube; every pass writes back into the cube, except the
        // compression's z pass, which writes the parent's FP64 block.  Thread mapping: x (Y, Z) =
        // (a, bq), y (X, Z) = (a, bq), z (X, Y) = (a, bq).
#pragma unroll 1
        for (int dim = 0; dim < 3; dim++) {
            __syncthreads();  // x: M^T ready, the previous node's cube and partials no longer read;
                              // y, z: the previous pass's stores are visible
            if (!active) continue;
            const int base = dim == 0 ? (bq * N2 + a) * RS : (dim == 1 ? bq * N2 * RS + a : a + bq * RS);
            const int stride = dim == 0 ? 1 : (dim == 1 ? RS : N2 * RS);
            float vh[N2], vl[N2];
            if (dim == 0) {
                const int cyz = (a >= K ? 2 : 0) | (bq >= K ? 4 : 0);
                const int r = (bq % K) * K * K + (a % K) * K;
#pragma unroll
                for (int X = 0; X < N2; X++) {
                    const int c = cyz | (X >= K ? 1 : 0);
                    const double d = MODE == 0 ? task.parent[(size_t)c * K3 + r + X % K]
                                               : task.child0[(size_t)c * 8 * K3 + r + X % K];
                    df_split(d, vh[X], vl[X]);
                }
            } else {
                // the whole line is in registers before the first store
#pragma unroll
                for (int i = 0; i < N2; i++) {
                    const float2 v = s_cube[base + i * stride];
                    vh[i] = v.x;
                    vl[i] = v.y;
                }
            }
            const bool to_parent = MODE == 1 && dim == 2;
            const int cxy = (a >= K ? 1 : 0) | (bq >= K ? 2 : 0);  // z pass: (X, Y) = (a, bq)
            const int r2 = (bq % K) * K + a % K;
            pdf_line<K>(vh, vl, s_mth, s_mtl, [&](int j, float h, float l) {
                if (to_parent) {
                    const int c = cxy | (j >= K ? 4 : 0);
                    // CUDA conversions here: the integer join made this pass spill at K = 9, 10
                    const double v = (double)h + (double)l;
                    task.parent[(size_t)c * K3 + (size_t)(j % K) * K * K + r2] = v;
                    if (j < K)
                        s0 = fma(v, v, s0);
                    else
                        s1 = fma(v, v, s1);
                } else {
                    s_cube[base + j * stride] = make_float2(h, l);
                }
            });
            if (to_parent) {
                s_red[cxy * K * K + r2] = s0;
                s_red[(cxy | 4) * K * K + r2] = s1;
            }
        }
        __syncthreads();
        if (MODE == 0) {
            // child c's scaling part += octant c of the cube
            for (int gi = tid; gi < 8 * K3; gi += blockDim.x) {
                const int c = gi / K3, r = gi - c * K3;
                const int ix = r % K, iy = (r / K) % K, iz = r / (K * K);
                const int X = (c & 1) * K + ix, Y = ((c >> 1) & 1) * K + iy, Z = (c >> 2) * K + iz;
                const float2 v = s_cube[(size_t)(Z * N2 + Y) * RS + X];
                task.child0[(size_t)c * 8 * K3 + r] += df_widen(v.x) + df_widen(v.y);
            }
        }
        if (MODE == 1) {
            // component c summed by one warp: lane-strided, then a fixed butterfly (deterministic)
            const int warp = tid >> 5, lane = tid & 31, nw = blockDim.x >> 5;
            for (int c = warp; c < 8; c += nw) {
                double s = 0.0;
                for (int j = lane; j < K * K; j += 32) s += s_red[c * K * K + j];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (lane == 0) cn[t][c] = sqrt(s);
            }
        }
    }
}

template <int K, int MODE>
void launch_post_df(const double *M, const PairTask *tasks, double *const *cn, int n, cudaStream_t s) {
    using G = PostGeo<K>;
    auto fn = post_df_kernel<K, MODE>;
    MWG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM));
    const int grid = n < 4096 ? n : 4096;
    fn<<<grid, G::THREADS, G::SMEM, s>>>(M, tasks, cn, n);
    MWG_CUDA(cudaGetLastError());
}

template <int MODE>
bool post_df(const DevBasis &b, const double *M, const PairTask *tasks, double *const *cn, int n, cudaStream_t s) {
    switch (b.K) {
        case 4: launch_post_df<4, MODE>(M, tasks, cn, n, s); return true;
        case 5: launch_post_df<5, MODE>(M, tasks, cn, n, s); return true;
        case 6: launch_post_df<6, MODE>(M, tasks, cn, n, s); return true;
        case 7: launch_post_df<7, MODE>(M, tasks, cn, n, s); return true;
        case 8: launch_post_df<8, MODE>(M, tasks, cn, n, s); return true;
        case 9: launch_post_df<9, MODE>(M, tasks, cn, n, s); return true;
        case 10: launch_post_df<10, MODE>(M, tasks, cn, n, s); return true;
        default: return false;
    }
}

}  // namespace

void k_topdown_df(const DevBasis &b, const PairTask *tasks, int n, cudaStream_t s) {
    if (n <= 0) return;
    if (!post_df<0>(b, b.WT, tasks, nullptr, n, s)) k_topdown(b, tasks, n, s);
}

void k_compress_df(const DevBasis &b, const PairTask *tasks, double *const *cn, int n, cudaStream_t s) {
    if (n <= 0) return;
    if (!post_df<1>(b, b.W, tasks, cn, n, s)) k_compress(b, tasks, cn, n, s);
}

}  // namespace mwg
