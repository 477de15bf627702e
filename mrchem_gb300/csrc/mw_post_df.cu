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
// One CTA per node, one thread per line of the cube: the CTA stages the FP64
// input as a cube of FP32 pairs in shared memory, then each pass transforms the
// threads' lines from one shared cube into the other (the last pass of the
// compression writes the parent's FP64 block and its norms).  Cube rows are
// padded to 2K + 1 pairs, which keeps the row-wise accesses free of bank
// conflicts.
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
    static constexpr int N2 = 2 * K, NC = N2 * N2, K3 = K * K * K, RS = N2 + 1, RH = K + 1;
    // one thread per line of the staged cube in the x pass, per half line in the y and z passes
    static constexpr int THREADS = ((NC + 31) / 32) * 32;
    // the full input cube (N2 x N2 rows of RS pairs; later the y pass's half cube), the half cube of
    // the x and z passes (N2 x N2 rows of RH pairs), M^T hi and lo (NC floats each), and the
    // compression's norm partials (4 components x K^2)
    static constexpr size_t SMEM = sizeof(float2) * (size_t)NC * RS + sizeof(float2) * (size_t)NC * RH +
                                   sizeof(float) * 2 * (size_t)NC + sizeof(double) * 4 * K * K;
};

// K outputs (half h of the 2K) of M v for one line of 2K values held in shared memory (element i at
// line[i * stride]), M^T in shared memory as hi / lo rows (M^T[k][j] = M[j][k]), handed to
// store(j, hi, lo) renormalised (|lo| <= ulp(hi) / 2).  The k loop is rolled: a few hundred
// instructions, where a fully unrolled transform (thousands) overflowed the instruction cache and
// stalled the small launches of the post-processing
template <int K>
__device__ __forceinline__ void pdf_half_line(const float2 *line, int stride, const float *mth, const float *mtl, int h,
                                              float (&oh)[K], float (&ol)[K]) {
    constexpr int N2 = 2 * K;
#pragma unroll
    for (int j = 0; j < K; j++) oh[j] = ol[j] = 0.0f;
#pragma unroll 1
    for (int k = 0; k < N2; k++) {
        const float2 v = line[k * stride];
#pragma unroll
        for (int j = 0; j < K; j++) pdf_fma(oh[j], ol[j], mth[k * N2 + h * K + j], mtl[k * N2 + h * K + j], v.x, v.y);
    }
#pragma unroll
    for (int j = 0; j < K; j++) {
        const float t = __fadd_rn(oh[j], ol[j]);
        ol[j] = __fsub_rn(ol[j], __fsub_rn(t, oh[j]));
        oh[j] = t;
    }
}

// MODE 0: top-down (M = W^T, input = the parent's block, children's scaling parts +=)
// MODE 1: bottom-up (M = W, input = the children's scaling parts, parent's block = and its norms)
//
// Two CTAs per node, one per half hx of the output's x range: a CTA transforms the whole staged
// cube along x into its half, then that half along y and z, so the two halves split the node's
// work with nothing computed twice, and a node of a small level finishes in half the time.  The
// CTA of half hx writes the four children (top-down) or parent components (compression) whose
// octant has x half hx.
template <int K, int MODE>
__global__ void __launch_bounds__(PostGeo<K>::THREADS, 2)
    post_df_kernel(const double *M, const PairTask *tasks, double *const *cn, int n) {
    using G = PostGeo<K>;
    constexpr int N2 = G::N2, NC = G::NC, K3 = G::K3, RS = G::RS, RH = G::RH;
    extern __shared__ __align__(16) float2 smem_post[];
    float2 *s_full = smem_post;                   // input cube[Z][Y][X] at (Z * N2 + Y) * RS + X; y pass out (half)
    float2 *s_half = s_full + (size_t)NC * RS;    // half cube[Z][Y][x'] at (Z * N2 + Y) * RH + x': x and z pass out
    float *s_mth = reinterpret_cast<float *>(s_half + (size_t)NC * RH);
    float *s_mtl = s_mth + NC;
    double *s_red = reinterpret_cast<double *>(s_mtl + NC);  // [component >> 1][K^2] (compression)
    const int tid = threadIdx.x;
    const bool active = tid < NC;
    // x pass: line (Y, Z); y and z passes: (x', the line's other coordinate, output half)
    const int xa = tid % N2, xb = tid / N2;
    const int px = tid % K, pl = (tid / K) % N2, ph = tid / (K * N2);

    for (int i = tid; i < NC; i += blockDim.x) {
        const int k = i / N2, j = i - k * N2;  // M^T[k][j] = M[j][k]
        float h, l;
        pdf_split(M[j * N2 + k], h, l);
        s_mth[i] = h;
        s_mtl[i] = l;
    }

    for (int u = blockIdx.x; u < 2 * n; u += gridDim.x) {
        const int t = u >> 1, hx = u & 1;
        const PairTask task = tasks[t];
        // the FP64 input, split into FP32 pairs, staged as a cube by all threads (coalesced reads):
        // top-down the parent's block, compression the children's scaling parts (child c in
        // octant c)
        __syncthreads();  // M^T ready; the previous node's cubes and partials are no longer read
        for (int gi = tid; gi < 8 * K3; gi += blockDim.x) {
            const int c = gi / K3, r = gi - c * K3;
            const int ix = r % K, iy = (r / K) % K, iz = r / (K * K);
            const int X = (c & 1) * K + ix, Y = ((c >> 1) & 1) * K + iy, Z = (c >> 2) * K + iz;
            const double d = MODE == 0 ? task.parent[gi] : task.child0[(size_t)c * 8 * K3 + r];
            float h, l;
            df_split(d, h, l);
            s_full[(size_t)(Z * N2 + Y) * RS + X] = make_float2(h, l);
        }
        __syncthreads();
        float oh[K], ol[K];
        if (active) {  // x pass: line (Y, Z) = (xa, xb), outputs X = hx K + j
            const int row = xb * N2 + xa;
            pdf_half_line<K>(s_full + row * RS, 1, s_mth, s_mtl, hx, oh, ol);
#pragma unroll
            for (int j = 0; j < K; j++) s_half[row * RH + j] = make_float2(oh[j], ol[j]);
        }
        __syncthreads();
        if (active) {  // y pass: line (x', Z) = (px, pl), outputs Y = ph K + j, into s_full as a half cube
            pdf_half_line<K>(s_half + pl * N2 * RH + px, RH, s_mth, s_mtl, ph, oh, ol);
#pragma unroll
            for (int j = 0; j < K; j++) s_full[(pl * N2 + ph * K + j) * RH + px] = make_float2(oh[j], ol[j]);
        }
        __syncthreads();
        if (active) {  // z pass: line (x', Y) = (px, pl), outputs Z = ph K + j
            pdf_half_line<K>(s_full + pl * RH + px, N2 * RH, s_mth, s_mtl, ph, oh, ol);
            if (MODE == 0) {
#pragma unroll
                for (int j = 0; j < K; j++) s_half[((ph * K + j) * N2 + pl) * RH + px] = make_float2(oh[j], ol[j]);
            } else {
                // parent component c = hx | (Y >= K) << 1 | ph << 2, element (Z % K, Y % K, x')
                const int c = hx | (pl >= K ? 2 : 0) | (ph << 2);
                const int r2 = (pl % K) * K + px;
                double s = 0.0;
#pragma unroll
                for (int j = 0; j < K; j++) {
                    const double v = df_widen(oh[j]) + df_widen(ol[j]);
                    task.parent[(size_t)c * K3 + (size_t)j * K * K + r2] = v;
                    s = fma(v, v, s);
                }
                s_red[(c >> 1) * K * K + r2] = s;
            }
        }
        __syncthreads();
        if (MODE == 0) {
            // child c's scaling part += octant c of the output, for the four children of half hx
            for (int gi = tid; gi < 4 * K3; gi += blockDim.x) {
                const int q = gi / K3, r = gi - q * K3;
                const int c = hx | (q << 1);
                const int ix = r % K, iy = (r / K) % K, iz = r / (K * K);
                const int Y = ((c >> 1) & 1) * K + iy, Z = (c >> 2) * K + iz;
                const float2 v = s_half[(size_t)(Z * N2 + Y) * RH + ix];
                task.child0[(size_t)c * 8 * K3 + r] += df_widen(v.x) + df_widen(v.y);
            }
        }
        if (MODE == 1) {
            // component c summed by one warp: lane-strided, then a fixed butterfly (deterministic)
            const int warp = tid >> 5, lane = tid & 31, nw = blockDim.x >> 5;
            for (int q = warp; q < 4; q += nw) {
                double s = 0.0;
                for (int j = lane; j < K * K; j += 32) s += s_red[q * K * K + j];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (lane == 0) cn[t][hx | (q << 1)] = sqrt(s);
            }
        }
    }
}

template <int K, int MODE>
void launch_post_df(const double *M, const PairTask *tasks, double *const *cn, int n, cudaStream_t s) {
    using G = PostGeo<K>;
    auto fn = post_df_kernel<K, MODE>;
    kernel_smem((const void *)fn, (int)G::SMEM);
    const int grid = 2 * n < 8192 ? 2 * n : 8192;
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
