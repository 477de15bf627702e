// mw_apply_df.cu -- double-FP32 tier of the NS-form apply.
//
// The contraction of apply_kernel (mw_kernels.cu) with every value held as an
// unevaluated pair of FP32 numbers (hi + lo, |lo| <= ulp(hi)/2), so that the
// items whose bound is too large for the FP32 and TF32 tiers run on the FP32
// pipe instead of GB300's FP64 pipe (1.06 TFLOP/s against 71 TFLOP/s FP32).
//
// Arithmetic (Dekker / Knuth error-free transformations, as used in double-
// double libraries): a product a*b is p + e with p = fl(ah*bh) and
// e = fma(ah, bh, -p) + ah*bl + al*bh (exact product error plus the cross
// terms, al*bl dropped); a running sum keeps its high part exact by TwoSum and
// collects every rounding error in its low part.  Every operation is an
// explicitly rounded intrinsic (__fmul_rn, __fadd_rn, ...), so the compiler
// cannot contract a product and a sum into one FMA and break the error terms.
// Per pass the result is within about (K + 4) 2^-48 of sum |a||x|, so an item
// is off by at most about 3e-13 b (b = its screening bound); the host gives
// this tier the items with 2e6 < b / tau <= 1e11.
//
// Inputs: FP32 shadows in cube order, hi cube followed by lo cube; operator
// blocks hi followed by lo.  Layout per CTA (one output node or chunk at a
// time, one thread per output column (Y', X')): the node accumulator in the
// thread's registers, one half (in Z) of the input cube, T1 and u as (hi, lo)
// float2 in shared memory, the y and z passes fused so that T2 is never
// stored.  113.6 KB of shared memory and at most 112 registers a thread at
// K = 10, so that a CTA of this tier (FP32 pipe) and one of the TF32 tier
// (tensor pipe) can run on the same SM.
#include "mw_chunks.cuh"
#include "mw_host.h"

namespace mwg {

namespace {

// (sh, sl) += (ah + al) * (bh + bl)
__device__ __forceinline__ void df_fma(float &sh, float &sl, float ah, float al, float bh, float bl) {
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

// (h, l) += (bh, bl)
__device__ __forceinline__ void df_add(float &h, float &l, float bh, float bl) {
    const float t = __fadd_rn(h, bh);
    const float bp = __fsub_rn(t, h);
    const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(t, bp)), __fsub_rn(bh, bp));
    l = __fadd_rn(l, __fadd_rn(err, bl));
    h = t;
}

// renormalise so that |l| <= ulp(h)/2
__device__ __forceinline__ float2 df_norm(float h, float l) {
    const float t = __fadd_rn(h, l);
    return make_float2(t, __fsub_rn(l, __fsub_rn(t, h)));
}

// (ah + al) * (bh + bl) as a renormalised pair
__device__ __forceinline__ float2 df_mul(float ah, float al, float bh, float bl) {
    const float p = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    return df_norm(p, e);
}

// Registers a thread may hold: with 416 threads at this cap, a CTA of this kernel and one CTA of
// the TF32 tier (288 threads x 64 registers) fit in an SM's 64K registers together.
constexpr int DF_MAXREG = 112;

template <int K>
struct DfGeo {
    static constexpr int N2 = 2 * K, NC = N2 * N2, C = NC * N2, K3 = K * K * K, HALF = K * NC;
    static constexpr int THREADS = ((NC + 31) / 32) * 32;
    // float2 units: IN (one half in Z: K x N2 x N2), T1 (C), U (K^3); then floats: A_x, A_y and
    // c A_z, high parts (3 NC), then low parts (3 NC).  113.6 KB at K = 10: a CTA of this kernel
    // and one of the TF32 tier (98.7 KB) share an SM.
    static constexpr size_t SMEM = sizeof(float2) * ((size_t)HALF + C + K3) + sizeof(float) * 6 * (size_t)NC;
    static_assert(SMEM <= 127 * 1024, "shares an SM with a TF32-tier CTA");
};

// One CTA per task (output node or chunk), thread (Y', X') owns the output column (Y', X', Z' =
// 0 .. 2K-1): its node accumulator stays in registers for all of the task's items.  Per item:
//   x pass, in two halves of Z (the input cube is staged half by half): T1[Z][Y][X'] and u,
//   added to the row's earlier items' (same term, ly and lz);
//   at the row's last item, y and z passes fused: for each Z the thread forms T2[Z][Y'][X'] (and
//   t2x for Z < K) and adds c A_z[Z'][Z] T2 to its 2K accumulators at once, so T2 is never stored.
template <int K>
__global__ void __maxnreg__(DF_MAXREG) apply_df_kernel(ApplyLaunch L) {
    using G = DfGeo<K>;
    constexpr int N2 = G::N2, NC = G::NC, C = G::C, K3 = G::K3, HALF = G::HALF;
    extern __shared__ __align__(16) float2 smem_df[];
    float2 *s_in = smem_df;        // IN[z][Y][X] of the current half (Z = h K + z)
    float2 *s_t1 = s_in + HALF;    // T1[Z][Y][X']
    float2 *s_u = s_t1 + C;        // u[Z][Y][X'], Z, Y, X' < K
    float *s_Ah = reinterpret_cast<float *>(s_u + K3);  // A_x, A_y, c A_z high parts
    float *s_Al = s_Ah + 3 * NC;                        // low parts
    __shared__ int s_node, s_redf;
    const int tid = threadIdx.x;
    const bool active = tid < NC;
    const int Yp = tid / N2, Xp = tid % N2;
    const bool excl = !L.root && active && (Yp < K) && (Xp < K);

    while (true) {
        if (tid == 0) s_node = atomicAdd(L.counter, 1);
        __syncthreads();
        const int w = s_node;
        if (w >= L.nnodes) break;
        float acc_h[N2], acc_l[N2];  // acc[Z'] of the thread's column (Y', X')
#pragma unroll
        for (int z = 0; z < N2; z++) acc_h[z] = acc_l[z] = 0.0f;
        const long long b0 = L.begin[w], b1 = L.end[w];
        int nrows = 0;  // rows of this task
        for (long long j = b0; j < b1; j++) {
            // rows: items of one term and (ly, lz) (the same A_y and A_z) follow one another in walk
            // order; their x passes add into T1 and u, and the row's last item runs the y and z passes
            // once on the sums (every thread reads the same pointers: `last` is uniform)
            const bool first = j == b0 || L.ay[j - 1] != L.ay[j] || L.az[j - 1] != L.az[j];
            const bool last = j + 1 == b1 || L.ay[j + 1] != L.ay[j] || L.az[j + 1] != L.az[j];
#pragma unroll 1
            for (int h = 0; h < 2; h++) {
                __syncthreads();  // the previous half's x pass, or the previous item, is done with smem
                {
                    // half h of the hi and lo cubes -> interleaved (hi, lo) pairs
                    const float4 *gh = reinterpret_cast<const float4 *>(L.in[j]) + (size_t)h * (HALF / 4);
                    const float4 *gl = gh + C / 4;
                    float4 *s4 = reinterpret_cast<float4 *>(s_in);
                    for (int i = tid; i < HALF / 4; i += blockDim.x) {
                        const float4 hv = __ldg(gh + i), lv = __ldg(gl + i);
                        s4[2 * i] = make_float4(hv.x, lv.x, hv.y, lv.y);
                        s4[2 * i + 1] = make_float4(hv.z, lv.z, hv.w, lv.w);
                    }
                    if (h == 0) {
                        const float *ax = reinterpret_cast<const float *>(L.ax[j]);
                        const float *ay = reinterpret_cast<const float *>(L.ay[j]);
                        const float *az = reinterpret_cast<const float *>(L.az[j]);
                        const double cfd = L.coef[j];
                        const float cfh = (float)cfd, cfl = (float)(cfd - (double)cfh);
                        for (int i = tid; i < 3 * NC; i += blockDim.x) {
                            const int d = i / NC, r = i - d * NC;
                            const float *op = d == 0 ? ax : (d == 1 ? ay : az);
                            float hv = __ldg(op + r), lv = __ldg(op + NC + r);
                            if (d == 2) {  // c A_z
                                const float2 m = df_mul(hv, lv, cfh, cfl);
                                hv = m.x;
                                lv = m.y;
                            }
                            s_Ah[i] = hv;
                            s_Al[i] = lv;
                        }
                    }
                }
                __syncthreads();
                if (active) {  // x pass of this half, thread (Y = Yp, X' = Xp)
                    float ah[N2], al[N2];
#pragma unroll
                    for (int X = 0; X < N2; X++) {
                        ah[X] = s_Ah[Xp * N2 + X];
                        al[X] = s_Al[Xp * N2 + X];
                    }
#pragma unroll 2
                    for (int z = 0; z < K; z++) {
                        const float2 *src = s_in + (z * N2 + Yp) * N2;
                        float s0h = 0.0f, s0l = 0.0f, s1h = 0.0f, s1l = 0.0f;
#pragma unroll
                        for (int X = 0; X < K; X++) {
                            const float2 v = src[X];
                            df_fma(s0h, s0l, ah[X], al[X], v.x, v.y);
                        }
#pragma unroll
                        for (int X = K; X < N2; X++) {
                            const float2 v = src[X];
                            df_fma(s1h, s1l, ah[X], al[X], v.x, v.y);
                        }
                        float th = s0h, tl = s0l;
                        df_add(th, tl, s1h, s1l);
                        const int Z = h * K + z;
                        float2 *t1 = s_t1 + (Z * N2 + Yp) * N2 + Xp;
                        if (!first) df_add(th, tl, t1->x, t1->y);  // this thread's own earlier value
                        *t1 = df_norm(th, tl);
                        if (excl && h == 0) {
                            float2 *u = s_u + (z * K + Yp) * K + Xp;
                            if (!first) df_add(s1h, s1l, u->x, u->y);
                            *u = df_norm(s1h, s1l);
                        }
                    }
                }
            }
            if (!last) continue;
            nrows++;
            __syncthreads();
            if (active) {  // y and z passes, thread (Y' = Yp, X' = Xp)
                const float *ayh = s_Ah + NC + Yp * N2, *ayl = s_Al + NC + Yp * N2;
                const float *czh = s_Ah + 2 * NC, *czl = s_Al + 2 * NC;  // c A_z[Z'][Z] at Z' N2 + Z
#pragma unroll 1
                for (int Z = 0; Z < N2; Z++) {
                    float s0h = 0.0f, s0l = 0.0f, s1h = 0.0f, s1l = 0.0f;
#pragma unroll
                    for (int Y = 0; Y < K; Y++) {
                        const float2 v = s_t1[(Z * N2 + Y) * N2 + Xp];
                        df_fma(s0h, s0l, ayh[Y], ayl[Y], v.x, v.y);
                    }
#pragma unroll
                    for (int Y = K; Y < N2; Y++) {
                        const float2 v = s_t1[(Z * N2 + Y) * N2 + Xp];
                        df_fma(s1h, s1l, ayh[Y], ayl[Y], v.x, v.y);
                    }
                    // t2x: u replaces T1 for Y < K (the scaling-scaling path in x and y left out)
                    float2 t2x = make_float2(0.0f, 0.0f);
                    if (Z < K) {
                        float xh = 0.0f, xl = 0.0f;
                        if (excl) {
#pragma unroll
                            for (int Y = 0; Y < K; Y++) {
                                const float2 v = s_u[(Z * K + Y) * K + Xp];
                                df_fma(xh, xl, ayh[Y], ayl[Y], v.x, v.y);
                            }
                        }
                        df_add(xh, xl, s1h, s1l);
                        t2x = df_norm(xh, xl);
                    }
                    df_add(s0h, s0l, s1h, s1l);
                    const float2 t2 = df_norm(s0h, s0l);
                    const bool use_x = excl && Z < K;
#pragma unroll
                    for (int Zp = 0; Zp < N2; Zp++) {
                        const float2 v = (use_x && Zp < K) ? t2x : t2;
                        df_fma(acc_h[Zp], acc_l[Zp], czh[Zp * N2 + Z], czl[Zp * N2 + Z], v.x, v.y);
                    }
                }
#pragma unroll
                for (int Zp = 0; Zp < N2; Zp++) {
                    const float2 a = df_norm(acc_h[Zp], acc_l[Zp]);
                    acc_h[Zp] = a.x;
                    acc_l[Zp] = a.y;
                }
            }
        }
        if (active) {
            double *out = L.out[w];
#pragma unroll
            for (int Zp = 0; Zp < N2; Zp++) {
                const int c = (Xp >= K ? 1 : 0) | (Yp >= K ? 2 : 0) | (Zp >= K ? 4 : 0);
                const int gi = c * K3 + (Zp % K) * K * K + (Yp % K) * K + (Xp % K);
                const double v = (double)acc_h[Zp] + (double)acc_l[Zp];
                if (L.set)
                    out[gi] = v;
                else
                    out[gi] += v;
            }
        }
        __syncthreads();
        if (tid == 0 && nrows > 0 && L.rows) atomicAdd(L.rows, nrows);
        finish_chunk(L, w, 8 * K3, &s_redf);
    }
}

template <int K>
void launch_df(const ApplyLaunch &L, int nsm, cudaStream_t s) {
    using G = DfGeo<K>;
    kernel_smem((const void *)apply_df_kernel<K>, (int)G::SMEM);
    // one CTA per task (tasks are ordered longest first and taken in that order): CTAs end
    // throughout the launch, so kernels of other streams get SM slots without waiting for it
    (void)nsm;
    const int grid = L.nnodes;
    if (grid < 1) return;
    apply_df_kernel<K><<<grid, G::THREADS, G::SMEM, s>>>(L);
    MWG_CUDA(cudaGetLastError());
}

}  // namespace

void k_apply_df(const DevBasis &b, const ApplyLaunch &L, int nsm, cudaStream_t s) {
    if (L.nnodes <= 0) return;
    switch (b.K) {
        case 4: launch_df<4>(L, nsm, s); break;
        case 5: launch_df<5>(L, nsm, s); break;
        case 6: launch_df<6>(L, nsm, s); break;
        case 7: launch_df<7>(L, nsm, s); break;
        case 8: launch_df<8>(L, nsm, s); break;
        case 9: launch_df<9>(L, nsm, s); break;
        case 10: launch_df<10>(L, nsm, s); break;
        default: throw Error(MW_ERR_ARG, "no double-FP32 apply kernel for this order");
    }
}

}  // namespace mwg
