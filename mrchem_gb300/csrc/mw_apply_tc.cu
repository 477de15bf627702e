// mw_apply_tc.cu -- TF32 tensor-core tier of the NS-form apply.
//
// The same item contraction as apply_kernel / apply32_kernel in mw_kernels.cu
// (c_t (A_z (x) A_y (x) A_x) in, scaling-scaling path left out below the root
// scale), written as three GEMMs on warp-level tensor-core MMAs
// (mma.sync m16n8k8 / m16n8k4, TF32 operands, FP32 accumulation):
//
//   x pass  T1[(Z,Y)][X'] = sum_X  IN[Z][Y][X]  A_x[X'][X]
//   y pass  T2[(Z,X')][Y'] = sum_Y T1[Z][Y][X'] A_y[Y'][Y]
//   z pass OUT[(Y',X')][Z'] += sum_Z T2[Z][Y'][X'] c A_z[Z'][Z]
//
// Each pass is (2K)^2 rows x 2K columns x 2K contraction.  Rows are ordered so
// that the K^2 rows whose two fixed indices are both in the scaling half come
// first: only the first ceil(K^2/16) row tiles take part in the exact
// exclusion of the scaling-scaling path, which uses the same u / t2x
// construction as the CUDA-core kernels (no subtraction):
//   u   = the wavelet-in-x part of T1 on the scaling octant,
//   t2x = the y pass in which u replaces T1 for Y < K (everything but the
//         (scaling x, scaling y) paths), used by the z pass for Z, Z' < K.
//
// The node accumulator stays in the MMA accumulator registers across all
// items of the node and is added once to the FP64 output block.  Operands are
// rounded to TF32 (cvt.rna, unit roundoff 2^-11): input values, the three
// operator blocks (A_z scaled by c_t) and the two intermediates, so an item
// is off by at most about 6 * 2^-11 * b (b = the item's screening bound); the
// host gives this tier only items below the root scale with b <= 2e3 x the
// screening threshold.
//
// Shared-memory layouts are chosen so that every fragment load and store of a
// warp touches 32 distinct banks (row strides = 8 mod 16 words where the
// fragment's thread-in-group index runs along the strided dimension).
#include "mw_async.cuh"
#include "mw_host.h"

namespace mwg {

namespace {

constexpr int pad8mod16(int x) { return x + ((8 - x % 16) + 16) % 16; }
constexpr int cmax(int a, int b) { return a > b ? a : b; }

template <int K>
struct TcGeo {
    static constexpr int N2 = 2 * K, NC = N2 * N2, C = NC * N2, KK = K * K, K3 = K * K * K, R = NC;
    static constexpr int MT = (R + 15) / 16;   // row tiles of 16
    static constexpr int NT = (N2 + 7) / 8;    // column tiles of 8
    static constexpr int NK8 = N2 / 8, REM = N2 % 8;
    static constexpr int NKS = NK8 + (REM ? 1 : 0);          // contraction steps
    static constexpr bool TAIL4 = REM > 0 && REM <= 4;       // last step is m16n8k4
    static constexpr int XT = (KK + 15) / 16;                 // row tiles holding scaling-octant rows
    static constexpr int NTS = (K + 7) / 8;                   // column tiles holding scaling columns
    static constexpr int W = MT < 5 ? MT : 5;                 // warps per CTA
    static constexpr int MPW = (MT + W - 1) / W;              // row tiles per warp
    static constexpr bool EVEN = MT % W == 0;                 // every warp has MPW row tiles
    // T1[Z][Y][X'] and u[Z][Y][X'] (Z, Y, X' < K): Y stride 24
    static constexpr int SY1 = 24, SZ1 = N2 * SY1, SZU = K * SY1;
    // T2[Z][Y'][X'] and t2x[Z][Y'][X']: Y' stride 20 (= 4 mod 16), Z stride = 8 mod 16
    static constexpr int SY2 = 20, SZ2 = pad8mod16(N2 * SY2), SZX = pad8mod16(K * SY2);
    // two regions that take turns: item j has IN and T2 in region j%2 and T1 in the other one,
    // so item j+1's input can be copied into that other region during item j's z pass
    static constexpr int REG = ((cmax(cmax(C, N2 * SZ1), N2 * SZ2) + 3) / 4) * 4;
    static constexpr int OU = 2 * REG;
    static constexpr int OT2X = OU + K * SZU;
    static constexpr int OA = ((OT2X + K * SZX + 3) / 4) * 4;  // two sets of A_x, A_y, A_z
    static constexpr int TOTAL = OA + 6 * NC;
    static constexpr uint32_t TX_BYTES = 4u * (C + 3 * NC);    // one item's copies
    static_assert(N2 <= SY2 && N2 <= SY1, "row strides too short for this order");
    static_assert(TX_BYTES < (1u << 20), "transaction count out of range");
};

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void mma_k8(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void mma_k4(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t b0) {
    asm("mma.sync.aligned.m16n8k4.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(b0));
}

// row r of a pass -> its two fixed cube indices (a, b): first the K^2 rows with
// a, b < K, then a < K <= b, then a >= K
template <int K>
__device__ __forceinline__ void row_ab(int r, int &a, int &b) {
    constexpr int KK = K * K, N2 = 2 * K;
    if (r < KK) {
        a = r / K;
        b = r - a * K;
    } else if (r < 2 * KK) {
        const int q = r - KK;
        a = q / K;
        b = K + (q - a * K);
    } else {
        const int q = r - 2 * KK;
        a = K + q / N2;
        b = q % N2;
    }
}

// B fragments of one pass for all column tiles and steps: B[k][n] = scale * M[n][k]
// (M = an operator block in shared memory, row = output index)
template <int K>
__device__ __forceinline__ void load_b(uint32_t (&bf)[TcGeo<K>::NT][TcGeo<K>::NKS][2], const float *M, float scale,
                                       int g, int t) {
    using G = TcGeo<K>;
#pragma unroll
    for (int nt = 0; nt < G::NT; nt++) {
        const int n = nt * 8 + g;
#pragma unroll
        for (int ks = 0; ks < G::NKS; ks++) {
            const int k0 = ks * 8 + t, k1 = k0 + 4;
            bf[nt][ks][0] = (n < G::N2 && k0 < G::N2) ? to_tf32(scale * M[n * G::N2 + k0]) : 0u;
            bf[nt][ks][1] = (n < G::N2 && k1 < G::N2) ? to_tf32(scale * M[n * G::N2 + k1]) : 0u;
        }
    }
}

// A fragments of one row tile for all steps.  fa(h, k) returns the element of
// fragment row g + 8h at contraction index k (zero outside the matrix); mode
// keeps all columns (0), only k < K (1) or only k >= K (2).
template <int K, int MODE, class FA>
__device__ __forceinline__ void load_a(uint32_t (&a)[TcGeo<K>::NKS][4], int t, FA fa) {
    using G = TcGeo<K>;
#pragma unroll
    for (int ks = 0; ks < G::NKS; ks++) {
        const int k0 = ks * 8 + t, k1 = k0 + 4;
        const bool p0 = MODE == 0 || (MODE == 1 ? k0 < K : k0 >= K);
        const bool p1 = MODE == 0 || (MODE == 1 ? k1 < K : k1 >= K);
        a[ks][0] = p0 ? to_tf32(fa(0, k0)) : 0u;
        a[ks][1] = p0 ? to_tf32(fa(1, k0)) : 0u;
        a[ks][2] = p1 ? to_tf32(fa(0, k1)) : 0u;
        a[ks][3] = p1 ? to_tf32(fa(1, k1)) : 0u;
    }
}

// c += A B over all steps for one column tile.  Steps that MODE masks out entirely are skipped.
template <int K, int MODE>
__device__ __forceinline__ void mma_steps(float (&c)[4], const uint32_t (&a)[TcGeo<K>::NKS][4],
                                          const uint32_t (&b)[TcGeo<K>::NKS][2], uint32_t bmask) {
    using G = TcGeo<K>;
#pragma unroll
    for (int ks = 0; ks < G::NKS; ks++) {
        const bool tail = G::TAIL4 && ks == G::NKS - 1;
        const int lo = ks * 8, hi = ks * 8 + (tail ? 4 : 8);
        if (MODE == 1 && lo >= K) continue;
        if (MODE == 2 && hi <= K) continue;
        if (tail)
            mma_k4(c, a[ks][0], a[ks][1], b[ks][0] & bmask);
        else
            mma_k8(c, a[ks], b[ks][0] & bmask, b[ks][1] & bmask);
    }
}


template <int K>
__global__ void __launch_bounds__(TcGeo<K>::W * 32, 2) apply_tc_kernel(ApplyLaunch L) {
    using G = TcGeo<K>;
    extern __shared__ __align__(16) float smem_tc[];
    float *s_u = smem_tc + G::OU;
    float *s_t2x = smem_tc + G::OT2X;
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ int s_node;
    __shared__ volatile int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    const bool excl = !L.root;
    // item j's input block and operator blocks -> region / operator set `buf` (thread 0 only)
    auto issue = [&](const void *in, const void *ax, const void *ay, const void *az, int buf) {
        float *A = smem_tc + G::OA + buf * 3 * G::NC;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&s_bar, G::TX_BYTES);
        bulk_copy(smem_tc + buf * G::REG, in, 4u * G::C, &s_bar);
        bulk_copy(A, ax, 4u * G::NC, &s_bar);
        bulk_copy(A + G::NC, ay, 4u * G::NC, &s_bar);
        bulk_copy(A + 2 * G::NC, az, 4u * G::NC, &s_bar);
    };
    if (tid == 0) {
        mbar_init(&s_bar);
        s_fail = 0;
    }
    __syncthreads();
    uint32_t parity = 0;

    while (true) {
        if (tid == 0) s_node = atomicAdd(L.counter, 1);
        __syncthreads();
        const int w = s_node;
        if (w >= L.nnodes) break;
        const long long b0 = L.begin[w], b1 = L.end[w];
        if (tid == 0 && b0 < b1) issue(L.in[b0], L.ax[b0], L.ay[b0], L.az[b0], 0);
        float acc[G::MPW][G::NT][4];
#pragma unroll
        for (int i = 0; i < G::MPW; i++)
#pragma unroll
            for (int nt = 0; nt < G::NT; nt++)
#pragma unroll
                for (int e = 0; e < 4; e++) acc[i][nt][e] = 0.0f;
        for (long long j = b0; j < b1; j++) {
            const int p = (int)((j - b0) & 1);
            float *s_in = smem_tc + p * G::REG;        // IN, then T2
            float *s_t2 = s_in;
            float *s_t1 = smem_tc + (p ^ 1) * G::REG;  // T1, then item j+1's input
            const float *s_A = smem_tc + G::OA + p * 3 * G::NC;
            // item j+1's pointers, read early so that their latency is hidden by the x and y passes
            const bool more = j + 1 < b1;
            const void *nin = nullptr, *nax = nullptr, *nay = nullptr, *naz = nullptr;
            if (tid == 0 && more) {
                nin = L.in[j + 1];
                nax = L.ax[j + 1];
                nay = L.ay[j + 1];
                naz = L.az[j + 1];
            }
            const float cf = float(L.coef[j]);
            mbar_wait(&s_bar, parity, &s_fail, L.status);
            parity ^= 1u;
            // ---- x pass: rows (Z, Y), contraction X, columns X'
            {
                uint32_t bf[G::NT][G::NKS][2];
                load_b<K>(bf, s_A, 1.0f, g, t);
#pragma unroll
                for (int i = 0; i < G::MPW; i++) {
                    const int mt = warp + G::W * i;
                    if (!G::EVEN && mt >= G::MT) break;
                    const int r0 = mt * 16 + g;
                    int z[2], y[2];
                    row_ab<K>(r0, z[0], y[0]);
                    row_ab<K>(r0 + 8, z[1], y[1]);
                    const bool v[2] = {r0 < G::R, r0 + 8 < G::R};
                    auto fa = [&](int h, int k) -> float {
                        return (v[h] && k < G::N2) ? s_in[(z[h] * G::N2 + y[h]) * G::N2 + k] : 0.0f;
                    };
                    float c[G::NT][4];
#pragma unroll
                    for (int nt = 0; nt < G::NT; nt++)
#pragma unroll
                        for (int e = 0; e < 4; e++) c[nt][e] = 0.0f;
                    if (excl && mt < G::XT) {
                        uint32_t a[G::NKS][4];
                        load_a<K, 2>(a, t, fa);
#pragma unroll
                        for (int nt = 0; nt < G::NT; nt++) mma_steps<K, 2>(c[nt], a, bf[nt], ~0u);
                        // u: rows in the scaling octant (r < K^2), columns X' < K
#pragma unroll
                        for (int h = 0; h < 2; h++) {
                            if (r0 + 8 * h >= G::KK) continue;
#pragma unroll
                            for (int nt = 0; nt < G::NTS; nt++)
#pragma unroll
                                for (int e = 0; e < 2; e++) {
                                    const int xp = nt * 8 + 2 * t + e;
                                    if (xp < K) s_u[z[h] * G::SZU + y[h] * G::SY1 + xp] = c[nt][2 * h + e];
                                }
                        }
                        load_a<K, 1>(a, t, fa);
#pragma unroll
                        for (int nt = 0; nt < G::NT; nt++) mma_steps<K, 1>(c[nt], a, bf[nt], ~0u);
                    } else {
                        uint32_t a[G::NKS][4];
                        load_a<K, 0>(a, t, fa);
#pragma unroll
                        for (int nt = 0; nt < G::NT; nt++) mma_steps<K, 0>(c[nt], a, bf[nt], ~0u);
                    }
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        if (!v[h]) continue;
                        float *row = s_t1 + z[h] * G::SZ1 + y[h] * G::SY1;
#pragma unroll
                        for (int nt = 0; nt < G::NT; nt++) {
                            const int xp = nt * 8 + 2 * t;
                            if (xp < G::N2) *reinterpret_cast<float2 *>(row + xp) = make_float2(c[nt][2 * h], c[nt][2 * h + 1]);
                        }
                    }
                }
            }
            __syncthreads();
            // ---- y pass: rows (Z, X'), contraction Y, columns Y'
            {
                uint32_t bf[G::NT][G::NKS][2];
                load_b<K>(bf, s_A + G::NC, 1.0f, g, t);
#pragma unroll
                for (int i = 0; i < G::MPW; i++) {
                    const int mt = warp + G::W * i;
                    if (!G::EVEN && mt >= G::MT) break;
                    const int r0 = mt * 16 + g;
                    int z[2], xp[2];
                    row_ab<K>(r0, z[0], xp[0]);
                    row_ab<K>(r0 + 8, z[1], xp[1]);
                    const bool v[2] = {r0 < G::R, r0 + 8 < G::R};
                    auto fa = [&](int h, int k) -> float {
                        return (v[h] && k < G::N2) ? s_t1[z[h] * G::SZ1 + k * G::SY1 + xp[h]] : 0.0f;
                    };
                    float c[G::NT][4];
#pragma unroll
                    for (int nt = 0; nt < G::NT; nt++)
#pragma unroll
                        for (int e = 0; e < 4; e++) c[nt][e] = 0.0f;
                    {
                        uint32_t a[G::NKS][4];
                        load_a<K, 0>(a, t, fa);
#pragma unroll
                        for (int nt = 0; nt < G::NT; nt++) mma_steps<K, 0>(c[nt], a, bf[nt], ~0u);
                    }
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        if (!v[h]) continue;
                        float *col = s_t2 + z[h] * G::SZ2 + xp[h];
#pragma unroll
                        for (int nt = 0; nt < G::NT; nt++)
#pragma unroll
                            for (int e = 0; e < 2; e++) {
                                const int yp = nt * 8 + 2 * t + e;
                                if (yp < G::N2) col[yp * G::SY2] = c[nt][2 * h + e];
                            }
                    }
                    if (excl && mt < G::XT) {
                        // t2x on the scaling octant: u replaces T1 for Y < K in rows r < K^2
                        auto fs = [&](int h, int k) -> float {
                            if (!v[h] || k >= G::N2) return 0.0f;
                            if (r0 + 8 * h < G::KK && k < K) return s_u[z[h] * G::SZU + k * G::SY1 + xp[h]];
                            return s_t1[z[h] * G::SZ1 + k * G::SY1 + xp[h]];
                        };
                        uint32_t a[G::NKS][4];
                        load_a<K, 0>(a, t, fs);
                        float cx[G::NTS][4];
#pragma unroll
                        for (int nt = 0; nt < G::NTS; nt++) {
#pragma unroll
                            for (int e = 0; e < 4; e++) cx[nt][e] = 0.0f;
                            mma_steps<K, 0>(cx[nt], a, bf[nt], ~0u);
                        }
#pragma unroll
                        for (int h = 0; h < 2; h++) {
                            if (r0 + 8 * h >= G::KK) continue;
#pragma unroll
                            for (int nt = 0; nt < G::NTS; nt++)
#pragma unroll
                                for (int e = 0; e < 2; e++) {
                                    const int yp = nt * 8 + 2 * t + e;
                                    if (yp < K) s_t2x[z[h] * G::SZX + yp * G::SY2 + xp[h]] = cx[nt][2 * h + e];
                                }
                        }
                    }
                }
            }
            __syncthreads();
            // T1's region is free: item j+1's blocks are copied into it during the z pass
            if (tid == 0 && more) issue(nin, nax, nay, naz, p ^ 1);
            // ---- z pass: rows (Y', X'), contraction Z, columns Z'; accumulate c_t * ... into acc
            {
                uint32_t bf[G::NT][G::NKS][2];
                load_b<K>(bf, s_A + 2 * G::NC, cf, g, t);
#pragma unroll
                for (int i = 0; i < G::MPW; i++) {
                    const int mt = warp + G::W * i;
                    if (!G::EVEN && mt >= G::MT) break;
                    const int r0 = mt * 16 + g;
                    int yp[2], xp[2];
                    row_ab<K>(r0, yp[0], xp[0]);
                    row_ab<K>(r0 + 8, yp[1], xp[1]);
                    const bool v[2] = {r0 < G::R, r0 + 8 < G::R};
                    auto fa = [&](int h, int k) -> float {
                        return (v[h] && k < G::N2) ? s_t2[k * G::SZ2 + yp[h] * G::SY2 + xp[h]] : 0.0f;
                    };
                    uint32_t a[G::NKS][4];
                    load_a<K, 0>(a, t, fa);
                    if (excl && mt < G::XT) {
                        // scaling-octant rows take t2x for Z < K in the columns Z' < K
                        auto fs = [&](int h, int k) -> float {
                            if (!v[h] || k >= G::N2) return 0.0f;
                            if (r0 + 8 * h < G::KK && k < K) return s_t2x[k * G::SZX + yp[h] * G::SY2 + xp[h]];
                            return s_t2[k * G::SZ2 + yp[h] * G::SY2 + xp[h]];
                        };
                        uint32_t as[G::NKS][4];
                        load_a<K, 0>(as, t, fs);
#pragma unroll
                        for (int nt = 0; nt < G::NT; nt++) {
                            if (nt * 8 + 8 <= K) {
                                mma_steps<K, 0>(acc[i][nt], as, bf[nt], ~0u);
                            } else if (nt * 8 >= K) {
                                mma_steps<K, 0>(acc[i][nt], a, bf[nt], ~0u);
                            } else {
                                // column n = nt*8 + g of the B fragment: scaling if n < K
                                const uint32_t ms = (nt * 8 + g < K) ? ~0u : 0u;
                                mma_steps<K, 0>(acc[i][nt], as, bf[nt], ms);
                                mma_steps<K, 0>(acc[i][nt], a, bf[nt], ~ms);
                            }
                        }
                    } else {
#pragma unroll
                        for (int nt = 0; nt < G::NT; nt++) mma_steps<K, 0>(acc[i][nt], a, bf[nt], ~0u);
                    }
                }
            }
            __syncthreads();  // item j+1's x pass writes T1 into this item's IN / T2 region
        }
        // ---- node epilogue: acc rows (Y', X'), columns Z' -> component-major FP64 block
        {
            double *out = L.out[w];
#pragma unroll
            for (int i = 0; i < G::MPW; i++) {
                const int mt = warp + G::W * i;
                if (!G::EVEN && mt >= G::MT) break;
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int r = mt * 16 + g + 8 * h;
                    if (r >= G::R) continue;
                    int yp, xp;
                    row_ab<K>(r, yp, xp);
#pragma unroll
                    for (int nt = 0; nt < G::NT; nt++)
#pragma unroll
                        for (int e = 0; e < 2; e++) {
                            const int zp = nt * 8 + 2 * t + e;
                            if (zp >= G::N2) continue;
                            const int c = (xp >= K ? 1 : 0) | (yp >= K ? 2 : 0) | (zp >= K ? 4 : 0);
                            const int gi = c * G::K3 + (zp % K) * K * K + (yp % K) * K + (xp % K);
                            const double val = double(acc[i][nt][2 * h + e]);
                            if (L.set)
                                out[gi] = val;
                            else
                                out[gi] += val;
                        }
                }
            }
        }
        __syncthreads();
    }
}

template <int K>
void launch_tc(const ApplyLaunch &L, int nsm, cudaStream_t s) {
    using G = TcGeo<K>;
    const int threads = G::W * 32;
    const size_t smem = sizeof(float) * (size_t)G::TOTAL;
    MWG_CUDA(cudaFuncSetAttribute(apply_tc_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    MWG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, apply_tc_kernel<K>, threads, smem));
    if (per_sm < 1) per_sm = 1;
    // one CTA per task (tasks are ordered longest first and taken in that order): CTAs end
    // throughout the launch, so kernels of other streams get SM slots without waiting for it
    (void)nsm;
    const int grid = L.nnodes;
    if (grid < 1) return;
    apply_tc_kernel<K><<<grid, threads, smem, s>>>(L);
    MWG_CUDA(cudaGetLastError());
}

}  // namespace

void k_apply_tc(const DevBasis &b, const ApplyLaunch &L, int nsm, cudaStream_t s) {
    if (L.nnodes <= 0) return;
    MWG_CUDA(cudaMemsetAsync(L.counter, 0, sizeof(int), s));
    MWG_CUDA(cudaMemsetAsync(L.status, 0, sizeof(int), s));
    switch (b.K) {
        case 4: launch_tc<4>(L, nsm, s); break;
        case 5: launch_tc<5>(L, nsm, s); break;
        case 6: launch_tc<6>(L, nsm, s); break;
        case 7: launch_tc<7>(L, nsm, s); break;
        case 8: launch_tc<8>(L, nsm, s); break;
        case 9: launch_tc<9>(L, nsm, s); break;
        case 10: launch_tc<10>(L, nsm, s); break;
        default: throw Error(MW_ERR_ARG, "no tensor-core apply kernel for this order");
    }
}

}  // namespace mwg
