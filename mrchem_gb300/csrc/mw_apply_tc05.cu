// mw_apply_tc05.cu -- TF32 tier of the NS-form apply on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory).
//
// The item contraction of the other tiers (mw_kernels.cu),
//
//   x pass  T1[(Z,Y)][X']  = sum_X IN[Z][Y][X]  A_x[X'][X]
//   y pass  T2[(X',Z)][Y'] = sum_Y T1[Z][Y][X'] A_y[Y'][Y]
//   z pass  OUT[(Y',X')][Z'] += sum_Z T2[Z][Y'][X'] c A_z[Z'][Z],
//
// as three GEMMs D[M x N] = A[M x 8k] B[N x 8k]^T of tcgen05.mma.kind::tf32 with M = 128,
// N = 32 (16 for K <= 5) and FP32 accumulation in tensor memory (TMEM).  The rows of a pass are
// its (2K)^2 index pairs, padded to whole tiles of 128; the columns are the 2K output indices.
// One thread issues the MMAs of a pass and commits them to an mbarrier; eight warps (sixteen in
// the split kernel where it has an SM to itself) then read
// the result out of TMEM (tcgen05.ld, one row per thread), round it to TF32 (cvt.rna) and store
// it as the A operand of the next pass.  The z pass accumulates into a second TMEM region that
// holds the output node for all of its items and is written to the FP64 block once.
//
// The scaling-scaling path is left out exactly below the root scale, as in the other tiers
// (no subtraction):
//   u   = the wavelet-in-x part of T1 on the scaling octant: K spare columns of the x pass get
//         the first K rows of A_x with the scaling columns zeroed (prepared with the operator
//         blocks), so one set of x MMAs yields T1 and u;
//   t2x = the y pass in which u replaces T1 for Y < K: K^2 extra rows (X', Z < K) of the y pass
//         (the row padding of the last tile has room for them);
//   the z pass takes t2x for Z < K in K^2 extra rows (Y', X' < K), whose columns Z' < K replace
//         those of the ordinary rows in the node epilogue.
//
// Operands in shared memory use the canonical K-major layout without swizzling: k-groups of 4
// columns, row r of a group at byte 16 r (8-row core matrices of 128 bytes, M-direction stride
// SBO = 128), groups LBO bytes apart.  The x pass's A (the input block) and every B (operator
// block) arrive in that layout, already rounded to TF32, by one bulk copy (TMA engine) each:
// the host prepares them once per input tree and per operator (mw_tc05_layout.h).  A_y and A_z
// are written by the epilogues into region R, whose LBO is padded to 80 mod 128 bytes so that
// the stores of a warp (one k per lane, rows shifted by one between the warp's runs of lanes)
// fall into distinct banks.  The coefficient c_t scales A_z (written by the y epilogue), so the
// operator blocks need no per-item scaling.
//
// Buffers: S (the input block, x pass), R (A_y, then A_z), a zero pad, and two sets of the
// three B operands.  The next item's copies (into S and the other B set) start as soon as the
// x MMAs have read S, so they run during this item's epilogues and y and z MMAs.
//
// Synchronisation: only the issuing thread waits for the copies (no other thread reads S or the
// B operands), so it cannot start the next item's copies while another thread still waits for
// the current ones.  A commit tracks every earlier MMA of the issuing thread, so the x pass's
// barrier also says that the previous item's z MMAs are done with R and their B set; the z MMAs
// get a commit of their own only at the end of a node.  The last k-step of a pass may read one k-group past
// its operand (2K is not a multiple of 8): the B operands are zero there, and the bytes read
// (S runs into R, R into the zero pad) are finite and not written while those MMAs run.  With
// about 97 KB of shared memory and 256 TMEM columns per CTA, two CTAs share an SM, so one CTA's
// MMAs run while the other's warps move data.
//
// Rounding: every operand is rounded to TF32 (unit roundoff 2^-11) as in the warp-level MMA
// version, so an item is off by at most about 6 * 2^-11 * b (b = its screening bound).  A row's
// items share the intermediates' roundings, which are relative to the row's sum: the row is off
// by at most the sum of its items' bounds, as the items would be one by one.
//
// Every wait on an mbarrier is bounded; one that runs out marks the launch failed (status word,
// reported by the host as MW_ERR_TIMEOUT) and the kernel ends normally, freeing its TMEM.
#include "mw_async.cuh"
#include "mw_chunks.cuh"
#include "mw_host.h"
#include "mw_tc05_layout.h"

#include <algorithm>

namespace mwg {

namespace {

template <int K>
struct T5Geo {
    static constexpr int N2 = 2 * K, NN = N2 * N2, KK = K * K, K3 = K * K * K;
    static constexpr int RE = NN + KK;                 // rows of the y and z passes (ordinary + extra)
    static constexpr int MT = (RE + 127) / 128;        // M tiles of the y and z passes
    static constexpr int MTX = (NN + 127) / 128;       // M tiles of the x pass
    static constexpr int N = tc5_n(K);                 // MMA N: 2K outputs + K columns of u
    static constexpr int KG = tc5_kg(K);               // k-groups holding data
    static constexpr int KS = tc5_ks(K);               // MMA k-steps of 8
    static constexpr int LBO_S = NN * 16;              // the input block as staged (x pass A)
    static constexpr int SX = KG * LBO_S;
    static constexpr int LBO_R = ((RE * 16 - 80 + 127) / 128) * 128 + 80;  // >= RE rows, 80 mod 128
    static constexpr int LBO_B = N * 16;
    static constexpr int BSZ = 2 * KS * LBO_B;         // bytes of one B operand (all k-steps)
    static constexpr int OR = SX, RSZ = KG * LBO_R;
    // bytes an MMA pass reads from the start of its A operand
    static constexpr int READ_S = (2 * KS - 1) * LBO_S + MTX * 2048;
    static constexpr int READ_R = (2 * KS - 1) * LBO_R + MT * 2048;
    static constexpr int ZPAD = READ_R > RSZ ? READ_R - RSZ : 0;
    static constexpr int OB = OR + RSZ + ZPAD;         // two sets of (B_x, B_y, B_z)
    static constexpr int SMEM = OB + 6 * BSZ;
    static constexpr int TMEM_COLS = 2 * MT * N <= 32 ? 32 : (2 * MT * N <= 64 ? 64 : (2 * MT * N <= 128 ? 128 : 256));
    static constexpr uint32_t STAGE_BYTES = (uint32_t)(SX + 3 * BSZ);
    // dynamic shared memory requested at launch: at least enough that no more CTAs share an SM
    // than its 512 TMEM columns serve (an allocation beyond them would wait for another CTA)
    static constexpr int MAX_CTAS = 512 / TMEM_COLS;
    static constexpr int SMEM_FLOOR = 228 * 1024 / (MAX_CTAS + 1);
    static constexpr int SMEM_LAUNCH = MAX_CTAS >= 8 || SMEM >= SMEM_FLOOR ? SMEM : SMEM_FLOOR;
    static_assert(N2 + K <= N, "u columns do not fit");
    static_assert(2 * MT * N <= 256, "TMEM budget");
    static_assert((size_t)SX == tc5_x_floats(K) * 4 && (size_t)BSZ == tc5_b_floats(K) * 4, "layouts");
    static_assert(LBO_R >= RE * 16 && LBO_R % 128 == 80, "R layout");
    static_assert(READ_S <= SX + RSZ, "the x pass reads past R");
    static_assert(SX % 16 == 0 && OB % 16 == 0 && BSZ % 16 == 0, "alignment");
    static_assert(SMEM <= 113 * 1024, "two CTAs per SM");
};

// Shared-memory layout of the kernel: SPLIT = 0 is the TF32 tier, SPLIT = 1 the split-TF32 tier,
// whose operands are stored twice (hi, then lo): S_hi S_lo | R_hi R_lo | zero pad | two sets of
// (B_x hi lo, B_y hi lo, B_z hi lo).  An MMA pass reads past its operand's end (last k-step):
// S_hi into S_lo, S_lo into R_hi, R_hi into R_lo, R_lo into the pad, all finite and not written
// while those MMAs run; the B operands are zero there.
template <int K, int SPLIT>
struct T5Mem {
    using G = T5Geo<K>;
    static constexpr int NP = SPLIT ? 2 : 1;  // stored parts per operand
    static constexpr int OR = NP * G::SX;      // R (hi) starts here; R lo at OR + RSZ
    static constexpr int OB = OR + NP * G::RSZ + G::ZPAD;
    static constexpr int BSET = 3 * NP * G::BSZ;  // one set of B operands
    static constexpr int SMEM = OB + 2 * BSET;
    static constexpr uint32_t STAGE_BYTES = (uint32_t)(NP * (G::SX + 3 * G::BSZ));
    // TMEM columns per M tile: the split tier's MMAs of width 2N put A_hi * B_hi in a tile's first N
    // columns and A_hi * B_lo in the next N; the epilogues add the two halves
    static constexpr bool WIDE = SPLIT && tc5_split_wide(K);
    static constexpr int NT = WIDE ? 2 * G::N : G::N;
    static constexpr int TMEM_COLS = WIDE ? (2 * G::MT * NT <= 64 ? 64 : (2 * G::MT * NT <= 128 ? 128 : (2 * G::MT * NT <= 256 ? 256 : 512)))
                                          : G::TMEM_COLS;
    // B operand k-group stride: the wide form's layout holds a group's N hi rows, then its N lo rows
    static constexpr int LBO_B = WIDE ? 2 * G::LBO_B : G::LBO_B;
    static_assert(2 * G::MT * NT <= 512, "TMEM budget");
    // as for the TF32 tier: request enough shared memory that no more CTAs share an SM than its 512
    // TMEM columns serve (a CTA whose allocation waits would hold its SM's resources idle)
    static constexpr int MAX_CTAS = SPLIT ? 512 / TMEM_COLS : G::MAX_CTAS;
    // CTAs per SM of the split tier with the narrow and the wide tiles (TMEM, shared memory, and
    // registers: about 90 a thread x 288 threads leave room for two CTAs); the wide form is used
    // only where it keeps the count
    static constexpr int fits(int tmem_cols) {
        return (512 / tmem_cols) < (228 * 1024 / SMEM) ? ((512 / tmem_cols) < 2 ? (512 / tmem_cols) : 2)
                                                       : ((228 * 1024 / SMEM) < 2 ? (228 * 1024 / SMEM) : 2);
    }
    static constexpr int WIDE_COLS = 2 * G::MT * 2 * G::N <= 64    ? 64
                                     : 2 * G::MT * 2 * G::N <= 128 ? 128
                                     : 2 * G::MT * 2 * G::N <= 256 ? 256
                                                                   : 512;
    static_assert(!SPLIT || tc5_split_wide(K) == (fits(WIDE_COLS) >= fits(G::TMEM_COLS)),
                  "tc5_split_wide: the wide tiles exactly where they keep the CTAs per SM");
    // epilogue warps: where the split kernel has an SM to itself (its shared memory admits one CTA)
    // sixteen, one TMEM tile quarter each per pass, so that its epilogues take half as long; else
    // eight (two CTAs per SM overlap one CTA's epilogues with the other's MMAs).  Warp w reads
    // lane quarter w % 4 of tiles w / 4, w / 4 + TS, ...
    static constexpr int EPI_WARPS = (SPLIT && SMEM > 114 * 1024) ? 16 : 8;
    static constexpr int TS = EPI_WARPS / 4;
    static constexpr int THREADS = 32 * EPI_WARPS + 32;  // + one warp that issues copies and MMAs
    static_assert(!(SPLIT && SMEM > 114 * 1024) || THREADS * 120 <= 65536, "registers for one CTA");
    static constexpr int SMEM_FLOOR = 228 * 1024 / (MAX_CTAS + 1);
    static constexpr int SMEM_LAUNCH = !SPLIT ? G::SMEM_LAUNCH : (MAX_CTAS >= 8 || SMEM >= SMEM_FLOOR ? SMEM : SMEM_FLOOR);
    static_assert(SPLIT || (OR == G::OR && OB == G::OB && SMEM == G::SMEM && STAGE_BYTES == G::STAGE_BYTES),
                  "the TF32 tier's layout");
    static_assert(OR % 16 == 0 && OB % 16 == 0 && BSET % 16 == 0 && G::RSZ % 16 == 0, "alignment");
    static_assert(SMEM <= 227 * 1024, "shared memory");
};

__device__ __forceinline__ float tf32r(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// shared-memory matrix descriptor: canonical K-major layout without swizzling
__device__ __forceinline__ uint64_t t5_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ void t5_mma(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void t5_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void t5_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void t5_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void async_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Loads of TMEM into registers.  tcgen05.ld is asynchronous: t5_ld* only start a load of 32
// (N = 32) or 16 (N = 16) consecutive columns of this warp's 32 lanes (r[j] = column j of lane
// base + lane); t5_wait ends every load of the thread and takes the registers of the load as
// in-out operands, so that no use of them is scheduled before it.
#define T5_R32(r)                                                                                          \
    "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), \
        "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]), "+r"(r[16]),   \
        "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]), "+r"(r[22]), "+r"(r[23]), "+r"(r[24]),  \
        "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]), "+r"(r[29]), "+r"(r[30]), "+r"(r[31])

__device__ __forceinline__ void t5_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%"
        "19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}

__device__ __forceinline__ void t5_ld16(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int j = 16; j < 32; j++) r[j] = 0u;
}

template <int K>
__device__ __forceinline__ void t5_ld(uint32_t taddr, uint32_t (&r)[32]) {
    if (T5Geo<K>::N == 32)
        t5_ld32(taddr, r);
    else
        t5_ld16(taddr, r);
}

__device__ __forceinline__ void t5_wait(uint32_t (&r)[32]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;" : T5_R32(r) : : "memory");
}


// element (row r, column k) of region R (k-group stride LBO_R, 16 bytes per row)
template <int K>
__device__ __forceinline__ float *r_at(uint8_t *R, int r, int k) {
    return reinterpret_cast<float *>(R + (k >> 2) * T5Geo<K>::LBO_R + 16 * r + 4 * (k & 3));
}

// the epilogue of one pass for the TMEM tiles of this warp (tiles half, half + TS, ... < tiles);
// WIDE: a tile is 2N columns wide and a row's value is the sum of its two halves
template <int K, bool WIDE, int TS, class Row>
__device__ __forceinline__ void t5_epilogue(uint32_t tcol, int tiles, int q, int half, int lane, Row row) {
    constexpr int N = T5Geo<K>::N, NT = WIDE ? 2 * N : N;
    for (int i = half; i < tiles; i += TS) {
        uint32_t a[32];
        const uint32_t t = tcol + ((uint32_t)(32 * q) << 16) + (uint32_t)(i * NT);
        t5_ld<K>(t, a);
        t5_wait(a);
        if (WIDE) {
            uint32_t b[32];
            t5_ld<K>(t + (uint32_t)N, b);
            t5_wait(b);
#pragma unroll
            for (int j = 0; j < N; j++) a[j] = __float_as_uint(__fadd_rn(__uint_as_float(a[j]), __uint_as_float(b[j])));
        }
        row(i * 128 + 32 * q + lane, a);
    }
}

// The TF32 tier at k >= 7 is held to 64 registers (it needs 71 at K = 10; no spills at 64): two
// of its CTAs (2 x 9 warps x 64) and one CTA of the double-FP32 tier (13 warps x 112) then fit in
// an SM's 65,536 registers together, as they do in shared memory, so the two tiers' kernels of
// different job groups can share SMs (tensor pipe and FP32 pipe side by side).
template <int K, int SPLIT>
__global__ void __launch_bounds__(T5Mem<K, SPLIT>::THREADS, SPLIT ? 1 : 2) __maxnreg__(SPLIT || K < 8 ? 128 : 64)
    apply_tc05_kernel(ApplyLaunch L) {
    using G = T5Geo<K>;
    using M = T5Mem<K, SPLIT>;
    constexpr int N2 = G::N2, NN = G::NN, KK = G::KK, K3 = G::K3, N = G::N;
    extern __shared__ __align__(1024) uint8_t smem5[];
    uint8_t *sS = smem5, *sR = smem5 + M::OR, *sB = smem5 + M::OB;
    // an epilogue value into the next pass's A operand: rounded to TF32, and for the split tier
    // the remainder rounded to TF32 in the lo copy of R
    auto put = [&](float *dst, float v) {
        const float h = tf32r(v);
        dst[0] = h;
        if (SPLIT) dst[G::RSZ / 4] = tf32r(__fsub_rn(v, h));
    };
    // barriers: 0 staging copies, 1 x MMAs (every item; the issuing thread waits), 2 y MMAs, 3 end
    // of a node, 4 draining after a failed wait, 5 x MMAs of a row's last item (the epilogue warps
    // wait).  A barrier's waiters tell its phases apart by parity only, so none may complete twice
    // before every waiter has seen the first: the items of a row sync nowhere, so the epilogue warps
    // wait on bar 5, which completes once per row, before a sync, and never on bar 1.
    __shared__ __align__(8) uint64_t bar[6];
    __shared__ uint32_t s_tmem;
    __shared__ int s_node, s_redf;
    __shared__ volatile int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool producer = warp == M::EPI_WARPS;  // copies and MMAs (lane 0)
    const bool issuer = producer && lane == 0;
    const int q = warp & 3, half = warp >> 2;  // epilogue warps: TMEM lane quarter, first tile
    const bool excl = !L.root;

    // zero everything once: padding rows, columns and k-groups are read by the MMAs
    for (int i = tid; i < M::SMEM / 16; i += blockDim.x) reinterpret_cast<float4 *>(smem5)[i] = make_float4(0, 0, 0, 0);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&s_tmem)),
                     "r"(M::TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int b = 0; b < 6; b++) mbar_init(&bar[b]);
        s_fail = 0;
    }
    async_fence();
    t5_before_sync();
    __syncthreads();
    t5_after_sync();
    const uint32_t tmem = s_tmem;
    const uint32_t tD = tmem, tACC = tmem + (uint32_t)(G::MT * M::NT);  // column offsets
    // instruction descriptors: F32 accumulator, TF32 A and B, M = 128, N = N (and 2N for the split
    // tier's MMAs that take B_hi and B_lo side by side)
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    const uint32_t idesc2 = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(M::NT >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    // descriptors of the operands' first core matrices; a tile / k-step adds its byte offset >> 4
    const uint64_t dS = t5_desc(smem_addr(sS), G::LBO_S, 128), dR = t5_desc(smem_addr(sR), G::LBO_R, 128);
    const uint64_t dB = t5_desc(smem_addr(sB), M::LBO_B, 128);
    uint32_t ph = 0;     // bit b: the parity of barrier b's next phase (a thread tracks the ones it waits on)
    uint32_t nitem = 0;  // items this CTA has started: B set nitem & 1

    auto stage = [&](const void *in, const void *ax, const void *ay, const void *az, uint32_t set) {
        if (s_fail) return;  // the issuing thread: the item's input block and B operands
        async_fence();
        mbar_expect_tx(&bar[0], M::STAGE_BYTES);
        uint8_t *B = sB + set * M::BSET;
        // each stored operand is hi, then lo (mw_tc05_layout.h): one copy of hi, or of hi and lo
        bulk_copy(sS, in, M::NP * G::SX, &bar[0]);
        bulk_copy(B, ax, M::NP * G::BSZ, &bar[0]);
        bulk_copy(B + M::NP * G::BSZ, ay, M::NP * G::BSZ, &bar[0]);
        bulk_copy(B + 2 * M::NP * G::BSZ, az, M::NP * G::BSZ, &bar[0]);
    };
    // status on a wait that runs out: 1 + barrier + 8 * (parity) + 16 * (items this CTA had started)
    auto wait = [&](int b) {
        const uint32_t p = (ph >> b) & 1u;
        mbar_wait(&bar[b], p, &s_fail, L.status, 1 + b + 8 * (int)p + 16 * (int)(nitem < 65535u ? nitem : 65535u));
        ph ^= 1u << b;
    };
    // all threads: the MMAs may read what was stored; the issuing thread then orders after the sync
    auto publish = [&]() {
        async_fence();
        t5_before_sync();
        __syncthreads();
        t5_after_sync();
    };
    // the issuing thread: tiles x k-steps of one pass, then a commit to barrier b (none if b < 0)
    // split tier, wide form: per tile and k-step, A_hi * [B_hi B_lo] (width 2N: hi * hi and hi * lo
    // side by side) and A_lo * B_hi (width N, into the first half); narrow form: hi * hi, hi * lo
    // and lo * hi into one accumulator of width N (B_lo BSZ bytes after B_hi).  lo * lo is dropped.
    // a_lo: the descriptor offset of A's lo copy
    auto issue_pass = [&](uint64_t da, int lbo_a, uint32_t a_lo, uint64_t db, int tiles, uint32_t dcol,
                          bool accumulate, int b) {
        if (s_fail) return;
        constexpr uint32_t b_lo = (uint32_t)(G::BSZ >> 4);
        for (int i = 0; i < tiles; i++)
#pragma unroll
            for (int s = 0; s < G::KS; s++) {
                const uint64_t a = da + (uint64_t)((2 * s * lbo_a + i * 2048) >> 4);
                const uint64_t bb = db + (uint64_t)((2 * s * M::LBO_B) >> 4);
                const uint32_t d = dcol + (uint32_t)(i * M::NT);
                t5_mma(d, a, bb, M::WIDE ? idesc2 : idesc, (accumulate || s > 0) ? 1u : 0u);
                if (SPLIT && !M::WIDE) t5_mma(d, a, bb + b_lo, idesc, 1u);
                if (SPLIT) t5_mma(d, a + a_lo, bb, idesc, 1u);
            }
        if (b >= 0) t5_commit(&bar[b]);
    };
    constexpr uint32_t S_LO = (uint32_t)(G::SX >> 4), R_LO = (uint32_t)(G::RSZ >> 4);

    while (true) {
        if (tid == 0) s_node = atomicAdd(L.counter, 1);
        __syncthreads();
        const int w = s_node;
        if (w >= L.nnodes) break;
        const long long b0 = L.begin[w], b1 = L.end[w];
        int nrows = 0;  // rows of this task
        if (issuer && b0 < b1) stage(L.in[b0], L.ax[b0], L.ay[b0], L.az[b0], nitem & 1u);
        bool acc_on = false;  // the node accumulator holds a row's z pass
        for (long long j = b0; j < b1; j++, nitem++) {
            const uint32_t set = nitem & 1u;
            const uint64_t dBs = dB + (uint64_t)((set * M::BSET) >> 4);
            constexpr uint32_t BPASS = (uint32_t)((M::NP * G::BSZ) >> 4);  // B_x -> B_y -> B_z
            // rows: a node's items come in walk order (term, then lz, ly, lx), so the items of one
            // term and (ly, lz), i.e. with the same B_y and B_z, follow one another.  Their x passes
            // accumulate into D (x is linear), and the row's last item runs the x epilogue and the y
            // and z passes once, on the sum.  Every thread reads the same pointers: `last` is uniform.
            const bool first = j == b0 || L.ay[j - 1] != L.ay[j] || L.az[j - 1] != L.az[j];
            const bool last = j + 1 == b1 || L.ay[j + 1] != L.ay[j] || L.az[j + 1] != L.az[j];
            if (producer) {
                if (lane == 0) {
                    const bool more = j + 1 < b1;
                    const void *nin = nullptr, *nax = nullptr, *nay = nullptr, *naz = nullptr;
                    if (more) {  // item j+1's pointers, read while item j's copies land
                        nin = L.in[j + 1];
                        nax = L.ax[j + 1];
                        nay = L.ay[j + 1];
                        naz = L.az[j + 1];
                    }
                    wait(0);  // item j's input block and B operands are in S and B set `set`
                    issue_pass(dS, G::LBO_S, S_LO, dBs, G::MTX, tD, !first, 1);
                    if (last && !s_fail) t5_commit(&bar[5]);
                    // the x MMAs, and every earlier MMA (the previous row's z pass), are done:
                    // S and the other B set are free for item j+1
                    wait(1);
                    if (more) stage(nin, nax, nay, naz, set ^ 1u);
                }
                __syncwarp();
            } else {
                // ---- x epilogue: D row (Z, Y) -> A_y rows (X', Z) and extra rows (X' < K, Z < K), k = Y
                if (last) wait(5);  // the row's x MMAs
                if (last) t5_after_sync();
                if (last) t5_epilogue<K, M::WIDE, M::TS>(tD, G::MTX, q, half, lane, [&](int r, const uint32_t (&v)[32]) {
                    if (r >= NN) return;
                    const int Z = r / N2, Y = r - Z * N2;
                    float *base = r_at<K>(sR, 0, Y);
#pragma unroll
                    for (int xp = 0; xp < N2; xp++) put(base + 4 * (xp * N2 + Z), __uint_as_float(v[xp]));
                    if (Z < K) {
#pragma unroll
                        for (int xp = 0; xp < K; xp++)
                            put(base + 4 * (NN + xp * K + Z), __uint_as_float(Y < K ? v[N2 + xp] : v[xp]));
                    }
                });
            }
            if (!last) continue;
            nrows++;
            publish();
            if (issuer) issue_pass(dR, G::LBO_R, R_LO, dBs + BPASS, G::MT, tD, false, 2);
            if (!producer) {
                // ---- y epilogue: D row (X', Z) -> c * A_z rows (Y', X') with k = Z; extra rows (Y', X' < K)
                const float cf = float(L.coef[j]);
                wait(2);
                t5_after_sync();
                t5_epilogue<K, M::WIDE, M::TS>(tD, G::MT, q, half, lane, [&](int r, const uint32_t (&v)[32]) {
                    if (r < NN) {
                        const int xp = r / N2, Z = r - xp * N2;
                        float *base = r_at<K>(sR, 0, Z);
#pragma unroll
                        for (int yp = 0; yp < N2; yp++) put(base + 4 * (yp * N2 + xp), cf * __uint_as_float(v[yp]));
                        if (Z >= K && xp < K) {
#pragma unroll
                            for (int yp = 0; yp < K; yp++) put(base + 4 * (NN + yp * K + xp), cf * __uint_as_float(v[yp]));
                        }
                    } else if (r < G::RE) {
                        const int e = r - NN, xp = e / K, Z = e - xp * K;
                        float *base = r_at<K>(sR, 0, Z);
#pragma unroll
                        for (int yp = 0; yp < K; yp++) put(base + 4 * (NN + yp * K + xp), cf * __uint_as_float(v[yp]));
                    }
                });
            }
            publish();
            if (issuer) issue_pass(dR, G::LBO_R, R_LO, dBs + 2 * BPASS, G::MT, tACC, acc_on, -1);
            acc_on = true;
        }
        // ---- node epilogue: accumulator rows (Y', X'), columns Z' -> component-major FP64 block
        if (b0 < b1 && issuer && !s_fail) t5_commit(&bar[3]);
        if (!producer) {
            if (b0 < b1) wait(3);
            t5_after_sync();
            double *out = L.out[w];
            auto row = [&](int r, const uint32_t (&v)[32]) {
                int yp = -1, xp = 0, zmax = 0, zmin = 0;
                if (r < NN) {
                    yp = r / N2;
                    xp = r - yp * N2;
                    zmax = N2;
                    zmin = (excl && yp < K && xp < K) ? K : 0;  // Z' < K from the extra row
                } else if (r < G::RE && excl) {
                    const int e = r - NN;
                    yp = e / K;
                    xp = e - yp * K;
                    zmax = K;
                }
                if (yp < 0) return;
                const int cxy = (xp >= K ? 1 : 0) | (yp >= K ? 2 : 0);
                const int off = (yp % K) * K + (xp % K);
#pragma unroll
                for (int zp = 0; zp < N2; zp++) {
                    if (zp < zmin || zp >= zmax) continue;
                    const int gi = (cxy | (zp >= K ? 4 : 0)) * K3 + (zp % K) * KK + off;
                    const double val = b0 < b1 ? double(__uint_as_float(v[zp])) : 0.0;
                    if (L.set)
                        out[gi] = val;
                    else
                        out[gi] += val;
                }
            };
            if (b0 < b1) {
                t5_epilogue<K, M::WIDE, M::TS>(tACC, G::MT, q, half, lane, row);
            } else {
                uint32_t zero[32] = {};
                for (int i = half; i < G::MT; i += M::TS) row(i * 128 + 32 * q + lane, zero);
            }
        }
        t5_before_sync();
        __syncthreads();
        t5_after_sync();
        if (tid == 0 && nrows > 0 && L.rows) atomicAdd(L.rows, nrows);
        finish_chunk(L, w, 8 * K3, &s_redf);
    }
    if (s_fail && issuer) {
        // a wait ran out: let whatever this CTA still has in flight end (bounded) before TMEM is freed
        t5_commit(&bar[4]);
        for (int it = 0; it < TMA_WAIT_LIMIT; it++)
            if (mbar_try_wait(&bar[4], 0)) break;
        for (int it = 0; it < TMA_WAIT_LIMIT; it++)
            if (mbar_try_wait(&bar[0], ph & 1u)) break;
    }
    t5_before_sync();
    __syncthreads();
    t5_after_sync();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(M::TMEM_COLS));
}

template <int K, int SPLIT>
void launch_tc05(const ApplyLaunch &L, cudaStream_t s) {
    using G = T5Geo<K>;
    using M = T5Mem<K, SPLIT>;
    kernel_smem((const void *)apply_tc05_kernel<K, SPLIT>, M::SMEM_LAUNCH);
    const int grid = L.nnodes;
    if (grid < 1) return;
    apply_tc05_kernel<K, SPLIT><<<grid, M::THREADS, M::SMEM_LAUNCH, s>>>(L);
    MWG_CUDA(cudaGetLastError());
}

// FP32 cube-order shadow -> x-pass operand: float4 (g, r) = row r = Z * 2K + Y, X = 4g .. 4g+3, per
// block the value rounded to TF32 (hi), then the remainder (the shadow's high cube minus hi, plus its
// low cube) rounded to TF32 (lo)
__global__ void to_tc_x_kernel(const float *cube32, float *out, size_t nblocks, int K) {
    const int N2 = 2 * K, NN = N2 * N2, KG = tc5_kg(K), C = NN * N2;
    const size_t per = (size_t)KG * NN, total = nblocks * per;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t blk = i / per;
        const int rem = (int)(i - blk * per), g = rem / NN, r = rem - g * NN;
        const float *src = cube32 + blk * 2 * (size_t)C + (size_t)r * N2 + 4 * g;
        const float *srl = src + C;  // the low cube
        float h[4], l[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const bool in = 4 * g + c < N2;
            const float v = in ? src[c] : 0.0f;
            h[c] = tf32r(v);
            l[c] = tf32r(in ? __fadd_rn(__fsub_rn(v, h[c]), srl[c]) : 0.0f);
        }
        float4 *o4 = reinterpret_cast<float4 *>(out);
        o4[2 * blk * per + rem] = make_float4(h[0], h[1], h[2], h[3]);
        o4[2 * blk * per + per + rem] = make_float4(l[0], l[1], l[2], l[3]);
    }
}

// throughput probe: one thread per CTA issues `iters` dense TF32 MMAs (M = 128, N = n, K = 8) on
// zeroed operands into one TMEM accumulator, then waits (bounded) for their commit
__global__ void __launch_bounds__(128) tc05_probe_kernel(int iters, int n, int *status) {
    extern __shared__ __align__(1024) uint8_t smp[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t s_tmem;
    __shared__ volatile int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int bytes_a = 128 * 32, bytes_b = n * 32;
    for (int i = tid; i < (bytes_a + bytes_b) / 16; i += blockDim.x)
        reinterpret_cast<float4 *>(smp)[i] = make_float4(0, 0, 0, 0);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_addr(&s_tmem)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        mbar_init(&bar);
        s_fail = 0;
    }
    async_fence();
    t5_before_sync();
    __syncthreads();
    t5_after_sync();
    const uint32_t tmem = s_tmem;
    if (tid == 0) {
        const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | (8u << 24);
        const uint64_t da = t5_desc(smem_addr(smp), 128, 256), db = t5_desc(smem_addr(smp + bytes_a), 128, 256);
        for (int i = 0; i < iters; i++) t5_mma(tmem, da, db, idesc, i > 0 ? 1u : 0u);
        t5_commit(&bar);
        mbar_wait(&bar, 0, &s_fail, status);
    }
    t5_before_sync();
    __syncthreads();
    t5_after_sync();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
}

}  // namespace

// Dense tcgen05 TF32 throughput (TFLOP/s, 2 flops per MAC) for MMAs of shape M = 128, N = n, K = 8.
double probe_tc05_tflops(int n, int nsm, cudaStream_t s) {
    if (n < 16 || n > 256 || n % 16) throw Error(MW_ERR_ARG, "probe: N must be a multiple of 16 in [16, 256]");
    // at most two CTAs per SM (512 TMEM columns): the shared memory asked for keeps a third out
    const int blocks = 2 * nsm, iters = 1 << 12, smem = 80 * 1024;
    MWG_CUDA(cudaFuncSetAttribute(tc05_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    int *status = nullptr;
    MWG_CUDA(cudaMalloc(&status, sizeof(int)));
    MWG_CUDA(cudaMemsetAsync(status, 0, sizeof(int), s));
    cudaEvent_t e0, e1;
    MWG_CUDA(cudaEventCreate(&e0));
    MWG_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        MWG_CUDA(cudaEventRecord(e0, s));
        tc05_probe_kernel<<<blocks, 128, smem, s>>>(iters, n, status);
        MWG_CUDA(cudaGetLastError());
        MWG_CUDA(cudaEventRecord(e1, s));
        MWG_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        MWG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0 && ms < best) best = ms;
    }
    int hs = 0;
    MWG_CUDA(cudaMemcpy(&hs, status, sizeof(int), cudaMemcpyDeviceToHost));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(status);
    if (hs) throw Error(MW_ERR_TIMEOUT, "probe: a bounded wait for the MMAs ran out");
    const double flops = 2.0 * 128.0 * n * 8.0 * (double)iters * blocks;
    return flops / (best * 1e-3) / 1e12;
}

void k_to_tc_x(const float *cube32, float *out, size_t nblocks, int K, cudaStream_t s) {
    if (nblocks == 0) return;
    const size_t total = nblocks * (size_t)tc5_kg(K) * (size_t)(4 * K * K);
    const int grid = (int)std::min<size_t>((total + 255) / 256, 4096);
    to_tc_x_kernel<<<grid, 256, 0, s>>>(cube32, out, nblocks, K);
    MWG_CUDA(cudaGetLastError());
}

template <int SPLIT>
void k_apply_tc05_t(int K, const ApplyLaunch &L, cudaStream_t s) {
    switch (K) {
        case 4: launch_tc05<4, SPLIT>(L, s); break;
        case 5: launch_tc05<5, SPLIT>(L, s); break;
        case 6: launch_tc05<6, SPLIT>(L, s); break;
        case 7: launch_tc05<7, SPLIT>(L, s); break;
        case 8: launch_tc05<8, SPLIT>(L, s); break;
        case 9: launch_tc05<9, SPLIT>(L, s); break;
        case 10: launch_tc05<10, SPLIT>(L, s); break;
        default: throw Error(MW_ERR_ARG, "no tensor-core apply kernel for this order");
    }
}

void k_apply_tc05(const DevBasis &b, const ApplyLaunch &L, bool split, cudaStream_t s) {
    if (L.nnodes <= 0) return;
    if (split)
        k_apply_tc05_t<1>(b.K, L, s);
    else
        k_apply_tc05_t<0>(b.K, L, s);
}

}  // namespace mwg
