// mw_screen.cu -- enumeration, screening and item lists of a batched apply on the GPU.
//
// For one level of one job group these kernels do what the host does in mw_apply.cpp
// (enumerate_node, the exact screening of generated inputs, the tier choice and the item
// lists), with the same floating-point operations in the same order, so that the items and
// their order, and therefore the apply's results, are identical to the host's:
//   screen_kernel<0>  one CTA per output node walks the candidate items (term t, then lz, ly,
//                     lx in the band L(t, n)) with the host's pruning of whole terms and rows
//                     (compacted level by level in shared memory),
//                     looks each input position up in the input tree's hash table (or walks up
//                     to its leaf ancestor), screens it with the item bound and counts the
//                     survivors; every missing input position that survives registers in the
//                     job's generation table (one slot per distinct position);
//   gen_tasks_kernel  the generation tasks of the registered positions;
//   screen_kernel<1>  the same walk after generation: generated inputs are screened again with
//                     their own norms, every item gets its tier, and the items are written in
//                     walk order (block-wide prefix sums per round of rows);
//   tier_offsets_kernel  per tier and node the first item (prefix sums in node order);
//   fill_kernel       the tier kernels' item arrays (input block, three operator blocks,
//                     coefficient), each tier's items in node order.
// Published method: the norm-product screening of the non-standard-form apply (Frediani et al.,
// Mol. Phys. 111 (2013) 1143), used by mrcpp::apply at CoulombPotential.cpp:131 and
// HelmholtzVector.cpp:149.  All integer sums are exact, so the kernels are deterministic.
#include <cuda_runtime.h>

#include "mw_host.h"

namespace mwg {

namespace {

constexpr int ST = 128;  // threads per CTA

// products and sums as the host's -ffp-contract=off code rounds them (no fused multiply-adds)
__device__ __forceinline__ double M(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double A(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dmax(double a, double b) { return a < b ? b : a; }  // std::max
__device__ __forceinline__ int floordiv2_d(int l) { return (l - (l & 1)) / 2; }

// mw_apply.cpp item_bound: b = sum_ft |in_ft| s(ft), the (0,0) pair left out below the root
__device__ double item_bound_d(const double *nx, const double *ny, const double *nz, const double *cn, bool root) {
    const double cx[2] = {A(nx[0], nx[2]), A(nx[1], nx[3])}, cy[2] = {A(ny[0], ny[2]), A(ny[1], ny[3])},
                 cz[2] = {A(nz[0], nz[2]), A(nz[1], nz[3])};
    double b = 0.0;
    if (cn[0] != 0.0) {
        double s = 0.0;
        if (root) {
            s = M(M(cx[0], cy[0]), cz[0]);
        } else {
            for (int gt = 1; gt < 8; gt++) s = A(s, M(M(nx[2 * (gt & 1)], ny[2 * ((gt >> 1) & 1)]), nz[2 * (gt >> 2)]));
        }
        b = A(b, M(cn[0], s));
    }
    for (int ft = 1; ft < 8; ft++)
        if (cn[ft] != 0.0) b = A(b, M(cn[ft], M(M(cx[ft & 1], cy[(ft >> 1) & 1]), cz[ft >> 2])));
    return b;
}

// mw_apply.cpp item_pairs: component pairs with a non-zero contraction
__device__ int item_pairs_d(const double *nx, const double *ny, const double *nz, const double *cn, bool root) {
    const int ex[2] = {(nx[0] != 0.0) + (nx[2] != 0.0), (nx[1] != 0.0) + (nx[3] != 0.0)},
              ey[2] = {(ny[0] != 0.0) + (ny[2] != 0.0), (ny[1] != 0.0) + (ny[3] != 0.0)},
              ez[2] = {(nz[0] != 0.0) + (nz[2] != 0.0), (nz[1] != 0.0) + (nz[3] != 0.0)};
    int p = 0;
    for (int ft = 0; ft < 8; ft++) {
        if (cn[ft] == 0.0) continue;
        p += ex[ft & 1] * ey[(ft >> 1) & 1] * ez[ft >> 2];
        if (!root && ft == 0 && nx[0] != 0.0 && ny[0] != 0.0 && nz[0] != 0.0) p--;
    }
    return p;
}

__device__ int hash_find(const ScreenJob &J, int n, int x, int y, int z) {
    unsigned h = key_hash(n, x, y, z) & (unsigned)J.hmask;
    for (int probe = 0; probe <= J.hmask; probe++) {
        const int4 k = J.hkey[h];
        if (k.x == n && k.y == x && k.z == y && k.w == z) return J.hval[h];
        if (k.x == HASH_EMPTY) return -1;
        h = (h + 1) & (unsigned)J.hmask;
    }
    return -1;
}

// position key in a job's generation table (translations relative to the world's corner at
// scale n; 21 bits each, checked by the host), never 0
__device__ __forceinline__ unsigned long long gen_key(const ScreenLevel &P, const int *p) {
    return ((unsigned long long)(p[0] - P.lo[0]) | ((unsigned long long)(p[1] - P.lo[1]) << 21) |
            ((unsigned long long)(p[2] - P.lo[2]) << 42)) + 1ull;
}
__device__ __forceinline__ unsigned gen_hash(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    return (unsigned)k;
}

// registers a missing input position (count pass); a full table raises the overflow flag
__device__ void gen_insert(const ScreenLevel &P, const ScreenNode &nd, const int *p, int anc, int an) {
    const unsigned long long key = gen_key(P, p);
    unsigned h = gen_hash(key) & (unsigned)nd.gmask;
    for (int probe = 0; probe <= nd.gmask; probe++) {
        const unsigned long long old = atomicCAS(&P.gkey[nd.gtab + h], 0ull, key);
        if (old == 0ull) {
            const int slot = atomicAdd(P.gen_cnt, 1);
            if (slot < P.gen_cap) {
                int *gi = P.gen_info + 6 * (size_t)slot;
                gi[0] = nd.job;
                gi[1] = anc;
                gi[2] = an;
                gi[3] = p[0];
                gi[4] = p[1];
                gi[5] = p[2];
                P.gval[nd.gtab + h] = slot;
            } else {
                atomicExch(P.overflow, 1);
            }
            return;
        }
        if (old == key) return;
        h = (h + 1) & (unsigned)nd.gmask;
    }
    atomicExch(P.overflow, 1);
}

// slot of a registered position (write pass, after the count pass completed); -1 if absent
__device__ int gen_find(const ScreenLevel &P, const ScreenNode &nd, const int *p) {
    const unsigned long long key = gen_key(P, p);
    unsigned h = gen_hash(key) & (unsigned)nd.gmask;
    for (int probe = 0; probe <= nd.gmask; probe++) {
        const unsigned long long k = P.gkey[nd.gtab + h];
        if (k == key) return P.gval[nd.gtab + h];
        if (k == 0ull) return -1;
        h = (h + 1) & (unsigned)nd.gmask;
    }
    return -1;
}

// exclusive prefix sum over the CTA (every thread calls it); *total gets the CTA's sum
template <typename U>
__device__ U block_scan(U v, U *wsum, U *total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    U x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const U y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    U before = 0, all = 0;
#pragma unroll
    for (int i = 0; i < ST / 32; i++) {
        if (i < w) before += wsum[i];
        all += wsum[i];
    }
    __syncthreads();
    *total = all;
    return x - v + before;
}

// FP32 estimate of item_bound_d (any rounding order).  With FP32 inputs and about 25 roundings
// it is within 2e-6 relative of the exact bound, plus products flushed below FP32's range; the
// host sets the node's fast flag only where that flush is far inside the decision margins.
__device__ float item_bound_f(const float *nx, const float *ny, const float *nz, const float *cn, bool root) {
    const float cx[2] = {nx[0] + nx[2], nx[1] + nx[3]}, cy[2] = {ny[0] + ny[2], ny[1] + ny[3]},
                cz[2] = {nz[0] + nz[2], nz[1] + nz[3]};
    float b = 0.0f;
    if (cn[0] != 0.0f) {
        float s;
        if (root) {
            s = cx[0] * cy[0] * cz[0];
        } else {
            const float yz0 = ny[0] * nz[0], yz1 = ny[2] * nz[0], yz2 = ny[0] * nz[2], yz3 = ny[2] * nz[2];
            s = nx[2] * yz0 + (nx[0] + nx[2]) * (yz1 + yz2 + yz3);
        }
        b = cn[0] * s;
    }
#pragma unroll
    for (int ft = 1; ft < 8; ft++) b += cn[ft] * (cx[ft & 1] * cy[(ft >> 1) & 1] * cz[ft >> 2]);
    return b;
}
// the scaling-only part: the bound of a block whose only non-zero norm is the scaling one
__device__ double scaling_bound_d(const double *nx, const double *ny, const double *nz, double a, bool root) {
    const double c[8] = {a, 0, 0, 0, 0, 0, 0, 0};
    return item_bound_d(nx, ny, nz, c, root);
}
__device__ float scaling_bound_f(const float *nx, const float *ny, const float *nz, float a, bool root) {
    if (root) return a * ((nx[0] + nx[2]) * (ny[0] + ny[2]) * (nz[0] + nz[2]));
    const float yz0 = ny[0] * nz[0], yz1 = ny[2] * nz[0], yz2 = ny[0] * nz[2], yz3 = ny[2] * nz[2];
    return a * (nx[2] * yz0 + (nx[0] + nx[2]) * (yz1 + yz2 + yz3));
}

// 1: the bound passes (>= thr) for certain, 0: it fails for certain, -1: FP64 must decide
__device__ __forceinline__ int fast_cmp(float b32, float lo, float hi) { return b32 < lo ? 0 : (b32 > hi ? 1 : -1); }

struct Row {  // the operator norms of one (t, lz, ly) row: FP64 for exact decisions, FP32 for estimates
    const double *ny, *nz;
    const float *ny32, *nz32;
};

// One candidate of the walk.  Returns true when it survives the first screen (the host's phase A:
// real inputs with their exact bound, missing ones with their leaf ancestor's block norm as the
// scaling norm); src / gen / an describe it.  The FP32 estimate decides where it is clear of the
// threshold, the host's FP64 arithmetic elsewhere, so the result is the host's.
__device__ bool candidate(const ScreenLevel &P, const ScreenJob &J, const ScreenNode &nd, const int *p,
                          const double *nx, const float *nx32, const Row &rw, int &src, int &gen, int &an) {
    for (int d = 0; d < 3; d++)
        if (p[d] < P.lo[d] || p[d] >= P.hi[d]) return false;
    const int i = hash_find(J, P.n, p[0], p[1], p[2]);
    if (i >= 0) {
        src = i;
        gen = 0;
        an = P.n;
    } else {
        int a = -1, al[3] = {p[0], p[1], p[2]};
        an = P.n;
        while (a < 0 && an > P.n0) {
            an--;
            for (int d = 0; d < 3; d++) al[d] = floordiv2_d(al[d]);
            a = hash_find(J, an, al[0], al[1], al[2]);
        }
        if (a < 0) return false;  // unreachable: the roots cover the world
        src = a;
        gen = 1;
    }
    if (P.root) return true;
    if (nd.flags & 4) {
        const float b32 = gen ? scaling_bound_f(nx32, rw.ny32, rw.nz32, J.bn32[src], false)
                              : item_bound_f(nx32, rw.ny32, rw.nz32, J.cn32 + 8 * (size_t)src, false);
        const int d = fast_cmp(b32, nd.thr_lo, nd.thr_hi);
        if (d >= 0) return d != 0;
    }
    const double bd = gen ? scaling_bound_d(nx, rw.ny, rw.nz, J.bn[src], false)
                          : item_bound_d(nx, rw.ny, rw.nz, J.cn + 8 * (size_t)src, false);
    return !(bd < nd.thr);
}

// An item after generation: a candidate that survives the first screen and the host's phase C
// (the exact bound, with a generated block's own norms, against thr2), and its tier.
struct Item {
    int src, gen, tier;
    const double *cn;
};
__device__ bool final_item(const ScreenLevel &P, const ScreenJob &J, const ScreenNode &nd, const int *p, int lx,
                           int ly, int lz, const double *nx, const float *nx32, const Row &rw, Item &it) {
    int an;
    if (!candidate(P, J, nd, p, nx, nx32, rw, it.src, it.gen, an)) return false;
    const float *cn32;
    if (!it.gen) {
        it.cn = J.cn + 8 * (size_t)it.src;
        cn32 = J.cn32 + 8 * (size_t)it.src;
    } else {
        it.src = gen_find(P, nd, p);
        if (it.src < 0) {  // unreachable after a count pass without overflow
            atomicExch(P.overflow, 2);
            return false;
        }
        it.cn = P.gcn + 8 * (size_t)it.src;
        cn32 = P.gcn32 + 8 * (size_t)it.src;
    }
    const bool root = P.root != 0, fast = (nd.flags & 4) != 0;
    const float b32 = fast ? item_bound_f(nx32, rw.ny32, rw.nz32, cn32, root) : 0.0f;
    double bd = 0.0;
    bool have = false;
    if (!root) {
        int d = fast ? fast_cmp(b32, nd.thr2_lo, nd.thr2_hi) : -1;
        if (d < 0) {
            bd = item_bound_d(nx, rw.ny, rw.nz, it.cn, false);
            have = true;
            d = !(bd < nd.thr2);
        }
        if (!d) return false;
    }
    const bool near = max(abs(lx), max(abs(ly), abs(lz))) <= 1;
    const double tthr = nd.tthr;
    if (!P.mixed || tthr < 0.0 || (P.near_fp64 && near)) {
        it.tier = 0;
        return true;
    }
    // above[k]: the bound exceeds boundary k (TIER_TF32, TIER_FP64, TIER_DF times tthr)
    bool above[3], clear = fast && !have;
    if (clear)
        for (int k = 0; k < 3; k++) {
            const int d = fast_cmp(b32, nd.tier_lo[k], nd.tier_hi[k]);
            if (d < 0) clear = false;
            above[k] = d == 1;
        }
    if (!clear) {
        if (!have) bd = item_bound_d(nx, rw.ny, rw.nz, it.cn, root);
        above[0] = !(bd <= M(P.tier_tf32, tthr));
        above[1] = bd > M(P.tier_fp64, tthr);
        above[2] = !(bd <= M(P.tier_df, tthr));
    }
    if (P.df_only)
        it.tier = above[2] ? 0 : 3;
    else if (above[1])
        it.tier = (P.dfp && !above[2]) ? 3 : 0;
    else if (P.tensor && (nd.flags & 2) && !above[0])
        it.tier = 2;
    else
        it.tier = 1;
    return true;
}

// last index i in [0, n) with pre[i] <= r (pre ascending, pre[n] > r)
__device__ __forceinline__ int last_le(const int *pre, int n, int r) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= r) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// One CTA per output node.  The walk prunes as the host does (mw_apply.cpp enumerate_node), level
// by level so that FP64 work is spent only on what survives: whole terms, then (t, lz) rows, then
// (t, lz, ly) rows, each with the host's expression; the surviving rows are compacted in walk
// order in shared memory, and every thread then walks the lx of one (t, lz, ly) row.
// PASS 0: count the first screen's survivors per node and register missing inputs.
// PASS 1: screen generated inputs with their own norms, choose tiers, write the items in walk order.
template <int PASS>
__global__ void __launch_bounds__(ST) screen_kernel(ScreenLevel P, int maxT, int zmax) {
    extern __shared__ int sm[];
    int *zpre = sm;                // [maxT + 1]: first z row of each term (live terms only)
    int *zlist = sm + maxT + 1;    // [zmax]: live z rows, t << 16 | (lz + L)
    int *ypre = zlist + zmax;      // [zmax + 1]: first y row of each live z row
    __shared__ unsigned wsum[ST / 32];
    __shared__ int s_cnt[8];
    const int q = blockIdx.x, tid = threadIdx.x;
    const ScreenNode nd = P.nodes[q];
    const ScreenJob &J = P.jobs[nd.job];
    const ScreenOp &op = J.op;
    const int T = op.T, S = op.S, s = P.sidx;
    const bool skip = !P.root && (nd.flags & 1);
    // the pruning tests are conservative bounds: with the fast flag they run in FP32 with a margin
    // (pruning at most what the host prunes; the extra candidates fail the exact screen)
    const bool fast = (nd.flags & 4) != 0;
    const double fm = nd.fm, thr = nd.thr;
    // translations whose input position lies in the world: lo <= l_o - l < hi (the walk skips the
    // others, which the host rejects one by one)
    int wlo[3], whi[3];
    for (int d = 0; d < 3; d++) {
        wlo[d] = nd.l[d] - P.hi[d] + 1;
        whi[d] = nd.l[d] - P.lo[d];
    }
    // terms
    for (int t = tid; t < T; t += ST) {
        const int L = op.band[t * S + s];
        bool live = L >= 0 && !skip;
        if (live && !P.root) {
            if (fast) {
                const float X = op.xmax32[t * S + s], Am = op.amax32[t * S + s];
                live = !(nd.fm32 * (3.0f * X * Am * Am) < nd.prune32);
            } else {
                const double X = op.xmax[t * S + s], Am = op.amax[t * S + s];
                live = !(M(M(M(M(fm, 3.0), X), Am), Am) < thr);
            }
        }
        // rows only where every direction has an in-world translation
        int rows = 1;
        for (int d = 0; d < 3; d++) rows = min(rows, min(L, whi[d]) - max(-L, wlo[d]) + 1);
        zpre[t] = (live && rows > 0) ? min(L, whi[2]) - max(-L, wlo[2]) + 1 : 0;
    }
    if (tid < 8) s_cnt[tid] = 0;
    __syncthreads();
    if (tid == 0) {
        int acc = 0;
        for (int t = 0; t < T; t++) {
            const int c = zpre[t];
            zpre[t] = acc;
            acc += c;
        }
        zpre[T] = acc;
    }
    __syncthreads();
    // z rows of the live terms
    const int Z = zpre[T];
    int nzr = 0;
    for (int z0 = 0; z0 < Z; z0 += ST) {
        const int z = z0 + tid;
        unsigned live = 0;
        int packed = 0, L = 0;
        if (z < Z) {
            const int t = last_le(zpre, T, z);
            L = op.band[t * S + s];
            const int lz = max(-L, wlo[2]) + z - zpre[t];
            live = 1;
            if (!P.root) {
                const size_t zb = 4 * (size_t)((long)op.off[t * S + s] + L + lz);
                if (fast) {
                    const float *nz = op.norms32 + zb;
                    const float X = op.xmax32[t * S + s], Am = op.amax32[t * S + s];
                    const float az = fmaxf(fmaxf(nz[0], nz[1]), fmaxf(nz[2], nz[3]));
                    const float xz = fmaxf(nz[1], fmaxf(nz[2], nz[3]));
                    live = !(nd.fm32 * (xz * Am * Am + 2.0f * az * X * Am) < nd.prune32);
                } else {
                    const double *nz = op.norms + zb;
                    const double X = op.xmax[t * S + s], Am = op.amax[t * S + s];
                    const double az = dmax(dmax(nz[0], nz[1]), dmax(nz[2], nz[3]));
                    const double xz = dmax(nz[1], dmax(nz[2], nz[3]));
                    live = !(M(fm, A(M(M(xz, Am), Am), M(M(M(2.0, az), X), Am))) < thr);
                }
            }
            packed = (t << 16) | (lz + L);
        }
        unsigned total;
        const unsigned pos = block_scan<unsigned>(live, wsum, &total);
        if (live) {
            zlist[nzr + pos] = packed;
            ypre[nzr + pos] = min(L, whi[1]) - max(-L, wlo[1]) + 1;  // >= 1: the term has rows
        }
        nzr += (int)total;
    }
    __syncthreads();
    // first y row of each live z row (in place: counts -> exclusive prefix sums)
    int ytot = 0;
    for (int i0 = 0; i0 < nzr; i0 += ST) {
        const int i = i0 + tid;
        const unsigned v = i < nzr ? (unsigned)ypre[i] : 0u;
        unsigned total;
        const unsigned pre = block_scan<unsigned>(v, wsum, &total);
        if (i < nzr) ypre[i] = ytot + (int)pre;
        ytot += (int)total;
    }
    if (tid == 0) ypre[nzr] = ytot;
    __syncthreads();
    // (t, lz, ly) rows: the y test, then the walk over lx
    int mine = 0;           // PASS 0: this thread's survivors
    long long written = 0;  // PASS 1: items written by earlier rounds
    const long long base = PASS ? P.cand_off[q] : 0;
    for (int r0 = 0; r0 < ytot; r0 += ST) {
        const int r = r0 + tid;
        int t = 0, L = -1, lz = 0, ly = 0;
        bool live = false;
        Row rw{nullptr, nullptr, nullptr, nullptr};
        long ob = 0;
        if (r < ytot) {
            const int i = last_le(ypre, nzr, r);
            const int packed = zlist[i];
            t = packed >> 16;
            L = op.band[t * S + s];
            lz = (packed & 0xffff) - L;
            ly = max(-L, wlo[1]) + r - ypre[i];
            ob = (long)op.off[t * S + s] + L;
            rw.nz = op.norms + 4 * (size_t)(ob + lz);
            rw.ny = op.norms + 4 * (size_t)(ob + ly);
            rw.nz32 = op.norms32 + 4 * (size_t)(ob + lz);
            rw.ny32 = op.norms32 + 4 * (size_t)(ob + ly);
            live = true;
            if (!P.root) {
                if (fast) {
                    const float *nz = rw.nz32, *ny = rw.ny32;
                    const float X = op.xmax32[t * S + s], Am = op.amax32[t * S + s];
                    const float az = fmaxf(fmaxf(nz[0], nz[1]), fmaxf(nz[2], nz[3]));
                    const float xz = fmaxf(nz[1], fmaxf(nz[2], nz[3]));
                    const float ay = fmaxf(fmaxf(ny[0], ny[1]), fmaxf(ny[2], ny[3]));
                    const float xy = fmaxf(ny[1], fmaxf(ny[2], ny[3]));
                    live = !(nd.fm32 * (xz * ay * Am + az * xy * Am + az * ay * X) < nd.prune32);
                } else {
                    const double *nz = rw.nz, *ny = rw.ny;
                    const double X = op.xmax[t * S + s], Am = op.amax[t * S + s];
                    const double az = dmax(dmax(nz[0], nz[1]), dmax(nz[2], nz[3]));
                    const double xz = dmax(nz[1], dmax(nz[2], nz[3]));
                    const double ay = dmax(dmax(ny[0], ny[1]), dmax(ny[2], ny[3]));
                    const double xy = dmax(ny[1], dmax(ny[2], ny[3]));
                    live = !(M(fm, A(A(M(M(xz, ay), Am), M(M(az, xy), Am)), M(M(az, ay), X))) < thr);
                }
            }
        }
        if (PASS == 0) {
            if (live) {
                for (int lx = max(-L, wlo[0]); lx <= min(L, whi[0]); lx++) {
                    const int p[3] = {nd.l[0] - lx, nd.l[1] - ly, nd.l[2] - lz};
                    int src, gen, an;
                    if (!candidate(P, J, nd, p, op.norms + 4 * (size_t)(ob + lx), op.norms32 + 4 * (size_t)(ob + lx), rw,
                                   src, gen, an))
                        continue;
                    mine++;
                    if (gen) gen_insert(P, nd, p, src, an);
                }
            }
        } else {
            // two walks of the row: screen and count its items, then write them at their place in
            // walk order.  Rows of at most 32 translations keep the first walk's survivors and tiers
            // in bit masks, so that the second walk only looks the inputs up again
            int c = 0;
            const int xlo = max(-L, wlo[0]), xhi = min(L, whi[0]);
            const bool keep = xhi - xlo < 32;
            unsigned surv = 0u;
            unsigned long long tiers = 0ull;
            if (live)
                for (int lx = xlo; lx <= xhi; lx++) {
                    const int p[3] = {nd.l[0] - lx, nd.l[1] - ly, nd.l[2] - lz};
                    const double *nx = op.norms + 4 * (size_t)(ob + lx);
                    Item it;
                    if (!final_item(P, J, nd, p, lx, ly, lz, nx, op.norms32 + 4 * (size_t)(ob + lx), rw, it)) continue;
                    c++;
                    if (keep) {
                        surv |= 1u << (lx - xlo);
                        tiers |= (unsigned long long)it.tier << (2 * (lx - xlo));
                    }
                    atomicAdd(&s_cnt[it.tier], 1);
                    atomicAdd(&s_cnt[4 + it.tier], item_pairs_d(nx, rw.ny, rw.nz, it.cn, P.root != 0));
                }
            unsigned total;
            const int pos = (int)block_scan<unsigned>((unsigned)c, wsum, &total);
            if (live && c > 0) {
                int k = 0;
                auto put = [&](int lx, int src, int gen, int tier) {
                    ScreenCand &cd = P.cand[base + written + pos + k];
                    cd.src = src;
                    cd.lx = (short)lx;
                    cd.ly = (short)ly;
                    cd.lz = (short)lz;
                    cd.tier = (unsigned char)tier;
                    cd.gen = (unsigned char)gen;
                    cd.t = t;
                    k++;
                };
                if (keep) {
                    for (unsigned m = surv; m; m &= m - 1) {
                        const int bit = __ffs(m) - 1, lx = xlo + bit;
                        const int p[3] = {nd.l[0] - lx, nd.l[1] - ly, nd.l[2] - lz};
                        // the input as final_item found it: a node of the input tree, or a generated slot
                        int src = hash_find(J, P.n, p[0], p[1], p[2]), gen = 0;
                        if (src < 0) {
                            src = gen_find(P, nd, p);
                            gen = 1;
                        }
                        put(lx, src, gen, (int)((tiers >> (2 * bit)) & 3ull));
                    }
                } else {
                    for (int lx = xlo; lx <= xhi; lx++) {
                        const int p[3] = {nd.l[0] - lx, nd.l[1] - ly, nd.l[2] - lz};
                        Item it;
                        if (!final_item(P, J, nd, p, lx, ly, lz, op.norms + 4 * (size_t)(ob + lx),
                                        op.norms32 + 4 * (size_t)(ob + lx), rw, it))
                            continue;
                        put(lx, it.src, it.gen, it.tier);
                    }
                }
            }
            written += total;
        }
    }
    if (PASS == 0) {
        unsigned total;
        block_scan<unsigned>((unsigned)mine, wsum, &total);
        if (tid == 0) P.cnt[q] = (int)total;
    } else {
        __syncthreads();
        if (tid < 8) P.tcnt[8 * (size_t)q + tid] = s_cnt[tid];
    }
}

// generation task of each registered position: its leaf ancestor's block and the path down to it
__global__ void gen_tasks_kernel(ScreenLevel P, GenTask *tasks, int ngen) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ngen) return;
    const int *gi = P.gen_info + 6 * (size_t)i;
    const ScreenJob &J = P.jobs[gi[0]];
    const int an = gi[2];
    GenTask tk;
    tk.anc = J.in64 + (size_t)gi[1] * P.bs;
    tk.out = P.g64 + (size_t)i * P.bs;
    tk.cn = P.gcn + 8 * (size_t)i;
    tk.steps = P.n - an;
    tk.path = 0;
    for (int s = 0; s < tk.steps; s++) {
        const int sh = P.n - (an + s + 1);
        uint64_t c = 0;
        for (int d = 0; d < 3; d++) c |= (uint64_t)((gi[3 + d] >> sh) & 1) << d;
        tk.path |= c << (3 * s);
    }
    tk.pad = 0;
    tasks[i] = tk;
}

__global__ void gen_norms32_kernel(ScreenLevel P, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) P.gcn32[i] = (float)P.gcn[i];
}

// per tier: the nodes' first items (prefix sums in node order), the tiers one after the other
__global__ void __launch_bounds__(1024) tier_offsets_kernel(ScreenLevel P) {
    __shared__ long long wpart[32];
    __shared__ long long s_base;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
    if (tid == 0) s_base = 0;
    __syncthreads();
    for (int k = 0; k < 4; k++) {
        long long run = s_base;
        for (int q0 = 0; q0 < P.nn; q0 += blockDim.x) {
            const int q = q0 + tid;
            const long long v = q < P.nn ? P.tcnt[8 * (size_t)q + k] : 0;
            long long x = v;
            for (int o = 1; o < 32; o <<= 1) {
                const long long y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) wpart[w] = x;
            __syncthreads();
            long long before = 0, all = 0;
            for (int i = 0; i < nw; i++) {
                if (i < w) before += wpart[i];
                all += wpart[i];
            }
            if (q < P.nn) P.tier_off[4 * (size_t)q + k] = run + x - v + before;
            run += all;
            __syncthreads();
        }
        if (tid == 0) {
            P.tier_tot[k] = run - s_base;
            s_base = run;
        }
        __syncthreads();
    }
}

// the tier kernels' item arrays: each node's items of a tier at its first item, in walk order
__global__ void __launch_bounds__(ST) fill_kernel(ScreenLevel P) {
    __shared__ unsigned wsum[ST / 32];
    __shared__ long long s_run[4];
    const int q = blockIdx.x, tid = threadIdx.x;
    const ScreenNode &nd = P.nodes[q];
    const ScreenJob &J = P.jobs[nd.job];
    const ScreenOp &op = J.op;
    const int S = op.S, s = P.sidx;
    const int *tc = P.tcnt + 8 * (size_t)q;
    const int m = tc[0] + tc[1] + tc[2] + tc[3];
    const long long c0 = P.cand_off[q];
    if (tid < 4) s_run[tid] = P.tier_off[4 * (size_t)q + tid];
    __syncthreads();
    for (int i0 = 0; i0 < m; i0 += ST) {
        const int i = i0 + tid;
        int tier = 0;
        unsigned onehot = 0;
        ScreenCand cd;
        if (i < m) {
            cd = P.cand[c0 + i];
            tier = cd.tier;
            onehot = 1u << (8 * tier);  // at most ST = 128 items of a tier per round: 8 bits each
        }
        unsigned total;
        const unsigned pre = block_scan<unsigned>(onehot, wsum, &total);
        if (i < m) {
            const long long dst = s_run[tier] + ((pre >> (8 * tier)) & 255);
            const long ob = (long)op.off[cd.t * S + s] + op.band[cd.t * S + s];
            const size_t bx = (size_t)(ob + cd.lx), by = (size_t)(ob + cd.ly), bz = (size_t)(ob + cd.lz);
            const size_t src = (size_t)cd.src;
            if (tier == 0) {
                P.in[dst] = cd.gen ? (const void *)(P.g64 + src * P.bs) : (const void *)(J.in64 + src * P.bs);
                P.ax[dst] = op.b64 + bx * P.bsz;
                P.ay[dst] = op.b64 + by * P.bsz;
                P.az[dst] = op.b64 + bz * P.bsz;
            } else if (tier == 2 || (tier == 1 && P.tensor)) {
                // the tensor-core tiers (TF32, and split-TF32 for tier 1 in the tensor modes)
                P.in[dst] = cd.gen ? (const void *)(P.gtc + P.tx * src) : (const void *)(J.intc + P.tx * src);
                const float *bt = tier == 1 ? op.btc2 : op.btc;  // the split tier's operator layout
                P.ax[dst] = bt + P.tb * bx;
                P.ay[dst] = bt + P.tb * by;
                P.az[dst] = bt + P.tb * bz;
            } else {
                P.in[dst] = cd.gen ? (const void *)(P.g32 + 2 * src * P.bs) : (const void *)(J.in32 + 2 * src * P.bs);
                P.ax[dst] = op.b32 + 2 * bx * P.bsz;
                P.ay[dst] = op.b32 + 2 * by * P.bsz;
                P.az[dst] = op.b32 + 2 * bz * P.bsz;
            }
            P.coef[dst] = op.c[cd.t];
        }
        __syncthreads();
        if (tid < 4) s_run[tid] += (total >> (8 * tid)) & 255;
        __syncthreads();
    }
}

}  // namespace

size_t screen_smem(int maxT, int zmax) { return sizeof(int) * ((size_t)maxT + 2 + 2 * (size_t)zmax); }

void k_screen_count(const ScreenLevel &P, int maxT, int zmax, cudaStream_t s) {
    if (P.nn <= 0) return;
    const size_t sm = screen_smem(maxT, zmax);
    if (sm > 48 * 1024) kernel_smem((const void *)screen_kernel<0>, (int)sm);
    screen_kernel<0><<<P.nn, ST, sm, s>>>(P, maxT, zmax);
}

void k_screen_gen_tasks(const ScreenLevel &P, GenTask *tasks, int ngen, cudaStream_t s) {
    if (ngen <= 0) return;
    gen_tasks_kernel<<<(ngen + 127) / 128, 128, 0, s>>>(P, tasks, ngen);
}

void k_screen_gen_norms32(const ScreenLevel &P, int ngen, cudaStream_t s) {
    if (ngen <= 0) return;
    gen_norms32_kernel<<<(8 * ngen + 255) / 256, 256, 0, s>>>(P, 8 * ngen);
}

void k_screen_write(const ScreenLevel &P, int maxT, int zmax, cudaStream_t s) {
    if (P.nn <= 0) return;
    const size_t sm = screen_smem(maxT, zmax);
    if (sm > 48 * 1024) kernel_smem((const void *)screen_kernel<1>, (int)sm);
    screen_kernel<1><<<P.nn, ST, sm, s>>>(P, maxT, zmax);
    tier_offsets_kernel<<<1, 1024, 0, s>>>(P);
}

void k_screen_fill(const ScreenLevel &P, cudaStream_t s) {
    if (P.nn <= 0) return;
    fill_kernel<<<P.nn, ST, 0, s>>>(P);
}

}  // namespace mwg
