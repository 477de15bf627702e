// mw_host.h -- host-side structures of the GB300 multiwavelet engine.
//
// Trees live on the device as SoA arrays (one FP64 block of 8*K^3
// coefficients per node, 8 component norms per node); the host keeps the
// integer structure (keys, parent/child links, Morton-sortable) and a copy of
// the component norms, which is all the refinement and screening decisions
// need.  Children of a node are always 8 consecutive nodes.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <map>
#include <stdexcept>
#include <tuple>
#include <string>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "../../include/mw_gb300.h"

namespace mwg {

constexpr int KMAX = 10;          // largest K = order + 1 with a GPU kernel
constexpr double SCREEN_FAC = 0.01;
constexpr double ZERO_EXP = 45.0;
constexpr double NS_CLEAN = 1e-13;

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define MWG_CUDA(call)                                                                                     \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess)                                                                             \
            throw ::mwg::Error(e_ == cudaErrorMemoryAllocation ? MW_ERR_OOM : MW_ERR_CUDA,                 \
                               std::string(#call) + ": " + cudaGetErrorString(e_));                        \
    } while (0)

struct Key {
    int n, l[3];
    bool operator==(const Key &o) const { return n == o.n && l[0] == o.l[0] && l[1] == o.l[1] && l[2] == o.l[2]; }
};

struct KeyHash {
    size_t operator()(const Key &k) const {
        uint64_t h = (uint64_t)(uint32_t)k.n * 0x9E3779B97F4A7C15ULL;
        h ^= (uint64_t)(uint32_t)k.l[0] * 0xC2B2AE3D27D4EB4FULL;
        h = (h << 21) | (h >> 43);
        h ^= (uint64_t)(uint32_t)k.l[1] * 0x165667B19E3779F9ULL;
        h = (h << 21) | (h >> 43);
        h ^= (uint64_t)(uint32_t)k.l[2] * 0xD6E8FEB86659FD93ULL;
        h ^= h >> 31;
        h *= 0xBF58476D1CE4E5B9ULL;
        h ^= h >> 29;
        return (size_t)h;
    }
};

inline int floordiv2(int l) { return (l - (l & 1)) / 2; }

// ---------------------------------------------------------------- basis
struct Basis {
    int n0, corner[3], boxes[3], k, K, type, max_depth, bs;
    std::vector<double> qx, qw, legq, c2v, v2c, integ, W, WT;
    void init(int root_scale, const int *corner, const int *boxes, int order, int type, int max_depth);
    void eval(double x, double *out) const;  // all K scaling functions at x in [0,1]
    bool in_world(int n, const int *l) const;
    int max_scale() const { return n0 + max_depth - 1; }
};

void gauss_legendre(int n, double *x, double *w);
void legendre_shifted(int n, double x, double *p);

// ---------------------------------------------------------------- device basis data
struct DevBasis {
    int K, type;
    const double *W, *WT, *c2v, *v2c, *qx, *qw, *legq;  // device
};

// ---------------------------------------------------------------- context
struct Ctx;

struct NodeInfo {
    int n, l[3];
    int parent, child0;
};

struct Tree {
    Ctx *ctx = nullptr;
    std::vector<NodeInfo> nodes;
    std::unordered_map<Key, int, KeyHash> map;
    std::vector<double> cn;       // 8 component norms per node (host copy)
    double *d_coefs = nullptr;    // cap * bs
    double *d_cn = nullptr;       // cap * 8
    float *d_coefs32 = nullptr;   // FP32 shadow (mixed-precision applies): cap32 x (high cube, low cube)
    float *d_coefs_tc = nullptr;  // TF32 x-pass operand of the tensor-core tier (mw_tc05_layout.h), cap_tc blocks
    size_t cap = 0, cap32 = 0, cap_tc = 0;
    int nroots = 0;

    int find(int n, const int *l) const {
        auto it = map.find(Key{n, {l[0], l[1], l[2]}});
        return it == map.end() ? -1 : it->second;
    }
    int nn() const { return (int)nodes.size(); }
    double *block(int i) const;
    void reserve(size_t n);
    int add(int n, const int *l, int parent);
    int split(int i);
    void reset_roots();
    void download_norms(int first, int count);
    double sqnorm_leaves() const;
    int max_scale() const;
    void free_device();
};

struct Oper {
    Ctx *ctx = nullptr;
    int kind = 0;  // 0 poisson, 1 helmholtz
    double mu = 0, prec = 0, eps = 0, rmin = 0, rmax = 0;
    int T = 0, S = 0;
    std::vector<double> c, a;
    std::vector<int> band;       // [T*S]
    std::vector<long> off;       // [T*S] block index of l = -band
    std::vector<double> norms;   // 4 per block, [g][f]
    std::vector<double> amax, xmax;  // per (t,s)
    long nblocks = 0;
    double *d_blocks = nullptr;  // (2K)^2 per block, FP64
    float *d_blocks32 = nullptr; // FP32 copy: per block the high part, then the low part (2 x (2K)^2)
    float *d_blocks_tc = nullptr; // TF32 B operand of the tensor-core tier per block (mw_tc05_layout.h)
    float *d_blocks_tc2 = nullptr; // ... in the split-TF32 tier's wide layout (tc5_split_wide(K) only)
    // the operator blocks the split-TF32 tier reads: the wide layout where the kernel uses it
    const float *split_blocks() const { return d_blocks_tc2 ? d_blocks_tc2 : d_blocks_tc; }
    // the screening tables on the device (bands, block offsets, sub-block norms, amax, xmax, term
    // coefficients), uploaded by the first apply that screens on the GPU (mw_screen.cu)
    void *d_screen = nullptr;
    void free_device();
    const double *norm(int t, int s, int l) const { return &norms[(size_t)(off[t * S + s] + l + band[t * S + s]) * 4]; }
    long block_index(int t, int s, int l) const { return off[t * S + s] + l + band[t * S + s]; }
    void build(const Basis &b);  // build_operators({this}, b)
};
// several operators of one context at once (mw_basis.cpp)
void build_operators(const std::vector<Oper *> &ops, const Basis &b);


// Device bump allocator for per-call scratch (task lists, items, generated
// blocks).  reset() keeps one chunk large enough for the previous peak.
struct Arena {
    struct Chunk {
        void *ptr = nullptr;
        size_t size = 0, used = 0;
    };
    std::vector<Chunk> chunks;   // device memory
    std::vector<Chunk> hchunks;  // pinned host staging for the copies that fill it
    size_t total = 0;
    void *alloc(size_t bytes);
    void *halloc(size_t bytes);
    // call only when the GPU no longer reads anything allocated since the last reset
    void reset();
    void release();
};

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    Basis basis;
    DevBasis dbasis{};
    double *d_basis = nullptr;
    std::string err;
    mw_stats last{};
    int nsm = 0;
    void *owner = nullptr;  // the C-ABI handle holding this context
    int live = 0;           // trees and operators created through the C ABI and not yet destroyed
    bool closing = false;   // destroyed by the caller; released when live drops to 0
    Arena arena;
    // extra streams and arenas: the batched apply splits its jobs into up to XGROUPS + 1 groups
    // (group 0 on `stream` / `arena`), so that the host prepares one group's level while the GPU
    // computes the others'
    static constexpr int XGROUPS = 7;
    static constexpr int DEFAULT_GROUPS = 4;
    cudaStream_t xstream[XGROUPS] = {};
    Arena xarena[XGROUPS];
    int groups = DEFAULT_GROUPS;  // job groups of a batched apply (1: no overlap)
    // where a batched apply enumerates, screens and lists its items: 1 on the GPU (mw_screen.cu,
    // the default), 0 on the host (OpenMP); both give the same items in the same order
    int screening = 1;
    // first size of a job's generation table in the GPU screening (slots; 0: 16 x the job's
    // output nodes at the level, at least 256).  A table that fills up is grown 8x and the level's
    // walk repeated.  MW_SCREEN_GEN_SLOTS in the environment at context creation sets it, which
    // the tests use to run the growth path.
    long screen_gen_slots = 0;
    Arena sarena;  // per-apply tables of the GPU screening (input hash tables and norms)
    // launch settings of a batched apply: job groups, and the largest number of items one CTA
    // task takes per tier (FP64, FP32, TF32, double-FP32) before a node is split into chunks
    struct Tuning {
        int groups = DEFAULT_GROUPS;
        long long chunk[4] = {4, 32, 96, 8};
    };
    // settings picked by the autotuner (mw_apply_batch_autotune) per (order K, jobs, precision
    // mode); a batched apply with the same key uses them unless overlap is off (groups == 1)
    std::map<std::tuple<int, int, int>, Tuning> tuned;
    // high-priority stream for the generation of missing input nodes, which the host waits for
    // in the middle of preparing a level; the contraction kernels run one CTA per task, so the
    // generation gets the next free slot instead of waiting for whole kernels of other groups
    cudaStream_t fast = nullptr;
    cudaEvent_t fast_done = nullptr;
    // copy stream of a batched apply from host buffers: every job group's input blocks go up on
    // it in group order, while the host builds the input trees' structures
    cudaStream_t ustream = nullptr;
    // high-priority streams, one per job group, that put the group's uploaded blocks into its
    // trees and derive the reduced copies and screening tables from them: their kernels take the
    // next free SM slots beside the other groups' contractions
    cudaStream_t pstream[XGROUPS + 1] = {};
    // k_fetch launches so far (packs of a few MB, screening tables); the batched apply and multiply
    // add theirs to their launch counts
    long long fetch_launches = 0;
    void *h_pinned = nullptr;
    size_t pinned_bytes = 0;
    void *pinned(size_t bytes);
    void sync();
    // Device buffers a tree outgrew during the current call (Tree::reserve).  Kernels queued
    // earlier, on any of the context's streams, may still read them, so they are released only
    // when the call has ended and every stream of the context is idle (release_retired).
    std::vector<void *> retired;
    std::mutex retired_mu;  // trees of one call may grow on several host threads
    void release_retired();
};

// Packs host arrays into the context's pinned buffer and ships them to the
// device with a single copy; ptr(i) is the device address of array i.
struct Packer {
    std::vector<size_t> offs, size;
    std::vector<const void *> srcs;
    char *dev = nullptr;
    void *add(const void *src, size_t bytes);
    void ship(Ctx &ctx, Arena &arena);
    void *ptr(size_t i) const { return dev + offs[i]; }
};

// ---------------------------------------------------------------- kernel interface (mw_kernels.cu)
struct GenTask {
    const double *anc;  // ancestor block
    double *out;        // generated block
    double *cn;         // 8 norms of the generated block
    uint64_t path;      // 3 bits per step, first step in the lowest bits
    int steps;
    int pad;
};

struct ProjFunc {
    int kind;  // 0 gaussian sum, 1 hydrogen
    int nterms;
    const mw_gterm *terms;  // device
    int hn, hl, hm;
    double Z, origin[3], hnorm;
};

struct ProjTask {
    int n, l[3];
    double *out;
    double *cn;
    int zero;
    int pad;
};

// a node whose items ran as several chunks: out (=|+=) the sum of its chunks' partial blocks, in order
struct ReduceTask {
    double *out;
    const double *part;  // count consecutive partial blocks
    int count;
    int set;
};

struct ApplyLaunch {
    int nnodes;
    int root;                     // 1: include the (0,0) component pair
    int set;                      // 1: write the block, 0: add to it
    double *const *out;           // per node: output block
    const long long *begin;       // per node: first item
    const long long *end;         // per node: one past the last item
    const void *const *in;        // per item: input block (double or float)
    const void *const *ax;        // per item: operator blocks (double or float)
    const void *const *ay;
    const void *const *az;
    const double *coef;           // per item
    int *counter;                 // dynamic node counter (persistent grid); zero at launch
    int *status;                  // 0, or non-zero when a bounded wait of the launch ran out (TF32 tier)
    int *rows = nullptr;          // rows processed (y and z passes run), summed over the launch's tasks
    // chunked nodes: per task the index of its node's ReduceTask (-1: the task is a whole node),
    // and per ReduceTask a counter of finished chunks (zero at launch).  The CTA that finishes a
    // node's last chunk sums the partials into the node's block (mw_chunks.cuh).
    const int *red_of = nullptr;
    const ReduceTask *red = nullptr;
    int *red_cnt = nullptr;
};

struct PairTask {  // parent -> children (8 consecutive blocks)
    double *parent;
    double *child0;
};

struct MulTask {
    const double *a, *b;
    double *out;
    double *cn;
    double scale;  // coef * 2^{3(n+1)/2}
};

struct AddTask {
    double *out;
    double *cn;
    int first, count;  // into the (src, coef) arrays
};

// Launch settings a kernel needs once per device, kept so that a launch makes no extra driver calls
// (the apply launches a few hundred to a few thousand kernels per call): the dynamic shared memory
// it may request (cudaFuncSetAttribute), and its resident CTAs per SM at a block size and request.
void kernel_smem(const void *fn, int bytes);
int kernel_ctas_per_sm(const void *fn, int threads, int bytes);

void k_project(const DevBasis &b, const ProjFunc &f, const ProjTask *tasks, int n, cudaStream_t s);
// K = 4 .. 10: generate_kernel_t<K> (shared memory, scratch unused); other K: scratch holds
// grid x generate_scratch_doubles(K) doubles (one slice per CTA)
void k_generate(const DevBasis &b, const GenTask *tasks, int n, double *scratch, int grid, int nsm, cudaStream_t s);
inline size_t generate_scratch_doubles(int K) {
    return (size_t)4 * K * K * K + (size_t)2 * K * K * K + (size_t)K * K * K;
}
void k_apply(const DevBasis &b, const ApplyLaunch &L, int fp32, int nsm, cudaStream_t s);
// TF32 tensor-core tier on the 5th-generation tensor cores (tcgen05.mma, accumulators in tensor
// memory); items point at the operand layouts of mw_tc05_layout.h
// split = false: the TF32 tier; split = true: the split-TF32 tier (hi * hi + hi * lo + lo * hi of
// the TF32-rounded operands and their remainders, FP32 accumulation), the tensor-core form of the
// FP32 tier.  Item pointers point at the hi copies of mw_tc05_layout.h's operand layouts.
void k_apply_tc05(const DevBasis &b, const ApplyLaunch &L, bool split, cudaStream_t s);
// FP32 cube-order shadows (high cube read) -> the tensor-core tier's x-pass operand layout
void k_to_tc_x(const float *cube32, float *out, size_t nblocks, int K, cudaStream_t s);
// round to TF32: nearest, ties away from zero (as cvt.rna.tf32.f32)
inline float tf32_round_host(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0x1000u) & ~0x1fffu;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}
// double-FP32 tier: reads the high and low parts of the same shadows and operator blocks
void k_apply_df(const DevBasis &b, const ApplyLaunch &L, int nsm, cudaStream_t s);
void k_norms(const DevBasis &b, double *const *blocks, double *const *cn, int n, cudaStream_t s);
void k_topdown(const DevBasis &b, const PairTask *tasks, int n, cudaStream_t s);
void k_compress(const DevBasis &b, const PairTask *tasks, double *const *cn, int n, cudaStream_t s);
// the same two passes with double-FP32 arithmetic on the FP32 pipe (mw_post_df.cu); FP64 blocks and norms
void k_topdown_df(const DevBasis &b, const PairTask *tasks, int n, cudaStream_t s);
void k_compress_df(const DevBasis &b, const PairTask *tasks, double *const *cn, int n, cudaStream_t s);
// the multiply's node kernel (mw_multiply_df.cu): double-FP32 transforms, FP64 blocks in and out
// the tree multiply split at its values (mw_multiply_df.cu): value cubes of blocks (2 (2K)^3 floats
// each, (hi, lo) pairs in cube order), and nodes from two value cubes
struct MulVTask {
    const float2 *a, *b;  // value cubes of the inputs at the node
    double *out;
    double *cn;
    double scale;         // coef * 2^{3(n+1)/2}
};
size_t mul_value_floats(int K);
void k_values_df(const DevBasis &b, const double *const *blocks, float2 *const *vals, int n, int nsm, cudaStream_t s);
void k_multiply_values_df(const DevBasis &b, const MulVTask *tasks, int n, int nsm, cudaStream_t s);
// dst[off[r] ..] = the len[r] doubles at src[r], for n ranges (one download of many small arrays)
void k_gather_ranges(const double *const *src, const long long *off, const int *len, int n, double *dst,
                     cudaStream_t s);
void k_add(const DevBasis &b, const AddTask *tasks, const double *const *src, const double *coefs, int n, int bs,
           cudaStream_t s);
void k_to_fp32(const double *in, float *out, size_t n, cudaStream_t s);
// operator construction on the GPU (mw_opbuild.cu)
struct OpBuildTask {  // one (term, scale): tau(m) = pref * (Legendre expansion . Gaussian moments of beta)
    double beta, pref;
    int root, cap;    // root scale: no early stop; cap: largest translation walked
    long nrm_off;     // first of this task's 4 (cap + 1) sub-block norms
};
struct OpBlockJob {  // one block pair NS(+l), NS(-l) of a task, at blocks + (off + band +- l) blocks
    int task, l, band, zero;  // zero: bit 2g+f marks sub-block (g, f) as cut
    long off;
    double *blocks;           // the operator's FP64 blocks
};
size_t op_build_smem();
constexpr int OP_NRM_HEAD = 64;  // translations per task whose norms phase 1 also writes compactly
void k_op_band(int K, const double *W, const double *cc, const double *gx, const double *gw, const OpBuildTask *tasks,
               int ntask, double *nrm, double *head, int *band, double *peak, cudaStream_t s);
void k_op_blocks(int K, const double *W, const double *cc, const double *gx, const double *gw, const OpBuildTask *tasks,
                 const OpBlockJob *jobs, int njob, cudaStream_t s);
void k_op_convert(const double *blocks, float *b32, float *btc, float *btc2, long nblocks, int K, int NB, int groups,
                  cudaStream_t s);
// FP32 shadow of whole blocks in cube order cube[Z][Y][X] (X = cx*K + ix): per block a high cube
// and a low cube (2 * 8K^3 floats, the low one holds the rounded remainder)
void k_to_fp32_cube(const double *in, float *out, size_t nblocks, int K, cudaStream_t s);
void k_dot(const double *const *a, const double *const *b, const int *start, int n, int bs, double *partial,
           cudaStream_t s);
void k_scale(double *x, size_t n, double c, cudaStream_t s);
// dst block j = src block map[j]; bs even
void k_permute_blocks(double *dst, const double *src, const int *map, int n, int bs, cudaStream_t s);
// device memory from pinned host memory (allocated by cudaMallocHost) with a kernel instead of
// a copy engine
void k_fetch(void *dst, const void *src_pinned, size_t bytes, cudaStream_t s);
// ---------------------------------------------------------------- screening on the GPU (mw_screen.cu)
// Hash of a node key, shared by the host (which fills an input tree's table) and the device (which
// looks positions up in it).
__host__ __device__ inline unsigned key_hash(int n, int x, int y, int z) {
    uint64_t h = (uint64_t)(uint32_t)n * 0x9E3779B97F4A7C15ULL;
    h ^= (uint64_t)(uint32_t)x * 0xC2B2AE3D27D4EB4FULL;
    h = (h << 21) | (h >> 43);
    h ^= (uint64_t)(uint32_t)y * 0x165667B19E3779F9ULL;
    h = (h << 21) | (h >> 43);
    h ^= (uint64_t)(uint32_t)z * 0xD6E8FEB86659FD93ULL;
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ULL;
    h ^= h >> 29;
    return (unsigned)h;
}
constexpr int HASH_EMPTY = (int)0x80000000;  // n of an empty slot of an input tree's table

struct ScreenOp {  // one operator's tables (device)
    const int *band, *off;             // [T*S]: band L(t, n), block index of l = -L
    const double *norms;               // 4 sub-block norms per block
    const float *norms32;              // the same rounded to FP32 (the fast path's estimates)
    const double *amax, *xmax, *c;     // [T*S], [T*S], [T]
    const float *amax32, *xmax32;
    const double *b64;                 // blocks in the tier kernels' layouts
    const float *b32, *btc, *btc2;
    int T, S;
};
struct ScreenJob {  // one job of the apply (device)
    ScreenOp op;
    const int4 *hkey;  // the input tree's hash table: key (n, l) per slot, n = HASH_EMPTY when free
    const int *hval;   // node index per slot
    int hmask, pad;
    const double *cn;  // the input's component norms (8 per node) and block norms, as the host has them
    const double *bn;
    const float *cn32, *bn32;  // the same rounded to FP32
    const double *in64;  // the input's blocks and shadows
    const float *in32, *intc;
};
struct ScreenNode {  // one output node of the level (device)
    double thr, thr2;      // screening threshold of the walk, and of the items after generation
    double tthr, fm;       // tier threshold (< 0: FP64 only), pruning norm
    int job, l[3];
    int flags;             // bit 0: zero weight below the root scale (no items), bit 1: TF32 allowed,
                           // bit 2: FP32 estimates decide where they are clear of the thresholds
    int gtab, gmask;       // the job's generation table: first slot, mask
    // FP32 decision bands: an FP32 bound below lo fails, above hi passes, in between FP64 decides
    float thr_lo, thr_hi, thr2_lo, thr2_hi;
    float tier_lo[3], tier_hi[3];  // around TIER_TF32, TIER_FP64 and TIER_DF times tthr
    float fm32, prune32;           // fm, and thr (1 - margin): prune where fm32 * expr < prune32
};
struct ScreenCand {  // one item in walk order
    int src;                    // input node, or generated slot when gen = 1
    short lx, ly, lz;
    unsigned char tier, gen;
    int t;
};
struct ScreenLevel {
    const ScreenNode *nodes;
    const ScreenJob *jobs;
    int nn, n, sidx, root, n0, bs, bsz;
    int lo[3], hi[3];  // the world's translations at scale n: lo <= l < hi
    int mixed, near_fp64, df_only, dfp, tensor;
    double tier_fp64, tier_tf32, tier_df;
    // generation tables: per job gmask + 1 keys (0 = free) and slots; slot counter, overflow flag;
    // per slot: job, ancestor, ancestor scale, l[3]
    unsigned long long *gkey;
    int *gval, *gen_cnt, *overflow, *gen_info;
    int gen_cap;
    int *cnt;                   // [nn] items before the exact screening of generated inputs
    const long long *cand_off;  // [nn] first ScreenCand of each node
    ScreenCand *cand;
    double *gcn;                // generated blocks' component norms
    float *gcn32;               // the same rounded to FP32
    int *tcnt;                  // [nn][8]: items per tier, then component pairs per tier
    long long *tier_off;        // [nn][4]: first item of each node in each tier's arrays
    long long *tier_tot;        // [4]
    const void **in, **ax, **ay, **az;  // item arrays, the tiers one after the other
    double *coef;
    double *g64;                // generated blocks and their shadows
    float *g32, *gtc;
    size_t tx, tb;              // floats per block in the TF32 layouts (input, operator)
};
// shared memory of the walk kernels: maxT = most terms of an operator, zmax = most (t, lz) rows of
// one at the level's scale (sum over terms of 2 L(t, n) + 1)
size_t screen_smem(int maxT, int zmax);
void k_screen_count(const ScreenLevel &P, int maxT, int zmax, cudaStream_t s);
void k_screen_gen_tasks(const ScreenLevel &P, GenTask *tasks, int ngen, cudaStream_t s);
// FP32 copies of the generated blocks' component norms (after the generation kernel)
void k_screen_gen_norms32(const ScreenLevel &P, int ngen, cudaStream_t s);
void k_screen_write(const ScreenLevel &P, int maxT, int zmax, cudaStream_t s);
void k_screen_fill(const ScreenLevel &P, cudaStream_t s);

// true when the GPU's DMA engines can read / write the host buffer directly (pinned memory)
bool host_is_pinned(const void *p);
double probe_fma_tflops(int fp64, int nsm, cudaStream_t s);
double probe_mma_tflops(int kind, int nsm, cudaStream_t s);
double probe_tc05_tflops(int n, int nsm, cudaStream_t s);
void k_eval(const DevBasis &b, const double *const *blocks, const int *keys, const double *pts, int npts,
            double *out, cudaStream_t s);

}  // namespace mwg
