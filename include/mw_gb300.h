/*
 * mw_gb300.h -- C ABI of the GB300-native multiwavelet apply engine.
 *
 * Drop-in boundary for the mrcpp:: calls MRChem makes on its hot path
 * (MRCPP commit 0e5b32003eed8e1abb22a44ba4e1a2ce9fd9ddb1, fetched by
 * external/upstream/fetch_mrcpp.cmake:39-42).  Plain pointers and sizes only.
 * Every entry returns an int status (MW_OK = 0); mw_last_error() gives the
 * message of the last failure on a context.  Calls on one context are
 * serialised on that context's CUDA stream; trees and operators belong to
 * the context that created them.
 *
 * Conventions:
 *   node key   int[4] = (n, lx, ly, lz): the box [2^-n l, 2^-n (l+1)]^3
 *   block      8 * K^3 doubles (K = order + 1): component c = cx|cy<<1|cz<<2
 *              (bit set = wavelet in that dimension), inner index
 *              ix + K*iy + K*K*iz.  Component 0 holds the node's scaling
 *              coefficients, components 1..7 its wavelet coefficients.
 *   tree       complete octree: every node has 0 or 8 children; host arrays
 *              are in canonical order (by scale, then Morton order with z
 *              most significant).
 */
#ifndef MW_GB300_H
#define MW_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MW_OK 0
#define MW_ERR_ARG 1
#define MW_ERR_OOM 2
#define MW_ERR_CUDA 3
#define MW_ERR_TIMEOUT 4
#define MW_ERR_STATE 5

#define MW_BASIS_LEGENDRE 0
#define MW_BASIS_INTERPOLATING 1

/* precision modes of mw_apply / mw_apply_batch */
#define MW_PREC_FP64 0   /* every contraction in FP64 */
/* norm-tiered by the item's bound b against the screening threshold tau: double-FP32 (pairs of
 * FP32 numbers, ~3e-13 b) when 2e6 tau < b <= 1e11 tau, FP64 above that, TF32 tensor cores (FP32
 * accumulation) when b <= 2e3 tau below the root scale, FP32 CUDA cores otherwise; root-scale
 * items under relative precision run in FP64 */
#define MW_PREC_MIXED 1
#define MW_PREC_MIXED_NEARFP64 2  /* as MW_PREC_MIXED, and every item with |l|_inf <= 1 in FP64 */
#define MW_PREC_MIXED_FP32 3      /* FP64 or FP32 only: no tensor-core and no double-FP32 tier */
#define MW_PREC_DF 4              /* double-FP32 for every item with b <= 1e11 tau, FP64 above that and for
                                   * root-scale items under relative precision (error ~3e-13 b per item) */

typedef struct mw_ctx_s *mw_ctx;
typedef struct mw_tree_s *mw_tree;
typedef struct mw_op_s *mw_op;

/* coef * (x-X)^px (y-Y)^py (z-Z)^pz * exp(-alpha |r-R|^2) */
typedef struct {
    double coef;
    double alpha;
    double pos[3];
    int pw[3];
    int pad;
} mw_gterm;

typedef struct {
    long long out_nodes;     /* output nodes computed */
    long long items;         /* (output node, input node, term) contractions */
    long long items_fp64;    /* ... of which in FP64 */
    long long items_fp32;    /* ... in FP32 */
    long long items_tf32;    /* ... in TF32 on the tensor cores */
    long long generated;     /* generated input nodes */
    long long levels;        /* refinement iterations */
    long long launches;      /* kernels launched */
    double flops;            /* algorithmic: 6 K^4 per surviving component pair */
    double flops_issued;     /* as executed by the kernels */
    double bytes;            /* algorithmic coefficient + operator bytes */
    double kernel_ms;        /* CUDA-event time of the contraction kernels */
    double host_ms;          /* wall time of the call */
    double flops_fp64;       /* algorithmic flops of the FP64 tier */
    double flops_fp32;       /* ... of the FP32 tier */
    double kernel_ms_fp64;   /* CUDA-event time of the FP64 contraction launches */
    double kernel_ms_fp32;   /* ... of the FP32 contraction launches */
    double host_enum_ms;     /* host: candidate enumeration (screening bounds, lookups); with GPU
                                screening, the wait for the GPU's candidate counts */
    double host_items_ms;    /* host: exact screening, tiers, item lists (GPU screening: the
                                per-tier node lists built from the GPU's counts) */
    double host_wait_ms;     /* host: waiting for the level's kernels and norm downloads */
    double flops_tf32;       /* algorithmic flops of the TF32 tier */
    double kernel_ms_tf32;   /* CUDA-event time of the TF32 contraction launches */
    long long items_df;      /* contractions in double-FP32 (pairs of FP32 numbers) */
    double flops_df;         /* algorithmic flops of the double-FP32 tier */
    double kernel_ms_df;     /* CUDA-event time of the double-FP32 contraction launches */
    double host_gen_ms;      /* host: generation requests and the generation of missing input nodes */
    double host_launch_ms;   /* host: ordering, chunking and packing the item lists, launches */
    double host_refine_ms;   /* host: refinement decisions after each level */
    double gpu_levels_ms;    /* GPU time from the call's first queued work to the end of its last level */
    double gpu_post_ms;      /* GPU time of the post-processing (sum over scales, compression, norms),
                                summed over the job groups, which overlap other groups' levels */
    long long screen_regrows; /* GPU screening: levels walked again after a generation table filled up */
    long long rows_fp64;      /* rows of the FP64 tier: runs of consecutive items of one node with the
                                 same term, ly and lz, whose x passes are summed before one y and one
                                 z pass */
    long long rows_fp32;      /* ... of the FP32-accuracy tier */
    long long rows_tf32;      /* ... of the TF32 tier */
    long long rows_df;        /* ... of the double-FP32 tier */
    double host_io_ms;        /* mw_apply_batch_host: host time building the input trees' structures,
                                 waiting for each job group's uploaded inputs and preparing them, and
                                 queueing the outputs' downloads */
} mw_stats;

/* ---- context (replaces MultiResolutionAnalysis<3>, src/mrenv.cpp:105-122) ---- */
int mw_ctx_create(int device, int root_scale, const int corner[3], const int boxes[3], int order, int basis,
                  int max_depth, mw_ctx *out);
/* Handles may be destroyed in any order: a destroyed context is released when the last of its
 * trees and operators is destroyed. */
int mw_ctx_destroy(mw_ctx ctx);
const char *mw_last_error(mw_ctx ctx);
int mw_ctx_basis(mw_ctx ctx, double *qx, double *qw, double *filter, double *c2v, double *v2c);
int mw_ctx_last_stats(mw_ctx ctx, mw_stats *st);
int mw_ctx_synchronize(mw_ctx ctx);
/* Batched applies split their jobs into up to four groups on their own streams and prepare one
 * group's level on the host while the GPU computes the others' (on = 1, the default).  With
 * on = 0 the groups are not formed: the tier kernels then run alone, so their CUDA-event times in
 * mw_stats are exclusive.  Results are bit-identical either way.  No counterpart in the reference
 * (its applies are one per call). */
int mw_ctx_set_overlap(mw_ctx ctx, int on);
/* The number of job groups (1..8) batched applies split into; mw_ctx_set_overlap sets 4 or 1. */
int mw_ctx_set_groups(mw_ctx ctx, int n);
/* Where applies enumerate their candidate items, screen them with the norm-product bound and
 * build the per-tier item lists: on = 1 on the GPU (the default), on = 0 on the host (OpenMP over
 * output nodes).  Both give the same items in the same order, so results are bit-identical.  Levels
 * more than 20 scales below the root and operators with bands above 32767 are screened on the
 * host either way.
 * Replaces the screening inside mrcpp::apply (CoulombPotential.cpp:131, HelmholtzVector.cpp:149),
 * which MRCPP runs on the host. */
int mw_ctx_set_screening(mw_ctx ctx, int on);

/* ---- trees (replaces FunctionTree<3>, src/qmfunctions/Orbital.h:51) ---- */
int mw_tree_create(mw_ctx ctx, mw_tree *out);
int mw_tree_destroy(mw_tree t);
int mw_tree_nnodes(mw_tree t, int *n);
int mw_tree_nleaves(mw_tree t, int *n);
int mw_tree_depth(mw_tree t, int *d);
int mw_tree_upload(mw_tree t, int nnodes, const int *keys, const double *coefs);
int mw_tree_download(mw_tree t, int *keys, double *coefs, unsigned char *is_leaf);
/* mw_tree_upload / mw_tree_download for n trees of one context with one synchronisation in all
 * (the reference moves orbitals one at a time, src/qmfunctions/orbital_utils.cpp:1218-1240).
 * Arrays of n per-tree pointers; a null keys / coefs / is_leaf entry skips that output. */
int mw_tree_upload_batch(int n, mw_tree *trees, const int *nnodes, const int *const *keys,
                         const double *const *coefs);
int mw_tree_download_batch(int n, mw_tree *trees, int *const *keys, double *const *coefs,
                           unsigned char *const *is_leaf);
/* Page-locks (pins) a host buffer for the context's GPU, or releases it.  When every coefficient
 * buffer of a batched upload or download is pinned, the GPU's copy engines move it directly and
 * the reordering into tree or canonical order runs on the device; otherwise the library stages
 * the blocks through its own pinned buffer.  No counterpart in the reference. */
int mw_pin_host(mw_ctx ctx, void *p, size_t bytes);
int mw_unpin_host(mw_ctx ctx, void *p);
int mw_tree_squared_norm(mw_tree t, double *out);
int mw_tree_integrate(mw_tree t, double *out);
int mw_tree_rescale(mw_tree t, double c);
int mw_tree_eval(mw_tree t, int npts, const double *xyz, double *out);
/* FunctionTree::clear / mrcpp::clear: back to the root nodes, zero coefficients */
int mw_tree_clear(mw_tree t);

/* mrcpp::project(prec, tree, GaussExp<3>) (src/qmfunctions/...; density_utils.cpp) */
int mw_project_gauss(double prec, mw_tree out, int nterms, const mw_gterm *terms, int abs_prec);
/* hydrogen-like orbital n, l (<= 1), m (x,y,z for l = 1), src/analyticfunctions/HydrogenFunction.cpp:35-198 */
int mw_project_hydrogen(double prec, mw_tree out, int n, int l, int m, double Z, const double origin[3], int abs_prec);

/* grids: mrcpp::copy_grid / build_grid / copy_func (src/qmfunctions/density_utils.cpp:72,85,87) */
int mw_copy_grid(mw_tree out, mw_tree inp);
int mw_build_grid(mw_tree out, int n, const mw_tree *trees);
int mw_copy_func(mw_tree out, mw_tree inp);
/* FunctionTree::crop(prec) (src/qmfunctions/density_utils.cpp:147) */
int mw_crop(mw_tree t, double prec, int abs_prec);
/* mrcpp::dot (src/qmfunctions/orbital_utils.cpp:79-82) */
int mw_dot(mw_tree a, mw_tree b, double *out);
/* The same inner product as mw_dot, for callers that cannot allocate at the moment they need it
 * (device memory held by another runtime's caching allocator; code that must not let cudaMalloc /
 * cudaFree synchronise the device).  No counterpart in the reference.  Allocates nothing: the
 * node-pair lists and partial sums live in a fixed 1 MiB device array that every GPU loading this
 * library holds until exit, so at most 32768 nodes common to both trees (MW_ERR_ARG beyond that).
 * All calls share that array: calls that overlap on the GPU or across host threads race.  The
 * array is reserved, and its address looked up, by mw_ctx_create on the context's device, not by
 * this call.  The call blocks until the result is on the host (it synchronises the context's
 * stream), so it must not be called while that stream is being captured. */
int mw_dot_noalloc(mw_tree a, mw_tree b, double *out);

/* ---- operators (src/driver.cpp:1131,1283; src/scf_solver/HelmholtzVector.cpp:144) ---- */
int mw_op_create_poisson(mw_ctx ctx, double prec, mw_op *out);
int mw_op_create_helmholtz(mw_ctx ctx, double mu, double prec, mw_op *out);
/* n Helmholtz operators built together (their NS blocks in shared GPU launches); the loop that
 * creates one operator per orbital in HelmholtzVector::apply, src/scf_solver/HelmholtzVector.cpp:144 */
int mw_op_create_helmholtz_batch(mw_ctx ctx, int n, const double *mu, double prec, mw_op *out);
int mw_op_destroy(mw_op op);
int mw_op_nterms(mw_op op, int *n);
int mw_op_terms(mw_op op, double *coefs, double *exps);
int mw_op_band(mw_op op, int term, int scale, int *band);
int mw_op_block(mw_op op, int term, int scale, int l, double *blk, double *norms4);

/* ---- the hot path ---- */
/* mrcpp::apply(prec, out, oper, inp[, precTrees], maxIter, absPrec)
 * (CoulombPotential.cpp:131,156; HelmholtzVector.cpp:149,154; ExchangePotential.cpp:200,204).
 * out must be empty (root nodes only); nprec = 0 for the plain call. */
int mw_apply(double prec, mw_tree out, mw_op op, mw_tree inp, int nprec, const mw_tree *prec_trees, int max_iter,
             int abs_prec, int precision_mode);
/* n independent applies (own operator, input, output, prec) in lockstep, one launch per level
 * (HelmholtzVector::operator(), src/scf_solver/HelmholtzVector.cpp:70-91; the exchange pair loop,
 * src/qmoperators/two_electron/ExchangePotentialD1.cpp:179-240).  nprec[i] precision-steering trees
 * of job i are consecutive in prec_trees (nprec may be NULL). */
int mw_apply_batch(int n, const double *precs, mw_tree *outs, mw_op *ops, mw_tree *inps, const int *nprec,
                   const mw_tree *prec_trees, int max_iter, int abs_prec, int precision_mode);
/* apply on a fixed output grid (the output's current grid, no refinement) */
/* mw_tree_upload_batch of the inputs, mw_apply_batch (no precision trees) and, optionally,
 * mw_tree_download_batch of the outputs, with the transfers overlapped: the job groups' input
 * blocks go up on one copy stream in group order while the host builds the input trees, each
 * group is prepared on its own high-priority stream and starts computing once its blocks have
 * landed; each group's outputs go down as soon as its post-processing is queued, beside the other
 * groups' work.
 * in_keys / in_coefs as in mw_tree_upload_batch.  Outputs (out_cap may be NULL for none): per job,
 * buffers for out_cap[i] nodes as mw_tree_download_batch fills them; out_nnodes[i] is the output's
 * node count when they were filled, minus it when the output did not fit or out_coefs[i] is not
 * pinned (then download it with mw_tree_download_batch).  The overlap needs distinct input trees
 * that are not outputs, and input buffers pinned with mw_pin_host; otherwise the inputs go up
 * first.  Results are bit-identical to the separate calls.  The reference has no counterpart
 * (HelmholtzVector::operator(), src/scf_solver/HelmholtzVector.cpp:70-91, applies orbitals that
 * already live in memory). */
int mw_apply_batch_host(int n, const double *precs, mw_tree *outs, mw_op *ops, mw_tree *inps, const int *in_nnodes,
                        const int *const *in_keys, const double *const *in_coefs, int max_iter, int abs_prec,
                        int precision_mode, const int *out_cap, int *const *out_keys, double *const *out_coefs,
                        unsigned char *const *out_leaf, int *out_nnodes);
/* Autotuner of the batched apply's launch settings (no counterpart in the reference): runs the
 * batch (as mw_apply_batch with no precision trees and max_iter = -1) `repeats` times for each
 * candidate -- job groups 2..6, then the chunk size of the TF32, FP32 and double-FP32 tiers, one
 * at a time -- and keeps the fastest (a candidate must beat the kept settings by 2%) in the context for this (order, n, precision_mode); later
 * batched applies with the same key use it.  The outputs hold the result of a last run with the
 * settings kept.  Returns the settings (groups, chunks[4] for FP64, FP32, TF32, double-FP32) and
 * their median wall time in ms.  Needs job-group overlap on (mw_ctx_set_overlap). */
int mw_apply_batch_autotune(int n, const double *precs, mw_tree *outs, mw_op *ops, mw_tree *inps, int abs_prec,
                            int precision_mode, int repeats, int *groups, long long *chunks, double *ms);
int mw_apply_fixed(double prec, mw_tree out, mw_op op, mw_tree inp, int abs_prec, int precision_mode);
/* L2-adjoint of the fixed-grid FP64 apply y = A x (output grid = seed's grid, absolute precision):
 * out <- A^T seed on x's grid, with the forward's item set (screened with x's norms).  Transposed
 * operator blocks, contraction grouped by input node (gather), then the forward's post-processing.
 * No MRCPP counterpart: it serves the gradient of the Coulomb energy J = 1/2 <rho, P rho>. */
int mw_apply_adjoint(double prec, mw_tree out, mw_op op, mw_tree x, mw_tree seed, int abs_prec);

/* mrcpp::multiply(prec, out, coef, a, b, maxIter, absPrec, useMaxNorms)
 * (QMPotential.cpp:147; ExchangePotential.cpp:175,213,223); out's current grid is the start grid */
int mw_multiply(double prec, mw_tree out, double coef, mw_tree a, mw_tree b, int max_iter, int abs_prec,
                int use_max_norms);
/* L2-adjoint of the fixed-grid product h = coef a b (mw_multiply with max_iter = 0 on h's grid)
 * in its first factor: out <- coef P_a(seed b), the product of the seed (on h's grid) and b on the
 * seed's grid, projected onto a's grid.  <seed, coef a b> = <out, a> to rounding.  No MRCPP
 * counterpart: it is the transpose of mrcpp::multiply (QMPotential.cpp:147,
 * density_utils.cpp:73) for gradients through orbital products and densities. */
int mw_multiply_adjoint(double prec, mw_tree out, double coef, mw_tree a, mw_tree b, mw_tree seed);
/* n independent products out_i = coef_i a_i b_i, level-synchronous (exchange pair products,
 * src/qmoperators/two_electron/ExchangePotential.cpp:175) */
int mw_multiply_batch(int n, const double *precs, mw_tree *outs, const double *coefs, mw_tree *as, mw_tree *bs,
                      int max_iter, int abs_prec, int use_max_norms);
/* mrcpp::square(prec, out, inp) (src/qmfunctions/density_utils.cpp:73) */
int mw_square(double prec, mw_tree out, mw_tree inp, int max_iter, int abs_prec);
/* mrcpp::add(prec, out, FunctionTreeVector, maxIter) on the union grid (density_utils.cpp:85-86) */
int mw_add(double prec, mw_tree out, int n, const double *coefs, const mw_tree *trees, int max_iter);

/* ---- composite steps around the path, device-resident ---- */
/* rho <- sum_i occ_i |phi_i|^2 (density::compute, src/qmfunctions/density_utils.cpp:64-150): squares
 * on copies of the orbitals' grids (one batched multiply), added on their union grid, cropped at
 * prec / sum(occ) when crop != 0 */
int mw_density(double prec, mw_tree rho, int n, const mw_tree *orbitals, const double *occ, int crop);
/* out_i <- sum_j U[i*nin + j] in_j on the inputs' union grid (orbital rotation,
 * src/qmfunctions/orbital_utils.cpp:242-248) */
int mw_rotate(int nout, mw_tree *outs, int nin, const mw_tree *ins, const double *U);
/* one tree to / from a file (checkpoint, src/qmfunctions/orbital_utils.cpp:1218-1240); format in mw_tree.cpp */
int mw_tree_save(mw_tree t, const char *path);
int mw_tree_load(mw_tree t, const char *path);

/* ---- diagnostics ---- */
/* measured FMA throughput of this GPU (TFLOP/s) in FP64 (fp64 = 1) or FP32 (fp64 = 0):
 * the denominator of the CUDA-core roofline of the contraction kernels */
int mw_probe_fma_peak(mw_ctx ctx, int fp64, double *tflops);
/* measured dense tensor-core throughput (TFLOP/s): kind 0 = warp-level mma.sync TF32 m16n8k8,
 * kind 1 = mma.sync BF16 m16n8k16, kind 2 = tcgen05.mma TF32 M128 N256 K8 (the device's dense TF32
 * rate), kind 3 = tcgen05.mma TF32 M128 N32 K8 (the shape of the TF32 apply tier) */
int mw_probe_mma_peak(mw_ctx ctx, int kind, double *tflops);

#ifdef __cplusplus
}
#endif
#endif
