// mw_internal.h -- driver-level declarations shared by the host translation units.
#pragma once

#include "mw_host.h"

namespace mwg {

// generated (reconstructed) blocks of one source tree at requested positions
struct GenSet {
    std::unordered_map<Key, int, KeyHash> slot;
    std::vector<Key> keys;
    std::vector<int> anc;
    std::vector<GenTask> tasks;
    double *base = nullptr;       // device blocks after generation
    std::vector<double> cn;       // their component norms
    void clear();
    int request(const Tree &src, int n, const int *l, int ancestor);
    double *generate(const Tree &src, Arena &arena, std::vector<double> &cn_out, mw_stats *st);
};

void generate_all(const std::vector<std::pair<GenSet *, const Tree *>> &sets, Arena &arena, mw_stats *st);
int find_ancestor(const Tree &t, int n, const int *l, int *an_out);
const double *block_at(const Tree &src, const GenSet &gs, const double *gbase, int n, const int *l);
bool key_less(const Basis &b, const NodeInfo &x, const NodeInfo &y);
std::vector<int> canonical_order(const Tree &t);

void tree_zero(Tree &t, int first, int count);
void tree_clear(Tree &t);
void tree_compress(Tree &t, Arena &arena, mw_stats *st);
void tree_norms_all(Tree &t, Arena &arena);
void tree_upload(Tree &t, int nnodes, const int *keys, const double *coefs, Arena &arena);
void tree_download(Tree &t, int *keys, double *coefs, unsigned char *leaf);
void tree_upload_batch(const std::vector<Tree *> &trees, const int *nnodes, const int *const *keys,
                       const double *const *coefs, Arena &arena);
void tree_norms_batch(const std::vector<Tree *> &trees, const int *nnodes, Arena &arena);
void tree_download_batch(const std::vector<Tree *> &trees, int *const *keys, double *const *coefs,
                         unsigned char *const *leaf);

void project_gauss(double prec, Tree &t, int nterms, const mw_gterm *terms, bool abs_prec, Arena &arena);
void project_hydrogen(double prec, Tree &t, int n, int l, int m, double Z, const double *origin, bool abs_prec,
                      Arena &arena);

void copy_grid(Tree &out, const Tree &inp);
void build_grid(Tree &out, const std::vector<const Tree *> &trees);
void combine_on_grid(Tree &out, const std::vector<const Tree *> &trees, const std::vector<double> &coefs, Arena &arena,
                     mw_stats *st);
void copy_func(Tree &out, const Tree &inp, Arena &arena);
void crop(Tree &t, double prec, bool abs_prec, Arena &arena);
double dot(const Tree &a, const Tree &b, Arena &arena);
double integrate(const Tree &t);
void rescale(Tree &t, double c);
void eval_points(const Tree &t, int npts, const double *xyz, double *out, Arena &arena);

struct ApplyJob {
    Tree *out;
    Oper *op;
    Tree *inp;
    double prec;
    bool abs_prec;
    int max_iter;
    std::vector<Tree *> prec_trees;
};

struct MulJob {
    Tree *out;
    Tree *a, *b;
    double coef, prec;
    int max_iter;
    bool abs_prec, use_max_norms;
};

// host inputs of a batched apply: per job, the input tree's keys and the caller's pinned
// coefficient blocks (in the keys' order); the input trees must be distinct
struct HostInputs {
    std::vector<int> nnodes;
    std::vector<const int *> keys;
    std::vector<const double *> coefs;
    // optional host outputs, per job: buffers for out_cap nodes (coefficients pinned).  When a job
    // group's post-processing is queued, each of its outputs that fits goes down in canonical
    // order on the group's stream; out_nnodes gets the node count, negative when it did not fit.
    std::vector<int *> out_keys;
    std::vector<double *> out_coefs;
    std::vector<unsigned char *> out_leaf;
    std::vector<int> out_cap;
    int *out_nnodes = nullptr;
};
void apply_batch(std::vector<ApplyJob> &jobs, int precision_mode, bool fixed_grid, mw_stats &st,
                 const HostInputs *hin = nullptr);
// the trees' structures from their keys, all trees in parallel (host work; the device arrays are
// sized first); per tree, the caller's block index of each tree node
std::vector<std::vector<int>> upload_structures(const std::vector<Tree *> &trees, const int *nnodes,
                                                const int *const *keys);
// on the context's current stream: the caller's blocks, already copied to the device in the
// caller's order (`staged`, tree after tree), permuted into the trees' order, the trees' norms,
// and the norms' download into pinned staging, returned (8 per node, tree after tree); read it
// after the stream has passed this point
double *upload_enqueue(const std::vector<Tree *> &trees, const std::vector<const int *> &maps,
                       const double *staged, Arena &arena);
// on the context's current stream: the trees' blocks in canonical order into the caller's pinned
// buffers; keys and leaf flags (host data, either may be null) are written before it returns
void download_enqueue(const std::vector<Tree *> &trees, int *const *keys, double *const *coefs,
                      unsigned char *const *leaf, Arena &arena);
void multiply_batch(std::vector<MulJob> &jobs, mw_stats &st);
void apply_adjoint(double prec, Tree &res, Oper &op, Tree &x, Tree &y, mw_stats &st);
void multiply_adjoint(double prec, Tree &out, double coef, const Tree &a, Tree &b, Tree &seed, mw_stats &st);
void density(double prec, Tree &rho, const std::vector<Tree *> &orbs, const std::vector<double> &occ, bool crop_sum,
             mw_stats &st);
void rotate(const std::vector<Tree *> &outs, const std::vector<const Tree *> &ins, const double *U, mw_stats &st);
double dot_noalloc(const Tree &a, const Tree &b);
// looks up the no-allocation scratch array's address on `device` (current), loading its module
void noalloc_setup(int device);
void tree_save(Tree &t, const char *path);
void tree_load(Tree &t, const char *path);
// bottom-up compression of several trees, one launch per scale; df: double-FP32 transforms
void compress_batch(const std::vector<Tree *> &trees, Arena &arena, mw_stats *st, bool df = false);
void add(Tree &out, const std::vector<const Tree *> &trees, const std::vector<double> &coefs, mw_stats &st);

}  // namespace mwg
