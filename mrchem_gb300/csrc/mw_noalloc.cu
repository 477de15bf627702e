// mw_noalloc.cu -- inner product of two trees that allocates no memory.
//
// Some callers cannot allocate GPU memory at the moment they need an overlap
// or an energy:
//  - a process whose device memory is already reserved by another runtime's
//    caching allocator, so cudaMalloc fails even though that memory sits idle;
//  - a code path that must not synchronise the device, since cudaMalloc and
//    cudaFree may block on other streams' work.
// mw_dot_noalloc serves them.  It computes the same sum as mw_dot with the same
// kernel, but stages the node-pair lists and the per-pair partial sums in a
// file-scope device array instead of memory it allocates.
//
// The array is a fixed 1 MiB, held on every GPU that loads the library until the
// process exits.  It takes at most NOALLOC_MAX_PAIRS node pairs (nodes present
// in both trees); a larger call is rejected with MW_ERR_ARG.  All calls share the
// array, and host staging is file-scope too: calls that overlap, on the GPU or
// from several host threads, race and must be serialised by the caller.
// Nothing needs clearing between calls, since each call writes every entry it
// later reads.  The array's device address is looked up (cudaGetSymbolAddress)
// when a context is created on a device, with that device current: with lazy
// module loading that lookup is what loads this file's module and reserves the
// 1 MiB, so it happens at mw_ctx_create, where the caller may still allocate,
// and never inside mw_dot_noalloc itself.  Each call copies its pair lists from
// host arrays and waits for its result on the host (a stream synchronisation),
// so it must not be called while the context's stream is being captured.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "mw_internal.h"

namespace mwg {

namespace {

constexpr size_t NOALLOC_BYTES = size_t(1) << 20;
constexpr int NOALLOC_MAX_PAIRS = 32768;
// per pair: two block pointers, one partial sum, one start offset
static_assert((size_t)NOALLOC_MAX_PAIRS * (3 * sizeof(void *) + sizeof(int)) <= NOALLOC_BYTES, "scratch too small");

__device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

constexpr int MAX_DEVICES = 64;
void *g_scratch_addr[MAX_DEVICES] = {nullptr};
std::mutex g_setup_mutex;

// host staging for the pair lists and the partial sums (file scope: no allocation per call)
const double *h_pa[NOALLOC_MAX_PAIRS];
const double *h_pb[NOALLOC_MAX_PAIRS];
int h_start[NOALLOC_MAX_PAIRS];
double h_part[NOALLOC_MAX_PAIRS];

// device address of the scratch array on `device` (which must be current); looked up once
char *scratch_on(int device) {
    if (device < 0 || device >= MAX_DEVICES) throw Error(MW_ERR_ARG, "mw_dot_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            throw Error(MW_ERR_CUDA, std::string("mw_dot_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
        g_scratch_addr[device] = p;
    }
    return static_cast<char *>(g_scratch_addr[device]);
}

}  // namespace

void noalloc_setup(int device) { scratch_on(device); }

double dot_noalloc(const Tree &a, const Tree &b) {
    Ctx &ctx = *a.ctx;
    const int K3 = ctx.basis.K * ctx.basis.K * ctx.basis.K;
    int n = 0;
    for (int i = 0; i < a.nn(); i++) {
        const NodeInfo &nd = a.nodes[i];
        int j = b.find(nd.n, nd.l);
        if (j < 0) continue;
        if (n == NOALLOC_MAX_PAIRS)
            throw Error(MW_ERR_ARG, "mw_dot_noalloc: the trees share more than " + std::to_string(NOALLOC_MAX_PAIRS) +
                                        " nodes, the most its fixed scratch holds; use mw_dot");
        h_pa[n] = a.block(i);
        h_pb[n] = b.block(j);
        h_start[n] = nd.n == ctx.basis.n0 ? 0 : K3;
        n++;
    }
    if (n == 0) return 0.0;
    char *base = scratch_on(ctx.device);
    // layout: [pointers a][pointers b][partials][starts], 8-byte aligned throughout
    const double **d_pa = reinterpret_cast<const double **>(base);
    const double **d_pb = d_pa + NOALLOC_MAX_PAIRS;
    double *d_part = reinterpret_cast<double *>(d_pb + NOALLOC_MAX_PAIRS);
    int *d_start = reinterpret_cast<int *>(d_part + NOALLOC_MAX_PAIRS);
    MWG_CUDA(cudaMemcpyAsync(d_pa, h_pa, sizeof(void *) * n, cudaMemcpyHostToDevice, ctx.stream));
    MWG_CUDA(cudaMemcpyAsync(d_pb, h_pb, sizeof(void *) * n, cudaMemcpyHostToDevice, ctx.stream));
    MWG_CUDA(cudaMemcpyAsync(d_start, h_start, sizeof(int) * n, cudaMemcpyHostToDevice, ctx.stream));
    k_dot(d_pa, d_pb, d_start, n, ctx.basis.bs, d_part, ctx.stream);
    MWG_CUDA(cudaMemcpyAsync(h_part, d_part, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    double s = 0.0;
    for (int i = 0; i < n; i++) s += h_part[i];
    return s;
}

}  // namespace mwg
