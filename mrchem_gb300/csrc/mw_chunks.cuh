// mw_chunks.cuh -- the end of a chunk task in the contraction kernels.
//
// A node with many items runs as several chunk tasks, each writing a partial block.  The CTA
// that finishes the last of a node's chunks sums all of them, in chunk order, into the node's
// block, so the result does not depend on which CTA ran which chunk or in what order they
// ended, and no separate reduction launch is needed.
#pragma once

#include "mw_host.h"

namespace mwg {
namespace {

// Called by every thread of the CTA after it has written task w's block (out of L.out[w]).
// flag: a shared int of the CTA.
__device__ __forceinline__ void finish_chunk(const ApplyLaunch &L, int w, int bs, int *flag) {
    if (!L.red_of) return;
    const int r = L.red_of[w];
    if (r < 0) return;
    __threadfence();  // this thread's stores of the partial block, before the count below
    __syncthreads();
    if (threadIdx.x == 0) {
        const int done = atomicAdd(&L.red_cnt[r], 1);
        __threadfence();
        *flag = done == L.red[r].count - 1;
    }
    __syncthreads();
    if (*flag) {
        const ReduceTask T = L.red[r];
        for (int i = threadIdx.x; i < bs; i += blockDim.x) {
            double v = T.set ? 0.0 : T.out[i];
            for (int c = 0; c < T.count; c++) v += __ldcg(T.part + (size_t)c * bs + i);  // written by other CTAs
            T.out[i] = v;
        }
    }
    __syncthreads();
}

}  // namespace
}  // namespace mwg
