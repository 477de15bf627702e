// mw_kernels.cu -- sm_103a kernels of the multiwavelet engine.
//
// Layouts: a node block is 8*K^3 doubles, component-major (component
// c = cx|cy<<1|cz<<2, inner index ix + K*iy + K*K*iz).  Inside a CTA a block
// is staged as the (2K)^3 "cube" cube[Z][Y][X] with X = cx*K + ix, so a
// multiwavelet transform or a non-standard-form operator application is three
// 2K x 2K matrix passes, one per dimension.
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <tuple>

#include "mw_chunks.cuh"
#include "mw_host.h"

namespace mwg {

namespace {

__device__ __forceinline__ int cube_of_block(int gi, int K) {
    int K3 = K * K * K;
    int c = gi / K3, r = gi - c * K3;
    int iz = r / (K * K), iy = (r / K) % K, ix = r % K;
    int X = (c & 1) * K + ix, Y = ((c >> 1) & 1) * K + iy, Z = (c >> 2) * K + iz;
    int N2 = 2 * K;
    return (Z * N2 + Y) * N2 + X;
}

// cube <- (M (x) M (x) M) cube, M 2K x 2K row-major; tmp is a second cube buffer
__device__ void cube_transform(double *cube, double *tmp, const double *M, int K) {
    int N2 = 2 * K, C = N2 * N2 * N2;
    for (int i = threadIdx.x; i < C; i += blockDim.x) {
        int X = i % N2, YZ = i / N2;
        const double *src = cube + YZ * N2;
        double s = 0.0;
        for (int k = 0; k < N2; k++) s += M[X * N2 + k] * src[k];
        tmp[i] = s;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < C; i += blockDim.x) {
        int X = i % N2, Y = (i / N2) % N2, Z = i / (N2 * N2);
        double s = 0.0;
        for (int k = 0; k < N2; k++) s += M[Y * N2 + k] * tmp[(Z * N2 + k) * N2 + X];
        cube[i] = s;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < C; i += blockDim.x) {
        int XY = i % (N2 * N2), Z = i / (N2 * N2);
        double s = 0.0;
        for (int k = 0; k < N2; k++) s += M[Z * N2 + k] * cube[k * N2 * N2 + XY];
        tmp[i] = s;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < C; i += blockDim.x) cube[i] = tmp[i];
    __syncthreads();
}

// per-dimension K x K map on each half of every dimension (children-wise map)
__device__ void cube_map_halves(double *cube, double *tmp, const double *A, int K) {
    int N2 = 2 * K, C = N2 * N2 * N2;
    for (int i = threadIdx.x; i < C; i += blockDim.x) {
        int X = i % N2, YZ = i / N2, hx = (X / K) * K, x = X % K;
        double s = 0.0;
        for (int k = 0; k < K; k++) s += A[x * K + k] * cube[YZ * N2 + hx + k];
        tmp[i] = s;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < C; i += blockDim.x) {
        int X = i % N2, Y = (i / N2) % N2, Z = i / (N2 * N2), hy = (Y / K) * K, y = Y % K;
        double s = 0.0;
        for (int k = 0; k < K; k++) s += A[y * K + k] * tmp[(Z * N2 + hy + k) * N2 + X];
        cube[i] = s;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < C; i += blockDim.x) {
        int XY = i % (N2 * N2), Z = i / (N2 * N2), hz = (Z / K) * K, z = Z % K;
        double s = 0.0;
        for (int k = 0; k < K; k++) s += A[z * K + k] * cube[(hz + k) * N2 * N2 + XY];
        tmp[i] = s;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < C; i += blockDim.x) cube[i] = tmp[i];
    __syncthreads();
}

__device__ void load_block(double *cube, const double *g, int K) {
    int n = 8 * K * K * K;
    for (int gi = threadIdx.x; gi < n; gi += blockDim.x) cube[cube_of_block(gi, K)] = g[gi];
    __syncthreads();
}

__device__ void store_block(double *g, const double *cube, int K) {
    int n = 8 * K * K * K;
    for (int gi = threadIdx.x; gi < n; gi += blockDim.x) g[gi] = cube[cube_of_block(gi, K)];
}

// 8 component norms of a block in global memory; deterministic fixed-order reduction
// the 8 component norms of a block: per thread strided sums of squares, a butterfly sum per warp,
// then the warps' sums in warp order (blockDim a multiple of 32; red holds 8 x warps doubles)
__device__ void block_norms(const double *g, double *cn, int K, double *red) {
    const int K3 = K * K * K, nt = blockDim.x, nw = nt >> 5, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int c = 0; c < 8; c++) {
        double s = 0.0;
        for (int i = threadIdx.x; i < K3; i += nt) {
            const double v = g[c * K3 + i];
            s += v * v;
        }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) red[c * nw + w] = s;
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        double s = 0.0;
        for (int i = 0; i < nw; i++) s += red[threadIdx.x * nw + i];
        cn[threadIdx.x] = sqrt(s);
    }
    __syncthreads();
}

__device__ void basis_eval(const DevBasis &b, double x, double *out) {
    int K = b.K;
    double p[KMAX];
    double t = 2.0 * x - 1.0;
    p[0] = 1.0;
    if (K > 1) p[1] = t;
    for (int j = 1; j + 1 < K; j++) p[j + 1] = ((2.0 * j + 1.0) * t * p[j] - j * p[j - 1]) / (j + 1.0);
    for (int j = 0; j < K; j++) p[j] *= sqrt(2.0 * j + 1.0);
    if (b.type == MW_BASIS_LEGENDRE) {
        for (int j = 0; j < K; j++) out[j] = p[j];
        return;
    }
    for (int j = 0; j < K; j++) {
        double s = 0.0;
        for (int i = 0; i < K; i++) s += b.legq[j * K + i] * p[i];
        out[j] = sqrt(b.qw[j]) * s;
    }
}

// ----------------------------------------------------------------- projection
__device__ double laguerre(int k, int a, double x) {
    if (k == 0) return 1.0;
    double l0 = 1.0, l1 = 1.0 + a - x;
    for (int j = 1; j < k; j++) {
        double l2 = ((2.0 * j + 1.0 + a - x) * l1 - (j + a) * l0) / (j + 1.0);
        l0 = l1;
        l1 = l2;
    }
    return l1;
}

__device__ double func_eval(const ProjFunc &f, double x, double y, double z) {
    if (f.kind == 0) {
        double v = 0.0;
        for (int t = 0; t < f.nterms; t++) {
            const mw_gterm &g = f.terms[t];
            double dx = x - g.pos[0], dy = y - g.pos[1], dz = z - g.pos[2];
            double e = g.alpha * (dx * dx + dy * dy + dz * dz);
            if (e > 700.0) continue;
            double p = g.coef;
            for (int i = 0; i < g.pw[0]; i++) p *= dx;
            for (int i = 0; i < g.pw[1]; i++) p *= dy;
            for (int i = 0; i < g.pw[2]; i++) p *= dz;
            v += p * exp(-e);
        }
        return v;
    }
    double q[3] = {x - f.origin[0], y - f.origin[1], z - f.origin[2]};
    double rr = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
    double rho = 2.0 * f.Z * rr / f.hn;
    double rad = f.hnorm * pow(rho, (double)f.hl) * laguerre(f.hn - f.hl - 1, 2 * f.hl + 1, rho) * exp(-0.5 * rho);
    double ang = 0.5 / sqrt(3.14159265358979323846);
    if (f.hl == 1) ang *= sqrt(3.0) * (rr > 0.0 ? q[f.hm] / rr : 0.0);
    return rad * ang;
}

__global__ void project_kernel(DevBasis b, ProjFunc f, const ProjTask *tasks, int n) {
    extern __shared__ double sm[];
    int K = b.K, N2 = 2 * K, C = N2 * N2 * N2;
    double *cube = sm, *tmp = sm + C, *red = sm + 2 * C;
    for (int t = blockIdx.x; t < n; t += gridDim.x) {
        ProjTask task = tasks[t];
        if (task.zero) {
            for (int i = threadIdx.x; i < C; i += blockDim.x) task.out[i] = 0.0;
            if (threadIdx.x < 8) task.cn[threadIdx.x] = 0.0;
            __syncthreads();
            continue;
        }
        double h = ldexp(1.0, -(task.n + 1));
        for (int i = threadIdx.x; i < C; i += blockDim.x) {
            int X = i % N2, Y = (i / N2) % N2, Z = i / (N2 * N2);
            double x = h * (2 * task.l[0] + X / K + b.qx[X % K]);
            double y = h * (2 * task.l[1] + Y / K + b.qx[Y % K]);
            double z = h * (2 * task.l[2] + Z / K + b.qx[Z % K]);
            cube[i] = func_eval(f, x, y, z);
        }
        __syncthreads();
        cube_map_halves(cube, tmp, b.v2c, K);
        double sc = pow(2.0, -1.5 * (task.n + 1));
        for (int i = threadIdx.x; i < C; i += blockDim.x) cube[i] *= sc;
        __syncthreads();
        cube_transform(cube, tmp, b.W, K);
        store_block(task.out, cube, K);
        __syncthreads();
        block_norms(task.out, task.cn, K, red);
    }
}

// ----------------------------------------------------------------- generated nodes
// Missing input nodes: a leaf's block reconstructed down a path of child steps
// to the requested node.  Each step keeps only the child's scaling part, so
// after the first step the block's wavelet parts are zero and the three passes
// contract over K instead of 2K.  The intermediates live in per-CTA scratch in
// global memory (L2-resident), so that the kernel needs no shared memory and
// fits on SMs beside the contraction CTAs: the host waits for it while
// preparing a level.  Every task writes the full block (wavelet parts zero)
// and its 8 component norms.
__global__ void __launch_bounds__(128) generate_kernel(DevBasis b, const GenTask *tasks, int n, double *scratch) {
    __shared__ double s_red[4];
    const int K = b.K, N2 = 2 * K, K3 = K * K * K, KK = K * K;
    const size_t per = (size_t)N2 * N2 * K + (size_t)N2 * K * K + K3;
    double *t1 = scratch + (size_t)blockIdx.x * per, *t2 = t1 + (size_t)N2 * N2 * K, *sc = t2 + (size_t)N2 * K * K;
    for (int t = blockIdx.x; t < n; t += gridDim.x) {
        const GenTask task = tasks[t];
        for (int s = 0; s < task.steps; s++) {
            const int c = (int)((task.path >> (3 * s)) & 7);
            const int bx = c & 1, by = (c >> 1) & 1, bz = (c >> 2) & 1;
            if (s == 0) {
                // from the ancestor's full block (component-major, components cx|cy<<1|cz<<2)
                for (int i = threadIdx.x; i < N2 * N2 * K; i += blockDim.x) {
                    const int x = i % K, YZ = i / K, Y = YZ % N2, Z = YZ / N2;
                    const int cyz = ((Y >= K) ? 2 : 0) | ((Z >= K) ? 4 : 0);
                    const double *row = task.anc + (Z % K) * KK + (Y % K) * K;
                    double acc = 0.0;
                    for (int X = 0; X < N2; X++)
                        acc += b.WT[(bx * K + x) * N2 + X] * row[(cyz | (X >= K ? 1 : 0)) * K3 + (X % K)];
                    t1[YZ * K + x] = acc;  // t1[Z][Y][x]
                }
                __syncthreads();
                for (int i = threadIdx.x; i < N2 * KK; i += blockDim.x) {
                    const int x = i % K, y = (i / K) % K, Z = i / KK;
                    double acc = 0.0;
                    for (int Y = 0; Y < N2; Y++) acc += b.WT[(by * K + y) * N2 + Y] * t1[(Z * N2 + Y) * K + x];
                    t2[i] = acc;  // t2[Z][y][x]
                }
                __syncthreads();
                for (int i = threadIdx.x; i < K3; i += blockDim.x) {
                    const int xy = i % KK, z = i / KK;
                    double acc = 0.0;
                    for (int Z = 0; Z < N2; Z++) acc += b.WT[(bz * K + z) * N2 + Z] * t2[Z * KK + xy];
                    sc[i] = acc;  // s[z][y][x]
                }
            } else {
                // from the previous step's scaling part (its wavelet parts are zero)
                for (int i = threadIdx.x; i < K3; i += blockDim.x) {
                    const int x = i % K, zy = i / K;
                    double acc = 0.0;
                    for (int X = 0; X < K; X++) acc += b.WT[(bx * K + x) * N2 + X] * sc[zy * K + X];
                    t1[i] = acc;  // t1[z][y][x']
                }
                __syncthreads();
                for (int i = threadIdx.x; i < K3; i += blockDim.x) {
                    const int x = i % K, y = (i / K) % K, z = i / KK;
                    double acc = 0.0;
                    for (int Y = 0; Y < K; Y++) acc += b.WT[(by * K + y) * N2 + Y] * t1[(z * K + Y) * K + x];
                    t2[i] = acc;  // t2[z][y'][x]
                }
                __syncthreads();
                for (int i = threadIdx.x; i < K3; i += blockDim.x) {
                    const int xy = i % KK, z = i / KK;
                    double acc = 0.0;
                    for (int Z = 0; Z < K; Z++) acc += b.WT[(bz * K + z) * N2 + Z] * t2[Z * KK + xy];
                    sc[i] = acc;  // s[z'][y][x]
                }
            }
            __syncthreads();
        }
        // the block: component 0 = s, components 1..7 = 0; norms likewise
        double ss = 0.0;
        for (int i = threadIdx.x; i < 8 * K3; i += blockDim.x) {
            const double v = i < K3 ? sc[i] : 0.0;
            task.out[i] = v;
            ss += v * v;
        }
        for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
        if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = ss;
        __syncthreads();
        if (threadIdx.x < 8) {
            double tot = 0.0;
            if (threadIdx.x == 0)
                for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += s_red[w];
            task.cn[threadIdx.x] = threadIdx.x == 0 ? sqrt(tot) : 0.0;
        }
        __syncthreads();
    }
}

// The same generation with K known at compile time: the filter matrix and the three
// intermediates in shared memory (56 KB at K = 10, four CTAs per SM), the loops unrolled.  The
// sums run in the same order as in generate_kernel, so the blocks and norms are identical.
template <int K>
__global__ void __launch_bounds__(256) generate_kernel_t(DevBasis b, const GenTask *tasks, int n) {
    constexpr int N2 = 2 * K, K3 = K * K * K, KK = K * K;
    extern __shared__ double gsm[];
    double *wt = gsm;                // W^T rows (c K + x) of length 2K, as b.WT
    double *t1 = wt + N2 * N2;       // t1[Z][Y][x] (first step) or t1[z][y][x']
    double *t2 = t1 + N2 * N2 * K;   // t2[Z][y][x] (first step) or t2[z][y'][x]
    double *sc = t2 + N2 * KK;       // s[z][y][x]
    __shared__ double s_red[8];
    for (int i = threadIdx.x; i < N2 * N2; i += blockDim.x) wt[i] = b.WT[i];
    __syncthreads();
    for (int t = blockIdx.x; t < n; t += gridDim.x) {
        const GenTask task = tasks[t];
        for (int s = 0; s < task.steps; s++) {
            const int c = (int)((task.path >> (3 * s)) & 7);
            const double *wx = wt + (c & 1) * K * N2, *wy = wt + ((c >> 1) & 1) * K * N2,
                         *wz = wt + ((c >> 2) & 1) * K * N2;
            if (s == 0) {
                for (int i = threadIdx.x; i < N2 * N2 * K; i += blockDim.x) {
                    const int x = i % K, YZ = i / K, Y = YZ % N2, Z = YZ / N2;
                    const int cyz = ((Y >= K) ? 2 : 0) | ((Z >= K) ? 4 : 0);
                    const double *row = task.anc + (Z % K) * KK + (Y % K) * K;
                    double acc = 0.0;
#pragma unroll
                    for (int X = 0; X < N2; X++) acc += wx[x * N2 + X] * row[(cyz | (X >= K ? 1 : 0)) * K3 + (X % K)];
                    t1[i] = acc;
                }
                __syncthreads();
                for (int i = threadIdx.x; i < N2 * KK; i += blockDim.x) {
                    const int x = i % K, y = (i / K) % K, Z = i / KK;
                    double acc = 0.0;
#pragma unroll
                    for (int Y = 0; Y < N2; Y++) acc += wy[y * N2 + Y] * t1[(Z * N2 + Y) * K + x];
                    t2[i] = acc;
                }
                __syncthreads();
                for (int i = threadIdx.x; i < K3; i += blockDim.x) {
                    const int xy = i % KK, z = i / KK;
                    double acc = 0.0;
#pragma unroll
                    for (int Z = 0; Z < N2; Z++) acc += wz[z * N2 + Z] * t2[Z * KK + xy];
                    sc[i] = acc;
                }
            } else {
                for (int i = threadIdx.x; i < K3; i += blockDim.x) {
                    const int x = i % K, zy = i / K;
                    double acc = 0.0;
#pragma unroll
                    for (int X = 0; X < K; X++) acc += wx[x * N2 + X] * sc[zy * K + X];
                    t1[i] = acc;
                }
                __syncthreads();
                for (int i = threadIdx.x; i < K3; i += blockDim.x) {
                    const int x = i % K, y = (i / K) % K, z = i / KK;
                    double acc = 0.0;
#pragma unroll
                    for (int Y = 0; Y < K; Y++) acc += wy[y * N2 + Y] * t1[(z * K + Y) * K + x];
                    t2[i] = acc;
                }
                __syncthreads();
                for (int i = threadIdx.x; i < K3; i += blockDim.x) {
                    const int xy = i % KK, z = i / KK;
                    double acc = 0.0;
#pragma unroll
                    for (int Z = 0; Z < K; Z++) acc += wz[z * N2 + Z] * t2[Z * KK + xy];
                    sc[i] = acc;
                }
            }
            __syncthreads();
        }
        double ss = 0.0;
        for (int i = threadIdx.x; i < 8 * K3; i += blockDim.x) {
            const double v = i < K3 ? sc[i] : 0.0;
            task.out[i] = v;
            ss += v * v;
        }
        for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
        if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = ss;
        __syncthreads();
        if (threadIdx.x < 8) {
            double tot = 0.0;
            if (threadIdx.x == 0)
                for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += s_red[w];
            task.cn[threadIdx.x] = threadIdx.x == 0 ? sqrt(tot) : 0.0;
        }
        __syncthreads();
    }
}

template <int K>
void launch_generate_t(const DevBasis &b, const GenTask *tasks, int n, int nsm, cudaStream_t s) {
    constexpr int N2 = 2 * K;
    constexpr size_t smem = sizeof(double) * ((size_t)N2 * N2 + (size_t)N2 * N2 * K + (size_t)N2 * K * K + (size_t)K * K * K);
    kernel_smem((const void *)generate_kernel_t<K>, (int)smem);
    const int grid = std::min(n, 4 * std::max(nsm, 1));
    generate_kernel_t<K><<<grid, 256, smem, s>>>(b, tasks, n);
    MWG_CUDA(cudaGetLastError());
}

// ----------------------------------------------------------------- NS-form apply
// One CTA per output node (persistent grid, dynamic node counter).  Thread
// (Yp, Xp) owns the output column cube[:, Yp, Xp] in registers.  Per item:
//   x pass  t1[Z][Y][X'] = sum_X Ax[X'][X] in[Z][Y][X]            (shared)
//   y pass  t2[Z]        = sum_Y Ay[Y'][Y] t1[Z][Y][X']           (registers)
//   z pass  acc[Z']     += c sum_Z Az[Z'][Z] t2[Z]
// Rows: consecutive items with the same Ay, Az (and so the same term and coefficient) add their
// x passes into t1 and u, and the row's last item runs the y and z passes once on the sums.
// Below the root scale the all-scaling path (f = 000 -> g = 000) is left out
// exactly: u holds the wavelet-in-x part of t1 on the scaling octant, and
// t2x the y pass that avoids the scaling-scaling path, used by g = 000.
template <typename T, int K>
__global__ void __launch_bounds__(((4 * K * K + 31) / 32) * 32) apply_kernel(ApplyLaunch L) {
    constexpr int N2 = 2 * K, NC = N2 * N2, C = NC * N2, K3 = K * K * K;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *s_in = reinterpret_cast<T *>(smem_raw);
    T *s_t1 = s_in + C;
    T *s_u = s_t1 + C;
    T *s_A = s_u + K3;
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
        T acc[N2];
#pragma unroll
        for (int z = 0; z < N2; z++) acc[z] = T(0);
        const long long b0 = L.begin[w], b1 = L.end[w];
        int nrows = 0;  // rows of this task
        for (long long j = b0; j < b1; j++) {
            const bool first = j == b0 || L.ay[j - 1] != L.ay[j] || L.az[j - 1] != L.az[j];
            const bool last = j + 1 == b1 || L.ay[j + 1] != L.ay[j] || L.az[j + 1] != L.az[j];
            __syncthreads();
            const T *gin = reinterpret_cast<const T *>(L.in[j]);
            for (int gi = tid; gi < 8 * K3; gi += blockDim.x) {
                int c = gi / K3, r = gi - c * K3;
                int iz = r / (K * K), iy = (r / K) % K, ix = r % K;
                int X = (c & 1) * K + ix, Y = ((c >> 1) & 1) * K + iy, Z = (c >> 2) * K + iz;
                s_in[(Z * N2 + Y) * N2 + X] = gin[gi];
            }
            const T *ax = reinterpret_cast<const T *>(L.ax[j]);
            const T *ay = reinterpret_cast<const T *>(L.ay[j]);
            const T *az = reinterpret_cast<const T *>(L.az[j]);
            for (int i = tid; i < NC; i += blockDim.x) {
                s_A[i] = ax[i];
                s_A[NC + i] = ay[i];
                s_A[2 * NC + i] = az[i];
            }
            const T cf = T(L.coef[j]);
            __syncthreads();
            if (active) {
                const T *arow = s_A + Xp * N2;
                T a[N2];
#pragma unroll
                for (int X = 0; X < N2; X++) a[X] = arow[X];
#pragma unroll 2
                for (int Z = 0; Z < N2; Z++) {
                    const T *src = s_in + (Z * N2 + Yp) * N2;
                    T s0 = T(0), s1 = T(0);
#pragma unroll
                    for (int X = 0; X < K; X++) s0 += a[X] * src[X];
#pragma unroll
                    for (int X = K; X < N2; X++) s1 += a[X] * src[X];
                    T *t1 = s_t1 + (Z * N2 + Yp) * N2 + Xp;  // this thread's own entries
                    *t1 = first ? s0 + s1 : *t1 + (s0 + s1);
                    if (excl && Z < K) {
                        T *u = s_u + (Z * K + Yp) * K + Xp;
                        *u = first ? s1 : *u + s1;
                    }
                }
            }
            if (!last) continue;
            nrows++;
            __syncthreads();
            if (active) {
                const T *arow = s_A + NC + Yp * N2;
                T t2[N2], t2x[K];
#pragma unroll
                for (int Z = 0; Z < N2; Z++) {
                    T s0 = T(0), s1 = T(0);
#pragma unroll
                    for (int Y = 0; Y < K; Y++) s0 += arow[Y] * s_t1[(Z * N2 + Y) * N2 + Xp];
#pragma unroll
                    for (int Y = K; Y < N2; Y++) s1 += arow[Y] * s_t1[(Z * N2 + Y) * N2 + Xp];
                    t2[Z] = s0 + s1;
                    if (Z < K) {
                        T su = T(0);
                        if (excl) {
#pragma unroll
                            for (int Y = 0; Y < K; Y++) su += arow[Y] * s_u[(Z * K + Y) * K + Xp];
                        }
                        t2x[Z] = su + s1;
                    }
                }
                const T *azm = s_A + 2 * NC;
#pragma unroll
                for (int Zp = 0; Zp < N2; Zp++) {
                    T s = T(0);
#pragma unroll
                    for (int Z = 0; Z < N2; Z++) {
                        T v = t2[Z];
                        if (Zp < K && Z < K) v = excl ? t2x[Z < K ? Z : 0] : v;
                        s += azm[Zp * N2 + Z] * v;
                    }
                    acc[Zp] += cf * s;
                }
            }
        }
        if (active) {
            double *out = L.out[w];
#pragma unroll
            for (int Zp = 0; Zp < N2; Zp++) {
                int c = (Xp >= K ? 1 : 0) | (Yp >= K ? 2 : 0) | (Zp >= K ? 4 : 0);
                int gi = c * K3 + (Zp % K) * K * K + (Yp % K) * K + (Xp % K);
                if (L.set)
                    out[gi] = double(acc[Zp]);
                else
                    out[gi] += double(acc[Zp]);
            }
        }
        __syncthreads();
        if (tid == 0 && nrows > 0 && L.rows) atomicAdd(L.rows, nrows);
        finish_chunk(L, w, 8 * K3, &s_redf);
    }
}

// N contiguous floats from shared memory, with the widest aligned vector loads
template <int N>
__device__ __forceinline__ void lds_row(float (&r)[N], const float *p) {
    if constexpr (N % 4 == 0) {
#pragma unroll
        for (int i = 0; i < N / 4; i++) {
            float4 v = reinterpret_cast<const float4 *>(p)[i];
            r[4 * i] = v.x;
            r[4 * i + 1] = v.y;
            r[4 * i + 2] = v.z;
            r[4 * i + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < N / 2; i++) {
            float2 v = reinterpret_cast<const float2 *>(p)[i];
            r[2 * i] = v.x;
            r[2 * i + 1] = v.y;
        }
    }
}

// FP32 tier of the NS-form apply.  Same contraction and exclusion as
// apply_kernel; each thread computes two outputs of every pass (indices i and
// i + K of one dimension), so that every row it reads from shared memory feeds
// twice the FMAs.  The x pass (thread (Y, X'), X' in [0, K)) reads rows of the
// input cube and stores t1 transposed as t1T[Z][X'][Y]; the y and z passes use
// (Y', X') with Y' in [0, K) fastest, so that the lanes of a warp read the same
// few rows of t1T, and hold their two A_y rows in registers; the node
// accumulator acc[Z'][X'][Y'] lives in shared memory (two CTAs per SM).  Each
// output's sums run in the same order as in the one-output form.  The FP32
// partial sum of the node is added once to its FP64 block.  Rows as in
// apply_kernel: a row's x passes add into t1T and u, its y and z passes run once.
template <int K>
__global__ void __launch_bounds__(((2 * K * K + 31) / 32) * 32, 2) apply32_kernel(ApplyLaunch L) {
    constexpr int N2 = 2 * K, NC = N2 * N2, C = NC * N2, K3 = K * K * K, U = ((K3 + 3) / 4) * 4;
    constexpr int NH = NC / 2;  // threads with work: (2K) x K
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *s_in = reinterpret_cast<float *>(smem_raw);
    float *s_t1 = s_in + C;   // t1T[Z][X'][Y]
    float *s_acc = s_t1 + C;  // node accumulator acc[Z'][X'][Y']
    float *s_u = s_acc + C;   // u[Z][X'][Y], Z, X', Y < K
    float *s_A = s_u + U;
    __shared__ int s_node, s_redf;
    const int tid = threadIdx.x;
    const bool active = tid < NH;
    // x pass: thread (Y = Yp, X' = Xh and Xh + K), Xh fastest
    const int Yp = tid / K, Xh = tid % K;
    const bool excl = !L.root && active && (Yp < K);  // u for X' = Xh (< K) on the scaling octant
    // y and z passes, epilogue: thread (Y' = Yh and Yh + K, X' = Xq), Yh fastest
    const int Xq = tid / K, Yh = tid % K;
    const bool exq = !L.root && active && (Xq < K);  // t2x for Y' = Yh (< K)

    while (true) {
        if (tid == 0) s_node = atomicAdd(L.counter, 1);
        __syncthreads();
        const int w = s_node;
        if (w >= L.nnodes) break;
        for (int i = tid; i < C; i += blockDim.x) s_acc[i] = 0.0f;
        const long long b0 = L.begin[w], b1 = L.end[w];
        int nrows = 0;  // rows of this task
        for (long long j = b0; j < b1; j++) {
            const bool first = j == b0 || L.ay[j - 1] != L.ay[j] || L.az[j - 1] != L.az[j];
            const bool last = j + 1 == b1 || L.ay[j + 1] != L.ay[j] || L.az[j + 1] != L.az[j];
            __syncthreads();
            // FP32 input blocks are stored in cube order: a straight 16-byte vector copy
            const float4 *gin4 = reinterpret_cast<const float4 *>(L.in[j]);
            float4 *sin4 = reinterpret_cast<float4 *>(s_in);
            for (int i = tid; i < C / 4; i += blockDim.x) sin4[i] = __ldg(gin4 + i);
            const float *ax = reinterpret_cast<const float *>(L.ax[j]);
            const float *ay = reinterpret_cast<const float *>(L.ay[j]);
            const float *az = reinterpret_cast<const float *>(L.az[j]);
            for (int i = tid; i < NC; i += blockDim.x) {
                s_A[i] = ax[i];
                s_A[NC + i] = ay[i];
                s_A[2 * NC + i] = az[i];
            }
            const float cf = float(L.coef[j]);
            __syncthreads();
            if (active) {  // x pass
                float a0[N2], a1[N2];
                lds_row<N2>(a0, s_A + Xh * N2);
                lds_row<N2>(a1, s_A + (Xh + K) * N2);
#pragma unroll 2
                for (int Z = 0; Z < N2; Z++) {
                    float row[N2];
                    lds_row<N2>(row, s_in + (Z * N2 + Yp) * N2);
                    float p0 = 0.0f, p1 = 0.0f, q0 = 0.0f, q1 = 0.0f;
#pragma unroll
                    for (int X = 0; X < K; X++) {
                        p0 = fmaf(a0[X], row[X], p0);
                        q0 = fmaf(a1[X], row[X], q0);
                    }
#pragma unroll
                    for (int X = K; X < N2; X++) {
                        p1 = fmaf(a0[X], row[X], p1);
                        q1 = fmaf(a1[X], row[X], q1);
                    }
                    float *t0 = s_t1 + (Z * N2 + Xh) * N2 + Yp, *t1 = s_t1 + (Z * N2 + Xh + K) * N2 + Yp;
                    *t0 = first ? p0 + p1 : *t0 + (p0 + p1);  // this thread's own entries
                    *t1 = first ? q0 + q1 : *t1 + (q0 + q1);
                    if (excl && Z < K) {
                        float *u = s_u + (Z * K + Xh) * K + Yp;
                        *u = first ? p1 : *u + p1;
                    }
                }
            }
            if (!last) continue;
            nrows++;
            __syncthreads();
            if (active) {  // y and z passes
                float ay0[N2], ay1[N2], t20[N2], t21[N2], t2x[K];
                lds_row<N2>(ay0, s_A + NC + Yh * N2);
                lds_row<N2>(ay1, s_A + NC + (Yh + K) * N2);
#pragma unroll
                for (int Z = 0; Z < N2; Z++) {
                    float row[N2];
                    lds_row<N2>(row, s_t1 + (Z * N2 + Xq) * N2);
                    float p0 = 0.0f, p1 = 0.0f, q0 = 0.0f, q1 = 0.0f;
#pragma unroll
                    for (int Y = 0; Y < K; Y++) {
                        p0 = fmaf(ay0[Y], row[Y], p0);
                        q0 = fmaf(ay1[Y], row[Y], q0);
                    }
#pragma unroll
                    for (int Y = K; Y < N2; Y++) {
                        p1 = fmaf(ay0[Y], row[Y], p1);
                        q1 = fmaf(ay1[Y], row[Y], q1);
                    }
                    t20[Z] = p0 + p1;
                    t21[Z] = q0 + q1;
                    if (Z < K) {
                        float su = 0.0f;
                        if (exq) {
                            const float *urow = s_u + (Z * K + Xq) * K;
#pragma unroll
                            for (int Y = 0; Y < K; Y++) su = fmaf(ay0[Y], urow[Y], su);
                        }
                        t2x[Z < K ? Z : 0] = su + p1;
                    }
                }
#pragma unroll
                for (int Zp = 0; Zp < N2; Zp++) {
                    float azr[N2];
                    lds_row<N2>(azr, s_A + 2 * NC + Zp * N2);
                    float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
                    for (int Z = 0; Z < N2; Z++) {
                        float v = t20[Z];
                        if (Zp < K && Z < K) v = exq ? t2x[Z < K ? Z : 0] : v;
                        s0 = fmaf(azr[Z], v, s0);
                        s1 = fmaf(azr[Z], t21[Z], s1);
                    }
                    float &a0_ = s_acc[(Zp * N2 + Xq) * N2 + Yh];
                    float &a1_ = s_acc[(Zp * N2 + Xq) * N2 + Yh + K];
                    a0_ = fmaf(cf, s0, a0_);
                    a1_ = fmaf(cf, s1, a1_);
                }
            }
        }
        __syncthreads();
        if (active) {
            double *out = L.out[w];
#pragma unroll 4
            for (int Zp = 0; Zp < N2; Zp++) {
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int Yq = Yh + h * K;
                    const int c = (Xq >= K ? 1 : 0) | (Yq >= K ? 2 : 0) | (Zp >= K ? 4 : 0);
                    const int gi = c * K3 + (Zp % K) * K * K + (Yq % K) * K + (Xq % K);
                    const double v = double(s_acc[(Zp * N2 + Xq) * N2 + Yq]);
                    if (L.set)
                        out[gi] = v;
                    else
                        out[gi] += v;
                }
            }
        }
        __syncthreads();
        if (tid == 0 && nrows > 0 && L.rows) atomicAdd(L.rows, nrows);
        finish_chunk(L, w, 8 * K3, &s_redf);
    }
}

template <typename T, int K>
void launch_apply_t(const ApplyLaunch &L, int nsm, cudaStream_t s) {
    constexpr int N2 = 2 * K, NC = N2 * N2, C = NC * N2, K3 = K * K * K;
    const bool f32 = sizeof(T) == 4;
    const int threads = f32 ? ((NC / 2 + 31) / 32) * 32 : ((NC + 31) / 32) * 32;
    const size_t smem = f32 ? sizeof(float) * (3 * C + ((K3 + 3) / 4) * 4 + 3 * NC) : sizeof(T) * (2 * C + K3 + 3 * NC);
    auto fn = f32 ? apply32_kernel<K> : apply_kernel<T, K>;
    kernel_smem((const void *)fn, (int)smem);
    int per_sm = kernel_ctas_per_sm((const void *)fn, threads, (int)smem);
    if (per_sm < 1) per_sm = 1;
    // one CTA per task (tasks are ordered longest first and taken in that order): CTAs end
    // throughout the launch, so kernels of other streams get SM slots without waiting for it
    (void)nsm;
    const int grid = L.nnodes;
    if (grid < 1) return;
    fn<<<grid, threads, smem, s>>>(L);
    MWG_CUDA(cudaGetLastError());
}

template <typename T>
void launch_apply_k(int K, const ApplyLaunch &L, int nsm, cudaStream_t s) {
    switch (K) {
        case 4: launch_apply_t<T, 4>(L, nsm, s); break;
        case 5: launch_apply_t<T, 5>(L, nsm, s); break;
        case 6: launch_apply_t<T, 6>(L, nsm, s); break;
        case 7: launch_apply_t<T, 7>(L, nsm, s); break;
        case 8: launch_apply_t<T, 8>(L, nsm, s); break;
        case 9: launch_apply_t<T, 9>(L, nsm, s); break;
        case 10: launch_apply_t<T, 10>(L, nsm, s); break;
        default: throw Error(MW_ERR_ARG, "no apply kernel for this order");
    }
}

// ----------------------------------------------------------------- post-processing
__global__ void norms_kernel(DevBasis b, double *const *blocks, double *const *cn, int n) {
    extern __shared__ double sm[];
    for (int t = blockIdx.x; t < n; t += gridDim.x) block_norms(blocks[t], cn[t], b.K, sm);
}

__global__ void topdown_kernel(DevBasis b, const PairTask *tasks, int n) {
    extern __shared__ double sm[];
    int K = b.K, N2 = 2 * K, C = N2 * N2 * N2, K3 = K * K * K;
    double *cube = sm, *tmp = sm + C;
    for (int t = blockIdx.x; t < n; t += gridDim.x) {
        PairTask task = tasks[t];
        load_block(cube, task.parent, K);
        cube_transform(cube, tmp, b.WT, K);
        // children's scaling parts += reconstruction; child c occupies octant c of the cube
        for (int gi = threadIdx.x; gi < 8 * K3; gi += blockDim.x) {
            int c = gi / K3, r = gi - c * K3;
            double *child = task.child0 + (size_t)c * 8 * K3;
            child[r] += cube[cube_of_block(gi, K)];
        }
        __syncthreads();
    }
}

__global__ void compress_kernel(DevBasis b, const PairTask *tasks, double *const *cn, int n) {
    extern __shared__ double sm[];
    int K = b.K, N2 = 2 * K, C = N2 * N2 * N2, K3 = K * K * K;
    double *cube = sm, *tmp = sm + C, *red = sm + 2 * C;
    for (int t = blockIdx.x; t < n; t += gridDim.x) {
        PairTask task = tasks[t];
        for (int gi = threadIdx.x; gi < 8 * K3; gi += blockDim.x) {
            int c = gi / K3, r = gi - c * K3;
            cube[cube_of_block(gi, K)] = task.child0[(size_t)c * 8 * K3 + r];
        }
        __syncthreads();
        cube_transform(cube, tmp, b.W, K);
        store_block(task.parent, cube, K);
        __syncthreads();
        block_norms(task.parent, cn[t], K, red);
    }
}

__global__ void add_kernel(DevBasis b, const AddTask *tasks, const double *const *src, const double *coefs, int n,
                           int bs) {
    extern __shared__ double sm[];
    for (int t = blockIdx.x; t < n; t += gridDim.x) {
        AddTask task = tasks[t];
        for (int i = threadIdx.x; i < bs; i += blockDim.x) {
            double s = 0.0;
            for (int k = 0; k < task.count; k++) s += coefs[task.first + k] * src[task.first + k][i];
            task.out[i] = s;
        }
        __syncthreads();
        block_norms(task.out, task.cn, b.K, sm);
    }
}

__global__ void to_fp32_kernel(const double *in, float *out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

// FP32 shadow of nblocks blocks, each written in cube order cube[Z][Y][X] as a high cube
// (the value rounded to FP32) followed by a low cube (the rounded remainder)
__global__ void to_fp32_cube_kernel(const double *in, float *out, size_t nblocks, int K) {
    const size_t bs = 8 * (size_t)K * K * K, n = nblocks * bs;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        size_t b = i / bs;
        int gi = (int)(i - b * bs);
        const double x = in[i];
        const float h = (float)x;
        float *o = out + 2 * b * bs + cube_of_block(gi, K);
        o[0] = h;
        o[bs] = (float)(x - (double)h);
    }
}

__global__ void scale_kernel(double *x, size_t n, double c) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        x[i] *= c;
}

__global__ void dot_kernel(const double *const *a, const double *const *bb, const int *start, int n, int bs,
                           double *partial) {
    extern __shared__ double sm[];
    for (int t = blockIdx.x; t < n; t += gridDim.x) {
        const double *x = a[t], *y = bb[t];
        double s = 0.0;
        for (int i = start[t] + threadIdx.x; i < bs; i += blockDim.x) s += x[i] * y[i];
        sm[threadIdx.x] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double tot = 0.0;
            for (int i = 0; i < (int)blockDim.x; i++) tot += sm[i];
            partial[t] = tot;
        }
        __syncthreads();
    }
}

// point evaluation: one CTA per point; blocks[p] is the leaf containing point p, keys[4p] its key
__global__ void eval_kernel(DevBasis b, const double *const *blocks, const int *keys, const double *pts, int npts,
                            double *out) {
    extern __shared__ double sm[];
    int K = b.K, N2 = 2 * K, C = N2 * N2 * N2, K3 = K * K * K;
    double *cube = sm, *tmp = sm + C, *red = sm + 2 * C;
    for (int p = blockIdx.x; p < npts; p += gridDim.x) {
        int n = keys[4 * p];
        load_block(cube, blocks[p], K);
        cube_transform(cube, tmp, b.WT, K);
        double h = ldexp(1.0, -(n + 1));
        int c = 0;
        double y[3];
        for (int d = 0; d < 3; d++) {
            double r = pts[3 * p + d];
            int cl = (int)floor(r / h);
            int lo = 2 * keys[4 * p + 1 + d];
            if (cl < lo) cl = lo;
            if (cl > lo + 1) cl = lo + 1;
            c |= (cl - lo) << d;
            y[d] = r / h - cl;
        }
        double ph[3][KMAX];
        for (int d = 0; d < 3; d++) basis_eval(b, y[d], ph[d]);
        double s = 0.0;
        for (int i = threadIdx.x; i < K3; i += blockDim.x) {
            int ix = i % K, iy = (i / K) % K, iz = i / (K * K);
            s += cube[cube_of_block(c * K3 + i, K)] * ph[0][ix] * ph[1][iy] * ph[2][iz];
        }
        red[threadIdx.x] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double tot = 0.0;
            for (int i = 0; i < (int)blockDim.x; i++) tot += red[i];
            out[p] = tot * pow(2.0, 1.5 * (n + 1));
        }
        __syncthreads();
    }
}

int grid_for(int n) { return n < 4096 ? (n > 0 ? n : 1) : 4096; }

size_t cube_bytes(int K) { return sizeof(double) * 8 * K * K * K; }

}  // namespace

void k_project(const DevBasis &b, const ProjFunc &f, const ProjTask *tasks, int n, cudaStream_t s) {
    if (n <= 0) return;
    size_t smem = 2 * cube_bytes(b.K) + 8 * 256 * sizeof(double);
    MWG_CUDA(cudaFuncSetAttribute(project_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    project_kernel<<<grid_for(n), 256, smem, s>>>(b, f, tasks, n);
    MWG_CUDA(cudaGetLastError());
}

void k_generate(const DevBasis &b, const GenTask *tasks, int n, double *scratch, int grid, int nsm, cudaStream_t s) {
    if (n <= 0) return;
    switch (b.K) {
        case 4: launch_generate_t<4>(b, tasks, n, nsm, s); return;
        case 5: launch_generate_t<5>(b, tasks, n, nsm, s); return;
        case 6: launch_generate_t<6>(b, tasks, n, nsm, s); return;
        case 7: launch_generate_t<7>(b, tasks, n, nsm, s); return;
        case 8: launch_generate_t<8>(b, tasks, n, nsm, s); return;
        case 9: launch_generate_t<9>(b, tasks, n, nsm, s); return;
        case 10: launch_generate_t<10>(b, tasks, n, nsm, s); return;
        default: break;
    }
    generate_kernel<<<grid, 128, 0, s>>>(b, tasks, n, scratch);
    MWG_CUDA(cudaGetLastError());
}

void k_apply(const DevBasis &b, const ApplyLaunch &L, int fp32, int nsm, cudaStream_t s) {
    if (L.nnodes <= 0) return;
    if (fp32)
        launch_apply_k<float>(b.K, L, nsm, s);
    else
        launch_apply_k<double>(b.K, L, nsm, s);
}

void k_norms(const DevBasis &b, double *const *blocks, double *const *cn, int n, cudaStream_t s) {
    if (n <= 0) return;
    norms_kernel<<<grid_for(n), 256, 8 * 256 * sizeof(double), s>>>(b, blocks, cn, n);
    MWG_CUDA(cudaGetLastError());
}

void k_topdown(const DevBasis &b, const PairTask *tasks, int n, cudaStream_t s) {
    if (n <= 0) return;
    size_t smem = 2 * cube_bytes(b.K);
    kernel_smem((const void *)topdown_kernel, (int)smem);
    topdown_kernel<<<grid_for(n), 256, smem, s>>>(b, tasks, n);
    MWG_CUDA(cudaGetLastError());
}

void k_compress(const DevBasis &b, const PairTask *tasks, double *const *cn, int n, cudaStream_t s) {
    if (n <= 0) return;
    size_t smem = 2 * cube_bytes(b.K) + 8 * 256 * sizeof(double);
    kernel_smem((const void *)compress_kernel, (int)smem);
    compress_kernel<<<grid_for(n), 256, smem, s>>>(b, tasks, cn, n);
    MWG_CUDA(cudaGetLastError());
}

// dst[off[r] .. off[r] + len[r]) = src[r][0 .. len[r]): one CTA per range
__global__ void gather_ranges_kernel(const double *const *src, const long long *off, const int *len, int n,
                                     double *dst) {
    for (int r = blockIdx.x; r < n; r += gridDim.x) {
        const double *s = src[r];
        double *d = dst + off[r];
        for (int i = threadIdx.x; i < len[r]; i += blockDim.x) d[i] = s[i];
    }
}

void k_gather_ranges(const double *const *src, const long long *off, const int *len, int n, double *dst,
                     cudaStream_t s) {
    if (n <= 0) return;
    gather_ranges_kernel<<<n < 4096 ? n : 4096, 128, 0, s>>>(src, off, len, n, dst);
    MWG_CUDA(cudaGetLastError());
}

void k_add(const DevBasis &b, const AddTask *tasks, const double *const *src, const double *coefs, int n, int bs,
           cudaStream_t s) {
    if (n <= 0) return;
    add_kernel<<<grid_for(n), 256, 8 * 256 * sizeof(double), s>>>(b, tasks, src, coefs, n, bs);
    MWG_CUDA(cudaGetLastError());
}

void k_to_fp32(const double *in, float *out, size_t n, cudaStream_t s) {
    if (n == 0) return;
    to_fp32_kernel<<<4096, 256, 0, s>>>(in, out, n);
    MWG_CUDA(cudaGetLastError());
}

void k_to_fp32_cube(const double *in, float *out, size_t nblocks, int K, cudaStream_t s) {
    if (nblocks == 0) return;
    to_fp32_cube_kernel<<<4096, 256, 0, s>>>(in, out, nblocks, K);
    MWG_CUDA(cudaGetLastError());
}

// dst block j = src block map[j] (blocks of bs doubles)
__global__ void permute_blocks_kernel(double *dst, const double *src, const int *map, int n, int bs) {
    for (int j = blockIdx.x; j < n; j += gridDim.x) {
        const double2 *s2 = reinterpret_cast<const double2 *>(src + (size_t)map[j] * bs);
        double2 *d2 = reinterpret_cast<double2 *>(dst + (size_t)j * bs);
        for (int i = threadIdx.x; i < bs / 2; i += blockDim.x) d2[i] = s2[i];
    }
}

// A pinned host buffer into device memory, read by the SMs over the host link: an upload of this
// kind never queues behind bulk copies on the copy engines (the input blocks of a host-buffer
// apply moving beside the first levels).  16-byte words where both ends are 16-byte aligned.
__global__ void fetch_kernel(char *dst, const char *src, size_t bytes, int vec) {
    const size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    size_t head = 0;
    if (vec) {
        const size_t n16 = bytes / 16;
        for (size_t i = tid; i < n16; i += stride) reinterpret_cast<uint4 *>(dst)[i] = reinterpret_cast<const uint4 *>(src)[i];
        head = n16 * 16;
    }
    for (size_t i = head + tid; i < bytes; i += stride) dst[i] = src[i];
}

void k_fetch(void *dst, const void *src_pinned, size_t bytes, cudaStream_t s) {
    if (bytes == 0) return;
    const int vec = ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src_pinned)) & 15) == 0;
    const size_t units = vec ? (bytes + 15) / 16 : bytes;
    const int blocks = (int)std::min<size_t>((units + 255) / 256, 1024);
    fetch_kernel<<<blocks, 256, 0, s>>>((char *)dst, (const char *)src_pinned, bytes, vec);
    MWG_CUDA(cudaGetLastError());
}

void k_permute_blocks(double *dst, const double *src, const int *map, int n, int bs, cudaStream_t s) {
    if (n <= 0) return;
    permute_blocks_kernel<<<std::min(n, 4096), 256, 0, s>>>(dst, src, map, n, bs);
    MWG_CUDA(cudaGetLastError());
}

void k_scale(double *x, size_t n, double c, cudaStream_t s) {
    if (n == 0) return;
    scale_kernel<<<4096, 256, 0, s>>>(x, n, c);
    MWG_CUDA(cudaGetLastError());
}

void k_dot(const double *const *a, const double *const *b, const int *start, int n, int bs, double *partial,
           cudaStream_t s) {
    if (n <= 0) return;
    dot_kernel<<<grid_for(n), 256, 256 * sizeof(double), s>>>(a, b, start, n, bs, partial);
    MWG_CUDA(cudaGetLastError());
}

void k_eval(const DevBasis &b, const double *const *blocks, const int *keys, const double *pts, int npts,
            double *out, cudaStream_t s) {
    if (npts <= 0) return;
    size_t smem = 2 * cube_bytes(b.K) + 256 * sizeof(double);
    MWG_CUDA(cudaFuncSetAttribute(eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    eval_kernel<<<grid_for(npts), 256, smem, s>>>(b, blocks, keys, pts, npts, out);
    MWG_CUDA(cudaGetLastError());
}

}  // namespace mwg

// ------------------------------------------------------------------ peak probe
namespace mwg {
namespace {
template <typename T>
__global__ void fma_probe_kernel(T *out, int iters, T seed) {
    T a0 = seed + threadIdx.x, a1 = a0 + T(1), a2 = a0 + T(2), a3 = a0 + T(3);
    T a4 = a0 + T(4), a5 = a0 + T(5), a6 = a0 + T(6), a7 = a0 + T(7);
    const T m = T(0.999999), c = T(1e-7);
    for (int i = 0; i < iters; i++) {
        a0 = a0 * m + c; a1 = a1 * m + c; a2 = a2 * m + c; a3 = a3 * m + c;
        a4 = a4 * m + c; a5 = a5 * m + c; a6 = a6 * m + c; a7 = a7 * m + c;
    }
    T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == T(-12345)) out[blockIdx.x] = s;  // never true; keeps the chain live
}
}  // namespace

namespace {
// register-only warp MMA chains: kind 0 = m16n8k8 TF32, kind 1 = m16n8k16 BF16 (FP32 accumulate)
__global__ void mma_probe_kernel(float *out, int iters, int kind) {
    uint32_t a[4], b[2];
    for (int i = 0; i < 4; i++) a[i] = 0x3c003c00u + threadIdx.x + i;
    for (int i = 0; i < 2; i++) b[i] = 0x3c003c00u + threadIdx.x * 3 + i;
    float c[4][4];
    for (int j = 0; j < 4; j++)
        for (int i = 0; i < 4; i++) c[j][i] = 0.0f;
    if (kind == 0) {
        for (int it = 0; it < iters; it++)
#pragma unroll
            for (int j = 0; j < 4; j++)
                asm volatile(
                    "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                    "{%0,%1,%2,%3};\n"
                    : "+f"(c[j][0]), "+f"(c[j][1]), "+f"(c[j][2]), "+f"(c[j][3])
                    : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
    } else {
        for (int it = 0; it < iters; it++)
#pragma unroll
            for (int j = 0; j < 4; j++)
                asm volatile(
                    "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                    "{%0,%1,%2,%3};\n"
                    : "+f"(c[j][0]), "+f"(c[j][1]), "+f"(c[j][2]), "+f"(c[j][3])
                    : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
    }
    float s = 0.0f;
    for (int j = 0; j < 4; j++)
        for (int i = 0; i < 4; i++) s += c[j][i];
    if (s == -12345.0f) out[blockIdx.x] = s;
}
}  // namespace

// Dense warp-MMA throughput (TFLOP/s, 2 flops per MAC) of the legacy mma.sync path.
double probe_mma_tflops(int kind, int nsm, cudaStream_t s) {
    if (kind == 2) return probe_tc05_tflops(256, nsm, s);
    if (kind == 3) return probe_tc05_tflops(32, nsm, s);
    const int threads = 256, blocks = nsm * 8, iters = 1 << 12;
    float *out = nullptr;
    MWG_CUDA(cudaMalloc(&out, sizeof(float) * blocks));
    cudaEvent_t e0, e1;
    MWG_CUDA(cudaEventCreate(&e0));
    MWG_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        MWG_CUDA(cudaEventRecord(e0, s));
        mma_probe_kernel<<<blocks, threads, 0, s>>>(out, iters, kind);
        MWG_CUDA(cudaGetLastError());
        MWG_CUDA(cudaEventRecord(e1, s));
        MWG_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        MWG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    const double macs_per_mma = kind == 0 ? 16.0 * 8 * 8 : 16.0 * 8 * 16;
    double flops = 2.0 * macs_per_mma * 4.0 * iters * (threads / 32.0) * blocks;
    return flops / (best * 1e-3) / 1e12;
}

double probe_fma_tflops(int fp64, int nsm, cudaStream_t s) {
    const int threads = 256, blocks = nsm * 8, iters = fp64 ? 1 << 13 : 1 << 16;
    void *out = nullptr;
    MWG_CUDA(cudaMalloc(&out, sizeof(double) * blocks));
    cudaEvent_t e0, e1;
    MWG_CUDA(cudaEventCreate(&e0));
    MWG_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        MWG_CUDA(cudaEventRecord(e0, s));
        if (fp64)
            fma_probe_kernel<double><<<blocks, threads, 0, s>>>((double *)out, iters, 1.0);
        else
            fma_probe_kernel<float><<<blocks, threads, 0, s>>>((float *)out, iters, 1.0f);
        MWG_CUDA(cudaGetLastError());
        MWG_CUDA(cudaEventRecord(e1, s));
        MWG_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        MWG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    double flops = 2.0 * 8.0 * iters * (double)threads * blocks;
    return flops / (best * 1e-3) / 1e12;
}
namespace {
std::mutex g_launch_mu;
std::map<std::pair<const void *, int>, int> g_smem_set;                    // (kernel, device) -> bytes
std::map<std::tuple<const void *, int, int, int>, int> g_ctas;               // (kernel, device, threads, bytes)
}  // namespace

void kernel_smem(const void *fn, int bytes) {
    int dev = 0;
    MWG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_launch_mu);
    int &have = g_smem_set[{fn, dev}];
    if (have >= bytes) return;
    MWG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    have = bytes;
}

int kernel_ctas_per_sm(const void *fn, int threads, int bytes) {
    int dev = 0;
    MWG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_launch_mu);
    auto key = std::make_tuple(fn, dev, threads, bytes);
    auto it = g_ctas.find(key);
    if (it != g_ctas.end()) return it->second;
    int per_sm = 0;
    MWG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, (size_t)bytes));
    g_ctas[key] = per_sm;
    return per_sm;
}

}  // namespace mwg
