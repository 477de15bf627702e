// mw_tc05_layout.h -- operand layouts of the tcgen05 TF32 tier (mw_apply_tc05.cu), shared by the
// host code that prepares them once per input tree and per operator.
//
// Both layouts are the canonical K-major shared-memory layout of tcgen05.mma without swizzling,
// stored contiguously in global memory so that one bulk copy lands them in shared memory ready
// for the MMAs: k-groups of 4 columns, group g after g groups of R rows x 16 bytes, row r of a
// group at byte 16 r.  Values are rounded to TF32 (round to nearest, ties away from zero).
//
//   input block (A of the x pass): rows r = Z * 2K + Y, k = X, element IN[Z][Y][X];
//                                  KG = ceil(2K / 4) groups of (2K)^2 rows
//   operator block (B of a pass):  rows n = output index, k = input index, element A[n][k];
//                                  rows 2K .. 3K-1 repeat rows 0 .. K-1 with the columns k < K
//                                  zeroed (the wavelet-in-x part the x pass needs); 2 KS groups
//                                  of N rows, the groups and rows past the data zero
//
// Every block is stored twice in a row: the value rounded to TF32 (hi), then the rounded
// remainder, value - hi, rounded to TF32 (lo).  The TF32 tier reads hi only; the split-TF32 tier
// (hi * hi + hi * lo + lo * hi on the tensor cores, the FP32-accuracy tier) reads both, lo at a
// fixed offset from hi.  Blocks are tc5_x_stride / tc5_b_stride floats apart.
#pragma once

#include <cstddef>

#if defined(__CUDACC__)
#define MWG_HD __host__ __device__
#else
#define MWG_HD
#endif

namespace mwg {

MWG_HD constexpr int tc5_n(int K) { return 3 * K <= 16 ? 16 : 32; }     // MMA N
MWG_HD constexpr int tc5_kg(int K) { return (2 * K + 3) / 4; }          // k-groups holding data
MWG_HD constexpr int tc5_ks(int K) { return (tc5_kg(K) + 1) / 2; }      // MMA k-steps of 8
MWG_HD constexpr size_t tc5_x_floats(int K) { return (size_t)tc5_kg(K) * 4 * (size_t)(2 * K) * (size_t)(2 * K); }
MWG_HD constexpr size_t tc5_b_floats(int K) { return (size_t)2 * tc5_ks(K) * tc5_n(K) * 4; }
// per-block strides of the stored layouts: hi, then lo
MWG_HD constexpr size_t tc5_x_stride(int K) { return 2 * tc5_x_floats(K); }
MWG_HD constexpr size_t tc5_b_stride(int K) { return 2 * tc5_b_floats(K); }

}  // namespace mwg
