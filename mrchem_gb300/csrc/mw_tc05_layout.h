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
//
// Where tc5_split_wide(K) holds, the split tier's operator blocks have a layout of their own with
// the same size: per k-group the group's N hi rows, then its N lo rows (k-group stride 2 N 16
// bytes), so that one MMA of width 2N takes B_hi and B_lo side by side (A_hi * B_hi in its first
// N columns, A_hi * B_lo in the others) and one of width N with the same descriptor reads B_hi
// alone.  Its TMEM tiles are then 2N columns wide; that is taken only at the orders where it
// leaves as many CTAs per SM as the three MMAs of width N do (at K = 8 the wide tiles need all
// 512 columns of an SM, where the narrow kernel fits two CTAs in shared memory and TMEM).
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
// the split tier's MMAs of width 2N on the interleaved operator layout (above)
MWG_HD constexpr bool tc5_split_wide(int K) { return K != 8; }
// per-block strides of the stored layouts: hi, then lo
MWG_HD constexpr size_t tc5_x_stride(int K) { return 2 * tc5_x_floats(K); }
MWG_HD constexpr size_t tc5_b_stride(int K) { return 2 * tc5_b_floats(K); }

}  // namespace mwg
