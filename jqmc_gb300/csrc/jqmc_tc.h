// Tensor-core (tcgen05) kernels of libjqmc_gpu: the exact-sum split GEMM of the
// mixed-precision table rebuild.  Internal to the library (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace jqmc_tc {

// Tile shape of the split GEMM: 128 rows (electrons) x 64 columns (AOs) per CTA,
// K (AOs) staged 32 at a time, six 8-bit slices per operand.
constexpr int kBM = 128, kBN = 64, kKC = 32, kSlices = 6, kStages = 3;
constexpr int kASliceBytes = kBM * kKC * 2;        // one slice of an A stage (bf16)
constexpr int kBSliceBytes = kBN * kKC * 2;
constexpr int kAStage = kSlices * kASliceBytes;    // 48 KiB
constexpr int kBStage = kSlices * kBSliceBytes;    // 24 KiB
constexpr int kMaxK = 768;                         // K <= 768: level 0 and levels 1, 2 by ranges exact
constexpr int kSmemBytes = kStages * (kAStage + kBStage) + 256;

// Byte offset of element (row, k) inside one slice block of `rows` x kKC bf16 in
// the tcgen05 canonical K-major layout without swizzle: 8 x 8 core matrices of
// 128 contiguous bytes, K-adjacent cores 128 B apart, 8-row groups 512 B apart.
__host__ __device__ inline int canon_offset(int row, int k) {
  return (row >> 3) * 512 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// The split of x (|x| < 1) into kSlices slices q_s = 2^-8s k_s with integers
// k_s in [-128, 128] and x = 2^-7 (q_0 + q_1 + q_2 + ...) up to 2^-48.  Each
// slice is exact in bf16 (8 significant bits, the exponent carries 2^-8s), so
// a product of slices s and t carries its level's scale 2^-8(s+t) and the
// levels merged into one accumulator add up correctly.
__host__ __device__ inline void split8(double x, float* q) {
  double y = x * 128.0;
  for (int s = 0; s < kSlices; ++s) {
    const double r = rint(y);
    q[s] = (float)ldexp(r, -8 * s);
    y = (y - r) * 256.0;
  }
}

// M[r][b] = sum_k Phi[r][k] L[k][b] for the rows of one chunk of one spin from
// the sliced operands:
//   a_slices  [row tile][k chunk][slice][kBM x kKC canonical]   (bf16 bits)
//   b_slices  [col tile][k chunk][slice][kBN x kKC canonical]
//   row_exp   per chunk row r: Phi[r][:] = 2^row_exp[r] * (|x| < 1)
//   col_exp   per column b: L[:][b] = 2^col_exp[b] * (|x| < 1)
// Output as float-float pairs (hi, lo) at out[((w * 2 + slot) * n + i) * ncols + b]
// for global row g = row0 + r, w = g / n, i = g % n, b < ncols; rows g >= rows_total
// are skipped.  On a wait that runs out (about 2 s) the tile's outputs are NaN and
// the walkers' status words get the bit `fail_bit`.  Returns 0, or a negative
// code for bad sizes (-1) or a failed launch (-3).
int ozaki_gemm(const uint16_t* a_slices, const uint16_t* b_slices, const int* row_exp, const int* col_exp, int nk_chunks,
               int n_col_tiles, int row_tiles, long long row0, long long rows_total, int n, int ncols, int slot,
               float2* out, int* status, int fail_bit, cudaStream_t stream);

}  // namespace jqmc_tc
