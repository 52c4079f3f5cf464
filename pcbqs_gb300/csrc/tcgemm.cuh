// The trailing update of the blocked complex64 LU on the tensor cores: C -= A B with FP32 complex operands split into
// BF16 parts and multiplied by a hand-written tcgen05 GEMM (TMA-fed shared memory, accumulators in tensor memory).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace pq {

// Scratch of one trailing update (the BF16 operand planes), sized by tc_update_scratch_bytes.
size_t tc_update_scratch_bytes(int64_t rows, int64_t cols, int k, int terms);

// C (rows x cols) -= A (rows x k) B (k x cols); all complex64 column-major with leading dimensions lda, ldb, ldc.
// Each FP32 value is split into BF16 parts x = h + m + l; `terms` = 3 multiplies h·h + h·m + m·h (relative error of
// a product about 2^-16), 6 adds h·l + m·m + l·h (about 2^-24, FP32's own level). The complex product runs as one
// real GEMM of inner dimension terms · 2k: A's rows [re | im] against B's columns [re; -im] (real part) and [im; re]
// (imaginary part). `scratch` holds tc_update_scratch_bytes; `a_packed` reuses the A planes packed by an
// earlier call with the same A (the LU packs its panel once per step for two updates). `error` (device int)
// receives ERR_TIMEOUT when a bounded wait of the GEMM gives up (limit `wait_cycles` SM clocks). Ordered on `stream`.
cudaError_t tc_update_c64(int64_t rows, int64_t cols, int k, const float2 *A, int64_t lda, const float2 *B,
                          int64_t ldb, float2 *C, int64_t ldc, int terms, void *scratch, bool a_packed,
                          int *error, unsigned long long wait_cycles, cudaStream_t stream);

// The same update with row-major operands and A packed once for many updates (the triangular solves' products with
// a fixed factor): C (rows x cols, row-major complex64, leading dimension ldc) -= A B, A's plane (rows x k, packed
// by tc_pack_rows_c64 from a row-major complex64 A with leading dimension lda, into tc_rows_plane_bytes; a plane of
// more rows may be used from any row on, its rows being tc_rows_row_bytes(k, terms) bytes apart) and B
// (k x cols, row-major complex64, leading dimension ldb) packed into `scratch` (tc_rows_scratch_bytes) per call.
size_t tc_rows_plane_bytes(int64_t rows, int k, int terms);
size_t tc_rows_row_bytes(int k, int terms);
size_t tc_rows_scratch_bytes(int64_t cols, int k, int terms);
cudaError_t tc_pack_rows_c64(int64_t rows, int k, const float2 *A, int64_t lda, int terms, void *plane,
                             cudaStream_t stream);
cudaError_t tc_update_rows_c64(int64_t rows, int64_t cols, int k, const void *aplane, const float2 *B, int64_t ldb,
                               float2 *C, int64_t ldc, int terms, void *scratch, int *error,
                               unsigned long long wait_cycles, cudaStream_t stream);

// The dense product over many right-hand sides on the same GEMM: Y (rows x cols complex128) = M (rows x kdim, real)
// X (kdim x cols complex128), X and Y row-major with leading dimensions ldx, ldy (in complex elements). M is
// packed once into its BF16 part plane (tc_pack_real into tc_real_plane_bytes) and reused by every product; each
// product packs X (rounded to FP32) into `scratch` (tc_real_scratch_bytes) and runs one real GEMM of inner
// dimension terms · kdim against X's real and imaginary columns side by side, writing Y whole. The result carries
// the relative error of the parts kept (terms 3: about 2^-16; 6: FP32's). `error`, `wait_cycles` and `stream` as in
// tc_update_c64.
size_t tc_real_plane_bytes(int64_t rows, int64_t kdim, int terms);
size_t tc_real_scratch_bytes(int64_t kdim, int64_t cols, int terms);
cudaError_t tc_pack_real(int64_t rows, int64_t kdim, const float *M, int64_t ldm, int terms, void *plane,
                         cudaStream_t stream);
cudaError_t tc_real_product(int64_t rows, int64_t kdim, const void *plane, int64_t cols, const double2 *X,
                            int64_t ldx, double2 *Y, int64_t ldy, int terms, void *scratch, int *error,
                            unsigned long long wait_cycles, cudaStream_t stream);

// The same product to FP64's accuracy from a real FP64 M and complex128 X: every row of M and every real column of X
// is cut into `slices` (2..7) integer slices of 8 bits under its own power-of-two scale, so each slice is exact in
// BF16 and every slice product sums exactly in FP32 over the tensor core's 256-long chunks; the levels of slice
// pairs are carried into Y in FP64. The truncation error is about 2^(-8 slices) of max_t |M[r, t]| times
// sum_t |X[t, c]| (slices 6: about 2^-48). M's plane (tc_slice_exact into tc_exact_plane_bytes) holds its slices and
// row exponents; `scratch` (tc_exact_scratch_bytes) X's. Non-finite entries make their rows or columns of Y
// non-finite.
size_t tc_exact_plane_bytes(int64_t rows, int64_t kdim, int slices);
size_t tc_exact_scratch_bytes(int64_t kdim, int64_t cols, int slices);
cudaError_t tc_slice_exact(int64_t rows, int64_t kdim, const double *M, int64_t ldm, int slices, void *plane,
                           cudaStream_t stream);
cudaError_t tc_exact_product(int64_t rows, int64_t kdim, const void *plane, int64_t cols, const double2 *X,
                             int64_t ldx, double2 *Y, int64_t ldy, int slices, void *scratch, int *error,
                             unsigned long long wait_cycles, cudaStream_t stream);

}  // namespace pq
