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

}  // namespace pq
