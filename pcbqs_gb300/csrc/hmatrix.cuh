// The compressed product Y = H X of an H-matrix packed by pcbqs_gb300.hmatrix.DeviceHMatrix (hmatrix.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace pq {

// X, Y: (n, k) complex128 row-major; slots: nslots x k complex128 scratch (the packing's slot count). Each block
// writes its contributions into its slots, then every row sums its slots in block order (deterministic).
cudaError_t hmatrix_apply(int64_t n, int64_t nb, const int64_t *meta, const int64_t *slot0, const int64_t *idx,
                          const double *store, const int64_t *row_ptr, const int64_t *slots_of_row, int max_rank,
                          int k, const double *x, double *y, double *slots, cudaStream_t st);

// The two passes of hmatrix_apply: the blocks' contributions into their slots (nb blocks of `meta`), and the rows'
// sums of their slots in block order.
cudaError_t hmatrix_blocks(int64_t nb, const int64_t *meta, const int64_t *slot0, const int64_t *idx,
                           const double *store, int max_rank, int k, const double *x, double *slots, cudaStream_t st);
cudaError_t hmatrix_rows(int64_t n, const int64_t *row_ptr, const int64_t *slots_of_row, int k, const double *slots,
                         double *y, cudaStream_t st);

}  // namespace pq
