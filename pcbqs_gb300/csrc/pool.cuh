// Stream-ordered device memory for the solver's large, short-lived buffers.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

namespace pq {

// Allocates from one memory pool per device that keeps freed memory reserved (release threshold: unlimited), so
// the dense system blocks, factors and Krylov bases of repeated solves reuse it instead of paying cudaMalloc and
// cudaFree (page mapping, device-wide synchronization) every time. Ordered on `stream` like cudaMallocAsync.
cudaError_t pool_alloc(void **ptr, size_t bytes, cudaStream_t stream);

// Returns `ptr` to its pool, ordered on `stream`; null is ignored.
void pool_free(void *ptr, cudaStream_t stream);

// Gives the reserved but unused memory of the current device's pool back to the device.
cudaError_t pool_trim();

template <class T> cudaError_t pool_alloc_n(T **ptr, size_t count, cudaStream_t stream) {
    return pool_alloc(reinterpret_cast<void **>(ptr), (count ? count : 1) * sizeof(T), stream);
}

}  // namespace pq
