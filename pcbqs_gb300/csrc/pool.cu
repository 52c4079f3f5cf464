// One retained memory pool per device for the solver's buffers (pool.cuh).
#include <cstdint>
#include <mutex>

#include "pool.cuh"

namespace pq {

namespace {

constexpr int MAX_DEVICES = 64;
std::mutex g_pool_mutex;
cudaMemPool_t g_pools[MAX_DEVICES] = {};

cudaError_t pool_of_current(cudaMemPool_t *out) {
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return e;
    if (device < 0 || device >= MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    if (!g_pools[device]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        cudaMemPool_t pool = nullptr;
        if ((e = cudaMemPoolCreate(&pool, &props)) != cudaSuccess) return e;
        uint64_t keep = UINT64_MAX;
        if ((e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess) {
            cudaMemPoolDestroy(pool);
            return e;
        }
        g_pools[device] = pool;
    }
    *out = g_pools[device];
    return cudaSuccess;
}

}  // namespace

cudaError_t pool_alloc(void **ptr, size_t bytes, cudaStream_t stream) {
    *ptr = nullptr;
    cudaMemPool_t pool = nullptr;
    cudaError_t e = pool_of_current(&pool);
    if (e != cudaSuccess) return e;
    return cudaMallocFromPoolAsync(ptr, bytes, pool, stream);
}

void pool_free(void *ptr, cudaStream_t stream) {
    if (ptr) cudaFreeAsync(ptr, stream);
}

cudaError_t pool_trim() {
    cudaMemPool_t pool = nullptr;
    cudaError_t e = pool_of_current(&pool);
    if (e != cudaSuccess) return e;
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return e;
    return cudaMemPoolTrimTo(pool, 0);
}

}  // namespace pq

#include "../../include/pcbqs_gb300.h"
#include "common.cuh"

extern "C" int pcbqs_gb300_release_memory(int device) {
    int previous = 0;
    cudaGetDevice(&previous);
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = pq::pool_trim();
    cudaSetDevice(previous);
    if (e != cudaSuccess) return pq::fail(pq::ERR_CUDA, "release_memory: %s", cudaGetErrorString(e));
    return pq::OK;
}
