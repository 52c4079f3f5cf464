// Partial inductances of plated via segments (pcbqs_gb300_via_inductance): each segment a straight filament along z
// at (x, y) from z0 to z1 with radius r, the matrix of their mutual inductances by Grover's formula for parallel
// filaments, M = scale [g(z1a - z0b) + g(z0a - z1b) - g(z1a - z1b) - g(z0a - z0b)], g(u) = u asinh(u / s) -
// sqrt(u^2 + s^2), s the axis distance; segments of one barrel (coaxial) and the self terms take the larger radius,
// so stacked segments add up to the whole barrel. Restates src/pcbqs/mqs.py:40-45 (filament_mutual) and :140-153
// (via_inductance). One thread per entry, FP64.
#include <algorithm>
#include <cmath>

#include "../../include/pcbqs_gb300.h"
#include "common.cuh"

namespace pq {

namespace {

__device__ __forceinline__ double grover_g(double u, double s) { return u * asinh(u / s) - sqrt(u * u + s * s); }

__global__ void k_via_inductance(int64_t nv, const double *seg, double scale, double *L, int64_t ld) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nv * nv; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / nv, j = t % nv;
        const double *a = seg + 5 * i, *b = seg + 5 * j;
        double s = hypot(a[0] - b[0], a[1] - b[1]);
        if (s < 1e-9) s = fmax(a[2], b[2]);
        L[i * ld + j] = scale * (grover_g(a[4] - b[3], s) + grover_g(a[3] - b[4], s) - grover_g(a[4] - b[4], s) -
                                 grover_g(a[3] - b[3], s));
    }
}

}  // namespace

}  // namespace pq

extern "C" int pcbqs_gb300_via_inductance(int64_t nv, const double *seg, double scale, double *L, int64_t ld,
                                          void *stream) {
    if (nv < 0 || (nv && (!seg || !L)) || ld < nv || !(scale > 0))
        return pq::fail(pq::ERR_ARGUMENT, "via_inductance: invalid argument");
    if (nv == 0) return pq::OK;
    const int64_t total = nv * nv;
    const unsigned blocks = (unsigned)std::min<int64_t>((total + 255) / 256, 4096);
    pq::k_via_inductance<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(nv, seg, scale, L, ld);
    pq::note_launches(1);
    const cudaError_t e = cudaGetLastError();
    if (e) return pq::fail(pq::ERR_CUDA, "via_inductance: %s", cudaGetErrorString(e));
    return pq::OK;
}
