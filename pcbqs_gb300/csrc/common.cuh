// Shared device-side definitions for the pcbqs GB300 static-fill and solve backend.
#pragma once
#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>

namespace pq {

// Status codes returned through the C ABI (include/pcbqs_gb300.h).
enum Status : int {
    OK = 0,
    ERR_ARGUMENT = 1,      // invalid argument (index out of range, bad size, null pointer)
    ERR_CUDA = 2,          // a CUDA runtime call failed
    ERR_NONFINITE = 3,     // a computed moment/entry was not finite
    ERR_MEMORY = 4,        // device allocation failed
    ERR_CONVERGENCE = 5,   // an iterative solve did not reach its tolerance
    ERR_TIMEOUT = 6,       // a bounded device wait gave up
};

// Record an error message for pcbqs_gb300_last_error() and return `code`.
int fail(int code, const char *fmt, ...);

// Count kernels launched by this library (reported by pcbqs_gb300_kernel_launches()).
void note_launches(long long count);

// Limit, in SM clocks, of the library's bounded device waits on the progress of other threads, blocks or copies
// (pcbqs_gb300_set_wait_cycles; DEFAULT_WAIT_CYCLES, about a second at 2 GHz, unless set).
constexpr unsigned long long DEFAULT_WAIT_CYCLES = 1ull << 31;
unsigned long long wait_cycles();
// Limit of the waits for a block's own asynchronous copies or products before it exits after giving up (these
// complete by themselves; about four seconds).
constexpr unsigned long long DRAIN_WAIT_CYCLES = 1ull << 33;

// Per-triangle records in HBM. One record per triangle, 16-byte aligned so a tile of consecutive triangles is
// one contiguous run that a bulk (TMA) copy can stage into shared memory.
//   FarRec   64 B: the three-point rule's points (x0,y0,x1,y1,x2,y2), area, z
//   ClsRec   32 B: centroid (cx, cy), bounding radius, z
//   SrcRec  192 B: vertices (6), edge tangents (6), outward normals (6), edge lengths (3), area, pad (2)
struct alignas(64) FarRec { double p[6]; double area; double z; };
struct alignas(32) ClsRec { double cx, cy, radius, z; };
struct alignas(64) SrcRec { double v[6]; double tau[6]; double un[6]; double len[3]; double area; double pad[2]; };
//   LocalRec 48 B (mixed precision): the centroid split in two floats (chi + clo), the three rule points as float
//   offsets from the centroid, area and z as floats.
struct alignas(16) LocalRec { float chi[2]; float clo[2]; float u[6]; float area; float z; };

// Device geometry of one mesh. Observation rules: obs[k] (nt, nq[k], 2) points, w[k] (nq[k]) weights.
struct Geometry {
    int nt;
    const FarRec *far;
    const ClsRec *cls;
    const SrcRec *src;
    const LocalRec *local;
    const double *obs[3];
    const double *w[3];
    int nq[3];
};

// FillEngine's near/far rule with every product rounded (no FMA contraction), so the quadrature choice is
// bit-identical to the reference's host rule: distance = sqrt((dx*dx + dy*dy) + d*d), size = r_p + r_q,
// far (-1) unless distance <= near*size (or all_near), level `outer` if distance <= size, else 0.
// Follows src/pcbqs/core/static_kernels.hpp:130-136 and src/pcbqs/static_backends.py:288-298.
__device__ __forceinline__ int classify(const ClsRec &a, const ClsRec &b, double d, double near, int all_near,
                                        int outer) {
    const double dx = __dsub_rn(a.cx, b.cx), dy = __dsub_rn(a.cy, b.cy);
    const double distance = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(d, d)));
    const double size = __dadd_rn(a.radius, b.radius);
    if (!all_near && !(distance <= __dmul_rn(near, size))) return -1;
    return distance <= size ? outer : 0;
}

}  // namespace pq
