// Internal launch interface of the fill kernels (fill.cu), used by the C ABI (capi.cu).
#pragma once
#include <algorithm>
#include "common.cuh"

namespace pq {

// Output moment planes M0, Mx, My, Mrr (row-major, leading dimension ld >= nt). scalar: M0 only.
template <class T> struct Planes {
    T *m0, *mx, *my, *mrr;
    int64_t ld;
    int scalar;
};
using FillPlanes = Planes<double>;

struct FillRule {
    double near;     // analytic when distance <= near * (r_p + r_q)
    int all_near;    // near = infinity: every pair analytic
    int outer;       // refinement level of pairs within the radii sum (0, 1 or 2)
    unsigned long long wait;   // limit (SM clocks) of the waits for a tile's geometry copies
};

// Compacted near pairs, one list per level slot (0: level 0, 1: level `outer`), and their counts.
struct NearLists {
    int2 *pair[2];
    unsigned long long *count;      // [2] device counters
    unsigned long long capacity;    // entries per list
};

cudaError_t launch_pairs(const Geometry &g, const int32_t *p, const int32_t *q, const double *d,
                         const int32_t *kind, int64_t n, int scalar, double *out, unsigned long long *count8,
                         int64_t *order, int *nonfinite, int *invalid, cudaStream_t stream);
cudaError_t launch_fill(const Geometry &g, const FillPlanes &out, const FillRule &rule, const NearLists &lists,
                        int *nonfinite, int *status, cudaStream_t stream);
cudaError_t launch_fill_near(const Geometry &g, const FillPlanes &out, const FillRule &rule, const NearLists &lists,
                             int *nonfinite, cudaStream_t stream);
// Mixed precision: FP32 planes of moments about each triangle's centroid (far pairs in FP32, near pairs FP64).
cudaError_t launch_fill_local(const Geometry &g, const Planes<float> &out, const FillRule &rule,
                              const NearLists &lists, int *nonfinite, int *status, cudaStream_t stream);
cudaError_t launch_fill_near_local(const Geometry &g, const Planes<float> &out, const FillRule &rule,
                                   const NearLists &lists, int *nonfinite, cudaStream_t stream);
size_t fill_smem_bytes();

}  // namespace pq
