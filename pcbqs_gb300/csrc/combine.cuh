// Internal launch interface of the combine and potential kernels (combine.cu).
#pragma once
#include <algorithm>
#include "common.cuh"

namespace pq {

// RWG basis on device: tri (2, ne) support triangles T+ / T-, alpha (2, ne) = +-l/(2A), vertex (2, ne, 2) the
// free vertices, scale (ne).
struct EdgeBasis {
    int64_t ne;
    const int32_t *tri;
    const double *alpha, *vertex, *scale;
};

struct MomentPlanes {
    const double *m0, *mx, *my, *mrr;
    int64_t ld;
};

// Mixed precision: FP32 basis with the supports' offsets off (2, ne, 2) = centroid - free vertex, and FP32 local
// moment planes.
struct EdgeBasisF {
    int64_t ne;
    const int32_t *tri;
    const float *alpha, *off, *scale;
};

struct MomentPlanesF {
    const float *m0, *mx, *my, *mrr;
    int64_t ld;
};

// Charge nodes: members of node a are members[start[a] .. start[a+1]), area[a] their summed area.
struct NodeGroups {
    int64_t nn;
    const int64_t *start;
    const int32_t *members;
    const double *area;
};

cudaError_t launch_edge_inductance(const EdgeBasis &e, const MomentPlanes &mo, double factor, double *L,
                                   int64_t ldl, cudaStream_t stream);
cudaError_t launch_potential(const NodeGroups &ng, const double *m0, int64_t ldm, double factor, double *P,
                             int64_t ldp, cudaStream_t stream);
cudaError_t launch_potential_single(const NodeGroups &ng, const float *m0, int64_t ldm, double factor, double *P,
                                    float *Pf, int64_t ldp, cudaStream_t stream);
cudaError_t launch_edge_inductance_local(const EdgeBasisF &e, const MomentPlanesF &mo, float factor, double *L,
                                         int64_t ldl, float *Lf, int64_t ldlf, cudaStream_t stream);

}  // namespace pq
