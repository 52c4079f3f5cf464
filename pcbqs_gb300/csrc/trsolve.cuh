// Triangular solves with a complex64 LU factor (cuSOLVER getrf layout). For a few right-hand sides one persistent
// cooperative kernel per 8 columns streams the factor once, with grid barriers between its dependent steps; for many,
// a blocked solve runs its off-diagonal products on the tcgen05 complex update (the factor read once for all
// columns). Which one a column count uses is timed once (per device, size and count) and remembered.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>

#include "solve.cuh"

namespace pq {

// The factor M = P L U of M = A^T (A the row-major system; M is its column-major view), as cuSOLVER getrf leaves
// it, prepared for solving A x = b = U^T L^T P^T x: the diagonal TRI_BLOCK x TRI_BLOCK blocks of U^T (lower) and
// L^T (unit upper) inverted once, and the row interchanges turned into one gather.
constexpr int TRI_BLOCK = 128;     // super-block of rows solved at once
constexpr int TRI_COLS = 8;        // right-hand sides per sweep over the factor
constexpr int TRI_PANEL = 1024;    // rows per step of the blocked solve

struct TriSolver {
    int64_t n = 0;
    int nblk = 0;
    const float2 *lu = nullptr;    // n x n, column-major (not owned)
    float2 *inv_lower = nullptr;   // nblk blocks of TRI_BLOCK^2, row-major inverses of U^T's diagonal blocks
    float2 *inv_upper = nullptr;   // the same for L^T
    int32_t *gather = nullptr;     // x[j] = z[gather[j]]
    // per right-hand-side count: work arrays, partial sums and the barrier words
    struct Plan {
        int kpad = 0;
        float2 *b = nullptr, *y = nullptr, *z = nullptr, *partial = nullptr;
        unsigned *sync = nullptr;     // barrier, solved quarters per sweep, status, panel items per step (padded)
        int method = -1;              // -1 not yet timed, 0 streaming sweeps, 1 blocked with tcgen05 updates
        void *planes = nullptr;       // the blocked solve's BF16 operand planes
        int *update_error = nullptr;  // its updates' timeout flag
    };
    std::map<int, Plan> plans;
    // The blocked solve's factor panels (TRI_PANEL columns of T = the row-major view of lu, all n rows each) as
    // BF16 part planes of `update_terms` products, packed at its first use and kept with the factor.
    int update_terms = 6;
    void *panel_planes = nullptr;
    std::map<int, int> method_by_bucket;     // the timed choice per power-of-two column bucket
    int grid = 0;                     // co-resident thread blocks of the sweep kernel

    // ipiv: the factor's 1-based pivots on the device (getrf output); synchronizes `s`.
    cudaError_t prepare(const float2 *lu, int64_t n, const int *ipiv, cudaStream_t s);
    // out (n, k) complex128 row-major = A^-1 in, both device arrays. deferred: no read-back of the barriers' status
    // (and no host synchronization), so the call can be captured into a graph; read_status checks it afterwards.
    // The first call with a column count (not deferred) times both methods and keeps the faster.
    cudaError_t solve(int k, const cd *in, cd *out, cudaStream_t s, bool deferred = false);
    // The method chosen for k columns (0 streaming, 1 blocked, -1 not chosen yet). `force` 0 or 1 makes every call
    // use that method (validation), without timing or remembering anything.
    int method_for(int k) const;
    int force = -1;
    // cudaErrorLaunchTimeout if a bounded wait of a deferred solve with k columns gave up; synchronizes `s`.
    cudaError_t read_status(int k, cudaStream_t s);
    void release();
    ~TriSolver() { release(); }

  private:
    cudaError_t plan_for(int k, Plan **out);
    cudaError_t solve_streaming(Plan *p, int k, const cd *in, cd *out, cudaStream_t s, bool deferred);
    cudaError_t solve_blocked(Plan *p, int k, const cd *in, cd *out, cudaStream_t s);
};

}  // namespace pq
