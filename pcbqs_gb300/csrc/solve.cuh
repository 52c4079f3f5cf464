// Batched GMRES (complex128) and the operators it runs on: internal interface (gmres.cu, peec_op.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

namespace pq {

// Vectors of k systems are stored (n, k) row-major as double2 (re, im): entry (r, s) at r * k + s.
using cd = double2;

// An operator applied to k systems at once: out = A_s in for each column s. `sys` gives each column's system
// (frequency) index, so one batch may hold several frequencies.
struct Operator {
    virtual ~Operator() = default;
    virtual int64_t n() const = 0;
    virtual cudaError_t apply(int k, const int32_t *sys, const cd *in, cd *out, cudaStream_t s) = 0;
};

// A right preconditioner: out = M_s^-1 in (out may not alias in).
struct Preconditioner {
    virtual ~Preconditioner() = default;
    virtual cudaError_t apply(int k, const int32_t *sys, const cd *in, cd *out, cudaStream_t s) = 0;
    // The same without any host synchronization or allocation (after one apply with this k), so that it can be
    // captured into a CUDA graph; whatever status it would have checked is read later by deferred_status.
    virtual cudaError_t apply_deferred(int k, const int32_t *sys, const cd *in, cd *out, cudaStream_t s) {
        return apply(k, sys, in, out, s);
    }
    virtual cudaError_t deferred_status(cudaStream_t) { return cudaSuccess; }
};

struct GmresOptions {
    double tol = 1e-8;       // relative residual |b - A x| / |b| per column
    int maxiter = 500;       // Arnoldi steps per column
    int restart = 100;
    // Each restart cycle (its Arnoldi steps, least squares and update) as one CUDA graph launch: the steps run in a
    // conditional WHILE node whose condition a kernel sets on the device (any column still active, steps left),
    // with no host synchronization between steps. The operator's and preconditioner's kernels must be capturable
    // (Preconditioner::apply_deferred) after one warm-up application. Same arithmetic, same result.
    bool captured = false;
};

struct GmresReport {
    std::vector<int> iterations;      // per column
    std::vector<double> residual;     // true relative residual per column at exit
    int cycles = 0;
    int launches = 0;                 // kernels launched by the GMRES loop itself (operator and preconditioner excluded)
};

// Solve A_s x_s = b_s for k columns (b, x on the device, (n, k) layout); x holds the initial guess on entry.
// Returns cudaSuccess; convergence is reported per column in `report` (residual > tol: not converged).
cudaError_t gmres_batched(Operator &A, Preconditioner *M, int k, const int32_t *sys_host, const cd *b, cd *x,
                          const GmresOptions &opt, GmresReport &report, cudaStream_t stream);

// Column helpers (device): norms (deterministic two-stage sums; scratch holds 64 * k doubles) and column moves.
cudaError_t column_norms(int64_t n, int k, const cd *x, double *out, double *scratch, cudaStream_t s);
cudaError_t gather_columns(int64_t n, int k, int ka, const int *act, const cd *full, cd *compact, cudaStream_t s);
cudaError_t scatter_add_columns(int64_t n, int k, int ka, const int *act, const cd *compact, cd *full,
                                cudaStream_t s);
cudaError_t subtract_from(int64_t count, const cd *b, cd *a, cudaStream_t s);     // a = b - a

// Mixed-precision refinement (the MixedLU scheme with a Krylov inner solve): the true residual r = b - A x with the
// FP64 operator, then an inner right-preconditioned GMRES on the single-precision operator A32 to `inner_tol` of
// |r|, x += correction, until |b - A x| / |b| <= tol per column or `max_outer` outer steps.
struct RefineOptions {
    double tol = 1e-8;
    double inner_tol = 1e-4;
    int max_outer = 8;
    int inner_maxiter = 200;
    int restart = 50;
    bool captured = false;   // the inner GMRES's cycles as graph launches (GmresOptions::captured)
};
cudaError_t refine_batched(Operator &A, Operator &A32, Preconditioner *M, int k, const int32_t *sys_host,
                           const cd *b, cd *x, const RefineOptions &opt, GmresReport &report, int &outer_steps,
                           cudaStream_t stream);

}  // namespace pq
