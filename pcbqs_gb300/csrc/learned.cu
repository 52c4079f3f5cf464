// A learned block preconditioner for the loop/tree systems: block-Jacobi plus one Neumann-type correction per
// selected pair of coupled blocks, each correction weighted by a gain that a small edge-level network predicts from
// the pair's features. No counterpart in the reference (its GMRES is preconditioned by sparse surrogates); block
// Jacobi (every gain zero) is both the starting point of the training and the fallback.
//
//   y   = D^-1 x                                         (block-Jacobi: the inverted diagonal blocks)
//   out = y - sum_{edges e = (b <- c)} g_e D_b^-1 A_bc y_c   (A_bc the off-diagonal block, g_e the learned gain)
//   g_e = w2 . tanh(W1 phi_e + b1) + b2                   (phi_e the edge's features; one hidden layer)
//
// Kernels: the network's forward and backward passes (deterministic parameter gradients: per-block partial sums in
// a fixed order, then one fixed-order reduction), the preconditioner's application (optionally keeping the
// correction vectors u_e = D_b^-1 A_bc y_c that the gains' gradients need), the gains' gradient dots, and a GMRES on
// a dense complex system with this preconditioner (or block-Jacobi alone) for the comparison. Everything FP64.
#include <algorithm>
#include <vector>

#include <cublas_v2.h>

#include "../../include/pcbqs_gb300.h"
#include "common.cuh"
#include "pool.cuh"
#include "solve.cuh"

namespace pq {

namespace {

constexpr int MLP_THREADS = 128;
constexpr int MAX_PARAMS = 1024;

// Blocks for a grid-stride loop over `total` items: enough to fill the GPU, capped.
int grid_of(int64_t total) { return (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 4096)); }

struct Mlp {
    int f, h;
    const double *W1, *b1, *W2, *b2;      // W1 (h, f) row-major
};

__device__ __forceinline__ Mlp mlp_of(int f, int h, const double *params) {
    return Mlp{f, h, params, params + h * f, params + h * f + h, params + h * f + 2 * h};
}

// g[e] = W2 . tanh(W1 phi[e] + b1) + b2; hidden[e] = tanh(...) (h values), one thread per edge.
__global__ void k_mlp_forward(int64_t nedge, int f, int h, const double *phi, const double *params, double *hidden,
                              double *g) {
    const Mlp m = mlp_of(f, h, params);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nedge; e += (int64_t)gridDim.x * blockDim.x) {
        const double *p = phi + e * f;
        double out = m.b2[0];
        for (int j = 0; j < h; ++j) {
            double a = m.b1[j];
            for (int i = 0; i < f; ++i) a += m.W1[j * f + i] * p[i];
            const double t = tanh(a);
            hidden[e * h + j] = t;
            out += m.W2[j] * t;
        }
        g[e] = out;
    }
}

// Parameter gradients for dL/dg (dg): each block accumulates its edges' contributions (grid-stride, fixed order) in
// shared memory, one parameter per thread, into partial[block]; k_sum_partials adds the blocks in order.
__global__ void k_mlp_backward(int64_t nedge, int f, int h, const double *phi, const double *params,
                               const double *hidden, const double *dg, double *partial) {
    const Mlp m = mlp_of(f, h, params);
    const int np = h * f + 2 * h + 1;
    for (int q = threadIdx.x; q < np; q += blockDim.x) {
        double acc = 0;
        for (int64_t e = blockIdx.x; e < nedge; e += gridDim.x) {
            const double d = dg[e];
            const double *hid = hidden + e * h;
            if (q < h * f) {                          // W1[j, i]
                const int j = q / f, i = q % f;
                acc += d * m.W2[j] * (1 - hid[j] * hid[j]) * phi[e * f + i];
            } else if (q < h * f + h) {               // b1[j]
                const int j = q - h * f;
                acc += d * m.W2[j] * (1 - hid[j] * hid[j]);
            } else if (q < h * f + 2 * h) {           // W2[j]
                acc += d * hid[q - h * f - h];
            } else {                                  // b2
                acc += d;
            }
        }
        partial[(int64_t)blockIdx.x * np + q] = acc;
    }
}

__global__ void k_sum_partials(int blocks, int np, const double *partial, double *grad) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < np; q += gridDim.x * blockDim.x) {
        double acc = 0;
        for (int b = 0; b < blocks; ++b) acc += partial[(int64_t)b * np + q];
        grad[q] = acc;
    }
}

// y[r, s] = sum_j Dinv[block(r)][r % bs][j] x[block(r) * bs + j, s] (the last block may be short).
__global__ void k_lp_block_jacobi(int64_t n, int bs, int k, const cd *dinv, const cd *in, cd *out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * k; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / k;
        const int s = (int)(t % k);
        const int64_t b = r / bs;
        const int rl = (int)(r - b * bs);
        const cd *M = dinv + (b * bs + rl) * bs;
        const int64_t c0 = b * bs;
        const int cn = (int)min((int64_t)bs, n - c0);
        double re = 0, im = 0;
        for (int c = 0; c < cn; ++c) {
            const cd mv = M[c], x = in[(c0 + c) * k + s];
            re += mv.x * x.x - mv.y * x.y;
            im += mv.x * x.y + mv.y * x.x;
        }
        out[t] = make_double2(re, im);
    }
}

// One block per (destination block b, column s), bs threads (one row each): for each edge e = (b <- c) of b,
// t = A_bc y_c, u = D_b^-1 t (kept in u_out[e][row][s] when given), out_b = y_b - sum_e g_e u. Edges grouped by
// destination (eptr CSR, ecol the source blocks), in their order: deterministic.
__global__ void k_lp_corrections(int64_t n, int bs, int64_t nblk, const int64_t *eptr, const int32_t *ecol,
                                 const cd *dinv, const cd *E, const double *g, int k, const cd *y, cd *out,
                                 cd *u_out) {
    extern __shared__ cd lp_smem[];
    cd *yc = lp_smem, *tv = lp_smem + bs;
    const int64_t b = blockIdx.x;
    const int s = blockIdx.y;
    const int i = threadIdx.x;
    const int64_t r = b * bs + i;
    const bool row = r < n;
    double ar = 0, ai = 0;
    for (int64_t e = eptr[b]; e < eptr[b + 1]; ++e) {
        const int64_t c = ecol[e];
        const int64_t rc = c * bs + i;
        yc[i] = rc < n ? y[rc * k + s] : make_double2(0, 0);
        __syncthreads();
        const cd *Ab = E + (e * bs + i) * bs;
        double tr = 0, ti = 0;
        for (int j = 0; j < bs; ++j) {
            const cd a = Ab[j], v = yc[j];
            tr += a.x * v.x - a.y * v.y;
            ti += a.x * v.y + a.y * v.x;
        }
        tv[i] = make_double2(tr, ti);
        __syncthreads();
        const cd *D = dinv + (b * bs + i) * bs;
        double ur = 0, ui = 0;
        for (int j = 0; j < bs; ++j) {
            const cd d = D[j], v = tv[j];
            ur += d.x * v.x - d.y * v.y;
            ui += d.x * v.y + d.y * v.x;
        }
        if (u_out) u_out[(e * bs + i) * k + s] = make_double2(ur, ui);
        ar += g[e] * ur;
        ai += g[e] * ui;
        __syncthreads();
    }
    if (row) {
        const cd yv = y[r * k + s];
        out[r * k + s] = make_double2(yv.x - ar, yv.y - ai);
    }
}

// dots[e] = sum_s sum_i Re(conj(S[b * bs + i, s]) u[e][i][s]) for the edges of every destination block b.
__global__ void k_lp_edge_dots(int64_t n, int bs, int64_t nblk, const int64_t *eptr, int k, const cd *S,
                               const cd *u, double *dots) {
    const int64_t b = blockIdx.x;
    for (int64_t e = eptr[b]; e < eptr[b + 1]; ++e) {
        double acc = 0;                       // one warp per edge: lanes over (row, column), fixed order
        for (int64_t t = threadIdx.x; t < (int64_t)bs * k; t += 32) {
            const int i = (int)(t / k), s = (int)(t % k);
            const int64_t r = b * bs + i;
            if (r < n) {
                const cd a = S[r * k + s], v = u[(e * bs + i) * k + s];
                acc += a.x * v.x + a.y * v.y;
            }
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) dots[e] = acc;
    }
}

struct LearnedPrecond : Preconditioner {
    int64_t n = 0, nblk = 0;
    int bs = 32;
    const int64_t *eptr = nullptr;
    const int32_t *ecol = nullptr;
    const cd *dinv = nullptr, *E = nullptr;
    const double *g = nullptr;          // null: block-Jacobi alone
    cd *y = nullptr;
    int cap = 0;
    ~LearnedPrecond() override { pool_free(y, nullptr); }
    cudaError_t apply(int k, const int32_t *, const cd *in, cd *out, cudaStream_t s) override {
        if (!g) {
            k_lp_block_jacobi<<<grid_of(n * k), 256, 0, s>>>(n, bs, k, dinv, in, out);
            note_launches(1);
            return cudaGetLastError();
        }
        if (k > cap) {
            pool_free(y, s);
            y = nullptr;
            cudaError_t e = pool_alloc_n(&y, (size_t)n * k, s);
            if (e) return e;
            cap = k;
        }
        k_lp_block_jacobi<<<grid_of(n * k), 256, 0, s>>>(n, bs, k, dinv, in, y);
        k_lp_corrections<<<dim3((unsigned)nblk, (unsigned)k), bs, 2 * bs * sizeof(cd), s>>>(n, bs, nblk, eptr, ecol,
                                                                                         dinv, E, g, k, y, out,
                                                                                         nullptr);
        note_launches(2);
        return cudaGetLastError();
    }
};

// y = A x for a dense complex row-major A (n x n, row stride lda) on (n, k) row-major columns: in column-major
// terms y^T = x^T A^T, one cuBLAS ZGEMM.
struct DenseComplexOp : Operator {
    int64_t n_ = 0, lda = 0;
    const cd *A = nullptr;
    cublasHandle_t blas = nullptr;
    ~DenseComplexOp() override {
        if (blas) cublasDestroy(blas);
    }
    int64_t n() const override { return n_; }
    cudaError_t apply(int k, const int32_t *, const cd *in, cd *out, cudaStream_t s) override {
        const cuDoubleComplex one = {1, 0}, zero = {0, 0};
        cublasSetStream(blas, s);
        if (cublasZgemm(blas, CUBLAS_OP_N, CUBLAS_OP_N, k, (int)n_, (int)n_, &one,
                        reinterpret_cast<const cuDoubleComplex *>(in), k, reinterpret_cast<const cuDoubleComplex *>(A),
                        (int)lda, &zero, reinterpret_cast<cuDoubleComplex *>(out), k) != CUBLAS_STATUS_SUCCESS)
            return cudaErrorUnknown;
        return cudaSuccess;
    }
};

}  // namespace

}  // namespace pq

using namespace pq;

extern "C" {

int pcbqs_gb300_learned_forward(int64_t nedge, int nfeat, int nhidden, const double *phi, const double *params,
                                double *hidden, double *gains, void *stream) {
    if (nedge < 0 || nfeat <= 0 || nhidden <= 0 || nhidden * nfeat + 2 * nhidden + 1 > MAX_PARAMS ||
        (nedge && (!phi || !params || !hidden || !gains)))
        return fail(ERR_ARGUMENT, "learned_forward: invalid argument");
    if (nedge == 0) return OK;
    k_mlp_forward<<<grid_of(nedge), MLP_THREADS, 0, static_cast<cudaStream_t>(stream)>>>(nedge, nfeat, nhidden, phi,
                                                                                       params, hidden, gains);
    note_launches(1);
    const cudaError_t e = cudaGetLastError();
    return e ? fail(ERR_CUDA, "learned_forward: %s", cudaGetErrorString(e)) : OK;
}

int pcbqs_gb300_learned_backward(int64_t nedge, int nfeat, int nhidden, const double *phi, const double *params,
                                 const double *hidden, const double *dgains, double *grad, void *stream) {
    const int np = nhidden * nfeat + 2 * nhidden + 1;
    if (nedge < 0 || nfeat <= 0 || nhidden <= 0 || np > MAX_PARAMS || !grad ||
        (nedge && (!phi || !params || !hidden || !dgains)))
        return fail(ERR_ARGUMENT, "learned_backward: invalid argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int blocks = (int)std::min<int64_t>(std::max<int64_t>(nedge, 1), 256);
    double *partial = nullptr;
    cudaError_t e = pool_alloc_n(&partial, (size_t)blocks * np, st);
    if (e) return fail(ERR_MEMORY, "learned_backward: %s", cudaGetErrorString(e));
    if (nedge) {
        k_mlp_backward<<<blocks, MLP_THREADS, 0, st>>>(nedge, nfeat, nhidden, phi, params, hidden, dgains, partial);
    } else {
        cudaMemsetAsync(partial, 0, sizeof(double) * blocks * np, st);
    }
    k_sum_partials<<<(np + 127) / 128, 128, 0, st>>>(blocks, np, partial, grad);
    note_launches(2);
    e = cudaGetLastError();
    pool_free(partial, st);
    return e ? fail(ERR_CUDA, "learned_backward: %s", cudaGetErrorString(e)) : OK;
}

int pcbqs_gb300_learned_apply(int64_t n, int bs, int64_t nblk, const int64_t *eptr, const int32_t *ecol,
                              const double *dinv, const double *E, const double *gains, int k, const double *in,
                              double *out, double *corrections, void *stream) {
    if (n <= 0 || bs <= 0 || bs > 64 || nblk != (n + bs - 1) / bs || k <= 0 || k > 65535 || !eptr || !dinv || !in ||
        !out || (gains && !ecol))
        return fail(ERR_ARGUMENT, "learned_apply: invalid argument (bs <= 64, nblk = ceil(n / bs))");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const cd *x = reinterpret_cast<const cd *>(in);
    cd *y = reinterpret_cast<cd *>(out);
    if (!gains) {
        k_lp_block_jacobi<<<grid_of(n * k), 256, 0, st>>>(n, bs, k, reinterpret_cast<const cd *>(dinv), x, y);
        note_launches(1);
    } else {
        cd *tmp = nullptr;
        cudaError_t e = pool_alloc_n(&tmp, (size_t)n * k, st);
        if (e) return fail(ERR_MEMORY, "learned_apply: %s", cudaGetErrorString(e));
        k_lp_block_jacobi<<<grid_of(n * k), 256, 0, st>>>(n, bs, k, reinterpret_cast<const cd *>(dinv), x, tmp);
        k_lp_corrections<<<dim3((unsigned)nblk, (unsigned)k), bs, 2 * bs * sizeof(cd), st>>>(
            n, bs, nblk, eptr, ecol, reinterpret_cast<const cd *>(dinv), reinterpret_cast<const cd *>(E), gains, k,
            tmp, y, reinterpret_cast<cd *>(corrections));
        note_launches(2);
        pool_free(tmp, st);
    }
    const cudaError_t e = cudaGetLastError();
    return e ? fail(ERR_CUDA, "learned_apply: %s", cudaGetErrorString(e)) : OK;
}

int pcbqs_gb300_learned_edge_dots(int64_t n, int bs, int64_t nblk, const int64_t *eptr, int k, const double *S,
                                  const double *corrections, double *dots, void *stream) {
    if (n <= 0 || bs <= 0 || bs > 64 || nblk != (n + bs - 1) / bs || k <= 0 || !eptr || !S || !corrections || !dots)
        return fail(ERR_ARGUMENT, "learned_edge_dots: invalid argument");
    k_lp_edge_dots<<<(unsigned)nblk, 32, 0, static_cast<cudaStream_t>(stream)>>>(
        n, bs, nblk, eptr, k, reinterpret_cast<const cd *>(S), reinterpret_cast<const cd *>(corrections), dots);
    note_launches(1);
    const cudaError_t e = cudaGetLastError();
    return e ? fail(ERR_CUDA, "learned_edge_dots: %s", cudaGetErrorString(e)) : OK;
}

int pcbqs_gb300_learned_gmres(int64_t n, const double *A, int64_t lda, int k, const double *b, double *x, double tol,
                              int maxiter, int restart, int bs, int64_t nblk, const int64_t *eptr,
                              const int32_t *ecol, const double *dinv, const double *E, const double *gains,
                              int32_t *iterations, double *residual, void *stream) {
    if (n <= 0 || !A || lda < n || k <= 0 || !b || !x || !(tol > 0) || maxiter <= 0 || restart <= 0 || bs <= 0 ||
        bs > 64 || nblk != (n + bs - 1) / bs || !eptr || !dinv || (gains && (!ecol || !E)))
        return fail(ERR_ARGUMENT, "learned_gmres: invalid argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DenseComplexOp op;
    op.n_ = n;
    op.lda = lda;
    op.A = reinterpret_cast<const cd *>(A);
    if (cublasCreate(&op.blas) != CUBLAS_STATUS_SUCCESS) return fail(ERR_CUDA, "learned_gmres: cuBLAS handle");
    LearnedPrecond M;
    M.n = n;
    M.nblk = nblk;
    M.bs = bs;
    M.eptr = eptr;
    M.ecol = ecol;
    M.dinv = reinterpret_cast<const cd *>(dinv);
    M.E = reinterpret_cast<const cd *>(E);
    M.g = gains;
    std::vector<int32_t> sys(k, 0);
    GmresOptions opt;
    opt.tol = tol;
    opt.maxiter = maxiter;
    opt.restart = restart;
    GmresReport rep;
    cudaError_t e = gmres_batched(op, &M, k, sys.data(), reinterpret_cast<const cd *>(b), reinterpret_cast<cd *>(x),
                                  opt, rep, st);
    if (!e) e = cudaStreamSynchronize(st);
    if (e) return fail(ERR_CUDA, "learned_gmres: %s", cudaGetErrorString(e));
    bool ok = true;
    for (int s = 0; s < k; ++s) {
        if (iterations) iterations[s] = rep.iterations[s];
        if (residual) residual[s] = rep.residual[s];
        ok = ok && rep.residual[s] <= tol;
    }
    return ok ? OK : fail(ERR_CONVERGENCE, "learned_gmres: not every column reached the tolerance");
}

}  // extern "C"
