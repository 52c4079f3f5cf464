// Blocked dense factorizations on the device: the complex64 LU with partial pivoting (cuSOLVER getrf's layout and
// pivot convention) and the FP32 Cholesky (potrf's layout), both with their trailing updates as large GEMMs.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace pq {

// Trailing-update arithmetic of the blocked LU.
enum LuMath : int {
    LU_GEMM_FP32 = 0,      // FP32 GEMMs on the CUDA cores
    LU_GEMM_BF16X9 = 1,    // FP32 GEMMs emulated on the tensor cores with three BF16 terms per operand
    LU_GEMM_TC3 = 2,       // this library's tcgen05 GEMM, three BF16 part products (about 16 correct bits)
    LU_GEMM_TC6 = 3,       // this library's tcgen05 GEMM, six BF16 part products (FP32's accuracy)
};

constexpr int MAX_BLOCK_PUBLIC = 4096;   // widest panel the blocked factorizations take

// Factors the n x n column-major complex64 matrix A (leading dimension n) in place as P A = L U, L unit lower,
// with ipiv[i] the 1-based row swapped with row i (the same layout and pivots as cusolverDnCgetrf, so the
// triangular solvers of that factor apply unchanged). Right-looking in `block`-column panels: each panel is
// factored by cuSOLVER on a second stream while the main stream finishes the previous step's trailing update
// (one step of lookahead), its row swaps are applied to the other columns by a gather kernel, the block row of U
// comes from a triangular solve and the trailing update from one large GEMM (`math`): cuBLAS into a scratch matrix
// and a subtract pass (LU_GEMM_FP32, LU_GEMM_BF16X9), or this library's tcgen05 update C -= A B with the subtraction
// fused (LU_GEMM_TC3, LU_GEMM_TC6: tc_update_c64, the panel's BF16 planes packed once per step). Returns
// cudaSuccess, or an error (cudaErrorLaunchTimeout: a bounded wait of the tcgen05 update gave up); *singular = the
// first zero pivot's 1-based index (0 if none). Ordered on `stream`; returns after the factor is complete.
// The trailing updates of the last tcgen05 factorization: their summed CUDA-event time on the main stream, their
// complex flops (8 rows cols k each) and how many there were.
struct LuUpdateStats {
    double ms = 0, flops = 0;
    int launches = 0;
};

cudaError_t getrf_blocked(int64_t n, float2 *A, int *ipiv, int block, int math, cudaStream_t stream, int *singular,
                          LuUpdateStats *stats = nullptr);

// The panel width of getrf_blocked for order n and `math`: the autotuner's choice (pcbqs_gb300_tune_lu_panel) when
// one is recorded for this device, else 2048.
int lu_panel_width(int64_t n, int math);

// Factors the n x n column-major symmetric positive definite FP32 matrix A (leading dimension lda >= n, best a
// multiple of 32 so that the GEMMs take their aligned forms; the lower triangle is read) in place as A = L L^T,
// L in the lower triangle (cusolverDnSpotrf's layout; the strict upper triangle is left with intermediate values). Right-looking in `block`-column panels: the diagonal block by
// cuSOLVER potrf and the panel below it by a triangular solve, both on a second stream one step ahead, and the
// trailing lower triangle by one GEMM per block column (`math`). *info = the 1-based order of the first leading
// minor that is not positive definite (0 if none). Ordered on `stream`; returns after the factor is complete.
cudaError_t potrf_blocked(int64_t n, float *A, int64_t lda, int block, int math, cudaStream_t stream, int *info);

}  // namespace pq
