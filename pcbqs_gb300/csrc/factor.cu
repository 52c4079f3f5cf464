// Blocked dense factorizations with one step of lookahead (declared in factor.cuh): the complex64 LU with partial
// pivoting (pq::getrf_blocked) and the FP32 Cholesky (pq::potrf_blocked).
//
// Why not cusolverDnCgetrf on the whole matrix: its trailing updates are GEMMs with a small inner dimension, which
// the BF16x9-emulated FP32 GEMM runs far below its rate (a 32k x 32k x 64 complex GEMM at 19 TFLOP/s against 141
// at an inner dimension of 1024, measured on GB300), and its panel factorizations sit on the critical path. Here
// the panels are wide (2048 columns in the PEEC factor), so each trailing update is one GEMM near the emulation's
// full rate, and the next panel is factored on a second, high-priority stream while the rest of the trailing
// matrix is updated.
//
// Step t (columns j .. j+jb of the n x n column-major matrix, rows j .. n):
//   panel stream: getrf of the panel (cuSOLVER, pivots relative to row j) -> k_lu_pivot_plan turns the pivots into
//                 global 1-based rows (the getrf convention) and the permutation of the rows they touch
//   main stream:  k_lu_swap_rows applies that permutation to every other column; triangular solve for the block
//                 row U12; the next panel's columns updated (GEMM into scratch, k_trailing_subtract); (event: the
//                 next panel may start); triangular solve and update of the remaining columns.
#include <algorithm>
#include <string>
#include <cstdio>
#include <vector>

#include <cublas_v2.h>
#include <cusolverDn.h>

#include "../../include/pcbqs_gb300.h"
#include "common.cuh"
#include "factor.cuh"
#include "tune.cuh"
#include "pool.cuh"
#include "tcgemm.cuh"

namespace pq {

namespace {

constexpr int MAX_BLOCK = MAX_BLOCK_PUBLIC;   // widest panel (the swap plan holds 2 * MAX_BLOCK rows)
constexpr int PLAN = 2 * MAX_BLOCK;
constexpr int HASH = 2 * MAX_BLOCK;        // open-addressing table of the rows below the panel (load <= 1/2)

// The panel's pivots (1-based, relative to row j) become global rows (1-based, as getrf reports them), and the
// sequence of swaps "row j+i <-> row piv[i]" becomes one permutation of the rows it touches: after it, row dst[e]
// holds what row src[e] held before. Rows of the panel take slots 0 .. jb-1; rows below it get the next slots
// through a small hash table. One block; the swap sequence itself is walked by one thread in shared memory.
constexpr size_t PLAN_SMEM = sizeof(int) * (2 * HASH + 2 * PLAN + MAX_BLOCK);

__global__ void k_lu_pivot_plan(int64_t n, int64_t j, int jb, int *ipiv, int *dst, int *src, int *count,
                                int *error) {
    extern __shared__ int plan_smem[];
    int *keys = plan_smem, *vals = keys + HASH, *content = vals + HASH, *rows = content + PLAN, *piv = rows + PLAN;
    __shared__ int used;
    for (int h = threadIdx.x; h < HASH; h += blockDim.x) keys[h] = -1;
    for (int s = threadIdx.x; s < jb; s += blockDim.x) {
        const int g = ipiv[j + s] + (int)j;
        ipiv[j + s] = g;
        piv[s] = g - 1;
        content[s] = rows[s] = (int)j + s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int c = jb;
        bool bad = false;
        for (int i = 0; i < jb; ++i) {
            const int p = piv[i];
            if (p < j + i || p >= n) {              // not a row at or below row j+i: leave it, report
                bad = true;
                continue;
            }
            int sp;
            if (p < j + jb) {
                sp = p - (int)j;
            } else {
                int h = (int)(((unsigned)p * 2654435761u) & (HASH - 1));
                while (keys[h] != -1 && keys[h] != p) h = (h + 1) & (HASH - 1);
                if (keys[h] == -1) {
                    keys[h] = p;
                    vals[h] = c;
                    content[c] = rows[c] = p;
                    ++c;
                }
                sp = vals[h];
            }
            const int t = content[i];
            content[i] = content[sp];
            content[sp] = t;
        }
        used = c;
        *count = c;
        if (bad) atomicExch(error, 1);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < used; e += blockDim.x) {
        dst[e] = rows[e];
        src[e] = content[e];
    }
}

// Applies the plan to the columns outside the panel, [0, j) and [j + jb, n): per column, every thread reads its
// entries of the touched rows, the block synchronises, then writes them to their new rows.
constexpr int SWAP_THREADS = 512;
constexpr size_t SWAP_SMEM = sizeof(int) * 2 * PLAN;
__global__ void __launch_bounds__(SWAP_THREADS) k_lu_swap_rows(int64_t n, int64_t j, int jb, float2 *A,
                                                               const int *dst, const int *src, const int *count) {
    extern __shared__ int swap_smem[];
    int *sd = swap_smem, *ss = swap_smem + PLAN;
    const int c = *count;
    for (int e = threadIdx.x; e < c; e += blockDim.x) {
        sd[e] = dst[e];
        ss[e] = src[e];
    }
    __syncthreads();
    const int64_t cols = n - jb;
    for (int64_t q = blockIdx.x; q < cols; q += gridDim.x) {
        const int64_t col = q < j ? q : q + jb;
        float2 *a = A + col * n;
        float2 v[PLAN / SWAP_THREADS];
#pragma unroll
        for (int r = 0; r < PLAN / SWAP_THREADS; ++r) {
            const int e = threadIdx.x + r * SWAP_THREADS;
            if (e < c) v[r] = a[ss[e]];
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < PLAN / SWAP_THREADS; ++r) {
            const int e = threadIdx.x + r * SWAP_THREADS;
            if (e < c) a[sd[e]] = v[r];
        }
    }
}

// The stream of the panel factorizations, at the device's highest priority: their small latency-bound kernels
// then take SMs as soon as the trailing GEMM's blocks retire, instead of queueing behind its later waves.
cudaError_t panel_stream(cudaStream_t *stream) {
    int least = 0, greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e) return e;
    return cudaStreamCreateWithPriority(stream, cudaStreamNonBlocking, greatest);
}

// C (rows x cols, column-major, leading dimension ldc) -= T (leading dimension rows): the second half of a trailing
// update whose product went to T. A separate pass because the emulated GEMM costs far more with beta = 1 than with
// beta = 0 (a 30k x 30k x 2048 complex update: 86.5 against 70.7 ms, measured), and this pass reads C and T and
// writes C once (3.3 ms for that size at HBM speed).
__global__ void k_trailing_subtract(int64_t rows, int64_t cols, float2 *C, int64_t ldc, const float2 *T) {
    for (int64_t c = blockIdx.y; c < cols; c += gridDim.y) {
        float2 *cc = C + c * ldc;
        const float2 *tc = T + c * rows;
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x) {
            const float2 t = tc[i];
            float2 v = cc[i];
            v.x -= t.x;
            v.y -= t.y;
            cc[i] = v;
        }
    }
}

struct Resources {
    cublasHandle_t blas = nullptr;
    cusolverDnHandle_t solver = nullptr;
    cudaStream_t panel = nullptr;
    cudaEvent_t ready = nullptr, next = nullptr;
    std::vector<cudaEvent_t> marks;          // around each tcgen05 update (when timed)
    float2 *work = nullptr, *product = nullptr;
    uint8_t *planes = nullptr;
    int *plan = nullptr, *info = nullptr;
    cudaStream_t main = nullptr;
    ~Resources() {
        if (main) cudaStreamSynchronize(main);
        if (panel) cudaStreamSynchronize(panel);
        pool_free(work, main);
        pool_free(product, main);
        pool_free(planes, main);
        pool_free(plan, main);
        pool_free(info, main);
        if (blas) cublasDestroy(blas);
        if (solver) cusolverDnDestroy(solver);
        if (ready) cudaEventDestroy(ready);
        if (next) cudaEventDestroy(next);
        for (cudaEvent_t e : marks) cudaEventDestroy(e);
        if (panel) cudaStreamDestroy(panel);
    }
};

}  // namespace

cudaError_t getrf_blocked(int64_t n, float2 *A, int *ipiv, int block, int math, cudaStream_t stream, int *singular,
                          LuUpdateStats *stats) {
    *singular = 0;
    if (n <= 0 || n > (int64_t)0x7fffffff || !A || !ipiv || block < 32 || block > MAX_BLOCK ||
        (math != LU_GEMM_FP32 && math != LU_GEMM_BF16X9 && math != LU_GEMM_TC3 && math != LU_GEMM_TC6))
        return cudaErrorInvalidValue;
    const bool tc = math == LU_GEMM_TC3 || math == LU_GEMM_TC6;
    const int terms = math == LU_GEMM_TC3 ? 3 : 6;
    if (stats) *stats = LuUpdateStats{};
    const int nb = (int)std::min<int64_t>(block, n);
    const int64_t steps = (n + nb - 1) / nb;
    Resources r;
    r.main = stream;
    cudaError_t e;
    if ((e = panel_stream(&r.panel)) || (e = cudaEventCreateWithFlags(&r.ready, cudaEventDisableTiming)) ||
        (e = cudaEventCreateWithFlags(&r.next, cudaEventDisableTiming)))
        return e;
    if (cublasCreate(&r.blas) != CUBLAS_STATUS_SUCCESS || cusolverDnCreate(&r.solver) != CUSOLVER_STATUS_SUCCESS)
        return cudaErrorNotSupported;
    cublasSetStream(r.blas, stream);
    cusolverDnSetStream(r.solver, r.panel);
    cublasComputeType_t compute = CUBLAS_COMPUTE_32F;
    if (math != LU_GEMM_FP32) {       // (the tcgen05 forms keep the emulated FP32 in the panels' own GEMMs)
        if (cublasSetEmulationStrategy(r.blas, CUBLAS_EMULATION_STRATEGY_EAGER) != CUBLAS_STATUS_SUCCESS ||
            cublasSetEmulationSpecialValuesSupport(r.blas, CUDA_EMULATION_SPECIAL_VALUES_SUPPORT_NONE) !=
                CUBLAS_STATUS_SUCCESS ||
            cublasSetMathMode(r.blas, CUBLAS_FP32_EMULATED_BF16X9_MATH) != CUBLAS_STATUS_SUCCESS ||
            cusolverDnSetMathMode(r.solver, CUSOLVER_FP32_EMULATED_BF16X9_MATH) != CUSOLVER_STATUS_SUCCESS)
            return cudaErrorNotSupported;
        compute = CUBLAS_COMPUTE_32F_EMULATED_16BFX9;
    }
    if ((e = cudaFuncSetAttribute(k_lu_pivot_plan, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PLAN_SMEM)) ||
        (e = cudaFuncSetAttribute(k_lu_swap_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SWAP_SMEM)))
        return e;
    int lwork = 0;
    if (cusolverDnCgetrf_bufferSize(r.solver, (int)n, nb, reinterpret_cast<cuComplex *>(A), (int)n, &lwork) !=
        CUSOLVER_STATUS_SUCCESS)
        return cudaErrorUnknown;
    // plan: dst (PLAN), src (PLAN), count, error, the tcgen05 update's timeout flag
    // cuBLAS: the trailing products go to a scratch matrix (beta = 0) and are subtracted by k_trailing_subtract; the
    // largest is (n - nb) x (n - nb). tcgen05: the BF16 planes of the largest update ((n - nb) rows and columns).
    const int64_t trail = n - nb;
    if ((e = pool_alloc_n(&r.work, (size_t)std::max(lwork, 1), stream)) ||
        (e = pool_alloc_n(&r.plan, (size_t)2 * PLAN + 3, stream)) ||
        (e = pool_alloc_n(&r.info, (size_t)steps, stream)))
        return e;
    if (trail > 0 && !tc && (e = pool_alloc_n(&r.product, (size_t)trail * trail, stream))) return e;
    if (trail > 0 && tc && (e = pool_alloc_n(&r.planes, tc_update_scratch_bytes(trail, trail, nb, terms), stream)))
        return e;
    int *dst = r.plan, *src = r.plan + PLAN, *count = r.plan + 2 * PLAN, *error = count + 1, *tc_error = count + 2;
    if ((e = cudaMemsetAsync(error, 0, 2 * sizeof(int), stream)) ||
        (e = cudaMemsetAsync(r.info, 0, sizeof(int) * steps, stream)))
        return e;
    auto at = [&](int64_t row, int64_t col) { return A + row + col * n; };
    const cuComplex one = {1.f, 0.f};
    int sms = 0, device = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    auto factor_panel = [&](int64_t j, int jb, int64_t t) -> cudaError_t {
        if (cusolverDnCgetrf(r.solver, (int)(n - j), jb, reinterpret_cast<cuComplex *>(at(j, j)), (int)n,
                             reinterpret_cast<cuComplex *>(r.work), ipiv + j, r.info + t) != CUSOLVER_STATUS_SUCCESS)
            return cudaErrorUnknown;
        k_lu_pivot_plan<<<1, 256, PLAN_SMEM, r.panel>>>(n, j, jb, ipiv, dst, src, count, error);
        note_launches(1);
        return cudaEventRecord(r.ready, r.panel);
    };
    const cuComplex zero = {0.f, 0.f};
    // a_packed: the panel's planes were packed by this step's first update
    auto gemm = [&](int64_t rows, int64_t cols, int k, const float2 *a, const float2 *b, float2 *c,
                    bool a_packed) -> bool {
        if (rows <= 0 || cols <= 0) return true;
        if (tc) {
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            if (stats && (cudaEventCreate(&e0) || cudaEventCreate(&e1) || cudaEventRecord(e0, stream))) return false;
            if (tc_update_c64(rows, cols, k, a, n, b, n, c, n, terms, r.planes, a_packed, tc_error, wait_cycles(),
                              stream) != cudaSuccess)
                return false;
            if (stats) {
                if (cudaEventRecord(e1, stream)) return false;
                r.marks.push_back(e0);
                r.marks.push_back(e1);
                stats->flops += 8.0 * (double)rows * (double)cols * (double)k;
                ++stats->launches;
            }
            return true;
        }
        if (rows > trail || cols > trail) return false;
        if (cublasGemmEx(r.blas, CUBLAS_OP_N, CUBLAS_OP_N, (int)rows, (int)cols, k, &one, a, CUDA_C_32F, (int)n, b,
                         CUDA_C_32F, (int)n, &zero, r.product, CUDA_C_32F, (int)rows, compute, CUBLAS_GEMM_DEFAULT) !=
            CUBLAS_STATUS_SUCCESS)
            return false;
        const dim3 grid((unsigned)std::min<int64_t>((rows + 255) / 256, 16),
                        (unsigned)std::min<int64_t>(cols, 65535));
        k_trailing_subtract<<<grid, 256, 0, stream>>>(rows, cols, c, n, r.product);
        note_launches(1);
        return true;
    };
    auto trsm = [&](int64_t j, int jb, int64_t c0, int64_t cols) -> bool {
        if (cols <= 0) return true;
        return cublasCtrsm(r.blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_UNIT, jb,
                           (int)cols, &one, reinterpret_cast<const cuComplex *>(at(j, j)), (int)n,
                           reinterpret_cast<cuComplex *>(at(j, c0)), (int)n) == CUBLAS_STATUS_SUCCESS;
    };
    // the panel stream starts after what the main stream queued before (the matrix's assembly)
    if ((e = cudaEventRecord(r.next, stream)) || (e = cudaStreamWaitEvent(r.panel, r.next, 0)) ||
        (e = factor_panel(0, nb, 0)))
        return e;
    for (int64_t t = 0; t < steps; ++t) {
        const int64_t j = t * nb;
        const int jb = (int)std::min<int64_t>(nb, n - j);
        const int64_t right = j + jb, rest = n - right;
        const int jb2 = (int)std::min<int64_t>(nb, rest);
        if ((e = cudaStreamWaitEvent(stream, r.ready, 0))) return e;
        const unsigned blocks = (unsigned)std::min<int64_t>(std::max<int64_t>(n - jb, 1), (int64_t)sms * 4);
        if (n > jb) {
            k_lu_swap_rows<<<blocks, SWAP_THREADS, SWAP_SMEM, stream>>>(n, j, jb, A, dst, src, count);
            note_launches(1);
        }
        if (rest <= 0) break;
        // next panel's columns first, so that its factorization overlaps the rest of the update
        if (!trsm(j, jb, right, jb2) || !gemm(rest, jb2, jb, at(right, j), at(j, right), at(right, right), false))
            return cudaErrorUnknown;
        if ((e = cudaEventRecord(r.next, stream)) || (e = cudaStreamWaitEvent(r.panel, r.next, 0)) ||
            (e = factor_panel(right, jb2, t + 1)))
            return e;
        if (!trsm(j, jb, right + jb2, rest - jb2) ||
            !gemm(rest, rest - jb2, jb, at(right, j), at(j, right + jb2), at(right, right + jb2), jb2 > 0))
            return cudaErrorUnknown;
    }
    if ((e = cudaGetLastError()) || (e = cudaStreamSynchronize(r.panel)) || (e = cudaStreamSynchronize(stream)))
        return e;
    std::vector<int> info((size_t)steps);
    int flags[2] = {0, 0};
    if ((e = cudaMemcpy(info.data(), r.info, sizeof(int) * steps, cudaMemcpyDeviceToHost)) ||
        (e = cudaMemcpy(flags, error, 2 * sizeof(int), cudaMemcpyDeviceToHost)))
        return e;
    if (flags[1]) return cudaErrorLaunchTimeout;
    if (flags[0]) return cudaErrorIllegalState;
    if (stats)
        for (size_t i = 0; i + 1 < r.marks.size(); i += 2) {
            float ms = 0;
            if (cudaEventElapsedTime(&ms, r.marks[i], r.marks[i + 1]) == cudaSuccess) stats->ms += ms;
        }
    for (int64_t t = 0; t < steps; ++t)
        if (info[t] > 0) {
            *singular = (int)(t * nb + info[t]);
            break;
        }
    return cudaSuccess;
}

namespace {

struct CholResources {
    cublasHandle_t blas = nullptr, blas_panel = nullptr;
    cusolverDnHandle_t solver = nullptr;
    cudaStream_t panel = nullptr, main = nullptr;
    cudaEvent_t ready = nullptr, next = nullptr;
    float *work = nullptr;
    int *info = nullptr;
    ~CholResources() {
        if (main) cudaStreamSynchronize(main);
        if (panel) cudaStreamSynchronize(panel);
        pool_free(work, main);
        pool_free(info, main);
        if (blas) cublasDestroy(blas);
        if (blas_panel) cublasDestroy(blas_panel);
        if (solver) cusolverDnDestroy(solver);
        if (ready) cudaEventDestroy(ready);
        if (next) cudaEventDestroy(next);
        if (panel) cudaStreamDestroy(panel);
    }
};

}  // namespace

// Step t (columns j .. j+jb):
//   panel stream: potrf of the diagonal block A[j:j+jb, j:j+jb]; L21 = A[j+jb:, j:j+jb] L11^-T (triangular solve)
//   main stream:  A[c:, c:c+w] -= L21[c-j-jb:] L21[c-j-jb : c-j-jb+w]^T for the block columns c of the trailing
//                 lower triangle, the next panel's block column first (then the panel stream may start it).
cudaError_t potrf_blocked(int64_t n, float *A, int64_t lda, int block, int math, cudaStream_t stream,
                          int *info_out) {
    *info_out = 0;
    if (n <= 0 || lda < n || lda > (int64_t)0x7fffffff || !A || block < 32 || block > MAX_BLOCK ||
        (math != LU_GEMM_FP32 && math != LU_GEMM_BF16X9))
        return cudaErrorInvalidValue;
    const int nb = (int)std::min<int64_t>(block, n);
    const int64_t steps = (n + nb - 1) / nb;
    CholResources r;
    r.main = stream;
    cudaError_t e;
    if ((e = panel_stream(&r.panel)) || (e = cudaEventCreateWithFlags(&r.ready, cudaEventDisableTiming)) ||
        (e = cudaEventCreateWithFlags(&r.next, cudaEventDisableTiming)))
        return e;
    if (cublasCreate(&r.blas) != CUBLAS_STATUS_SUCCESS || cublasCreate(&r.blas_panel) != CUBLAS_STATUS_SUCCESS ||
        cusolverDnCreate(&r.solver) != CUSOLVER_STATUS_SUCCESS)
        return cudaErrorNotSupported;
    cublasSetStream(r.blas, stream);
    cublasSetStream(r.blas_panel, r.panel);
    cusolverDnSetStream(r.solver, r.panel);
    cublasComputeType_t compute = CUBLAS_COMPUTE_32F;
    if (math == LU_GEMM_BF16X9) {
        if (cublasSetEmulationStrategy(r.blas, CUBLAS_EMULATION_STRATEGY_EAGER) != CUBLAS_STATUS_SUCCESS ||
            cublasSetEmulationSpecialValuesSupport(r.blas, CUDA_EMULATION_SPECIAL_VALUES_SUPPORT_NONE) !=
                CUBLAS_STATUS_SUCCESS ||
            cublasSetMathMode(r.blas, CUBLAS_FP32_EMULATED_BF16X9_MATH) != CUBLAS_STATUS_SUCCESS ||
            cublasSetMathMode(r.blas_panel, CUBLAS_FP32_EMULATED_BF16X9_MATH) != CUBLAS_STATUS_SUCCESS ||
            cusolverDnSetMathMode(r.solver, CUSOLVER_FP32_EMULATED_BF16X9_MATH) != CUSOLVER_STATUS_SUCCESS)
            return cudaErrorNotSupported;
        compute = CUBLAS_COMPUTE_32F_EMULATED_16BFX9;
    }
    int lwork = 0;
    if (cusolverDnSpotrf_bufferSize(r.solver, CUBLAS_FILL_MODE_LOWER, nb, A, (int)lda, &lwork) !=
        CUSOLVER_STATUS_SUCCESS)
        return cudaErrorUnknown;
    if ((e = pool_alloc_n(&r.work, (size_t)std::max(lwork, 1), stream)) ||
        (e = pool_alloc_n(&r.info, (size_t)steps, stream)) ||
        (e = cudaMemsetAsync(r.info, 0, sizeof(int) * steps, stream)))
        return e;
    auto at = [&](int64_t row, int64_t col) { return A + row + col * lda; };
    const float one = 1.f, minus = -1.f;
    auto factor_panel = [&](int64_t j, int jb, int64_t t) -> cudaError_t {
        if (cusolverDnSpotrf(r.solver, CUBLAS_FILL_MODE_LOWER, jb, at(j, j), (int)lda, r.work, lwork, r.info + t) !=
            CUSOLVER_STATUS_SUCCESS)
            return cudaErrorUnknown;
        const int64_t below = n - j - jb;
        if (below > 0 &&
            cublasStrsm(r.blas_panel, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT,
                        (int)below, jb, &one, at(j, j), (int)lda, at(j + jb, j), (int)lda) != CUBLAS_STATUS_SUCCESS)
            return cudaErrorUnknown;
        return cudaEventRecord(r.ready, r.panel);
    };
    // A[c:, c:c+w] -= L21[c-r0:] L21[c-r0 : c-r0+w]^T, L21 = A[r0:, j:j+jb]
    auto update = [&](int64_t j, int jb, int64_t c, int64_t w) -> bool {
        const int64_t rows = n - c;
        if (rows <= 0 || w <= 0) return true;
        return cublasGemmEx(r.blas, CUBLAS_OP_N, CUBLAS_OP_T, (int)rows, (int)w, jb, &minus, at(c, j), CUDA_R_32F,
                            (int)lda, at(c, j), CUDA_R_32F, (int)lda, &one, at(c, c), CUDA_R_32F, (int)lda, compute,
                            CUBLAS_GEMM_DEFAULT) == CUBLAS_STATUS_SUCCESS;
    };
    if ((e = cudaEventRecord(r.next, stream)) || (e = cudaStreamWaitEvent(r.panel, r.next, 0)) ||
        (e = factor_panel(0, nb, 0)))
        return e;
    for (int64_t t = 0; t < steps; ++t) {
        const int64_t j = t * nb;
        const int jb = (int)std::min<int64_t>(nb, n - j);
        const int64_t right = j + jb;
        if ((e = cudaStreamWaitEvent(stream, r.ready, 0))) return e;
        if (right >= n) break;
        const int64_t w0 = std::min<int64_t>(nb, n - right);
        if (!update(j, jb, right, w0)) return cudaErrorUnknown;
        if ((e = cudaEventRecord(r.next, stream)) || (e = cudaStreamWaitEvent(r.panel, r.next, 0)) ||
            (e = factor_panel(right, (int)w0, t + 1)))
            return e;
        for (int64_t c = right + w0; c < n; c += nb)
            if (!update(j, jb, c, std::min<int64_t>(nb, n - c))) return cudaErrorUnknown;
    }
    if ((e = cudaGetLastError()) || (e = cudaStreamSynchronize(r.panel)) || (e = cudaStreamSynchronize(stream)))
        return e;
    std::vector<int> info((size_t)steps);
    if ((e = cudaMemcpy(info.data(), r.info, sizeof(int) * steps, cudaMemcpyDeviceToHost))) return e;
    for (int64_t t = 0; t < steps; ++t)
        if (info[t] > 0) {
            *info_out = (int)(t * nb + info[t]);
            break;
        }
    return cudaSuccess;
}

}  // namespace pq

extern "C" int pcbqs_gb300_cholesky_f32(int64_t n, float *a, int64_t lda, int block, int math, int32_t *info,
                                        void *stream) {
    if (n <= 0 || lda < n || !a || !info || block < 32 || block > pq::MAX_BLOCK_PUBLIC || (math != 0 && math != 1))
        return pq::fail(pq::ERR_ARGUMENT, "cholesky_f32: invalid argument (lda >= n, block 32..%d, math 0 or 1)",
                        pq::MAX_BLOCK_PUBLIC);
    int order = 0;
    const cudaError_t e = pq::potrf_blocked(n, a, lda, block, math, static_cast<cudaStream_t>(stream), &order);
    *info = order;
    if (e) return pq::fail(pq::ERR_CUDA, "cholesky_f32: %s", cudaGetErrorString(e));
    return pq::OK;
}

namespace pq {

namespace {
std::string panel_key(int64_t n, int math) {
    return "lu_panel n=" + std::to_string(n) + " math=" + std::to_string(math);
}

// A diagonally dominant complex64 matrix for timing the factorization: a hashed value in [-1, 1) off the diagonal,
// n on it.
__global__ void k_timing_matrix(int64_t n, unsigned seed, float2 *A) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n; t += (int64_t)gridDim.x * blockDim.x) {
        unsigned h = (unsigned)(t * 2654435761ull) ^ seed;
        h ^= h >> 16;
        h *= 0x7feb352du;
        h ^= h >> 15;
        const float a = (float)(h & 0xffff) / 32768.f - 1.f, b = (float)(h >> 16) / 32768.f - 1.f;
        A[t] = (t / n == t % n) ? make_float2((float)n, 0.f) : make_float2(a, b);
    }
}
}  // namespace

int lu_panel_width(int64_t n, int math) {
    const int w = tune_get(panel_key(n, math));
    return w >= 32 && w <= MAX_BLOCK_PUBLIC ? w : 2048;
}

}  // namespace pq

extern "C" int pcbqs_gb300_tune_lu_panel(int64_t n, int math, const int32_t *widths, int count, int32_t *best,
                                         void *stream) {
    if (n <= 0 || math < 0 || math > 3 || !widths || count <= 0 || !best)
        return pq::fail(pq::ERR_ARGUMENT, "tune_lu_panel: invalid argument (math 0..3)");
    for (int i = 0; i < count; ++i)
        if (widths[i] < 32 || widths[i] > pq::MAX_BLOCK_PUBLIC)
            return pq::fail(pq::ERR_ARGUMENT, "tune_lu_panel: widths 32..%d", pq::MAX_BLOCK_PUBLIC);
    auto st = static_cast<cudaStream_t>(stream);
    float2 *A = nullptr;
    int *ipiv = nullptr;
    cudaError_t e;
    if ((e = pq::pool_alloc_n(&A, (size_t)n * n, st)) || (e = pq::pool_alloc_n(&ipiv, (size_t)n, st))) {
        pq::pool_free(A, st);
        return pq::fail(pq::ERR_MEMORY, "tune_lu_panel: %s", cudaGetErrorString(e));
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best_ms = 1e30f;
    int choice = -1;
    for (int i = 0; i < count && !e; ++i) {
        int zero = 0;
        pq::k_timing_matrix<<<152 * 8, 256, 0, st>>>(n, 12345u, A);
        pq::note_launches(1);
        if ((e = cudaEventRecord(e0, st))) break;
        if ((e = pq::getrf_blocked(n, A, ipiv, widths[i], math, st, &zero))) break;
        if ((e = cudaEventRecord(e1, st)) || (e = cudaEventSynchronize(e1))) break;
        float ms = 0;
        if ((e = cudaEventElapsedTime(&ms, e0, e1))) break;
        if (ms < best_ms) {
            best_ms = ms;
            choice = widths[i];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    pq::pool_free(A, st);
    pq::pool_free(ipiv, st);
    if (e) return pq::fail(e == cudaErrorLaunchTimeout ? pq::ERR_TIMEOUT : pq::ERR_CUDA, "tune_lu_panel: %s",
                           cudaGetErrorString(e));
    pq::tune_put(pq::panel_key(n, math), choice);
    *best = choice;
    return pq::OK;
}

extern "C" int pcbqs_gb300_lu_factor_c64(int64_t n, void *a, int32_t *ipiv, int block, int math, int32_t *singular,
                                         void *stream) {
    if (n <= 0 || !a || !ipiv || !singular || block < 32 || block > pq::MAX_BLOCK_PUBLIC || math < 0 || math > 3)
        return pq::fail(pq::ERR_ARGUMENT, "lu_factor_c64: invalid argument (block 32..%d, math 0..3)",
                        pq::MAX_BLOCK_PUBLIC);
    int zero = 0;
    const cudaError_t e = pq::getrf_blocked(n, static_cast<float2 *>(a), ipiv, block, math,
                                            static_cast<cudaStream_t>(stream), &zero);
    *singular = zero;
    if (e == cudaErrorLaunchTimeout)
        return pq::fail(pq::ERR_TIMEOUT, "lu_factor_c64: a bounded wait of the tensor-core update gave up");
    if (e) return pq::fail(pq::ERR_CUDA, "lu_factor_c64: %s", cudaGetErrorString(e));
    return pq::OK;
}

extern "C" int pcbqs_gb300_complex_update(int64_t rows, int64_t cols, int k, const void *a, int64_t lda,
                                          const void *b, int64_t ldb, void *c, int64_t ldc, int terms,
                                          uint64_t wait_cycles, void *stream) {
    if (rows < 0 || cols < 0 || k < 0 || !a || !b || !c || lda < rows || ldb < k || ldc < rows ||
        (terms != 3 && terms != 6) || wait_cycles == 0)
        return pq::fail(pq::ERR_ARGUMENT, "complex_update: invalid argument (terms 3 or 6, lda >= rows, ldb >= k, "
                                          "ldc >= rows, wait_cycles > 0)");
    if (rows == 0 || cols == 0 || k == 0) return pq::OK;
    auto st = static_cast<cudaStream_t>(stream);
    uint8_t *scratch = nullptr;
    int *flag = nullptr;
    cudaError_t e;
    if ((e = pq::pool_alloc_n(&scratch, pq::tc_update_scratch_bytes(rows, cols, k, terms), st)) ||
        (e = pq::pool_alloc_n(&flag, 1, st))) {
        pq::pool_free(scratch, st);
        return pq::fail(pq::ERR_MEMORY, "complex_update: scratch: %s", cudaGetErrorString(e));
    }
    int timed_out = 0;
    if (!(e = cudaMemsetAsync(flag, 0, sizeof(int), st)))
        e = pq::tc_update_c64(rows, cols, k, static_cast<const float2 *>(a), lda, static_cast<const float2 *>(b), ldb,
                              static_cast<float2 *>(c), ldc, terms, scratch, false, flag,
                              (unsigned long long)wait_cycles, st);
    if (!e) e = cudaMemcpyAsync(&timed_out, flag, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    pq::pool_free(scratch, st);
    pq::pool_free(flag, st);
    if (e) return pq::fail(pq::ERR_CUDA, "complex_update: %s", cudaGetErrorString(e));
    if (timed_out) return pq::fail(pq::ERR_TIMEOUT, "complex_update: a bounded wait of the tensor-core GEMM gave up");
    return pq::OK;
}
