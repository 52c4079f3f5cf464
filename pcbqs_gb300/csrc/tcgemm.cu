// C -= A B for complex64 matrices on the tcgen05 tensor cores (declared in tcgemm.cuh).
//
// The complex product is one real GEMM. With A = Ar + i Ai (rows x k) and B = Br + i Bi (k x cols):
//   Re C -= [Ar | Ai] [Br; -Bi],   Im C -= [Ar | Ai] [Bi; Br].
// Each FP32 value is split into BF16 parts x = h + m + l (h = bf16(x), m = bf16(x - h), l = bf16(x - h - m)), and
// the part products kept (3: hh, hm, mh; 6: also hl, mm, lh) are laid side by side along the inner dimension:
// A's plane holds, for every row, the segments [a_p(s) of Ar | Ai] and B's plane, for every output column (real
// and imaginary columns interleaved: plane row 2j is Re of column j, 2j + 1 its Im), the matching [b_q(s)]. One
// BF16 GEMM with FP32 accumulation of inner dimension K = terms · 2k then yields the FP32-accurate product
// (terms = 6) or one with about 16 correct bits (terms = 3).
//
// The GEMM: one CTA per 128 x 256 tile of the real product (128 rows of C by 128 of its complex columns), ten
// warps. Warp 8's elected thread streams 64-wide K slices of both planes into a 4-stage shared-memory ring by TMA
// (128-byte swizzle, one mbarrier per stage carrying the transaction bytes); warp 9's elected thread issues the
// tcgen05.mma (kind::f16, BF16 inputs, M 128, N 256, K 16: four per slice) and frees each stage through
// tcgen05.commit. Every 4 slices the sum restarts in the other of two 256-column tensor-memory buffers, and warps
// 0-7 add the finished buffer into FP32 registers (tcgen05.ld 32x32b, 128 sums a thread): the tensor core's own
// accumulation then never runs over more than 256 of the inner dimension, which keeps the six-term product at
// FP32's accuracy. At the end warps 0-7 subtract their sums from C, a warp's 32 rows of one column being 256
// contiguous bytes. One tile per CTA (not persistent) so that the LU's high-priority panel factorizations get SMs as
// tiles retire. Every wait is bounded in SM clocks; on timeout the CTA records ERR_TIMEOUT, waits (bounded) for its
// own copies and products in flight, frees its tensor memory and exits.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "tcgemm.cuh"
#include "tma.cuh"

namespace pq {

namespace {

constexpr int BM = 128, BN = 256, BK = 64, STAGES = 4;
constexpr int FOLD_WARPS = 8, PRODUCER_WARP = 8, MMA_WARP = 9, THREADS = 320;
constexpr int FOLD_THREADS = FOLD_WARPS * 32;
constexpr int A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2, STAGE_BYTES = A_BYTES + B_BYTES;
// The accumulator is promoted to FP32 registers every CHUNK K slices (256 of the inner dimension): the tensor
// core's own FP32 accumulation over a long inner dimension loses accuracy with every product it adds (measured: a
// normwise error of 1.25e-6 over 24,576 terms against cuBLAS FP32's 1.6e-8), so each chunk starts a fresh sum in
// one of two 256-column tensor-memory buffers while the fold warps add the previous chunk's into registers.
constexpr int CHUNK = 4;
constexpr int TMEM_COLS = 2 * BN;
constexpr size_t SMEM = (size_t)STAGES * STAGE_BYTES + 1024 + 256;   // ring, 1024-byte alignment slack, barriers
constexpr int KPAD = 32;                                             // k padded to a multiple of 32 (K % 64 == 0)
// limit of the waits for this CTA's own copies and products in flight before it exits (these complete on their
// own; the caller's limit only bounds the waits on the pipeline's progress)
constexpr unsigned long long DRAIN_CYCLES = DRAIN_WAIT_CYCLES;

// part indices of A and B in each product segment
__constant__ int8_t SEG_A[6] = {0, 0, 1, 0, 1, 2};
__constant__ int8_t SEG_B[6] = {0, 1, 0, 2, 1, 0};

__device__ __forceinline__ void split3(float x, __nv_bfloat16 &h, __nv_bfloat16 &m, __nv_bfloat16 &l) {
    h = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(h);
    m = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(m);
    l = __float2bfloat16_rn(r2);
}

__device__ __forceinline__ __nv_bfloat16 pick(int p, __nv_bfloat16 h, __nv_bfloat16 m, __nv_bfloat16 l) {
    return p == 0 ? h : (p == 1 ? m : l);
}

// A's plane: row r, segment s, position 2t + c = part SEG_A[s] of component c (re, im) of A[r, t]; zero for t >= k.
// 32 rows x 32 k per block, transposed through shared memory so both the column-major reads and the row writes
// are contiguous.
__global__ void __launch_bounds__(256) k_pack_a(int64_t rows, int k, int kp, int terms, const float2 *A, int64_t lda,
                                                __nv_bfloat162 *out) {
    __shared__ float2 tile[32][33];
    const int64_t r0 = (int64_t)blockIdx.x * 32;
    const int t0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int j = ty; j < 32; j += 8) {
        const int64_t r = r0 + tx;
        const int t = t0 + j;
        tile[j][tx] = (r < rows && t < k) ? A[r + (int64_t)t * lda] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int64_t K2 = (int64_t)kp;          // bf16 pairs per segment (kp complex values)
    for (int j = ty; j < 32; j += 8) {
        const int64_t r = r0 + j;
        if (r >= rows) continue;
        const int t = t0 + tx;
        const float2 v = tile[tx][j];
        __nv_bfloat16 rh, rm, rl, ih, im, il;
        split3(v.x, rh, rm, rl);
        split3(v.y, ih, im, il);
        __nv_bfloat162 *row = out + r * (K2 * terms);
        for (int s = 0; s < terms; ++s) {
            const int p = SEG_A[s];
            row[s * K2 + t] = __halves2bfloat162(pick(p, rh, rm, rl), pick(p, ih, im, il));
        }
    }
}

// B's plane: row 2j (Re of column j) holds (Br, -Bi) at positions (2t, 2t + 1), row 2j + 1 (Im) holds (Bi, Br),
// each value's part SEG_B[s] in segment s. B's columns are contiguous in t, as are the plane's rows.
__global__ void __launch_bounds__(256) k_pack_b(int64_t cols, int k, int kp, int terms, const float2 *B, int64_t ldb,
                                                __nv_bfloat162 *out) {
    const int64_t K2 = (int64_t)kp;
    for (int64_t j = blockIdx.y; j < cols; j += gridDim.y) {
        const float2 *col = B + j * ldb;
        __nv_bfloat162 *re = out + (2 * j) * (K2 * terms), *imr = re + K2 * terms;
        for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < kp; t += gridDim.x * blockDim.x) {
            const float2 v = t < k ? col[t] : make_float2(0.f, 0.f);
            __nv_bfloat16 rh, rm, rl, ih, im, il;
            split3(v.x, rh, rm, rl);
            split3(v.y, ih, im, il);
            for (int s = 0; s < terms; ++s) {
                const int q = SEG_B[s];
                const __nv_bfloat16 br = pick(q, rh, rm, rl), bi = pick(q, ih, im, il);
                re[s * K2 + t] = __halves2bfloat162(br, __hneg(bi));
                imr[s * K2 + t] = __halves2bfloat162(bi, br);
            }
        }
    }
}

// ---- the low-rank product (the H-matrix's far blocks) ----
// X (n x k complex128, row-major) into its transposed BF16 plane: row c = real column c (2c' = Re, 2c' + 1 = Im of
// column c'), part h at pad_pos[i], part m at n_pad + pad_pos[i]. 32 x 32 blocks transposed through shared memory.
__global__ void __launch_bounds__(256) k_pack_xt(int64_t n, int ncols, const double *X, const int32_t *pad_pos,
                                                 int64_t n_pad, __nv_bfloat16 *out) {
    __shared__ float tile[32][33];
    const int64_t i0 = (int64_t)blockIdx.x * 32;
    const int c0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int r = ty; r < 32; r += 8) {
        const int64_t i = i0 + r;
        const int c = c0 + tx;
        tile[r][tx] = (i < n && c < ncols) ? (float)X[i * ncols + c] : 0.f;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int c = c0 + r;
        const int64_t i = i0 + tx;
        if (c >= ncols || i >= n) continue;
        __nv_bfloat16 h, m, l;
        split3(tile[tx][r], h, m, l);
        __nv_bfloat16 *row = out + (int64_t)c * 2 * n_pad;
        const int64_t p = pad_pos[i];
        row[p] = h;
        row[n_pad + p] = m;
    }
}

// ---- the row-major complex update (the triangular solves' products) ----
// A's plane from a row-major complex64 A (row r contiguous in t): the same layout as k_pack_a.
__global__ void __launch_bounds__(256) k_pack_a_rows(int64_t rows, int k, int kp, int terms, const float2 *A,
                                                     int64_t lda, __nv_bfloat162 *out) {
    const int64_t K2 = kp;
    for (int64_t r = blockIdx.y; r < rows; r += gridDim.y) {
        const float2 *src = A + r * lda;
        __nv_bfloat162 *row = out + r * (K2 * terms);
        for (int t = blockIdx.x * 256 + threadIdx.x; t < kp; t += gridDim.x * 256) {
            const float2 v = t < k ? src[t] : make_float2(0.f, 0.f);
            __nv_bfloat16 rh, rm, rl, ih, im, il;
            split3(v.x, rh, rm, rl);
            split3(v.y, ih, im, il);
            for (int s = 0; s < terms; ++s) {
                const int p = SEG_A[s];
                row[s * K2 + t] = __halves2bfloat162(pick(p, rh, rm, rl), pick(p, ih, im, il));
            }
        }
    }
}

// B's plane from a row-major complex64 B (k x cols, leading dimension ldb): the layout of k_pack_b, each 32 x 32
// block transposed through shared memory.
__global__ void __launch_bounds__(256) k_pack_b_rows(int64_t cols, int k, int kp, int terms, const float2 *B,
                                                     int64_t ldb, __nv_bfloat162 *out) {
    __shared__ float2 tile[32][33];
    const int64_t t0 = (int64_t)blockIdx.x * 32, j0 = (int64_t)blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int i = ty; i < 32; i += 8) {
        const int64_t t = t0 + i, j = j0 + tx;
        tile[i][tx] = (t < k && j < cols) ? B[t * ldb + j] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int64_t K2 = kp;
    for (int i = ty; i < 32; i += 8) {
        const int64_t j = j0 + i;
        if (j >= cols) continue;
        const int64_t t = t0 + tx;
        const float2 v = tile[tx][i];
        __nv_bfloat16 rh, rm, rl, ih, im, il;
        split3(v.x, rh, rm, rl);
        split3(v.y, ih, im, il);
        __nv_bfloat162 *re = out + (2 * j) * (K2 * terms), *imr = re + K2 * terms;
        for (int s = 0; s < terms; ++s) {
            const int q = SEG_B[s];
            const __nv_bfloat16 br = pick(q, rh, rm, rl), bi = pick(q, ih, im, il);
            re[s * K2 + t] = __halves2bfloat162(br, __hneg(bi));
            imr[s * K2 + t] = __halves2bfloat162(bi, br);
        }
    }
}

// ---- the FP64-accurate product (integer slices) ----
// A value x of a row (column) whose entries are all below 2^e in magnitude is x = 2^(e-7) sum_s a_s 2^(-8s) + r with
// integer slices |a_s| <= 128 (exact in BF16) and |r| <= 2^(e-7) 2^(-8S-1) after S slices: a_0 = rint(x 2^(7-e)),
// then each remainder times 256 rounded again. A product of two slices is an integer below 2^14 in magnitude, so a
// chunk of 256 of them sums exactly in the tensor core's FP32 accumulator; the fold warps add the chunks as 32-bit
// integers and carry the sum of every level (slice pairs (i, j) of equal i + j, weight 2^(-8(i+j))) into the FP64
// result. Pairs above level S - 1 are dropped; they weigh less than the representation error.
constexpr int MAX_SLICES = 7;
constexpr int MAX_PAIRS = MAX_SLICES * (MAX_SLICES + 1) / 2;
// the pairs (i, j) in order of level i + j: the first S (S + 1) / 2 are those of S slices
__constant__ int8_t PAIR_A[MAX_PAIRS] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3, 0, 1, 2, 3, 4, 0, 1, 2, 3, 4, 5, 0, 1, 2, 3, 4, 5, 6};
__constant__ int8_t PAIR_B[MAX_PAIRS] = {0, 1, 0, 2, 1, 0, 3, 2, 1, 0, 4, 3, 2, 1, 0, 5, 4, 3, 2, 1, 0, 6, 5, 4, 3, 2, 1, 0};
__constant__ int8_t PAIR_LEVEL[MAX_PAIRS] = {0, 1, 1, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 4,
                                             5, 5, 5, 5, 5, 5, 6, 6, 6, 6, 6, 6, 6};

// e such that |x| < 2^e (-1022 for zero and subnormals)
__device__ __forceinline__ int bound_exponent(double x) {
    return (int)((__double_as_longlong(x) >> 52) & 0x7ff) - 1022;
}

// x's slices under bound exponent e, most significant first, in integer arithmetic on x's bits (the FP64 pipe is
// slow): q = x 2^(7 - e + 8 (slices - 1)) rounded to an integer (|q| <= 2^(7 + 8 (slices - 1))), then q's balanced
// base-256 digits (the lower ones in [-128, 127], the leading one in [-128, 128]). NaN and infinity give zeros (their
// rows and columns are marked by their exponent 1025).
__device__ __forceinline__ void slice_digits(double x, int e, int slices, int (&d)[MAX_SLICES]) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int E = (int)((bits >> 52) & 0x7ff);
    long long q = 0;
    if (E != 0x7ff) {
        unsigned long long m = bits & 0xFFFFFFFFFFFFFull;
        if (E) m |= 1ull << 52;
        const int ex = E ? E - 1075 : -1074;                   // x = +-m 2^ex
        const int sh = -(ex + 7 - e + 8 * (slices - 1));       // q = m 2^-sh
        unsigned long long mag;
        if (sh <= 0) mag = m << (-sh);                         // sh >= -2 since |x| < 2^e and slices <= 7
        else if (sh >= 60) mag = 0;                            // m < 2^53: rounds to zero
        else mag = (m + (1ull << (sh - 1))) >> sh;
        q = (bits >> 63) ? -(long long)mag : (long long)mag;
    }
#pragma unroll
    for (int s = MAX_SLICES - 1; s >= 1; --s) {
        if (s < slices) {
            const long long digit = ((q + 128) & 255) - 128;
            d[s] = (int)digit;
            q = (q - digit) / 256;                             // exact
        }
    }
    d[0] = (int)q;
}

__device__ __forceinline__ void write_slices(double x, int e, int slices, int64_t kp, int64_t t, __nv_bfloat16 *row) {
    int d[MAX_SLICES];
    slice_digits(x, e, slices, d);
#pragma unroll
    for (int s = 0; s < MAX_SLICES; ++s)
        if (s < slices) row[s * kp + t] = __int2bfloat16_rn(d[s]);
}

// M's slice plane (rows x slices x kp, row-major FP64 M with leading dimension ldm) and its row exponents; one
// block per row: the row's bound exponent, then its slices (zero for kdim <= t < kp).
__global__ void __launch_bounds__(256) k_slice_rows(int64_t rows, int64_t kdim, int64_t kp, int slices,
                                                    const double *M, int64_t ldm, __nv_bfloat16 *out, int *row_exp) {
    __shared__ int part[8];
    for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
        const double *src = M + r * ldm;
        int e = -1022;
        for (int64_t t = threadIdx.x; t < kdim; t += 256) e = max(e, bound_exponent(src[t]));
        for (int o = 16; o; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
        if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = e;
        __syncthreads();
        e = part[0];
        for (int w = 1; w < 8; ++w) e = max(e, part[w]);
        __syncthreads();
        // two neighbouring entries per thread, stored as BF16 pairs (kp is even)
        __nv_bfloat162 *row = reinterpret_cast<__nv_bfloat162 *>(out + r * kp * slices);
        const int64_t half = kp / 2;
        for (int64_t u = threadIdx.x; u < half; u += 256) {
            const int64_t t = 2 * u;
            int d0[MAX_SLICES], d1[MAX_SLICES];
            slice_digits(t < kdim ? src[t] : 0.0, e, slices, d0);
            slice_digits(t + 1 < kdim ? src[t + 1] : 0.0, e, slices, d1);
#pragma unroll
            for (int s = 0; s < MAX_SLICES; ++s)
                if (s < slices)
                    row[s * half + u] = __halves2bfloat162(__int2bfloat16_rn(d0[s]), __int2bfloat16_rn(d1[s]));
        }
        if (threadIdx.x == 0) row_exp[r] = e;
    }
}

// Column bound exponents of X (kdim x ncols real, row-major, leading dimension ldxr) into col_exp (preset to a value
// below -1022): 32 columns (one per lane) by stretches of 256 rows, gridDim.x stretches apart.
__global__ void __launch_bounds__(256) k_column_exponents(int64_t kdim, int64_t ncols, const double *X, int64_t ldxr,
                                                          int *col_exp) {
    __shared__ int part[8][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t j = (int64_t)blockIdx.y * 32 + lane;
    int e = -1022;
    if (j < ncols)
        for (int64_t t0 = (int64_t)blockIdx.x * 256; t0 < kdim; t0 += (int64_t)gridDim.x * 256)
            for (int64_t t = t0 + w; t < kdim && t < t0 + 256; t += 8) e = max(e, bound_exponent(X[t * ldxr + j]));
    part[w][lane] = e;
    __syncthreads();
    if (w == 0 && j < ncols) {
        for (int i = 1; i < 8; ++i) e = max(e, part[i][lane]);
        atomicMax(col_exp + j, e);
    }
}

// X's slice plane: plane row j (X's real column j) holds its slices along t, scaled by its column exponent; 32 x 32
// blocks transposed through shared memory.
__global__ void __launch_bounds__(256) k_slice_cols(int64_t kdim, int64_t kp, int64_t ncols, int slices,
                                                    const double *X, int64_t ldxr, const int *col_exp,
                                                    __nv_bfloat16 *out) {
    __shared__ double tile[32][33];
    const int64_t t0 = (int64_t)blockIdx.x * 32, j0 = (int64_t)blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int i = ty; i < 32; i += 8) {
        const int64_t t = t0 + i, j = j0 + tx;
        tile[i][tx] = (t < kdim && j < ncols) ? X[t * ldxr + j] : 0.0;
    }
    __syncthreads();
    for (int i = ty; i < 32; i += 8) {
        const int64_t j = j0 + i;
        if (j >= ncols) continue;
        write_slices(tile[tx][i], max(col_exp[j], -1022), slices, kp, t0 + tx, out + j * kp * slices);
    }
}

// Y (rows x cols complex128) times 2^(row exponent + column exponent - 14): the slices' scales. A bound exponent
// of 1025 marks a NaN or infinity in the row or column: its results are NaN.
__device__ __forceinline__ double scaled(double v, int er, int ec) {
    return (er > 1024 || ec > 1024) ? __longlong_as_double(0x7ff8000000000000LL) : ldexp(v, er + ec - 14);
}

__global__ void k_exact_scale(int64_t rows, int64_t cols, double2 *Y, int64_t ldy, const int *row_exp,
                              const int *col_exp) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows * cols;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / cols, c = i - r * cols;
        double2 *p = Y + r * ldy + c;
        double2 v = *p;
        v.x = scaled(v.x, row_exp[r], max(col_exp[2 * c], -1022));
        v.y = scaled(v.y, row_exp[r], max(col_exp[2 * c + 1], -1022));
        *p = v;
    }
}

// The real operand's plane (the dense product Y = M X): row r, segment s, position t = part SEG_A[s] of M[r, t] (M
// row-major FP32, leading dimension ldm); zero for kdim <= t < kp.
__global__ void __launch_bounds__(256) k_pack_rows(int64_t rows, int64_t kdim, int64_t kp, int terms, const float *M,
                                                   int64_t ldm, __nv_bfloat16 *out) {
    for (int64_t r = blockIdx.y; r < rows; r += gridDim.y) {
        const float *src = M + r * ldm;
        __nv_bfloat16 *row = out + r * kp * terms;
        for (int64_t t = (int64_t)blockIdx.x * 256 + threadIdx.x; t < kp; t += (int64_t)gridDim.x * 256) {
            __nv_bfloat16 h, m, l;
            split3(t < kdim ? src[t] : 0.f, h, m, l);
            for (int s = 0; s < terms; ++s) row[s * kp + t] = pick(SEG_A[s], h, m, l);
        }
    }
}

// The right-hand sides' plane: X (kdim x cols complex128, row-major, leading dimension ldx) seen as the real
// kdim x 2cols matrix Xr; plane row j holds column j of Xr (so rows 2c, 2c + 1 are Re and Im of column c), each
// value rounded to FP32 and its part SEG_B[s] written in segment s. 32 x 32 blocks transposed through shared memory.
__global__ void __launch_bounds__(256) k_pack_cols(int64_t kdim, int64_t kp, int64_t ncols, int terms,
                                                   const double *X, int64_t ldxr, __nv_bfloat16 *out) {
    __shared__ float tile[32][33];
    const int64_t t0 = (int64_t)blockIdx.x * 32, j0 = (int64_t)blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int i = ty; i < 32; i += 8) {
        const int64_t t = t0 + i, j = j0 + tx;
        tile[i][tx] = (t < kdim && j < ncols) ? (float)X[t * ldxr + j] : 0.f;
    }
    __syncthreads();
    for (int i = ty; i < 32; i += 8) {
        const int64_t j = j0 + i;
        if (j >= ncols) continue;
        const int64_t t = t0 + tx;
        __nv_bfloat16 h, m, l;
        split3(tile[tx][i], h, m, l);
        __nv_bfloat16 *row = out + j * kp * terms;
        for (int s = 0; s < terms; ++s) row[s * kp + t] = pick(SEG_B[s], h, m, l);
    }
}

// ---- tcgen05 / TMA primitives (inline PTX, sm_100 family) ----

// Shared-memory matrix descriptor of a K-major operand tile in the 128-byte swizzle layout that TMA writes with
// CU_TENSOR_MAP_SWIZZLE_128B: rows of 128 bytes, 8-row groups 1024 bytes apart (stride byte offset), the leading
// byte offset unused for this layout, descriptor version 1, layout type 2 (128-byte swizzle). The tile base is
// 1024-byte aligned; a K step of 16 elements inside the 128-byte row adds 32 bytes to the start address.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1), both
// K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tma_prefetch(const CUtensorMap *map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(a), "l"(b), "r"(IDESC), "r"(accumulate)
        : "memory");
}

// Arrive on `bar` once every tcgen05.mma issued so far by this thread has completed.
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Wait for phase parity `parity` of `bar`, giving up after `limit` SM clocks or, when `abort` is given, as soon as
// another thread of the CTA has given up (*abort set). Returns false on giving up.
__device__ __forceinline__ bool wait_bounded(uint64_t *bar, uint32_t parity, unsigned long long limit,
                                             volatile int *abort) {
    const long long t0 = clock64();
    const bool probe = limit < PROBE_BELOW_CYCLES;
    for (uint32_t i = 0;; ++i) {
        if (probe ? mbar_test_wait(bar, parity) : mbar_try_wait(bar, parity)) return true;
        if ((unsigned long long)(clock64() - t0) > limit || ((i & 15) == 15 && abort && *abort)) return false;
    }
}

struct TileArgs {
    int64_t rows, cols;          // C's size (complex); the low-rank modes: cols = right-hand sides
    const LrGroup *groups;       // the low-rank modes' groups
    const int *tile_group, *tile_m;   // MODE 5: each tile's group and row tile
    int a_pitch, b_pitch;        // the low-rank modes: part pitch (elements) of the A and B planes along K
    __nv_bfloat16 *tplane;       // MODE 4's output: the T plane (MODE 5's B operand)
    double2 *slots;              // MODE 5's output rows
    float2 *C;
    int64_t ldc;
    double2 *Y;                  // the real-operand product's output (row-major, leading dimension ldy)
    int64_t ldy;
    int kblocks;                 // K / 64
    int seg_kblocks;             // the FP64-accurate product: 64-wide K slices per slice segment
    int tiles_m, tiles_n;        // row and column tiles
    int *error;
    unsigned long long wait;
};

// MODE 6: the dense leaves, Y[I] = D_g X[J_g] over (group, row tile) tiles: A = the dense plane at a_row0 (K: J's
// padded range in parts of dpitch), B = X's transposed plane at J's padded range; stored into the slot rows.
// MODE 4 / 5: the two phases of the low-rank product (LrGroup): 4 T_g = R_g X[J_g] (A = R's plane, 128 rows
// of which rank_g hold R_g; B = X's transposed plane at J_g's padded range; K = 3 part segments of kb slices), its
// tile written as the BF16 parts of T_g^T into the T plane; 5 Y[I_g] = L_g T_g (A = L's plane at a_row0, B = the
// T plane at t_row0, K = 3 one-slice segments), each tile stored into its group's slot rows.
// MODE 0: C -= D into a column-major complex64 C (the complex update); 3: the same into a row-major C; 1: Y = D into a row-major complex128 Y, D's
// columns 2c, 2c + 1 being column c's real and imaginary parts (the real-operand product); 2: the same Y from
// integer slices (the FP64-accurate product): K runs over the slice pairs in level order, each pair a segment of
// seg_kblocks slices of its A and B slice planes, and the fold warps keep 32-bit integer sums that they carry into Y
// (FP64) at every change of level, before 511 chunks could overflow them, and at the end.
template <int MODE>
__global__ void __launch_bounds__(THREADS, 1) k_tc_update(const __grid_constant__ CUtensorMap map_a,
                                                          const __grid_constant__ CUtensorMap map_b, TileArgs args) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE_BYTES);
    uint64_t *empty = full + STAGES;
    uint64_t *cfull = empty + STAGES;      // [2] a chunk's sum is complete in tensor-memory buffer b
    uint64_t *cempty = cfull + 2;          // [2] the fold warps have read buffer b
    uint64_t *drained = cempty + 2;        // every product issued has completed
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(drained + 1);
    volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // tiles in groups of GROUP row tiles, the row tile fastest within a group: the CTAs resident at one time share
    // a few A strips and B strips in L2
    constexpr int GROUP = 16;
    const int per_group = GROUP * args.tiles_n;
    const int first_m = (int)(blockIdx.x / per_group) * GROUP;
    const int in_group = (int)(blockIdx.x % per_group);
    const int gm = min(GROUP, args.tiles_m - first_m);
    int m_tile = first_m + in_group % gm, n_tile = in_group / gm;
    int kb_total = args.kblocks;
    LrGroup grp{};
    if (MODE == 4) {                       // one tile per group
        grp = args.groups[blockIdx.x];
        m_tile = 0;
        n_tile = 0;
        kb_total = 3 * grp.kb;
    } else if (MODE == 5) {
        grp = args.groups[args.tile_group[blockIdx.x]];
        m_tile = args.tile_m[blockIdx.x];
        n_tile = 0;
        kb_total = 3;
    } else if (MODE == 6) {
        grp = args.groups[args.tile_group[blockIdx.x]];
        m_tile = args.tile_m[blockIdx.x];
        n_tile = 0;
        kb_total = 3 * grp.kb;
    }
    const int64_t m0 = (int64_t)m_tile * BM;
    const int nchunks = (kb_total + CHUNK - 1) / CHUNK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&cfull[b], 1);
            mbar_init(&cempty[b], FOLD_THREADS);
        }
        mbar_init(drained, 1);
        *abort = 0;
        mbar_fence_init();
        tma_prefetch(&map_a);
        tma_prefetch(&map_b);
    }
    __syncwarp();
    if (warp == PRODUCER_WARP) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const uint32_t ring = smem_addr(smem);

    if (warp == PRODUCER_WARP) {
        if (lane == 0) {
            // producer: slice kb into stage kb % STAGES once the MMA has released it
            bool ok = true;
            int issued_last[STAGES];
            for (int s = 0; s < STAGES; ++s) issued_last[s] = -1;
            for (int kb = 0; kb < kb_total; ++kb) {
                const int s = kb % STAGES;
                if (!wait_bounded(&empty[s], ((kb / STAGES) & 1) ^ 1, args.wait, abort)) {
                    ok = false;
                    break;
                }
                mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
                const uint32_t a_dst = ring + s * STAGE_BYTES, b_dst = a_dst + A_BYTES;
                int xa = kb * BK, xb = kb * BK, ya = (int)m0, yb = n_tile * BN;
                if (MODE == 2) {
                    const int p = kb / args.seg_kblocks, off = (kb - p * args.seg_kblocks) * BK;
                    xa = PAIR_A[p] * args.seg_kblocks * BK + off;
                    xb = PAIR_B[p] * args.seg_kblocks * BK + off;
                } else if (MODE == 4) {
                    const int sg = kb / grp.kb, off = (kb - sg * grp.kb) * BK;
                    xa = SEG_A[sg] * args.a_pitch + grp.b_x0 + off;
                    xb = SEG_B[sg] * args.b_pitch + grp.a_x0 + off;
                    ya = 0;
                    yb = 0;
                } else if (MODE == 5) {
                    xa = SEG_A[kb] * BK;
                    xb = SEG_B[kb] * BK;
                    ya = grp.a_row0 + (int)m0;
                    yb = grp.t_row0;
                } else if (MODE == 6) {
                    const int sg = kb / grp.kb, off = (kb - sg * grp.kb) * BK;
                    xa = SEG_A[sg] * args.a_pitch + off;
                    xb = SEG_B[sg] * args.b_pitch + grp.a_x0 + off;
                    ya = grp.a_row0 + (int)m0;
                    yb = 0;
                }
                tma_load_2d(a_dst, &map_a, xa, ya, smem_addr(&full[s]));
                tma_load_2d(b_dst, &map_b, xb, yb, smem_addr(&full[s]));
                issued_last[s] = kb;
            }
            if (!ok) {
                *abort = 1;
                atomicExch(args.error, ERR_TIMEOUT);
            }
            // every copy issued has landed before the CTA may exit (already true when the MMA consumed them all)
            for (int s = 0; s < STAGES; ++s)
                if (issued_last[s] >= 0)
                    wait_bounded(&full[s], (issued_last[s] / STAGES) & 1, DRAIN_CYCLES, nullptr);
        }
    } else if (warp == MMA_WARP) {
        if (lane == 0) {
            // MMA issuer: chunk c accumulates afresh in buffer c & 1 once the fold warps have read its last use
            bool ok = true;
            for (int kb = 0; kb < kb_total; ++kb) {
                const int c = kb / CHUNK, buf = c & 1;
                const bool first = kb % CHUNK == 0;
                if (first) {
                    if (!wait_bounded(&cempty[buf], ((c >> 1) & 1) ^ 1, args.wait, abort)) {
                        ok = false;
                        break;
                    }
                    fence_after_sync();
                }
                const int s = kb % STAGES;
                if (!wait_bounded(&full[s], (kb / STAGES) & 1, args.wait, abort)) {
                    ok = false;
                    break;
                }
                fence_after_sync();
                const uint32_t a_base = ring + s * STAGE_BYTES, b_base = a_base + A_BYTES;
                const uint32_t d = tmem + buf * BN;
#pragma unroll
                for (int kk = 0; kk < BK / 16; ++kk)
                    mma_bf16(d, sw128_desc(a_base + kk * 32), sw128_desc(b_base + kk * 32), !first || kk != 0);
                mma_commit(smem_addr(&empty[s]));
                if (kb % CHUNK == CHUNK - 1 || kb == kb_total - 1) mma_commit(smem_addr(&cfull[buf]));
            }
            if (!ok) {
                *abort = 1;
                atomicExch(args.error, ERR_TIMEOUT);
            }
            mma_commit(smem_addr(drained));       // after every product issued (also on the way out)
        }
    } else {
        // fold warps: warp w reads tensor-memory lanes (tile rows) 32 (w % 4) .. + 31, columns 128 (w / 4) .. + 127,
        // and keeps their running FP32 sums in registers; then subtracts them from C, a warp's 32 rows of one
        // column being 256 contiguous bytes
        const int q = warp & 3, h = warp >> 2;
        const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + h * (BN / 2);
        float acc[BN / 2];        // MODE 2: the bits of 32-bit integer sums
#pragma unroll
        for (int i = 0; i < BN / 2; ++i) acc[i] = 0.f;
        bool good = true;
        if (MODE == 2) {
            // runs of chunks of one level (at most 511: |sum| < 2^31), each carried into Y after its last chunk
            bool stored = false;  // Y holds this tile's earlier runs
            for (int c = 0; c < nchunks && good;) {
                const int level = PAIR_LEVEL[(c * CHUNK) / args.seg_kblocks];
                int end = c + 1;
                while (end < nchunks && end - c < 511 && PAIR_LEVEL[(end * CHUNK) / args.seg_kblocks] == level) ++end;
                // an integer-valued FP32 sum |v| <= 2^22 as an integer: the bits of v + 1.5 * 2^23 are
                // v + 0x4B400000; the sums carry that offset once per chunk (wrapping), removed at the carry
                const unsigned offset = (unsigned)(end - c) * 0x4B400000u;
                for (; c < end; ++c) {
                    const int buf = c & 1;
                    const bool landed = wait_bounded(&cfull[buf], (c >> 1) & 1, args.wait, abort);
                    if (!__all_sync(0xffffffffu, landed)) {
                        good = false;
                        break;
                    }
                    fence_after_sync();
#pragma unroll
                    for (int j = 0; j < BN / 2 / 16; ++j) {
                        uint32_t r[16];
                        tmem_ld16(taddr + buf * BN + j * 16, r);
#pragma unroll
                        for (int i = 0; i < 16; ++i)
                            acc[j * 16 + i] = __int_as_float(__float_as_int(acc[j * 16 + i]) +
                                                             __float_as_int(__uint_as_float(r[i]) + 12582912.0f));
                    }
                    fence_before_sync();
                    mbar_arrive(&cempty[buf]);
                }
                if (!good) break;
                const int64_t row = m0 + q * 32 + lane;
                const int64_t c0 = (int64_t)n_tile * (BN / 2) + h * (BN / 4);
                const double w = __longlong_as_double((long long)(1023 - 8 * level) << 52);
                if (row < args.rows) {
                    double2 *base = args.Y + row * args.ldy + c0;
#pragma unroll
                    for (int j = 0; j < BN / 4; ++j)
                        if (c0 + j < args.cols) {
                            double2 v = stored ? base[j] : make_double2(0.0, 0.0);
                            v.x = fma((double)(int)(__float_as_uint(acc[2 * j]) - offset), w, v.x);
                            v.y = fma((double)(int)(__float_as_uint(acc[2 * j + 1]) - offset), w, v.y);
                            base[j] = v;
                        }
                }
#pragma unroll
                for (int i = 0; i < BN / 2; ++i) acc[i] = 0.f;
                stored = true;
            }
        } else {
            for (int c = 0; c < nchunks; ++c) {
                const int buf = c & 1;
                const bool landed = wait_bounded(&cfull[buf], (c >> 1) & 1, args.wait, abort);
                if (!__all_sync(0xffffffffu, landed)) {
                    good = false;
                    break;
                }
                fence_after_sync();
#pragma unroll
                for (int j = 0; j < BN / 2 / 32; ++j) {
                    uint32_t r[32];
                    tmem_ld32(taddr + buf * BN + j * 32, r);
#pragma unroll
                    for (int i = 0; i < 32; ++i) acc[j * 32 + i] += __uint_as_float(r[i]);
                }
                fence_before_sync();
                mbar_arrive(&cempty[buf]);
            }
        }
        if (!good) {
            if (lane == 0) {
                *abort = 1;
                atomicExch(args.error, ERR_TIMEOUT);
            }
        } else if (MODE == 2) {
            // Y complete (its scales applied by k_exact_scale)
        } else if (!*abort && MODE == 4) {
            // rows of D: ranks j; columns: the right-hand sides' real columns c. T^T's plane row c holds the parts
            // h, m of T[j, c] at j and 64 + j (zero from the group's rank to 64).
            const int j = q * 32 + lane;
            if (j < 64) {
                const int c0 = h * (BN / 2);
                __nv_bfloat16 *trow = args.tplane + (int64_t)grp.t_row0 * 128;
#pragma unroll
                for (int i = 0; i < BN / 2; ++i) {
                    const int c = c0 + i;
                    if (c < 2 * args.cols) {
                        __nv_bfloat16 vh, vm, vl;
                        split3(j < grp.rank ? acc[i] : 0.f, vh, vm, vl);
                        trow[(int64_t)c * 128 + j] = vh;
                        trow[(int64_t)c * 128 + 64 + j] = vm;
                    }
                }
            }
        } else if (!*abort && (MODE == 5 || MODE == 6)) {
            const int64_t row = m0 + q * 32 + lane;
            const int64_t c0 = h * (BN / 4);
            if (row < grp.rows) {
                double2 *base = args.slots + (grp.slot0 + row) * args.cols;
#pragma unroll
                for (int j = 0; j < BN / 4; ++j)
                    if (c0 + j < args.cols) base[c0 + j] = make_double2(acc[2 * j], acc[2 * j + 1]);
            }
        } else if (!*abort && MODE == 3) {
            const int64_t row = m0 + q * 32 + lane;
            const int64_t c0 = (int64_t)n_tile * (BN / 2) + h * (BN / 4);
            if (row < args.rows) {
                float2 *base = args.C + row * args.ldc;
#pragma unroll
                for (int j = 0; j < BN / 4; ++j)
                    if (c0 + j < args.cols) {
                        float2 v = base[c0 + j];
                        v.x -= acc[2 * j];
                        v.y -= acc[2 * j + 1];
                        base[c0 + j] = v;
                    }
            }
        } else if (!*abort && MODE == 1) {
            const int64_t row = m0 + q * 32 + lane;
            const int64_t c0 = (int64_t)n_tile * (BN / 2) + h * (BN / 4);
            if (row < args.rows) {
                double2 *base = args.Y + row * args.ldy;
#pragma unroll
                for (int j = 0; j < BN / 4; ++j)
                    if (c0 + j < args.cols) base[c0 + j] = make_double2(acc[2 * j], acc[2 * j + 1]);
            }
        } else if (!*abort) {
            const int64_t row = m0 + q * 32 + lane;
            const int64_t c0 = (int64_t)n_tile * (BN / 2) + h * (BN / 4);
            if (row < args.rows) {
                float2 *base = args.C + row;
#pragma unroll
                for (int j = 0; j < BN / 4; ++j) {
                    const int64_t col = c0 + j;
                    if (col < args.cols) {
                        float2 *p = base + col * args.ldc;
                        float2 v = *p;
                        v.x -= acc[2 * j];
                        v.y -= acc[2 * j + 1];
                        *p = v;
                    }
                }
            }
        }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == PRODUCER_WARP) {
        __syncwarp();
        // the products in flight finish before the tensor memory is freed (at once on the normal path; after an
        // abort the MMA thread committed `drained` behind its last product)
        wait_bounded(drained, 0, args.wait + DRAIN_CYCLES, nullptr);
        __syncwarp();
        fence_after_sync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// A row-major BF16 plane (rows x K, K contiguous) as a TMA map of 64 x box_rows tiles, 128-byte swizzle.
bool plane_map(CUtensorMap *map, const void *base, int64_t rows, int64_t K, int box_rows) {
    auto encode = encode_fn();
    if (!encode) return false;
    cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)K * 2};
    cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int64_t padded_k(int k) { return ((int64_t)k + KPAD - 1) / KPAD * KPAD; }
int64_t align1k(int64_t b) { return (b + 1023) / 1024 * 1024; }
// the real product's inner dimension per segment: a whole number of 64-wide K slices
int64_t padded_real(int64_t kdim) { return (kdim + BK - 1) / BK * BK; }
// the FP64-accurate product's segment: whole chunks, so no chunk mixes two slice pairs
int64_t padded_exact(int64_t kdim) { return (kdim + CHUNK * BK - 1) / (CHUNK * BK) * (CHUNK * BK); }

cudaError_t configure() {
    static bool configured[64] = {};
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e) return e;
    if (device < 64 && !configured[device]) {
        if ((e = cudaFuncSetAttribute(k_tc_update<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM)) ||
            (e = cudaFuncSetAttribute(k_tc_update<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM)) ||
            (e = cudaFuncSetAttribute(k_tc_update<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM)) ||
            (e = cudaFuncSetAttribute(k_tc_update<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM)) ||
            (e = cudaFuncSetAttribute(k_tc_update<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM)) ||
            (e = cudaFuncSetAttribute(k_tc_update<5>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM)) ||
            (e = cudaFuncSetAttribute(k_tc_update<6>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM)))
            return e;
        configured[device] = true;
    }
    return cudaSuccess;
}

}  // namespace

size_t tc_update_scratch_bytes(int64_t rows, int64_t cols, int k, int terms) {
    const int64_t K = terms * 2 * padded_k(k);
    return (size_t)(align1k(rows * K * 2) + align1k(2 * cols * K * 2));
}

cudaError_t tc_update_c64(int64_t rows, int64_t cols, int k, const float2 *A, int64_t lda, const float2 *B,
                          int64_t ldb, float2 *C, int64_t ldc, int terms, void *scratch, bool a_packed, int *error,
                          unsigned long long wait_cycles, cudaStream_t stream) {
    if (rows <= 0 || cols <= 0 || k <= 0) return cudaSuccess;
    if ((terms != 3 && terms != 6) || !A || !B || !C || !scratch || !error || lda < rows || ldb < k || ldc < rows ||
        rows > (int64_t)0x7fffff00 || 2 * cols > (int64_t)0x7fffff00)
        return cudaErrorInvalidValue;
    cudaError_t e = configure();
    if (e) return e;
    const int kp = (int)padded_k(k);
    const int64_t K = (int64_t)terms * 2 * kp;
    auto *pa = static_cast<__nv_bfloat162 *>(scratch);
    auto *pb = reinterpret_cast<__nv_bfloat162 *>(static_cast<uint8_t *>(scratch) + align1k(rows * K * 2));
    if (!a_packed) {
        const dim3 grid((unsigned)((rows + 31) / 32), (unsigned)(kp / 32));
        k_pack_a<<<grid, 256, 0, stream>>>(rows, k, kp, terms, A, lda, pa);
        note_launches(1);
    }
    {
        const dim3 grid((unsigned)std::max<int64_t>(1, (kp + 255) / 256), (unsigned)std::min<int64_t>(cols, 65535));
        k_pack_b<<<grid, 256, 0, stream>>>(cols, k, kp, terms, B, ldb, pb);
        note_launches(1);
    }
    CUtensorMap ma, mb;
    if (!plane_map(&ma, pa, rows, K, BM) || !plane_map(&mb, pb, 2 * cols, K, BN)) return cudaErrorNotSupported;
    TileArgs args;
    args.rows = rows;
    args.cols = cols;
    args.C = C;
    args.ldc = ldc;
    args.Y = nullptr;
    args.ldy = 0;
    args.kblocks = (int)(K / BK);
    args.seg_kblocks = 1;
    args.tiles_m = (int)((rows + BM - 1) / BM);
    args.tiles_n = (int)((2 * cols + BN - 1) / BN);
    args.error = error;
    args.wait = wait_cycles;
    const int64_t tiles = (int64_t)args.tiles_m * args.tiles_n;
    if (tiles > 0x7fffffff) return cudaErrorInvalidValue;
    k_tc_update<0><<<(unsigned)tiles, THREADS, SMEM, stream>>>(ma, mb, args);
    note_launches(1);
    return cudaGetLastError();
}

size_t tc_real_plane_bytes(int64_t rows, int64_t kdim, int terms) {
    return (size_t)align1k(rows * terms * padded_real(kdim) * 2);
}

size_t tc_real_scratch_bytes(int64_t kdim, int64_t cols, int terms) {
    return (size_t)align1k(2 * cols * terms * padded_real(kdim) * 2);
}

cudaError_t tc_pack_real(int64_t rows, int64_t kdim, const float *M, int64_t ldm, int terms, void *plane,
                         cudaStream_t stream) {
    if (rows <= 0 || kdim <= 0) return cudaSuccess;
    if ((terms != 3 && terms != 6) || !M || !plane || ldm < kdim) return cudaErrorInvalidValue;
    const int64_t kp = padded_real(kdim);
    const dim3 grid((unsigned)std::min<int64_t>((kp + 255) / 256, 64), (unsigned)std::min<int64_t>(rows, 65535));
    k_pack_rows<<<grid, 256, 0, stream>>>(rows, kdim, kp, terms, M, ldm, static_cast<__nv_bfloat16 *>(plane));
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t tc_real_product(int64_t rows, int64_t kdim, const void *plane, int64_t cols, const double2 *X,
                            int64_t ldx, double2 *Y, int64_t ldy, int terms, void *scratch, int *error,
                            unsigned long long wait_cycles, cudaStream_t stream) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    if ((terms != 3 && terms != 6) || kdim <= 0 || !plane || !X || !Y || !scratch || !error || ldx < cols ||
        ldy < cols || rows > (int64_t)0x7fffff00 || 2 * cols > (int64_t)0x7fffff00 || (2 * cols + 31) / 32 > 65535)
        return cudaErrorInvalidValue;
    cudaError_t e = configure();
    if (e) return e;
    const int64_t kp = padded_real(kdim), K = terms * kp;
    {
        const dim3 grid((unsigned)(kp / 32), (unsigned)((2 * cols + 31) / 32));
        k_pack_cols<<<grid, 256, 0, stream>>>(kdim, kp, 2 * cols, terms, reinterpret_cast<const double *>(X),
                                              2 * ldx, static_cast<__nv_bfloat16 *>(scratch));
        note_launches(1);
    }
    CUtensorMap ma, mb;
    if (!plane_map(&ma, plane, rows, K, BM) || !plane_map(&mb, scratch, 2 * cols, K, BN))
        return cudaErrorNotSupported;
    TileArgs args;
    args.rows = rows;
    args.cols = cols;
    args.C = nullptr;
    args.ldc = 0;
    args.Y = Y;
    args.ldy = ldy;
    args.kblocks = (int)(K / BK);
    args.seg_kblocks = 1;
    args.tiles_m = (int)((rows + BM - 1) / BM);
    args.tiles_n = (int)((2 * cols + BN - 1) / BN);
    args.error = error;
    args.wait = wait_cycles;
    const int64_t tiles = (int64_t)args.tiles_m * args.tiles_n;
    if (tiles > 0x7fffffff || K / BK > 0x7fffffff) return cudaErrorInvalidValue;
    k_tc_update<1><<<(unsigned)tiles, THREADS, SMEM, stream>>>(ma, mb, args);
    note_launches(1);
    return cudaGetLastError();
}

size_t tc_exact_plane_bytes(int64_t rows, int64_t kdim, int slices) {
    return (size_t)(align1k(rows * slices * padded_exact(kdim) * 2) + align1k(rows * 4));
}

size_t tc_exact_scratch_bytes(int64_t kdim, int64_t cols, int slices) {
    return (size_t)(align1k(2 * cols * slices * padded_exact(kdim) * 2) + align1k(2 * cols * 4));
}

cudaError_t tc_slice_exact(int64_t rows, int64_t kdim, const double *M, int64_t ldm, int slices, void *plane,
                           cudaStream_t stream) {
    if (rows <= 0 || kdim <= 0) return cudaSuccess;
    if (slices < 2 || slices > MAX_SLICES || !M || !plane || ldm < kdim) return cudaErrorInvalidValue;
    const int64_t kp = padded_exact(kdim);
    auto *out = static_cast<__nv_bfloat16 *>(plane);
    int *row_exp = reinterpret_cast<int *>(static_cast<uint8_t *>(plane) + align1k(rows * slices * kp * 2));
    k_slice_rows<<<(unsigned)std::min<int64_t>(rows, 1 << 20), 256, 0, stream>>>(rows, kdim, kp, slices, M, ldm, out,
                                                                                row_exp);
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t tc_exact_product(int64_t rows, int64_t kdim, const void *plane, int64_t cols, const double2 *X,
                             int64_t ldx, double2 *Y, int64_t ldy, int slices, void *scratch, int *error,
                             unsigned long long wait_cycles, cudaStream_t stream) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    const int64_t kp = padded_exact(kdim);
    const int pairs = slices * (slices + 1) / 2;
    if (slices < 2 || slices > MAX_SLICES || kdim <= 0 || !plane || !X || !Y || !scratch || !error || ldx < cols ||
        ldy < cols || rows > (int64_t)0x7fffff00 || 2 * cols > (int64_t)0x7fffff00 ||
        (2 * cols + 31) / 32 > 65535 || (int64_t)slices * kp > (int64_t)0x7fffff00 ||
        (int64_t)pairs * (kp / BK) > (int64_t)0x7fffffff)
        return cudaErrorInvalidValue;
    cudaError_t e = configure();
    if (e) return e;
    const int64_t ncols = 2 * cols, K = (int64_t)slices * kp;
    auto *bplane = static_cast<__nv_bfloat16 *>(scratch);
    int *col_exp = reinterpret_cast<int *>(static_cast<uint8_t *>(scratch) + align1k(ncols * slices * kp * 2));
    const int *row_exp =
        reinterpret_cast<const int *>(static_cast<const uint8_t *>(plane) + align1k(rows * slices * kp * 2));
    const double *Xr = reinterpret_cast<const double *>(X);
    if ((e = cudaMemsetAsync(col_exp, 0x80, (size_t)ncols * sizeof(int), stream))) return e;   // below -1022
    {
        const dim3 grid((unsigned)std::min<int64_t>((kdim + 255) / 256, 65535), (unsigned)((ncols + 31) / 32));
        k_column_exponents<<<grid, 256, 0, stream>>>(kdim, ncols, Xr, 2 * ldx, col_exp);
        const dim3 g2((unsigned)(kp / 32), (unsigned)((ncols + 31) / 32));
        k_slice_cols<<<g2, 256, 0, stream>>>(kdim, kp, ncols, slices, Xr, 2 * ldx, col_exp, bplane);
        note_launches(2);
    }
    CUtensorMap ma, mb;
    if (!plane_map(&ma, plane, rows, K, BM) || !plane_map(&mb, bplane, ncols, K, BN)) return cudaErrorNotSupported;
    TileArgs args;
    args.rows = rows;
    args.cols = cols;
    args.C = nullptr;
    args.ldc = 0;
    args.Y = Y;
    args.ldy = ldy;
    args.kblocks = (int)(pairs * (kp / BK));
    args.seg_kblocks = (int)(kp / BK);
    args.tiles_m = (int)((rows + BM - 1) / BM);
    args.tiles_n = (int)((ncols + BN - 1) / BN);
    args.error = error;
    args.wait = wait_cycles;
    const int64_t tiles = (int64_t)args.tiles_m * args.tiles_n;
    if (tiles > 0x7fffffff) return cudaErrorInvalidValue;
    k_tc_update<2><<<(unsigned)tiles, THREADS, SMEM, stream>>>(ma, mb, args);
    k_exact_scale<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((rows * cols + 255) / 256, 152 * 16)), 256, 0,
                    stream>>>(rows, cols, Y, ldy, row_exp, col_exp);
    note_launches(2);
    return cudaGetLastError();
}

size_t tc_rows_plane_bytes(int64_t rows, int k, int terms) {
    return (size_t)align1k(rows * terms * 2 * padded_k(k) * 2);
}

size_t tc_rows_row_bytes(int k, int terms) { return (size_t)(terms * 2 * padded_k(k) * 2); }

size_t tc_rows_scratch_bytes(int64_t cols, int k, int terms) {
    return (size_t)align1k(2 * cols * terms * 2 * padded_k(k) * 2);
}

cudaError_t tc_pack_rows_c64(int64_t rows, int k, const float2 *A, int64_t lda, int terms, void *plane,
                             cudaStream_t stream) {
    if (rows <= 0 || k <= 0) return cudaSuccess;
    if ((terms != 3 && terms != 6) || !A || !plane || lda < k) return cudaErrorInvalidValue;
    const int kp = (int)padded_k(k);
    const dim3 grid((unsigned)std::max(1, std::min((kp + 255) / 256, 64)), (unsigned)std::min<int64_t>(rows, 65535));
    k_pack_a_rows<<<grid, 256, 0, stream>>>(rows, k, kp, terms, A, lda, static_cast<__nv_bfloat162 *>(plane));
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t tc_update_rows_c64(int64_t rows, int64_t cols, int k, const void *aplane, const float2 *B, int64_t ldb,
                               float2 *C, int64_t ldc, int terms, void *scratch, int *error,
                               unsigned long long wait_cycles, cudaStream_t stream) {
    if (rows <= 0 || cols <= 0 || k <= 0) return cudaSuccess;
    if ((terms != 3 && terms != 6) || !aplane || !B || !C || !scratch || !error || ldb < cols || ldc < cols ||
        rows > (int64_t)0x7fffff00 || 2 * cols > (int64_t)0x7fffff00 || (cols + 31) / 32 > 65535)
        return cudaErrorInvalidValue;
    cudaError_t e = configure();
    if (e) return e;
    const int kp = (int)padded_k(k);
    const int64_t K = (int64_t)terms * 2 * kp;
    auto *pb = static_cast<__nv_bfloat162 *>(scratch);
    {
        const dim3 grid((unsigned)(kp / 32), (unsigned)((cols + 31) / 32));
        k_pack_b_rows<<<grid, 256, 0, stream>>>(cols, k, kp, terms, B, ldb, pb);
        note_launches(1);
    }
    CUtensorMap ma, mb;
    if (!plane_map(&ma, aplane, rows, K, BM) || !plane_map(&mb, pb, 2 * cols, K, BN)) return cudaErrorNotSupported;
    TileArgs args;
    args.rows = rows;
    args.cols = cols;
    args.C = C;
    args.ldc = ldc;
    args.Y = nullptr;
    args.ldy = 0;
    args.kblocks = (int)(K / BK);
    args.seg_kblocks = 1;
    args.tiles_m = (int)((rows + BM - 1) / BM);
    args.tiles_n = (int)((2 * cols + BN - 1) / BN);
    args.error = error;
    args.wait = wait_cycles;
    const int64_t tiles = (int64_t)args.tiles_m * args.tiles_n;
    if (tiles > 0x7fffffff) return cudaErrorInvalidValue;
    k_tc_update<3><<<(unsigned)tiles, THREADS, SMEM, stream>>>(ma, mb, args);
    note_launches(1);
    return cudaGetLastError();
}

size_t tc_lowrank_scratch_bytes(int64_t n_pad, int ngroups) {
    return (size_t)(align1k(256 * 2 * n_pad * 2) + align1k((int64_t)ngroups * 256 * 128 * 2));
}

cudaError_t tc_lowrank_product(const LowRankPlan &p, int k, const double2 *X, double2 *slots, void *scratch,
                               int *error, unsigned long long wait_cycles, cudaStream_t stream) {
    if (p.ngroups <= 0 && p.ndgroups <= 0) return cudaSuccess;
    if (p.ndgroups > 0 && (!p.dplane || !p.dgroups || !p.dtile_group || !p.dtile_m || p.ndtiles <= 0 ||
                           p.drows < BM || p.dpitch % BK))
        return cudaErrorInvalidValue;
    if (k <= 0 || k > BN / 2 || !X || !slots || !scratch || !error || !p.pad_pos || p.n <= 0 || p.n_pad <= 0 ||
        p.n_pad % BK)
        return cudaErrorInvalidValue;
    if (p.ngroups > 0 && (!p.lplane || !p.rplane || !p.groups || !p.tile_group || !p.tile_m || p.rwidth % BK ||
                          p.lrows < BM || p.ntiles <= 0))
        return cudaErrorInvalidValue;
    cudaError_t e = configure();
    if (e) return e;
    auto *xt = static_cast<__nv_bfloat16 *>(scratch);
    auto *tplane = reinterpret_cast<__nv_bfloat16 *>(static_cast<uint8_t *>(scratch) + align1k(256 * 2 * p.n_pad * 2));
    {
        const dim3 grid((unsigned)((p.n + 31) / 32), (unsigned)((2 * k + 31) / 32));
        k_pack_xt<<<grid, 256, 0, stream>>>(p.n, 2 * k, reinterpret_cast<const double *>(X), p.pad_pos, p.n_pad, xt);
        note_launches(1);
    }
    CUtensorMap ma, mb;
    TileArgs args{};
    args.cols = k;
    args.groups = p.groups;
    args.error = error;
    args.wait = wait_cycles;
    args.tiles_m = 1;
    args.tiles_n = 1;
    args.seg_kblocks = 1;
    if (p.ndgroups > 0) {         // the dense leaves: D_g X[J_g] into their slot rows
        if (!plane_map(&ma, p.dplane, p.drows, 2 * p.dpitch, BM) || !plane_map(&mb, xt, 256, 2 * p.n_pad, BN))
            return cudaErrorNotSupported;
        TileArgs d = args;
        d.groups = p.dgroups;
        d.tile_group = p.dtile_group;
        d.tile_m = p.dtile_m;
        d.a_pitch = (int)p.dpitch;
        d.b_pitch = (int)p.n_pad;
        d.slots = slots;
        k_tc_update<6><<<(unsigned)p.ndtiles, THREADS, SMEM, stream>>>(ma, mb, d);
        note_launches(1);
    }
    if (p.ngroups <= 0) return cudaGetLastError();
    // phase one: T_g = R_g X[J_g], one tile per group
    if (!plane_map(&ma, p.rplane, BM, 2 * p.rwidth, BM) || !plane_map(&mb, xt, 256, 2 * p.n_pad, BN))
        return cudaErrorNotSupported;
    args.a_pitch = (int)p.rwidth;
    args.b_pitch = (int)p.n_pad;
    args.tplane = tplane;
    k_tc_update<4><<<(unsigned)p.ngroups, THREADS, SMEM, stream>>>(ma, mb, args);
    // phase two: L_g T_g into the slots
    if (!plane_map(&ma, p.lplane, p.lrows, 128, BM) || !plane_map(&mb, tplane, (int64_t)p.ngroups * 256, 128, BN))
        return cudaErrorNotSupported;
    args.tile_group = p.tile_group;
    args.tile_m = p.tile_m;
    args.slots = slots;
    k_tc_update<5><<<(unsigned)p.ntiles, THREADS, SMEM, stream>>>(ma, mb, args);
    note_launches(2);
    return cudaGetLastError();
}

}  // namespace pq
