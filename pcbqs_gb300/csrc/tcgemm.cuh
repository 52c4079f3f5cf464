// The trailing update of the blocked complex64 LU on the tensor cores: C -= A B with FP32 complex operands split into
// BF16 parts and multiplied by a hand-written tcgen05 GEMM (TMA-fed shared memory, accumulators in tensor memory).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace pq {

// One low-rank contribution Y[I] += L (R X[J]) of an H-matrix product on the tensor cores (tc_lowrank_product):
// L (|I| x rank) and R (rank x |J|) are a block's factors (U and V, or V^T and U^T for its transposed half), R X[J]
// summed over J's range of the padded cluster order. Layout shared with pcbqs_gb300.hmatrix (40 bytes).
struct LrGroup {
    int32_t a_row0;   // first row of L in the left plane
    int32_t rows;     // |I|
    int32_t a_x0;     // J's padded start in the right-hand sides' plane (a multiple of 64)
    int32_t b_x0;     // R's start in the right plane (a multiple of 64)
    int32_t kb;       // 64-wide slices of J's padded range
    int32_t t_row0;   // the group's 256 rows in the T plane
    int32_t rank;     // <= 64
    int32_t pad;
    int64_t slot0;    // first slot row of the output
};

// One H-matrix's low-rank blocks packed for the tensor cores (device arrays): the left factors' plane (lrows x 128
// BF16: parts h and m of L at 0 and 64, zero from the rank on), the right factors' plane (128 x 2 rwidth BF16: part
// h at 0, m at rwidth; group g's R in rows 0 .. rank - 1 from b_x0, at the padded positions of J), the groups, and
// the phase-two tiles (group, row tile); pad_pos: each row's position in the padded cluster order (n_pad wide).
struct LowRankPlan {
    const void *lplane = nullptr;
    int64_t lrows = 0;
    const void *rplane = nullptr;
    int64_t rwidth = 0;
    const LrGroup *groups = nullptr;
    int ngroups = 0;
    const int32_t *tile_group = nullptr, *tile_m = nullptr;
    int ntiles = 0;
    const int32_t *pad_pos = nullptr;
    int64_t n = 0, n_pad = 0;
    // the dense leaves on the tensor cores too (optional): their plane (drows x 2 dpitch BF16: parts h at 0, m at
    // dpitch; group g's block in rows a_row0 .., its columns at J's padded positions), groups and tiles
    const void *dplane = nullptr;
    int64_t drows = 0, dpitch = 0;
    const LrGroup *dgroups = nullptr;
    int ndgroups = 0;
    const int32_t *dtile_group = nullptr, *dtile_m = nullptr;
    int ndtiles = 0;
};

// Scratch of tc_lowrank_product: the right-hand sides' transposed plane (256 x 2 n_pad BF16) and the T plane
// (ngroups x 256 x 128 BF16); zeroed once when allocated (padding positions are never written).
size_t tc_lowrank_scratch_bytes(int64_t n_pad, int ngroups);
// The low-rank blocks' contributions to Y = H X (and the dense leaves', when the plan holds them: MODE 6, Y[I] = D X[J]
// in three part products, one group per block and direction, written to its slot rows) (X: n x k complex128 row-major, k <= 128) in BF16 three-part
// products with FP32 accumulation: phase one T_g = R_g X[J_g] for every group (one tile each), written as T_g^T's
// BF16 parts; phase two L_g T_g into the group's slot rows (slots: complex128, k wide), summed with the dense blocks'
// slots afterwards. `error`, `wait_cycles`, `stream` as in tc_update_c64.
cudaError_t tc_lowrank_product(const LowRankPlan &plan, int k, const double2 *X, double2 *slots, void *scratch,
                               int *error, unsigned long long wait_cycles, cudaStream_t stream);

// Scratch of one trailing update (the BF16 operand planes), sized by tc_update_scratch_bytes.
size_t tc_update_scratch_bytes(int64_t rows, int64_t cols, int k, int terms);

// C (rows x cols) -= A (rows x k) B (k x cols); all complex64 column-major with leading dimensions lda, ldb, ldc.
// Each FP32 value is split into BF16 parts x = h + m + l; `terms` = 3 multiplies h·h + h·m + m·h (relative error of
// a product about 2^-16), 6 adds h·l + m·m + l·h (about 2^-24, FP32's own level). The complex product runs as one
// real GEMM of inner dimension terms · 2k: A's rows [re | im] against B's columns [re; -im] (real part) and [im; re]
// (imaginary part). `scratch` holds tc_update_scratch_bytes; `a_packed` reuses the A planes packed by an
// earlier call with the same A (the LU packs its panel once per step for two updates). `error` (device int)
// receives ERR_TIMEOUT when a bounded wait of the GEMM gives up (limit `wait_cycles` SM clocks). Ordered on `stream`.
cudaError_t tc_update_c64(int64_t rows, int64_t cols, int k, const float2 *A, int64_t lda, const float2 *B,
                          int64_t ldb, float2 *C, int64_t ldc, int terms, void *scratch, bool a_packed,
                          int *error, unsigned long long wait_cycles, cudaStream_t stream);

// The same update with row-major operands and A packed once for many updates (the triangular solves' products with
// a fixed factor): C (rows x cols, row-major complex64, leading dimension ldc) -= A B, A's plane (rows x k, packed
// by tc_pack_rows_c64 from a row-major complex64 A with leading dimension lda, into tc_rows_plane_bytes; a plane of
// more rows may be used from any row on, its rows being tc_rows_row_bytes(k, terms) bytes apart) and B
// (k x cols, row-major complex64, leading dimension ldb) packed into `scratch` (tc_rows_scratch_bytes) per call.
size_t tc_rows_plane_bytes(int64_t rows, int k, int terms);
size_t tc_rows_row_bytes(int k, int terms);
size_t tc_rows_scratch_bytes(int64_t cols, int k, int terms);
cudaError_t tc_pack_rows_c64(int64_t rows, int k, const float2 *A, int64_t lda, int terms, void *plane,
                             cudaStream_t stream);
cudaError_t tc_update_rows_c64(int64_t rows, int64_t cols, int k, const void *aplane, const float2 *B, int64_t ldb,
                               float2 *C, int64_t ldc, int terms, void *scratch, int *error,
                               unsigned long long wait_cycles, cudaStream_t stream);

// The dense product over many right-hand sides on the same GEMM: Y (rows x cols complex128) = M (rows x kdim, real)
// X (kdim x cols complex128), X and Y row-major with leading dimensions ldx, ldy (in complex elements). M is
// packed once into its BF16 part plane (tc_pack_real into tc_real_plane_bytes) and reused by every product; each
// product packs X (rounded to FP32) into `scratch` (tc_real_scratch_bytes) and runs one real GEMM of inner
// dimension terms · kdim against X's real and imaginary columns side by side, writing Y whole. The result carries
// the relative error of the parts kept (terms 3: about 2^-16; 6: FP32's). `error`, `wait_cycles` and `stream` as in
// tc_update_c64.
size_t tc_real_plane_bytes(int64_t rows, int64_t kdim, int terms);
size_t tc_real_scratch_bytes(int64_t kdim, int64_t cols, int terms);
cudaError_t tc_pack_real(int64_t rows, int64_t kdim, const float *M, int64_t ldm, int terms, void *plane,
                         cudaStream_t stream);
cudaError_t tc_real_product(int64_t rows, int64_t kdim, const void *plane, int64_t cols, const double2 *X,
                            int64_t ldx, double2 *Y, int64_t ldy, int terms, void *scratch, int *error,
                            unsigned long long wait_cycles, cudaStream_t stream);

// The same product to FP64's accuracy from a real FP64 M and complex128 X: every row of M and every real column of X
// is cut into `slices` (2..7) integer slices of 8 bits under its own power-of-two scale, so each slice is exact in
// BF16 and every slice product sums exactly in FP32 over the tensor core's 256-long chunks; the levels of slice
// pairs are carried into Y in FP64. The truncation error is about 2^(-8 slices) of max_t |M[r, t]| times
// sum_t |X[t, c]| (slices 6: about 2^-48). M's plane (tc_slice_exact into tc_exact_plane_bytes) holds its slices and
// row exponents; `scratch` (tc_exact_scratch_bytes) X's. Non-finite entries make their rows or columns of Y
// non-finite.
size_t tc_exact_plane_bytes(int64_t rows, int64_t kdim, int slices);
size_t tc_exact_scratch_bytes(int64_t kdim, int64_t cols, int slices);
cudaError_t tc_slice_exact(int64_t rows, int64_t kdim, const double *M, int64_t ldm, int slices, void *plane,
                           cudaStream_t stream);
cudaError_t tc_exact_product(int64_t rows, int64_t kdim, const void *plane, int64_t cols, const double2 *X,
                             int64_t ldx, double2 *Y, int64_t ldy, int slices, void *scratch, int *error,
                             unsigned long long wait_cycles, cudaStream_t stream);

}  // namespace pq
