// The compressed-free PEEC operator in loop/tree coordinates, its block-Jacobi preconditioner, a dense symmetric
// operator (for P^-1 B), and their C ABI.
//
// Operator (src/pcbqs/peec_iterative.py:267-278): for system s at angular frequency w_s,
//   branch = K (D_s y),  D_s = diag(1 on loop unknowns, j w_s alpha_s on tree unknowns), alpha_s = zscale_s/pscale
//   out    = K^T (r_s R branch + j w_s L branch) / zscale_s + T^T P T y / pscale
// with K (branches x unknowns) the loop/tree basis, T = A K_tree (nodes x unknowns, zero on loop columns), R the
// sparse sheet resistance (r_s its per-frequency factor, 1 at DC), L, P the dense partial-inductance and potential
// matrices on the device (P complex, P_re + j P_im, for a lossy dielectric stack). The dense products run in this
// file's symmetric dense kernels (FP64, or FP32 for the inner products of the mixed solve), every sparse product
// and combination in its CSR kernels.
//
// Block-Jacobi: the unknowns are ordered so that consecutive runs of `bs` are geometric clusters; each diagonal
// block of the operator, (r K^T R K + j w K^T L K)_blk D_blk / zscale + (T^T P T)_blk / pscale, is formed on the
// device (K^T L K and T^T P T blocks gathered from the dense matrices), inverted (Gauss-Jordan with partial
// pivoting), and applied to every column of its system.
#include <algorithm>
#include <type_traits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include <cublas_v2.h>
#include <cusolverDn.h>

#include "../../include/pcbqs_gb300.h"
#include "common.cuh"
#include "factor.cuh"
#include "pool.cuh"
#include "solve.cuh"
#include "hmatrix.cuh"
#include "tcgemm.cuh"
#include "trsolve.cuh"
#include "tune.cuh"

namespace pq {

struct Csr {
    int64_t rows = 0, cols = 0;
    const int64_t *ptr = nullptr;
    const int32_t *idx = nullptr;
    const double *val = nullptr;
};

// Y[r, s] = (acc ? Y[r, s] : 0) + scale[sys[s]] * sum_j val_j X[idx_j, s]   (scale nullable: 1)
__global__ void k_spmm(Csr S, int k, const cd *X, cd *Y, const double *scale, const int *sys, int accumulate) {
    const int64_t total = S.rows * k;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / k;
        const int s = (int)(t % k);
        double re = 0, im = 0;
        for (int64_t j = S.ptr[r]; j < S.ptr[r + 1]; ++j) {
            const double v = S.val[j];
            const cd x = X[(int64_t)S.idx[j] * k + s];
            re += v * x.x;
            im += v * x.y;
        }
        if (scale) {
            const double f = scale[sys[s]];
            re *= f;
            im *= f;
        }
        if (accumulate) {
            Y[t].x += re;
            Y[t].y += im;
        } else {
            Y[t] = make_double2(re, im);
        }
    }
}

// U = D_s Y: tree rows times j w_s alpha_s.
__global__ void k_tree_scale(int64_t n, int k, const int8_t *is_tree, const double *walpha, const int *sys,
                             const cd *Y, cd *U) {
    const int64_t total = n * k;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / k;
        const cd y = Y[t];
        if (is_tree[r]) {
            const double f = walpha[sys[(int)(t % k)]];     // j f y = (-f y.im, f y.re)
            U[t] = make_double2(-f * y.y, f * y.x);
        } else {
            U[t] = y;
        }
    }
}

// V[e, s] = sum_f R[e, f] B[f, s] + j w_s LB[e, s] for copper rows e < ne; other passive rows (lumped parts with no
// impedance here) are zero.
__global__ void k_impedance(Csr R, int64_t nb, int k, const cd *B, const cd *LB, const double *omega,
                            const cd *rscale, int64_t nscaled, const int *sys, cd *V) {
    const int64_t total = nb * k;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = t / k;
        const int s = (int)(t % k);
        double re = 0, im = 0;
        if (e < R.rows) {
            for (int64_t j = R.ptr[e]; j < R.ptr[e + 1]; ++j) {
                const cd b = B[(int64_t)R.idx[j] * k + s];
                re += R.val[j] * b.x;
                im += R.val[j] * b.y;
            }
            const cd rs = e < nscaled ? rscale[sys[s]] : make_double2(1.0, 0.0);
            const double rr = re * rs.x - im * rs.y, ri = re * rs.y + im * rs.x;
            const double w = omega[sys[s]];
            const cd lb = LB[t];
            re = rr - w * lb.y;
            im = ri + w * lb.x;
        }
        V[t] = make_double2(re, im);
    }
}

// y += j z (the imaginary part of a complex matrix applied through its real view).
__global__ void k_add_times_j(int64_t count, const cd *z, cd *y) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x) {
        const cd a = z[t];
        y[t] = make_double2(y[t].x - a.y, y[t].y + a.x);
    }
}

// Diagonal blocks of S^T M S for a dense symmetric M: out[b][i][j] = sum_{e in col i} sum_{f in col j}
// S_ei S_fj M[e, f], columns of S given as rows of S^T (CSR St). One CTA per block.
__global__ void k_block_gather(int64_t n, int bs, Csr St, const double *M, int64_t ldm, double *out) {
    const int64_t b = blockIdx.x;
    const int64_t c0 = b * bs;
    for (int t = threadIdx.x; t < bs * bs; t += blockDim.x) {
        const int i = t / bs, j = t % bs;
        const int64_t ci = c0 + i, cj = c0 + j;
        double acc = 0;
        if (ci < n && cj < n) {
            for (int64_t a = St.ptr[ci]; a < St.ptr[ci + 1]; ++a) {
                const double sa = St.val[a];
                const double *row = M + (int64_t)St.idx[a] * ldm;
                double part = 0;
                for (int64_t c = St.ptr[cj]; c < St.ptr[cj + 1]; ++c) part += St.val[c] * row[St.idx[c]];
                acc += sa * part;
            }
        }
        out[(b * bs + i) * bs + j] = acc;
    }
}

// Form and invert every (system, block): A = (KRK + j w KLK) D / zscale + TPT / pscale; padding rows beyond n
// are identity. Gauss-Jordan with partial pivoting on [A | I] in shared memory; one warp per matrix row group.
__global__ void k_block_invert(int64_t n, int bs, int64_t nblk, const double *krk, const double *klk,
                               const double *tpt, const double *tpt_im, const int8_t *is_tree, const double *omega,
                               const double *zscale, const cd *rscale, double pscale, cd *inv, int *singular) {
    extern __shared__ cd aug[];     // bs x 2bs
    const int64_t b = blockIdx.x;
    const int s = blockIdx.y;
    const int w2 = 2 * bs;
    const double w = omega[s], zs = zscale[s], alpha = zs / pscale;
    const int64_t c0 = b * bs;
    for (int t = threadIdx.x; t < bs * w2; t += blockDim.x) {
        const int i = t / w2, j = t % w2;
        cd v = make_double2(0, 0);
        if (j < bs) {
            const int64_t ci = c0 + i, cj = c0 + j;
            if (ci < n && cj < n) {
                const size_t at = (b * bs + i) * bs + j;
                const cd rs = rscale[s];
                double re = rs.x * krk[at] / zs, im = (rs.y * krk[at] + w * klk[at]) / zs;
                if (is_tree[cj]) {       // column scaled by j w alpha
                    const double f = w * alpha;
                    const double r2 = -f * im, i2 = f * re;
                    re = r2;
                    im = i2;
                }
                if (is_tree[ci] && is_tree[cj]) {
                    re += tpt[at] / pscale;
                    if (tpt_im) im += tpt_im[at] / pscale;
                }
                v = make_double2(re, im);
            } else if (i == j) {
                v = make_double2(1, 0);
            }
        } else {
            v = make_double2(j - bs == i ? 1 : 0, 0);
        }
        aug[t] = v;
    }
    __syncthreads();
    __shared__ int piv;
    for (int c = 0; c < bs; ++c) {
        if (threadIdx.x == 0) {
            int best = c;
            double bv = -1;
            for (int r = c; r < bs; ++r) {
                const cd a = aug[r * w2 + c];
                const double m = a.x * a.x + a.y * a.y;
                if (m > bv) { bv = m; best = r; }
            }
            piv = best;
            if (!(bv > 0)) *singular = 1;
        }
        __syncthreads();
        const int p = piv;
        if (p != c)
            for (int j = threadIdx.x; j < w2; j += blockDim.x) {
                const cd tmp = aug[c * w2 + j];
                aug[c * w2 + j] = aug[p * w2 + j];
                aug[p * w2 + j] = tmp;
            }
        __syncthreads();
        const cd d = aug[c * w2 + c];
        const double dd = d.x * d.x + d.y * d.y;
        const cd dinv = dd > 0 ? make_double2(d.x / dd, -d.y / dd) : make_double2(0, 0);
        __syncthreads();
        for (int j = threadIdx.x; j < w2; j += blockDim.x) {
            const cd a = aug[c * w2 + j];
            aug[c * w2 + j] = make_double2(a.x * dinv.x - a.y * dinv.y, a.x * dinv.y + a.y * dinv.x);
        }
        __syncthreads();
        for (int t = threadIdx.x; t < bs * w2; t += blockDim.x) {
            const int r = t / w2, j = t % w2;
            if (r == c) continue;
            const cd f = aug[r * w2 + c];
            const cd pv = aug[c * w2 + j];
            if (j != c) {
                aug[t].x -= f.x * pv.x - f.y * pv.y;
                aug[t].y -= f.x * pv.y + f.y * pv.x;
            }
        }
        __syncthreads();
        for (int r = threadIdx.x; r < bs; r += blockDim.x)
            if (r != c) aug[r * w2 + c] = make_double2(0, 0);
        __syncthreads();
    }
    cd *out = inv + ((size_t)s * nblk + b) * bs * bs;
    for (int t = threadIdx.x; t < bs * bs; t += blockDim.x) out[t] = aug[(t / bs) * w2 + bs + t % bs];
}

// out[r, s] = sum_{c in block(r)} Inv[sys s][blk][r_l][c_l] in[c, s]
__global__ void k_block_apply(int64_t n, int bs, int64_t nblk, int k, const cd *inv, const int *sys, const cd *in,
                              cd *out) {
    const int64_t total = n * k;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / k;
        const int s = (int)(t % k);
        const int64_t b = r / bs;
        const int rl = (int)(r - b * bs);
        const cd *M = inv + (((size_t)sys[s] * nblk + b) * bs + rl) * bs;
        const int64_t c0 = b * bs;
        const int cn = (int)std::min<int64_t>(bs, n - c0);
        double re = 0, im = 0;
        for (int c = 0; c < cn; ++c) {
            const cd m = M[c], x = in[(c0 + c) * k + s];
            re += m.x * x.x - m.y * x.y;
            im += m.x * x.y + m.y * x.x;
        }
        out[t] = make_double2(re, im);
    }
}

// Jacobi: out = in / d
__global__ void k_diag_apply(int64_t n, int k, const double *d, const cd *in, cd *out) {
    const int64_t total = n * k;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const double f = 1.0 / d[t / k];
        out[t] = make_double2(in[t].x * f, in[t].y * f);
    }
}

__global__ void k_diag_extract(int64_t n, const double *A, int64_t lda, double *d) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = fabs(A[i * lda + i]);
        d[i] = v > 0 ? A[i * lda + i] : 1.0;
    }
}

static int grid_of(int64_t total) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, (int64_t)sms * 16));
}

// Y = M X for a dense symmetric real M (rows x rows, leading dimension ld, FP64 or its FP32 copy) and complex128
// X, Y (rows x k, row-major): the real view X (rows x 2k) in passes of up to DENSE_NC real columns. Thread block of
// 8 warps on 8 * RW rows; every warp streams its rows' entries along i (coalesced) against a 256-entry chunk of X
// staged in shared memory column by column (conflict-free), so each M entry costs exactly its NC multiply-adds:
// the FP64 product runs at the FP64 pipe's rate with no padding of the 2k columns, the FP32 one at HBM speed.
constexpr int DENSE_NC = 16;
constexpr int DENSE_CHUNK = 256;

template <class T, int RW>
__global__ void __launch_bounds__(256) k_dense_sym_apply(int64_t rows, const T *__restrict__ M, int64_t ld,
                                                         const double *__restrict__ X, int xcols, int c0, int nc,
                                                         double *__restrict__ Y) {
    __shared__ T xs[DENSE_NC][DENSE_CHUNK];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t r0 = ((int64_t)blockIdx.x * 8 + warp) * RW;
    T acc[RW][DENSE_NC];
#pragma unroll
    for (int r = 0; r < RW; ++r)
#pragma unroll
        for (int c = 0; c < DENSE_NC; ++c) acc[r][c] = 0;
    const T *mrow[RW];
#pragma unroll
    for (int r = 0; r < RW; ++r) mrow[r] = M + (r0 + r < rows ? r0 + r : 0) * ld;
    for (int64_t i0 = 0; i0 < rows; i0 += DENSE_CHUNK) {
        __syncthreads();
        for (int t = threadIdx.x; t < DENSE_CHUNK * DENSE_NC; t += 256) {
            const int ii = t / DENSE_NC, c = t % DENSE_NC;
            const int64_t i = i0 + ii;
            xs[c][ii] = (i < rows && c < nc) ? (T)X[i * xcols + c0 + c] : (T)0;
        }
        __syncthreads();
        const int span = rows - i0 < DENSE_CHUNK ? (int)(rows - i0) : DENSE_CHUNK;
        for (int ii = lane; ii < span; ii += 32) {
            T mv[RW];
#pragma unroll
            for (int r = 0; r < RW; ++r) mv[r] = mrow[r][i0 + ii];
#pragma unroll
            for (int c = 0; c < DENSE_NC; ++c) {
                const T xv = xs[c][ii];
#pragma unroll
                for (int r = 0; r < RW; ++r) acc[r][c] += mv[r] * xv;
            }
        }
    }
#pragma unroll
    for (int r = 0; r < RW; ++r)
#pragma unroll
        for (int c = 0; c < DENSE_NC; ++c) {
            T v = acc[r][c];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0 && r0 + r < rows && c < nc) Y[(r0 + r) * xcols + c0 + c] = (double)v;
        }
}

// The FP32 product is bound by streaming M (4 B an entry), so it skips the shared-memory staging: X is first
// packed into FP32 rows of DENSE_NC values (64 B, 16-byte aligned), which every warp reads with vector loads that
// the 8 warps of a block share through L1; each lane then keeps RW x 16 sums and issues its loads for two columns
// before the multiply-adds.
__global__ void k_pack_x_f32(int64_t rows, const double *X, int xcols, int c0, int nc, float *Xf) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < rows * DENSE_NC;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / DENSE_NC;
        const int c = (int)(t % DENSE_NC);
        Xf[t] = c < nc ? (float)X[i * xcols + c0 + c] : 0.0f;
    }
}

template <int RW, int U>
__global__ void __launch_bounds__(256) k_dense_apply_f32(int64_t rows, const float *__restrict__ M, int64_t ld,
                                                         const float *__restrict__ Xf, int xcols, int c0, int nc,
                                                         double *__restrict__ Y) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t r0 = ((int64_t)blockIdx.x * 8 + warp) * RW;
    float acc[RW][DENSE_NC];
#pragma unroll
    for (int r = 0; r < RW; ++r)
#pragma unroll
        for (int c = 0; c < DENSE_NC; ++c) acc[r][c] = 0.f;
    const float *mrow[RW];
#pragma unroll
    for (int r = 0; r < RW; ++r) mrow[r] = M + (r0 + r < rows ? r0 + r : 0) * ld;
    for (int64_t i = lane; i < rows; i += 32 * U) {
        float mv[U][RW];
        float4 xv[U][DENSE_NC / 4];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t iu = i + 32 * u;
            const bool in = iu < rows;
#pragma unroll
            for (int r = 0; r < RW; ++r) mv[u][r] = in ? __ldg(mrow[r] + iu) : 0.f;
            const float4 *xp = reinterpret_cast<const float4 *>(Xf + (in ? iu : 0) * DENSE_NC);
#pragma unroll
            for (int q = 0; q < DENSE_NC / 4; ++q) xv[u][q] = in ? __ldg(xp + q) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int q = 0; q < DENSE_NC / 4; ++q)
#pragma unroll
                for (int r = 0; r < RW; ++r) {
                    acc[r][4 * q] += mv[u][r] * xv[u][q].x;
                    acc[r][4 * q + 1] += mv[u][r] * xv[u][q].y;
                    acc[r][4 * q + 2] += mv[u][r] * xv[u][q].z;
                    acc[r][4 * q + 3] += mv[u][r] * xv[u][q].w;
                }
    }
#pragma unroll
    for (int r = 0; r < RW; ++r)
#pragma unroll
        for (int c = 0; c < DENSE_NC; ++c) {
            float v = acc[r][c];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0 && r0 + r < rows && c < nc) Y[(r0 + r) * xcols + c0 + c] = (double)v;
        }
}

// The FP32 product's shape (rows per warp RW, columns in flight per lane U) is chosen per device and matrix size
// by timing the candidates once on first use (the pick is cached), since which of register reuse and loads in
// flight limits it depends on the size.
using DenseF32Kernel = void (*)(int64_t, const float *, int64_t, const float *, int, int, int, double *);
struct DenseF32Variant {
    int rw, u;
    DenseF32Kernel kernel;
};
static const DenseF32Variant DENSE_F32_VARIANTS[] = {
    {2, 2, k_dense_apply_f32<2, 2>}, {2, 4, k_dense_apply_f32<2, 4>}, {4, 1, k_dense_apply_f32<4, 1>},
    {4, 2, k_dense_apply_f32<4, 2>}, {4, 4, k_dense_apply_f32<4, 4>}};
constexpr int DENSE_F32_COUNT = sizeof(DENSE_F32_VARIANTS) / sizeof(DENSE_F32_VARIANTS[0]);


static cudaError_t launch_dense_f32(int v, int64_t rows, const float *M, int64_t ld, const float *xf, int xcols,
                                   int c0, int nc, double *Y, cudaStream_t s) {
    const DenseF32Variant &d = DENSE_F32_VARIANTS[v];
    const unsigned grid = (unsigned)((rows + 8 * d.rw - 1) / (8 * d.rw));
    d.kernel<<<grid, 256, 0, s>>>(rows, M, ld, xf, xcols, c0, nc, Y);
    return cudaGetLastError();
}

static cudaError_t tuned_dense_f32(int64_t rows, const float *M, int64_t ld, const float *xf, int xcols, int c0,
                                   int nc, double *Y, cudaStream_t s, int &choice) {
    const std::string key = "dense_f32 rows=" + std::to_string(rows);
    const int known = tune_get(key);
    if (known >= 0 && known < DENSE_F32_COUNT) {
        choice = known;
        return cudaSuccess;
    }
    cudaEvent_t e0, e1;
    cudaError_t e;
    if ((e = cudaEventCreate(&e0)) || (e = cudaEventCreate(&e1))) return e;
    float best = 1e30f;
    choice = 0;
    for (int v = 0; v < DENSE_F32_COUNT && !e; ++v) {
        float ms = 0;
        for (int rep = 0; rep < 2 && !e; ++rep) {      // the second run is timed
            cudaEventRecord(e0, s);
            e = launch_dense_f32(v, rows, M, ld, xf, xcols, c0, nc, Y, s);
            cudaEventRecord(e1, s);
            if (!e) e = cudaEventSynchronize(e1);
            if (!e) e = cudaEventElapsedTime(&ms, e0, e1);
        }
        note_launches(2);
        if (!e && ms < best) {
            best = ms;
            choice = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e) return e;
    tune_put(key, choice);
    return cudaSuccess;
}

template <class T, int RW>
static cudaError_t dense_sym_apply(int64_t rows, int k, const T *M, int64_t ld, const cd *X, cd *Y, cudaStream_t s,
                                   float *xf = nullptr) {
    const int xcols = 2 * k;
    const unsigned grid = (unsigned)((rows + 8 * RW - 1) / (8 * RW));
    for (int c0 = 0; c0 < xcols; c0 += DENSE_NC) {
        const int nc = std::min(DENSE_NC, xcols - c0);
        if constexpr (std::is_same<T, float>::value) {
            k_pack_x_f32<<<grid_of(rows * DENSE_NC), 256, 0, s>>>(rows, reinterpret_cast<const double *>(X), xcols,
                                                                 c0, nc, xf);
            note_launches(1);
            int v = 0;
            cudaError_t e = tuned_dense_f32(rows, M, ld, xf, xcols, c0, nc, reinterpret_cast<double *>(Y), s, v);
            if (!e) e = launch_dense_f32(v, rows, M, ld, xf, xcols, c0, nc, reinterpret_cast<double *>(Y), s);
            if (e) return e;
            note_launches(1);
        } else {
            k_dense_sym_apply<T, RW><<<grid, 256, 0, s>>>(rows, M, ld, reinterpret_cast<const double *>(X), xcols,
                                                          c0, nc, reinterpret_cast<double *>(Y));
            note_launches(1);
        }
    }
    return cudaGetLastError();
}

// Device buffers come from the retained stream-ordered pool (pool.cuh): the dense blocks, factors and work arrays
// of one solve are reused by the next instead of being mapped and unmapped each time. Buffers that outlive a call
// are released on the legacy stream, after the call that used them has synchronized its stream.
template <class T> static cudaError_t dev_alloc(T **p, size_t count, cudaStream_t s = nullptr) {
    return pool_alloc_n(p, count, s);
}

static void dev_free(void *p, cudaStream_t s = nullptr) { pool_free(p, s); }

__global__ void k_to_f32(int64_t count, const double *in, float *out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x)
        out[t] = (float)in[t];
}

__global__ void k_to_f64(int64_t count, const float *in, double *out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x)
        out[t] = (double)in[t];
}

struct PeecOp : Operator {
    int64_t n_ = 0, nb = 0, ne = 0, nn = 0;
    Csr K, Kt, T, Tt, R;
    const double *L = nullptr, *P = nullptr;
    const double *Pim = nullptr;          // imaginary part of P (lossy dielectric stack), or null
    int64_t ldl = 0, ldp = 0;
    const int8_t *is_tree = nullptr;
    double pscale = 1;
    int nsys = 0;
    double *omega = nullptr, *zscale = nullptr, *walpha = nullptr, *inv_z = nullptr, *inv_p = nullptr;
    cd *rscale = nullptr;                 // per system factor on R (device)
    std::vector<cd> rscale_host;
    int64_t nscaled = 0;                  // rows of R the factor applies to (the rest keep theirs)
    int cap = 0;               // columns the scratch holds
    cd *u = nullptr, *branch = nullptr, *lb = nullptr, *v = nullptr, *tq = nullptr, *pq = nullptr, *pq2 = nullptr;
    int64_t launches = 0;

    int64_t n() const override { return n_; }

    cudaError_t reserve(int k, cudaStream_t s) {
        if (k <= cap) return cudaSuccess;
        for (cd *p : {u, branch, lb, v, tq, pq, pq2}) dev_free(p, s);
        u = branch = lb = v = tq = pq = pq2 = nullptr;
        cudaError_t e;
        if ((e = dev_alloc(&u, (size_t)n_ * k, s)) || (e = dev_alloc(&branch, (size_t)nb * k, s)) ||
            (e = dev_alloc(&lb, (size_t)ne * k, s)) || (e = dev_alloc(&v, (size_t)nb * k, s)) ||
            (e = dev_alloc(&tq, (size_t)nn * k, s)) || (e = dev_alloc(&pq, (size_t)nn * k, s)) ||
            (e = dev_alloc(&pq2, (size_t)nn * k, s)))
            return e;
        cap = k;
        return cudaSuccess;
    }

    // Single-precision copies of L and P for the inner products of the mixed solve (set by peec_single).
    const float *Lf = nullptr, *Pf = nullptr, *Pfim = nullptr;
    int64_t ldlf = 0, ldpf = 0;

    // y (rows x k complex128) = M x for a dense symmetric M, in FP64 or through its single-precision copy when
    // `single` (k_dense_sym_apply / k_dense_apply_f32).
    float *xf = nullptr;       // packed FP32 right-hand sides of the single-precision products
    int64_t capf = 0;

    // The single-precision products over at least TC_MIN_COLUMNS right-hand sides run on the tensor cores
    // (tc_real_product): L's, P's and P's imaginary part's BF16 part planes (tc_terms parts) are packed on first use
    // after peec_single, the right-hand sides per product. tc_terms = 0 keeps the FP32 product throughout.
    static constexpr int TC_MIN_COLUMNS = 16;
    int tc_terms = 3;
    void *plane[3] = {};
    size_t plane_cap[3] = {};
    bool packed[3] = {};
    void *tcs = nullptr;       // the right-hand sides' plane
    size_t tcs_cap = 0;
    int *tc_error = nullptr;   // ERR_TIMEOUT from a product whose bounded wait gave up

    cudaError_t tensor_product(int which, int64_t rows, int k, const float *Mf, int64_t ldf, const cd *x, cd *y,
                               cudaStream_t s) {
        cudaError_t e;
        if (!tc_error) {
            if ((e = dev_alloc(&tc_error, 1, s)) || (e = cudaMemsetAsync(tc_error, 0, sizeof(int), s))) return e;
        }
        const size_t pb = tc_real_plane_bytes(rows, rows, tc_terms);
        if (!packed[which] || plane_cap[which] < pb) {
            if (plane_cap[which] < pb) {
                dev_free(plane[which], s);
                plane[which] = nullptr;
                plane_cap[which] = 0;
                if ((e = dev_alloc(reinterpret_cast<uint8_t **>(&plane[which]), pb, s))) return e;
                plane_cap[which] = pb;
            }
            if ((e = tc_pack_real(rows, rows, Mf, ldf, tc_terms, plane[which], s))) return e;
            packed[which] = true;
        }
        const size_t sb = tc_real_scratch_bytes(rows, k, tc_terms);
        if (sb > tcs_cap) {
            dev_free(tcs, s);
            tcs = nullptr;
            tcs_cap = 0;
            if ((e = dev_alloc(reinterpret_cast<uint8_t **>(&tcs), sb, s))) return e;
            tcs_cap = sb;
        }
        return tc_real_product(rows, rows, plane[which], k, reinterpret_cast<const double2 *>(x), k,
                               reinterpret_cast<double2 *>(y), k, tc_terms, tcs, tc_error, wait_cycles(), s);
    }

    void unpack() {
        for (bool &p : packed) p = false;
    }

    // The FP64 products over at least EXACT_MIN_COLUMNS right-hand sides on the tensor cores when exact_slices > 0
    // (tc_exact_product: L's, P's and P's imaginary part's integer slice planes, packed on first use; FP64's
    // accuracy); exact_slices = 0 keeps them on the FP64 pipe.
    static constexpr int EXACT_MIN_COLUMNS = 4;
    int exact_slices = 0;
    void *xplane[3] = {};
    size_t xplane_cap[3] = {};
    bool xpacked[3] = {};
    void *xs = nullptr;        // the right-hand sides' slices
    size_t xs_cap = 0;

    cudaError_t sliced_product(int which, int64_t rows, int k, const double *M, int64_t ld, const cd *x, cd *y,
                               cudaStream_t s) {
        cudaError_t e;
        if (!tc_error) {
            if ((e = dev_alloc(&tc_error, 1, s)) || (e = cudaMemsetAsync(tc_error, 0, sizeof(int), s))) return e;
        }
        const size_t pb = tc_exact_plane_bytes(rows, rows, exact_slices);
        if (!xpacked[which] || xplane_cap[which] < pb) {
            if (xplane_cap[which] < pb) {
                dev_free(xplane[which], s);
                xplane[which] = nullptr;
                xplane_cap[which] = 0;
                if ((e = dev_alloc(reinterpret_cast<uint8_t **>(&xplane[which]), pb, s))) return e;
                xplane_cap[which] = pb;
            }
            if ((e = tc_slice_exact(rows, rows, M, ld, exact_slices, xplane[which], s))) return e;
            xpacked[which] = true;
        }
        const size_t sb = tc_exact_scratch_bytes(rows, k, exact_slices);
        if (sb > xs_cap) {
            dev_free(xs, s);
            xs = nullptr;
            xs_cap = 0;
            if ((e = dev_alloc(reinterpret_cast<uint8_t **>(&xs), sb, s))) return e;
            xs_cap = sb;
        }
        return tc_exact_product(rows, rows, xplane[which], k, reinterpret_cast<const double2 *>(x), k,
                                reinterpret_cast<double2 *>(y), k, exact_slices, xs, tc_error, wait_cycles(), s);
    }

    // The compressed operator (pcbqs_gb300_peec_set_compressed): L's edge rows from an H-matrix with the via
    // segments' dense block after them, P = W^T H W from the triangle potential's H-matrix; every product of the
    // operator (FP64, single view included) then goes through them.
    struct HMat {
        int64_t n = 0, nblocks = 0, nslots = 0;
        const int64_t *meta = nullptr, *slot0 = nullptr, *idx = nullptr, *row_ptr = nullptr, *slots_of_row = nullptr;
        const double *store = nullptr;
        int max_rank = 0;
        // the single view's low-rank blocks on the tensor cores (pcbqs_gb300_peec_set_lowrank)
        bool lr = false;
        LowRankPlan plan;
        const int64_t *meta_dense = nullptr, *slot0_dense = nullptr;
        int64_t ndense = 0;
        void *scratch = nullptr;      // tc_lowrank_scratch_bytes, zeroed when allocated
    };
    bool compressed = false;
    HMat hl, hp;
    int64_t nvia = 0;
    const double *via = nullptr;      // nvia x nvia, leading dimension nvia
    Csr W, Wt;                        // triangles x nodes and its transpose
    cd *hslots = nullptr, *tri_x = nullptr, *tri_y = nullptr;
    int64_t hcap = 0;                 // columns the three buffers hold

    cudaError_t hm_apply(HMat &H, bool single, int k, const cd *x, cd *y, cudaStream_t s) {
        if (!single || !H.lr || k > 128)
            return hmatrix_apply(H.n, H.nblocks, H.meta, H.slot0, H.idx, H.store, H.row_ptr, H.slots_of_row,
                                 H.max_rank, k, reinterpret_cast<const double *>(x), reinterpret_cast<double *>(y),
                                 reinterpret_cast<double *>(hslots), s);
        cudaError_t e;
        if (!tc_error) {
            if ((e = dev_alloc(&tc_error, 1, s)) || (e = cudaMemsetAsync(tc_error, 0, sizeof(int), s))) return e;
        }
        if (!H.scratch) {
            const size_t bytes = tc_lowrank_scratch_bytes(H.plan.n_pad, H.plan.ngroups);
            if ((e = dev_alloc(reinterpret_cast<uint8_t **>(&H.scratch), bytes, s)) ||
                (e = cudaMemsetAsync(H.scratch, 0, bytes, s)))
                return e;
        }
        if ((e = hmatrix_blocks(H.ndense, H.meta_dense, H.slot0_dense, H.idx, H.store, H.max_rank, k,
                                reinterpret_cast<const double *>(x), reinterpret_cast<double *>(hslots), s)) ||
            (e = tc_lowrank_product(H.plan, k, reinterpret_cast<const double2 *>(x), reinterpret_cast<double2 *>(hslots),
                                    H.scratch, tc_error, wait_cycles(), s)))
            return e;
        return hmatrix_rows(H.n, H.row_ptr, H.slots_of_row, k, reinterpret_cast<const double *>(hslots),
                            reinterpret_cast<double *>(y), s);
    }

    cudaError_t compressed_product(int which, bool single, int k, const cd *x, cd *y, cudaStream_t s) {
        if (which == 2) return cudaErrorNotSupported;       // no complex P with the compressed operator
        cudaError_t e;
        if (k > hcap) {
            for (cd *p : {hslots, tri_x, tri_y}) dev_free(p, s);
            hslots = tri_x = tri_y = nullptr;
            hcap = 0;
            const int64_t slots = std::max<int64_t>(1, std::max(hl.nslots, hp.nslots));
            if ((e = dev_alloc(&hslots, (size_t)slots * k, s)) ||
                (e = dev_alloc(&tri_x, (size_t)std::max<int64_t>(1, hp.n) * k, s)) ||
                (e = dev_alloc(&tri_y, (size_t)std::max<int64_t>(1, hp.n) * k, s)))
                return e;
            hcap = k;
        }
        if (which == 0) {
            if ((e = hm_apply(hl, single, k, x, y, s))) return e;
            if (nvia) return dense_sym_apply<double, 2>(nvia, k, via, nvia, x + hl.n * k, y + hl.n * k, s);
            return cudaSuccess;
        }
        k_spmm<<<grid_of(hp.n * k), 256, 0, s>>>(W, k, x, tri_x, nullptr, nullptr, 0);
        if ((e = hm_apply(hp, single, k, tri_x, tri_y, s))) return e;
        k_spmm<<<grid_of(nn * k), 256, 0, s>>>(Wt, k, tri_y, y, nullptr, nullptr, 0);
        note_launches(2);
        return cudaGetLastError();
    }

    // which: 0 L, 1 P, 2 P's imaginary part
    cudaError_t dense(int which, bool single, int64_t rows, int k, const double *M, int64_t ld, const float *Mf,
                      int64_t ldf, const cd *x, cd *y, cudaStream_t s) {
        if (compressed) return compressed_product(which, single, k, x, y, s);
        if (!M) return cudaErrorInvalidValue;
        if (!single) {
            if (exact_slices && k >= EXACT_MIN_COLUMNS) return sliced_product(which, rows, k, M, ld, x, y, s);
            return dense_sym_apply<double, 2>(rows, k, M, ld, x, y, s);
        }
        if (!Mf) return cudaErrorInvalidValue;
        if (tc_terms && k >= TC_MIN_COLUMNS) return tensor_product(which, rows, k, Mf, ldf, x, y, s);
        const int64_t need = std::max(ne, nn) * (int64_t)DENSE_NC;
        if (need > capf) {
            dev_free(xf, s);
            xf = nullptr;
            cudaError_t e = dev_alloc(&xf, (size_t)need, s);
            if (e) return e;
            capf = need;
        }
        return dense_sym_apply<float, 4>(rows, k, Mf, ldf, x, y, s, xf);
    }

    cudaError_t apply_impl(bool single, int k, const int32_t *sys, const cd *in, cd *out, cudaStream_t s) {
        cudaError_t e = reserve(k, s);
        if (e) return e;
        k_tree_scale<<<grid_of(n_ * k), 256, 0, s>>>(n_, k, is_tree, walpha, sys, in, u);
        k_spmm<<<grid_of(nb * k), 256, 0, s>>>(K, k, u, branch, nullptr, sys, 0);
        if ((e = dense(0, single, ne, k, L, ldl, Lf, ldlf, branch, lb, s))) return e;
        k_impedance<<<grid_of(nb * k), 256, 0, s>>>(R, nb, k, branch, lb, omega, rscale, nscaled, sys, v);
        k_spmm<<<grid_of(n_ * k), 256, 0, s>>>(Kt, k, v, out, inv_z, sys, 0);
        if (nn > 0) {
            k_spmm<<<grid_of(nn * k), 256, 0, s>>>(T, k, in, tq, nullptr, sys, 0);
            if ((e = dense(1, single, nn, k, P, ldp, Pf, ldpf, tq, pq, s))) return e;
            if (Pim) {          // complex P: P_re q + j (P_im q)
                if ((e = dense(2, single, nn, k, Pim, ldp, Pfim, ldpf, tq, pq2, s))) return e;
                k_add_times_j<<<grid_of(nn * k), 256, 0, s>>>(nn * k, pq2, pq);
                note_launches(1);
            }
            k_spmm<<<grid_of(n_ * k), 256, 0, s>>>(Tt, k, pq, out, inv_p, sys, 1);
        }
        launches += nn > 0 ? 6 : 3;
        note_launches(nn > 0 ? 6 : 3);
        return cudaGetLastError();
    }

    cudaError_t apply(int k, const int32_t *sys, const cd *in, cd *out, cudaStream_t s) override {
        return apply_impl(false, k, sys, in, out, s);
    }

    ~PeecOp() override {
        for (cd *p : {u, branch, lb, v, tq, pq, pq2}) dev_free(p);
        for (double *p : {omega, zscale, walpha, inv_z, inv_p}) dev_free(p);
        dev_free(rscale);
        dev_free(xf);
        for (void *p : plane) dev_free(p);
        for (void *p : xplane) dev_free(p);
        dev_free(xs);
        for (cd *p : {hslots, tri_x, tri_y}) dev_free(p);
        dev_free(hl.scratch);
        dev_free(hp.scratch);
        dev_free(tcs);
        dev_free(tc_error);
    }
};

// The same operator with its dense products in single precision (the inner products of the mixed solve).
struct SingleView : Operator {
    PeecOp *op = nullptr;
    int64_t n() const override { return op->n_; }
    cudaError_t apply(int k, const int32_t *sys, const cd *in, cd *out, cudaStream_t s) override {
        return op->apply_impl(true, k, sys, in, out, s);
    }
};

struct BlockJacobi : Preconditioner {
    int64_t n = 0, nblk = 0;
    int bs = 32;
    cd *inv = nullptr;
    ~BlockJacobi() override { dev_free(inv); }
    cudaError_t apply(int k, const int32_t *sys, const cd *in, cd *out, cudaStream_t s) override {
        k_block_apply<<<grid_of(n * k), 256, 0, s>>>(n, bs, nblk, k, inv, sys, in, out);
        note_launches(1);
        return cudaGetLastError();
    }
};

// ---- dense loop/tree system and its single-precision LU (the MixedLU precedent, src/pcbqs/kernels.py:125-181) ----

// out[j, c] = sum_{a in row j of St} St.val[a] M[St.idx[a], c]  for c < ncols: rows of M combined along the columns of
// S (St = S^T in CSR). Grid: (column chunks, rows j strided by gridDim.y).
__global__ void k_rows_combine(Csr St, const double *M, int64_t ldm, int64_t ncols, double *out, int64_t ldo) {
    for (int64_t j = blockIdx.y; j < St.rows; j += gridDim.y) {
        const int64_t a0 = St.ptr[j], a1 = St.ptr[j + 1];
        for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncols;
             c += (int64_t)gridDim.x * blockDim.x) {
            double acc = 0;
            for (int64_t a = a0; a < a1; ++a) acc += St.val[a] * M[(int64_t)St.idx[a] * ldm + c];
            out[j * ldo + c] = acc;
        }
    }
}

// The same with two columns per thread as one 16-byte load and store (ncols, ldm and ldo even, M and out 16-byte
// aligned): half the memory instructions for the FP64 pipe's and the memory system's queues.
__global__ void k_rows_combine2(Csr St, const double *M, int64_t ldm, int64_t ncols, double *out, int64_t ldo) {
    const int64_t half = ncols / 2;
    for (int64_t j = blockIdx.y; j < St.rows; j += gridDim.y) {
        const int64_t a0 = St.ptr[j], a1 = St.ptr[j + 1];
        for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < half;
             c += (int64_t)gridDim.x * blockDim.x) {
            double2 acc = make_double2(0.0, 0.0);
            for (int64_t a = a0; a < a1; ++a) {
                const double v = St.val[a];
                const double2 m = reinterpret_cast<const double2 *>(M + (int64_t)St.idx[a] * ldm)[c];
                acc.x += v * m.x;
                acc.y += v * m.y;
            }
            reinterpret_cast<double2 *>(out + j * ldo)[c] = acc;
        }
    }
}

// Grid of (x, rows) blocks with the row count within the launch limit; the kernels stride over the rows.
static dim3 row_grid(unsigned x, int64_t rows) {
    return dim3(x, (unsigned)std::min<int64_t>(std::max<int64_t>(rows, 1), 65535));
}

// out (cols x rows) = W^T for W (rows x cols, leading dimension ldw): 32 x 32 tiles through shared memory so that
// both the reads and the writes are coalesced. Block (32, 8), grid (cols / 32, rows / 32).
__global__ void k_transpose(const double *W, int64_t rows, int64_t cols, int64_t ldw, double *out, int64_t ldo) {
    __shared__ double tile[32][33];
    const int64_t c0 = (int64_t)blockIdx.x * 32, r0 = (int64_t)blockIdx.y * 32;
    for (int dy = threadIdx.y; dy < 32; dy += 8) {
        const int64_t r = r0 + dy, c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[dy][threadIdx.x] = W[r * ldw + c];
    }
    __syncthreads();
    for (int dy = threadIdx.y; dy < 32; dy += 8) {
        const int64_t c = c0 + dy, r = r0 + threadIdx.x;
        if (r < rows && c < cols) out[c * ldo + r] = tile[threadIdx.x][dy];
    }
}

// A[i, j] = (j w KLK[i,j]) d_j / zs + TPT[i,j] / ps as complex64, d_j = 1 (loop) or j w alpha (tree). Grid
// (column chunks, rows strided by gridDim.y). The scalings are products with precomputed factors (a division per
// entry costs the slow FP64 pipe more than the whole pass's memory traffic; the result is rounded to FP32).
__global__ void k_assemble_c64(int64_t n, const double *klk, const double *tpt, const double *tpt_im,
                               const int8_t *is_tree, double w, double zs, double ps, float2 *A) {
  const double f = w * zs / ps, wz = w / zs, ips = 1.0 / ps;
  for (int64_t i = blockIdx.y; i < n; i += gridDim.y) {
    const bool tree_i = is_tree[i];
    const double *krow = klk + i * n, *trow = tpt + i * n, *tirow = tpt_im ? tpt_im + i * n : nullptr;
    float2 *arow = A + i * n;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        double re = 0, im = wz * krow[j];
        const bool tree_j = is_tree[j];
        if (tree_j) {                // times j f
            const double r2 = -f * im;
            im = f * re;
            re = r2;
        }
        if (tree_i && tree_j) {
            re += ips * trow[j];
            if (tirow) im += ips * tirow[j];
        }
        arow[j] = make_float2((float)re, (float)im);
    }
  }
}

// A[i, j] += KRK[i, j] d_j / zs for the sparse K^T R K.
__global__ void k_add_krk_c64(Csr S, const int8_t *is_tree, double w, double zs, double ps, cd rs, float2 *A) {
    const double f = w * zs / ps;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < S.rows; i += (int64_t)gridDim.x * blockDim.x)
        for (int64_t a = S.ptr[i]; a < S.ptr[i + 1]; ++a) {
            const int64_t j = S.idx[a];
            const double v = S.val[a] / zs;
            float2 &e = A[i * S.cols + j];
            if (is_tree[j]) {           // times j f
                e.x += (float)(-f * rs.y * v);
                e.y += (float)(f * rs.x * v);
            } else {
                e.x += (float)(rs.x * v);
                e.y += (float)(rs.y * v);
            }
        }
}

// Row-major (n, k) complex128 <-> column-major (n, k) complex64.
__global__ void k_to_c64_cols(int64_t n, int k, const cd *in, float2 *out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * k; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / k;
        const int s = (int)(t % k);
        out[(int64_t)s * n + r] = make_float2((float)in[t].x, (float)in[t].y);
    }
}

__global__ void k_from_c64_cols(int64_t n, int k, const float2 *in, cd *out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * k; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / k;
        const int s = (int)(t % k);
        const float2 v = in[(int64_t)s * n + r];
        out[t] = make_double2(v.x, v.y);
    }
}

struct LuPrecond : Preconditioner {
    int64_t n = 0;
    float2 *lu = nullptr;        // complex64 factor of the row-major system (the transpose, column-major)
    int *ipiv = nullptr, *info = nullptr;
    float2 *work = nullptr;      // right-hand sides, column-major (library solve)
    int cap = 0;
    cusolverDnHandle_t solver = nullptr;
    TriSolver tri;               // streaming triangular solves (the solve every GMRES step uses)
    ~LuPrecond() override {
        tri.release();
        dev_free(lu);
        dev_free(ipiv);
        dev_free(info);
        dev_free(work);
        if (solver) cusolverDnDestroy(solver);
    }
    cudaError_t apply(int k, const int32_t *, const cd *in, cd *out, cudaStream_t s) override {
        return tri.solve(k, in, out, s);
    }
    int deferred_k = 0;
    cudaError_t apply_deferred(int k, const int32_t *, const cd *in, cd *out, cudaStream_t s) override {
        deferred_k = k;
        return tri.solve(k, in, out, s, true);
    }
    cudaError_t deferred_status(cudaStream_t s) override {
        return deferred_k ? tri.read_status(deferred_k, s) : cudaSuccess;
    }
    // The same solve through cuSOLVER getrs, for validation of the streaming solver.
    cudaError_t apply_library(int k, const cd *in, cd *out, cudaStream_t s) {
        if (k > cap) {
            dev_free(work, s);
            work = nullptr;
            cudaError_t e = dev_alloc(&work, (size_t)n * k, s);
            if (e) return e;
            cap = k;
        }
        cusolverDnSetStream(solver, s);
        k_to_c64_cols<<<grid_of(n * k), 256, 0, s>>>(n, k, in, work);
        if (cusolverDnCgetrs(solver, CUBLAS_OP_T, (int)n, k, reinterpret_cast<cuComplex *>(lu), (int)n, ipiv,
                             reinterpret_cast<cuComplex *>(work), (int)n, info) != CUSOLVER_STATUS_SUCCESS)
            return cudaErrorUnknown;
        k_from_c64_cols<<<grid_of(n * k), 256, 0, s>>>(n, k, work, out);
        note_launches(2);
        return cudaGetLastError();
    }
};

// The FP32 Cholesky factor of P in the LU layout of the streaming triangular solver: P = L L^T = (L D^-1)(D L^T),
// D = diag(L), so with M = P^T = P the column-major array holds the unit lower L D^-1 below the diagonal and the
// upper D L^T on and above it (no pivoting), as complex64 with zero imaginary parts.
__global__ void k_cholesky_to_lu(int64_t n, const float *chol, int64_t ldc, float2 *lu) {
    for (int64_t j = blockIdx.y; j < n; j += gridDim.y) {   // column j of the column-major arrays
        const float djj = chol[j + j * ldc];
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
             i += (int64_t)gridDim.x * blockDim.x) {
            const float v = i > j ? chol[i + j * ldc] / djj : chol[i + i * ldc] * chol[j + i * ldc];
            lu[i + j * n] = make_float2(v, 0.f);
        }
    }
}

__global__ void k_identity_pivots(int64_t n, int *ipiv) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        ipiv[t] = (int)(t + 1);
}

constexpr int CHOL_BLOCK = 1024;   // panel width of the blocked Cholesky

// Row-major (n, k) complex128 -> column-major (n, 2k) FP32: the real parts in columns 0..k-1, the imaginary parts
// in k..2k-1 (real right-hand sides for a real factor); and back.
__global__ void k_split_cols_f32(int64_t n, int k, const cd *in, float *out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * k; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / k;
        const int c = (int)(t % k);
        out[(int64_t)c * n + r] = (float)in[t].x;
        out[(int64_t)(k + c) * n + r] = (float)in[t].y;
    }
}

__global__ void k_join_cols_f32(int64_t n, int k, const float *in, cd *out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * k; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / k;
        const int c = (int)(t % k);
        out[t] = make_double2(in[(int64_t)c * n + r], in[(int64_t)(k + c) * n + r]);
    }
}

// out (n x n, leading dimension ldo) = in (n x n, leading dimension ldi) in FP32.
__global__ void k_to_f32_strided(int64_t n, const double *in, int64_t ldi, float *out, int64_t ldo) {
    for (int64_t r = blockIdx.y; r < n; r += gridDim.y)
        for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
            out[r * ldo + c] = (float)in[r * ldi + c];
}

struct CholPrecond : Preconditioner {
    int64_t n = 0, ldc = 0;      // the FP32 factor's leading dimension: n rounded up to 32 (aligned GEMM forms)
    float *chol = nullptr;
    float2 *lu = nullptr;
    int *ipiv = nullptr;
    TriSolver tri;
    // library = true: solves with cuBLAS triangular solves on the FP32 factor instead of the streaming sweeps.
    // Slower alone, but ordinary kernels, so the solve may run beside other work on the device (the sweeps are
    // cooperative kernels that must have it to themselves).
    bool library = false;
    cublasHandle_t blas = nullptr;
    float *work = nullptr;
    int cap = 0;
    ~CholPrecond() override {
        tri.release();
        dev_free(chol);
        dev_free(lu);
        dev_free(ipiv);
        dev_free(work);
        if (blas) cublasDestroy(blas);
    }
    cudaError_t factor(int64_t n_, const double *A, int64_t lda, cudaStream_t s, int &host_info) {
        n = n_;
        ldc = (n + 31) / 32 * 32;
        cudaError_t e;
        if ((e = dev_alloc(&chol, (size_t)n * ldc, s))) return e;
        // A symmetric: its rows are the columns of the column-major copy
        k_to_f32_strided<<<row_grid((unsigned)std::min<int64_t>((n + 255) / 256, 8), n), 256, 0, s>>>(n, A, lda, chol,
                                                                                                     ldc);
        note_launches(1);
        // blocked, FP32 arithmetic emulated with BF16x9 products on the tensor cores (FP32 accuracy)
        if ((e = potrf_blocked(n, chol, ldc, CHOL_BLOCK, LU_GEMM_BF16X9, s, &host_info)) || host_info) return e;
        if (library) {
            if (cublasCreate(&blas) != CUBLAS_STATUS_SUCCESS) return cudaErrorNotSupported;
            return cudaStreamSynchronize(s);
        }
        // the factor in the triangular solver's layout; the FP32 copy is not needed afterwards
        if ((e = dev_alloc(&lu, (size_t)n * n, s)) || (e = dev_alloc(&ipiv, (size_t)n, s))) return e;
        k_cholesky_to_lu<<<row_grid((unsigned)std::min<int64_t>((n + 255) / 256, 8), n), 256, 0, s>>>(n, chol, ldc,
                                                                                                     lu);
        k_identity_pivots<<<grid_of(n), 256, 0, s>>>(n, ipiv);
        note_launches(2);
        if ((e = tri.prepare(lu, n, ipiv, s))) return e;
        dev_free(chol, s);
        chol = nullptr;
        return cudaStreamSynchronize(s);
    }
    cudaError_t apply(int k, const int32_t *, const cd *in, cd *out, cudaStream_t s) override {
        if (!library) return tri.solve(k, in, out, s);
        if (2 * k > cap) {
            dev_free(work, s);
            work = nullptr;
            cudaError_t e = dev_alloc(&work, (size_t)n * 2 * k, s);
            if (e) return e;
            cap = 2 * k;
        }
        const float one = 1.f;
        cublasSetStream(blas, s);
        k_split_cols_f32<<<grid_of(n * k), 256, 0, s>>>(n, k, in, work);
        if (cublasStrsm(blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, (int)n,
                        2 * k, &one, chol, (int)ldc, work, (int)n) != CUBLAS_STATUS_SUCCESS ||
            cublasStrsm(blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, (int)n,
                        2 * k, &one, chol, (int)ldc, work, (int)n) != CUBLAS_STATUS_SUCCESS)
            return cudaErrorUnknown;
        k_join_cols_f32<<<grid_of(n * k), 256, 0, s>>>(n, k, work, out);
        note_launches(2);
        return cudaGetLastError();
    }
};

struct DenseSym : Operator {
    int64_t n_ = 0, ld = 0;
    const double *A = nullptr, *Aim = nullptr;   // real and (nullable) imaginary parts, both symmetric
    cd *tmp = nullptr;
    int cap = 0;
    int64_t n() const override { return n_; }
    ~DenseSym() override { dev_free(tmp); }
    cudaError_t apply(int k, const int32_t *, const cd *in, cd *out, cudaStream_t s) override {
        cudaError_t e = dense_sym_apply<double, 2>(n_, k, A, ld, in, out, s);
        if (e || !Aim) return e;
        if (k > cap) {
            dev_free(tmp, s);
            tmp = nullptr;
            if ((e = dev_alloc(&tmp, (size_t)n_ * k, s))) return e;
            cap = k;
        }
        if ((e = dense_sym_apply<double, 2>(n_, k, Aim, ld, in, tmp, s))) return e;
        k_add_times_j<<<grid_of(n_ * k), 256, 0, s>>>(n_ * k, tmp, out);
        note_launches(1);
        return cudaGetLastError();
    }
};

struct Jacobi : Preconditioner {
    int64_t n = 0;
    double *d = nullptr;
    cudaError_t apply(int k, const int32_t *, const cd *in, cd *out, cudaStream_t s) override {
        k_diag_apply<<<grid_of(n * k), 256, 0, s>>>(n, k, d, in, out);
        note_launches(1);
        return cudaGetLastError();
    }
};

// P alone (nn x nn) through the operator's own P products (dense or compressed), for the equilibrium charge.
struct PotentialView : Operator {
    PeecOp *op = nullptr;
    int64_t n() const override { return op->nn; }
    cudaError_t apply(int k, const int32_t *, const cd *in, cd *out, cudaStream_t s) override {
        return op->dense(1, false, op->nn, k, op->P, op->ldp, nullptr, 0, in, out, s);
    }
};

// ---- graph preconditioner (src/pcbqs/peec_iterative.py:19-84, without face-sheet pairs) ----
//
// For y (n x k, the operator's order), with d the passive branches' own impedance (zdiag), Dinv = 1/d, zs the
// system's zscale, ps the potential scale, and kept nodes all but each component's root:
//   trial_j = zs dinv_b(j) y_j on each loop j (b(j) its defining branch), v = G^-1 (Ap trial)[keep],
//   G = Ap Dinv Ap^T [keep][:, keep] (dense complex64 LU, optionally one FP64 residual correction);
//   out_j = trial_j - dinv_b(j) (v_a - v_b) on each loop (a, b the ends of b(j), v = 0 at a root);
//   rt_j = y_j - d_b(j) / zs (K_loops out)_b(j) on each tree unknown;
//   v2 = T[keep]^-T rt, m_c = sum_{i in c} pinv_i v2_i / total_c, charge_i = pinv_i (v2_i - m_c(i));
//   out_j = ps (T[keep]^-1 charge)_j on each tree unknown.
// Every kernel below takes (rows x k) row-major complex128 arrays, one thread per (row, column).

static __device__ __forceinline__ cd zmul(cd a, cd b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// G (nkeep x nkeep, row-major = column-major: G is symmetric) from the branches at each kept node: the diagonal the
// sum of their 1/d, -1/d at the other end's column (none at a root). One thread per row; G zeroed beforehand.
__global__ void k_graph_laplacian(int64_t nkeep, const int64_t *lap_ptr, const int32_t *lap_branch,
                                  const int32_t *lap_other, const cd *dinv, float2 *G) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nkeep; i += (int64_t)gridDim.x * blockDim.x) {
        double re = 0, im = 0;
        float2 *row = G + i * nkeep;
        for (int64_t a = lap_ptr[i]; a < lap_ptr[i + 1]; ++a) {
            const cd w = dinv[lap_branch[a]];
            re += w.x;
            im += w.y;
            const int32_t o = lap_other[a];
            if (o >= 0) {
                row[o].x -= (float)w.x;
                row[o].y -= (float)w.y;
            }
        }
        row[i].x += (float)re;
        row[i].y += (float)im;
    }
}

// rhs[i, c] = sum over the loops j incident to kept node i of ac_ij zs dinv_b(j) y[j, c]   (Ap trial)
__global__ void k_graph_node_rhs(Csr ac, int k, const int32_t *branch, const cd *dinv, double zs, const cd *y,
                                 cd *rhs) {
    const int64_t total = ac.rows * k;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / k;
        const int c = (int)(t % k);
        cd acc = make_double2(0, 0);
        for (int64_t a = ac.ptr[i]; a < ac.ptr[i + 1]; ++a) {
            const int32_t j = ac.idx[a];
            const cd w = dinv[branch[j]];
            const double f = zs * ac.val[a];
            const cd p = zmul(make_double2(f * w.x, f * w.y), y[(int64_t)j * k + c]);
            acc.x += p.x;
            acc.y += p.y;
        }
        rhs[t] = acc;
    }
}

// r = rhs - G v with G from the branches in FP64 (the Laplacian solve's residual correction).
__global__ void k_graph_residual(int64_t nkeep, int k, const int64_t *lap_ptr, const int32_t *lap_branch,
                                 const int32_t *lap_other, const cd *dinv, const cd *v, const cd *rhs, cd *r) {
    const int64_t total = nkeep * k;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / k;
        const int c = (int)(t % k);
        const cd vi = v[t];
        cd acc = rhs[t];
        for (int64_t a = lap_ptr[i]; a < lap_ptr[i + 1]; ++a) {
            const int32_t o = lap_other[a];
            const cd vo = o >= 0 ? v[(int64_t)o * k + c] : make_double2(0, 0);
            const cd p = zmul(dinv[lap_branch[a]], make_double2(vi.x - vo.x, vi.y - vo.y));
            acc.x -= p.x;
            acc.y -= p.y;
        }
        r[t] = acc;
    }
}

__global__ void k_graph_add(int64_t count, const cd *x, cd *y) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x) {
        y[t].x += x[t].x;
        y[t].y += x[t].y;
    }
}

// The loop unknowns' outputs: trial_j - dinv_b(j) (v_a - v_b).
__global__ void k_graph_loops(int64_t n, int k, const int8_t *is_tree, const int32_t *branch, const int32_t *ends,
                              const cd *dinv, double zs, const cd *y, const cd *v, cd *out) {
    const int64_t total = n * k;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = t / k;
        if (is_tree[j]) continue;
        const int c = (int)(t % k);
        const cd w = dinv[branch[j]];
        const int32_t a = ends[2 * j], b = ends[2 * j + 1];
        const cd va = a >= 0 ? v[(int64_t)a * k + c] : make_double2(0, 0);
        const cd vb = b >= 0 ? v[(int64_t)b * k + c] : make_double2(0, 0);
        const cd trial = zmul(make_double2(zs * w.x, zs * w.y), y[t]);
        const cd drop = zmul(w, make_double2(va.x - vb.x, va.y - vb.y));
        out[t] = make_double2(trial.x - drop.x, trial.y - drop.y);
    }
}

// The tree unknowns' right-hand side: rt_j = y_j - d_b / zs sum over the loop columns of K's row b of K_bl out_l,
// b = branch[j] (K: passive branches x unknowns). Loop rows of rt are set to zero.
__global__ void k_graph_tree_rhs(int64_t n, int k, const int8_t *is_tree, const int32_t *branch, Csr K,
                                 const cd *zdiag, double inv_zs, const cd *y, const cd *out, cd *rt) {
    const int64_t total = n * k;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = t / k;
        if (!is_tree[j]) {
            rt[t] = make_double2(0, 0);
            continue;
        }
        const int c = (int)(t % k);
        const int32_t b = branch[j];
        cd acc = make_double2(0, 0);
        for (int64_t a = K.ptr[b]; a < K.ptr[b + 1]; ++a) {
            const int32_t l = K.idx[a];
            if (is_tree[l]) continue;
            const cd x = out[(int64_t)l * k + c];
            acc.x += K.val[a] * x.x;
            acc.y += K.val[a] * x.y;
        }
        const cd z = zdiag[b];
        const cd p = zmul(make_double2(z.x * inv_zs, z.y * inv_zs), acc);
        rt[t] = make_double2(y[t].x - p.x, y[t].y - p.y);
    }
}

// m[c, col] = rtotal_c sum over component c's kept rows i of pinv_i v2[i, col]. Block (32 columns, 16 row
// strides) per (component, 32-column chunk); a fixed summation order.
__global__ void __launch_bounds__(512) k_graph_common(int k, const int64_t *member_ptr, const int32_t *members,
                                                      const cd *pinv, const cd *rtotal, const cd *v2, cd *m) {
    __shared__ cd part[16][32];
    const int comp = blockIdx.x;
    const int c = blockIdx.y * 32 + threadIdx.x;
    cd acc = make_double2(0, 0);
    if (c < k)
        for (int64_t a = member_ptr[comp] + threadIdx.y; a < member_ptr[comp + 1]; a += 16) {
            const int32_t i = members[a];
            const cd p = zmul(pinv[i], v2[(int64_t)i * k + c]);
            acc.x += p.x;
            acc.y += p.y;
        }
    part[threadIdx.y][threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.y == 0 && c < k) {
        cd s = part[0][threadIdx.x];
        for (int r = 1; r < 16; ++r) {
            s.x += part[r][threadIdx.x].x;
            s.y += part[r][threadIdx.x].y;
        }
        m[(int64_t)comp * k + c] = zmul(s, rtotal[comp]);
    }
}

// charge (in place of v2) = pinv_i (v2_i - m_comp(i)).
__global__ void k_graph_charge(int64_t nkeep, int k, const int32_t *comp, const cd *pinv, const cd *m, cd *v2) {
    const int64_t total = nkeep * k;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / k;
        const int c = (int)(t % k);
        const cd mm = m[(int64_t)comp[i] * k + c];
        v2[t] = zmul(pinv[i], make_double2(v2[t].x - mm.x, v2[t].y - mm.y));
    }
}

// The tree unknowns' outputs: ps (T[keep]^-1 charge)_j; loop rows and the long rows (k_graph_tree_out_long)
// untouched.
__global__ void k_graph_tree_out(int64_t n, int k, const int8_t *is_tree, const int8_t *long_row, Csr tinv, double ps,
                                 const cd *charge, cd *out) {
    const int64_t total = n * k;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = t / k;
        if (!is_tree[j] || long_row[j]) continue;
        const int c = (int)(t % k);
        double re = 0, im = 0;
        for (int64_t a = tinv.ptr[j]; a < tinv.ptr[j + 1]; ++a) {
            const cd x = charge[(int64_t)tinv.idx[a] * k + c];
            re += tinv.val[a] * x.x;
            im += tinv.val[a] * x.y;
        }
        out[t] = make_double2(ps * re, ps * im);
    }
}

// The graph Laplacian's solve, x = G^-1 r for k columns ((nkeep, k) complex128 row-major, kept-row order).
struct LapSolver {
    virtual ~LapSolver() = default;
    // deferred: capturable (no host synchronization or allocation; after one call with this k)
    virtual cudaError_t solve(int k, const cd *r, cd *x, cudaStream_t s, bool deferred) = 0;
    virtual cudaError_t status(int k, cudaStream_t s) { return cudaSuccess; }
};

// G dense in complex64, LU-factored by getrf_blocked (tcgen05 updates), solved by the streaming/blocked TriSolver.
struct DenseLap : LapSolver {
    float2 *G = nullptr;
    int *ipiv = nullptr;
    TriSolver tri;
    ~DenseLap() override {
        tri.release();
        dev_free(G);
        dev_free(ipiv);
    }
    cudaError_t solve(int k, const cd *r, cd *x, cudaStream_t s, bool deferred) override {
        return tri.solve(k, r, x, s, deferred);
    }
    cudaError_t status(int k, cudaStream_t s) override { return tri.read_status(k, s); }
};

// rows new position p of `in` (kept-row order) -> out[p] = in[perm[p]]; and back.
__global__ void k_rows_gather(int64_t rows, int k, const int64_t *perm, const cd *in, cd *out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < rows * k; t += (int64_t)gridDim.x * blockDim.x)
        out[t] = in[perm[t / k] * k + t % k];
}

__global__ void k_rows_scatter(int64_t rows, int k, const int64_t *perm, const cd *in, cd *out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < rows * k; t += (int64_t)gridDim.x * blockDim.x)
        out[perm[t / k] * k + t % k] = in[t];
}

// out (n, k) row-major complex128 += in (n x k column-major complex64)
__global__ void k_from_c64_cols_add(int64_t n, int k, const float2 *in, cd *out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * k; t += (int64_t)gridDim.x * blockDim.x) {
        const float2 v = in[(t % k) * n + t / k];
        out[t].x += v.x;
        out[t].y += v.y;
    }
}

// One domain's block of G (nd x nd, rows = columns: symmetric), zeroed beforehand: the diagonal sums every branch of
// the row's node, the off-diagonal entries only the branches to the domain's own interior.
__global__ void k_domain_block(int64_t off, int64_t nd, const int64_t *perm, const int64_t *pos,
                               const int64_t *lap_ptr, const int32_t *lap_branch, const int32_t *lap_other,
                               const cd *dinv, float2 *A) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t kr = perm[off + i];
        double re = 0, im = 0;
        for (int64_t a = lap_ptr[kr]; a < lap_ptr[kr + 1]; ++a) {
            const cd w = dinv[lap_branch[a]];
            re += w.x;
            im += w.y;
            const int32_t o = lap_other[a];
            if (o < 0) continue;
            const int64_t q = pos[o] - off;
            if (q >= 0 && q < nd) {
                A[i * nd + q].x -= (float)w.x;
                A[i * nd + q].y -= (float)w.y;
            }
        }
        A[i * nd + i].x += (float)re;
        A[i * nd + i].y += (float)im;
    }
}

__global__ void k_identity_c64(int64_t n, float2 *A) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n; t += (int64_t)gridDim.x * blockDim.x)
        A[t] = make_float2(t / n == t % n ? 1.f : 0.f, 0.f);
}

// The separator block G_SS (ns x ns, zeroed beforehand): rows at new positions n_int + p.
__global__ void k_separator_block(int64_t ns, int64_t n_int, const int64_t *perm, const int64_t *pos,
                                  const int64_t *lap_ptr, const int32_t *lap_branch, const int32_t *lap_other,
                                  const cd *dinv, float2 *S) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < ns; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t kr = perm[n_int + p];
        double re = 0, im = 0;
        for (int64_t a = lap_ptr[kr]; a < lap_ptr[kr + 1]; ++a) {
            const cd w = dinv[lap_branch[a]];
            re += w.x;
            im += w.y;
            const int32_t o = lap_other[a];
            if (o < 0) continue;
            const int64_t q = pos[o] - n_int;
            if (q >= 0) {
                S[p * ns + q].x -= (float)w.x;
                S[p * ns + q].y -= (float)w.y;
            }
        }
        S[p * ns + p].x += (float)re;
        S[p * ns + p].y += (float)im;
    }
}

// One domain's Schur term: S[bnd_p, bnd_q] -= sum_{i ~ p} sum_{j ~ q} w_pi Ainv[i, j] w_qj over its m boundary
// entries (nptr: each entry's interior neighbours, local rows and branches). One thread per (p, q).
__global__ void k_schur_domain(int64_t m, const int32_t *bnd, const int64_t *nptr, const int32_t *local,
                               const int32_t *branch, const cd *dinv, const float2 *Ainv, int64_t nd, float2 *S,
                               int64_t ns) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m * m; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = t / m, q = t % m;
        cd acc = make_double2(0, 0);
        for (int64_t a = nptr[p]; a < nptr[p + 1]; ++a) {
            const cd wa = dinv[branch[a]];
            cd row = make_double2(0, 0);
            for (int64_t b = nptr[q]; b < nptr[q + 1]; ++b) {
                const float2 v = Ainv[(int64_t)local[a] + (int64_t)local[b] * nd];
                const cd pr = zmul(make_double2(v.x, v.y), dinv[branch[b]]);
                row.x += pr.x;
                row.y += pr.y;
            }
            const cd pr = zmul(wa, row);
            acc.x += pr.x;
            acc.y += pr.y;
        }
        float2 &e = S[(int64_t)bnd[p] * ns + bnd[q]];
        e.x -= (float)acc.x;
        e.y -= (float)acc.y;
    }
}

// r_S = r_S + sum over each separator row's interior neighbours of w y_I   (r_S - G_SI y_I)
__global__ void k_separator_rhs(int64_t ns, int k, int64_t n_int, const int64_t *perm, const int64_t *pos,
                                const int64_t *lap_ptr, const int32_t *lap_branch, const int32_t *lap_other,
                                const cd *dinv, const cd *rn, const cd *yI, cd *rS) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ns * k; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = t / k;
        const int c = (int)(t % k);
        const int64_t kr = perm[n_int + p];
        cd acc = rn[(n_int + p) * k + c];
        for (int64_t a = lap_ptr[kr]; a < lap_ptr[kr + 1]; ++a) {
            const int32_t o = lap_other[a];
            if (o < 0) continue;
            const int64_t q = pos[o];
            if (q >= n_int) continue;
            const cd pr = zmul(dinv[lap_branch[a]], yI[q * k + c]);
            acc.x += pr.x;
            acc.y += pr.y;
        }
        rS[t] = acc;
    }
}

// t_I = sum over each interior row's separator neighbours of w x_S   (-G_IS x_S)
__global__ void k_interior_coupling(int64_t n_int, int k, const int64_t *perm, const int64_t *pos,
                                    const int64_t *lap_ptr, const int32_t *lap_branch, const int32_t *lap_other,
                                    const cd *dinv, const cd *xS, cd *tI) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_int * k;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = t / k;
        const int c = (int)(t % k);
        const int64_t kr = perm[p];
        cd acc = make_double2(0, 0);
        for (int64_t a = lap_ptr[kr]; a < lap_ptr[kr + 1]; ++a) {
            const int32_t o = lap_other[a];
            if (o < 0) continue;
            const int64_t q = pos[o];
            if (q < n_int) continue;
            const cd pr = zmul(dinv[lap_branch[a]], xS[(q - n_int) * k + c]);
            acc.x += pr.x;
            acc.y += pr.y;
        }
        tI[t] = acc;
    }
}

// G split into `parts` domain interiors (no edges between them) and a separator S:
//   G = [A_I  G_IS; G_SI  G_SS],  A_I = diag(A_d),  Schur S = G_SS - sum_d G_Sd A_d^-1 G_dS,
//   y_I = A_I^-1 r_I,  x_S = S^-1 (r_S - G_SI y_I),  x_I = y_I - A_I^-1 G_IS x_S.
// The domains' inverses are explicit in complex64 (cuSOLVER getrf + getrs against the identity at set-up), applied
// per domain as cuBLAS complex64 GEMMs over all columns; S is dense in complex64, LU-factored by getrf_blocked and
// solved by the TriSolver. Not capturable (its cuBLAS calls stay outside CUDA graphs).
struct DomainLap : LapSolver {
    int64_t nk = 0, n_int = 0, ns = 0, parts = 0;
    std::vector<int64_t> dom_ptr, bnd_ptr, blk_off;
    const int64_t *perm = nullptr, *pos = nullptr, *lap_ptr = nullptr;
    const int32_t *lap_branch = nullptr, *lap_other = nullptr;
    const cd *dinv = nullptr;
    float2 *Ainv = nullptr, *S = nullptr;
    int *ipiv = nullptr;
    TriSolver tri;
    cublasHandle_t blas = nullptr;
    int cap = 0;
    cd *rn = nullptr, *yI = nullptr, *rS = nullptr, *xS = nullptr, *tI = nullptr;
    float2 *f1 = nullptr, *f2 = nullptr;
    void free_work() {
        for (void *p : {(void *)rn, (void *)yI, (void *)rS, (void *)xS, (void *)tI, (void *)f1, (void *)f2}) dev_free(p);
        rn = yI = rS = xS = tI = nullptr;
        f1 = f2 = nullptr;
        cap = 0;
    }
    ~DomainLap() override {
        tri.release();
        free_work();
        dev_free(Ainv);
        dev_free(S);
        dev_free(ipiv);
        if (blas) cublasDestroy(blas);
    }
    cudaError_t reserve(int k, cudaStream_t s) {
        if (k <= cap) return cudaSuccess;
        free_work();
        cudaError_t e;
        if ((e = dev_alloc(&rn, (size_t)nk * k, s)) || (e = dev_alloc(&yI, (size_t)n_int * k, s)) ||
            (e = dev_alloc(&rS, (size_t)ns * k, s)) || (e = dev_alloc(&xS, (size_t)ns * k, s)) ||
            (e = dev_alloc(&tI, (size_t)n_int * k, s)) || (e = dev_alloc(&f1, (size_t)n_int * k, s)) ||
            (e = dev_alloc(&f2, (size_t)n_int * k, s))) {
            free_work();
            return e;
        }
        cap = k;
        return cudaSuccess;
    }
    // f2 = A_I^-1 f1, both (n_int x k) column-major complex64
    cudaError_t domains_apply(int k, cudaStream_t s) {
        cublasSetStream(blas, s);
        const cuComplex one = make_cuComplex(1.f, 0.f), zero = make_cuComplex(0.f, 0.f);
        for (int64_t d = 0; d < parts; ++d) {
            const int64_t off = dom_ptr[d], nd = dom_ptr[d + 1] - off;
            if (!nd) continue;
            if (cublasCgemm(blas, CUBLAS_OP_N, CUBLAS_OP_N, (int)nd, k, (int)nd, &one,
                            reinterpret_cast<const cuComplex *>(Ainv + blk_off[d]), (int)nd,
                            reinterpret_cast<const cuComplex *>(f1 + off), (int)n_int, &zero,
                            reinterpret_cast<cuComplex *>(f2 + off), (int)n_int) != CUBLAS_STATUS_SUCCESS)
                return cudaErrorUnknown;
        }
        return cudaSuccess;
    }
    cudaError_t solve(int k, const cd *r, cd *x, cudaStream_t s, bool deferred) override {
        if (deferred) return cudaErrorNotSupported;
        cudaError_t e;
        if ((e = reserve(k, s))) return e;
        k_rows_gather<<<grid_of(nk * k), 256, 0, s>>>(nk, k, perm, r, rn);
        k_to_c64_cols<<<grid_of(n_int * k), 256, 0, s>>>(n_int, k, rn, f1);
        if ((e = domains_apply(k, s))) return e;
        k_from_c64_cols<<<grid_of(n_int * k), 256, 0, s>>>(n_int, k, f2, yI);
        k_separator_rhs<<<grid_of(ns * k), 256, 0, s>>>(ns, k, n_int, perm, pos, lap_ptr, lap_branch, lap_other,
                                                         dinv, rn, yI, rS);
        if ((e = tri.solve(k, rS, xS, s, false))) return e;
        k_interior_coupling<<<grid_of(n_int * k), 256, 0, s>>>(n_int, k, perm, pos, lap_ptr, lap_branch, lap_other,
                                                                dinv, xS, tI);
        k_to_c64_cols<<<grid_of(n_int * k), 256, 0, s>>>(n_int, k, tI, f1);
        if ((e = domains_apply(k, s))) return e;
        k_from_c64_cols_add<<<grid_of(n_int * k), 256, 0, s>>>(n_int, k, f2, yI);
        k_rows_scatter<<<grid_of(n_int * k), 256, 0, s>>>(n_int, k, perm, yI, x);
        k_rows_scatter<<<grid_of(ns * k), 256, 0, s>>>(ns, k, perm + n_int, xS, x);
        note_launches(10 + 2 * (int)parts);
        return cudaGetLastError();
    }
};

// The same for the rows of T[keep]^-1 longer than GRAPH_LONG_ROW entries (the branches near a root: their subtrees
// hold most of the nodes), one thread block per row: the threads stride over the row's entries with
// GRAPH_ROW_COLS columns at a time in registers, then a fixed-order tree reduction in shared memory.
constexpr int GRAPH_LONG_ROW = 512;
constexpr int GRAPH_ROW_COLS = 8;

__global__ void __launch_bounds__(256) k_graph_tree_out_long(const int32_t *rows, int k, Csr tinv, double ps,
                                                             const cd *charge, cd *out) {
    __shared__ cd part[256][GRAPH_ROW_COLS];
    const int64_t j = rows[blockIdx.x];
    const int64_t a0 = tinv.ptr[j], a1 = tinv.ptr[j + 1];
    for (int c0 = 0; c0 < k; c0 += GRAPH_ROW_COLS) {
        const int nc = min(GRAPH_ROW_COLS, k - c0);
        cd acc[GRAPH_ROW_COLS];
        for (int c = 0; c < GRAPH_ROW_COLS; ++c) acc[c] = make_double2(0, 0);
        for (int64_t a = a0 + threadIdx.x; a < a1; a += blockDim.x) {
            const double v = tinv.val[a];
            const cd *x = charge + (int64_t)tinv.idx[a] * k + c0;
            for (int c = 0; c < GRAPH_ROW_COLS; ++c)
                if (c < nc) {
                    acc[c].x += v * x[c].x;
                    acc[c].y += v * x[c].y;
                }
        }
        for (int c = 0; c < GRAPH_ROW_COLS; ++c) part[threadIdx.x][c] = acc[c];
        __syncthreads();
        for (int stride = blockDim.x / 2; stride > 0; stride >>= 1) {
            if ((int)threadIdx.x < stride)
                for (int c = 0; c < GRAPH_ROW_COLS; ++c) {
                    part[threadIdx.x][c].x += part[threadIdx.x + stride][c].x;
                    part[threadIdx.x][c].y += part[threadIdx.x + stride][c].y;
                }
            __syncthreads();
        }
        if ((int)threadIdx.x < nc)
            out[j * k + c0 + threadIdx.x] = make_double2(ps * part[0][threadIdx.x].x, ps * part[0][threadIdx.x].y);
        __syncthreads();
    }
}

struct GraphPrecond : Preconditioner {
    int64_t n = 0, nkeep = 0, ncomp = 0, nbranch = 0;
    int32_t *long_rows = nullptr;     // the tree unknowns whose row of T[keep]^-1 is longer than GRAPH_LONG_ROW
    int8_t *long_flag = nullptr;      // n: 1 on those rows
    int64_t nlong = 0;
    Csr ac, tinv, tinvt, K;
    const int64_t *lap_ptr = nullptr, *member_ptr = nullptr;
    const int32_t *lap_branch = nullptr, *lap_other = nullptr, *branch = nullptr, *loop_ends = nullptr,
                  *comp = nullptr, *members = nullptr;
    const int8_t *is_tree = nullptr;
    cd *zdiag = nullptr, *dinv = nullptr, *pinv = nullptr, *rtotal = nullptr;   // owned (rtotal = 1 / total)
    double zs = 1, ps = 1;
    int refine = 0;          // FP64 residual corrections of each Laplacian solve
    LapSolver *lap = nullptr;
    int cap = 0, deferred_k = 0;
    cd *rhs = nullptr, *v = nullptr, *corr = nullptr, *rt = nullptr, *v2 = nullptr, *m = nullptr;

    void free_work() {
        for (cd *p : {rhs, v, corr, rt, v2, m}) dev_free(p);
        rhs = v = corr = rt = v2 = m = nullptr;
        cap = 0;
    }
    ~GraphPrecond() override {
        delete lap;
        free_work();
        for (void *p : {(void *)zdiag, (void *)dinv, (void *)pinv, (void *)rtotal, (void *)long_rows,
                        (void *)long_flag})
            dev_free(p);
    }
    cudaError_t reserve(int k, cudaStream_t s) {
        if (k <= cap) return cudaSuccess;
        free_work();
        cudaError_t e;
        if ((e = dev_alloc(&rhs, (size_t)nkeep * k, s)) || (e = dev_alloc(&v, (size_t)nkeep * k, s)) ||
            (e = dev_alloc(&corr, (size_t)nkeep * k, s)) || (e = dev_alloc(&rt, (size_t)n * k, s)) ||
            (e = dev_alloc(&v2, (size_t)nkeep * k, s)) || (e = dev_alloc(&m, (size_t)ncomp * k, s))) {
            free_work();
            return e;
        }
        cap = k;
        return cudaSuccess;
    }
    cudaError_t run(int k, const cd *in, cd *out, cudaStream_t s, bool deferred) {
        cudaError_t e;
        k_graph_node_rhs<<<grid_of(nkeep * k), 256, 0, s>>>(ac, k, branch, dinv, zs, in, rhs);
        if ((e = lap->solve(k, rhs, v, s, deferred))) return e;
        for (int it = 0; it < refine; ++it) {
            k_graph_residual<<<grid_of(nkeep * k), 256, 0, s>>>(nkeep, k, lap_ptr, lap_branch, lap_other, dinv, v,
                                                                rhs, corr);
            if ((e = lap->solve(k, corr, v2, s, deferred))) return e;
            k_graph_add<<<grid_of(nkeep * k), 256, 0, s>>>(nkeep * k, v2, v);
            note_launches(2);
        }
        k_graph_loops<<<grid_of(n * k), 256, 0, s>>>(n, k, is_tree, branch, loop_ends, dinv, zs, in, v, out);
        k_graph_tree_rhs<<<grid_of(n * k), 256, 0, s>>>(n, k, is_tree, branch, K, zdiag, 1.0 / zs, in, out, rt);
        k_spmm<<<grid_of(nkeep * k), 256, 0, s>>>(tinvt, k, rt, v2, nullptr, nullptr, 0);
        k_graph_common<<<dim3((unsigned)ncomp, (unsigned)((k + 31) / 32)), dim3(32, 16), 0, s>>>(
            k, member_ptr, members, pinv, rtotal, v2, m);
        k_graph_charge<<<grid_of(nkeep * k), 256, 0, s>>>(nkeep, k, comp, pinv, m, v2);
        k_graph_tree_out<<<grid_of(n * k), 256, 0, s>>>(n, k, is_tree, long_flag, tinv, ps, v2, out);
        if (nlong) k_graph_tree_out_long<<<(unsigned)nlong, 256, 0, s>>>(long_rows, k, tinv, ps, v2, out);
        note_launches(nlong ? 8 : 7);
        return cudaGetLastError();
    }
    cudaError_t apply(int k, const int32_t *, const cd *in, cd *out, cudaStream_t s) override {
        cudaError_t e = reserve(k, s);
        return e ? e : run(k, in, out, s, false);
    }
    cudaError_t apply_deferred(int k, const int32_t *, const cd *in, cd *out, cudaStream_t s) override {
        if (k > cap) return cudaErrorInvalidValue;      // one apply with this k comes first (no allocation here)
        deferred_k = k;
        return run(k, in, out, s, true);
    }
    cudaError_t deferred_status(cudaStream_t s) override {
        return deferred_k ? lap->status(deferred_k, s) : cudaSuccess;
    }
};

}  // namespace pq

using namespace pq;

struct pcbqs_gb300_peec {
    PeecOp op;
    BlockJacobi *bj = nullptr;
    LuPrecond *lu = nullptr;
    GraphPrecond *graph = nullptr;
    double *klk = nullptr, *tpt = nullptr;   // dense K^T L K and T^T P T (n x n), made once for the factors
    double *tpt_im = nullptr;                // T^T P_im T when P is complex
    float assemble_ms = 0, getrf_ms = 0;     // CUDA-event times of the last factorization's two stages
    bool captured = false;                   // GMRES restart cycles as CUDA graph launches
    LuUpdateStats updates;                   // its tcgen05 trailing updates (math 4, 5)
    ~pcbqs_gb300_peec() {
        delete bj;
        delete lu;
        delete graph;
        dev_free(klk);
        dev_free(tpt);
        dev_free(tpt_im);
    }
};

namespace {
#define pfail pq::fail

// A failed CUDA call's status: 6 when a bounded device wait gave up (cudaErrorLaunchTimeout from this library's
// own kernels), 2 otherwise.
static int cuda_status(cudaError_t e) { return e == cudaErrorLaunchTimeout ? ERR_TIMEOUT : ERR_CUDA; }
constexpr int LU_BLOCK = 2048;     // panel width of the blocked factorization (math 2 .. 5)
Csr csr_of(const pcbqs_gb300_csr &c) {
    Csr out;
    out.rows = c.rows;
    out.cols = c.cols;
    out.ptr = c.ptr;
    out.idx = c.idx;
    out.val = c.val;
    return out;
}
}  // namespace

extern "C" {

int pcbqs_gb300_peec_create(const pcbqs_gb300_peec_desc *d, pcbqs_gb300_peec **out) {
    if (!d || !out) return pfail(ERR_ARGUMENT, "peec_create: null argument");
    *out = nullptr;
    if (d->n <= 0 || d->nb <= 0 || d->ne < 0 || d->ne > d->nb || d->nn < 0 || d->nsys <= 0 || !d->omega ||
        !d->zscale || !d->is_tree || !(d->pscale > 0))
        return pfail(ERR_ARGUMENT, "peec_create: invalid sizes or arrays");
    if (d->K.rows != d->nb || d->K.cols != d->n || d->Kt.rows != d->n || d->Kt.cols != d->nb ||
        d->R.rows != d->ne || (d->nn > 0 && (d->T.rows != d->nn || d->T.cols != d->n || d->Tt.rows != d->n)))
        return pfail(ERR_ARGUMENT, "peec_create: sparse shapes do not match");
    auto *h = new (std::nothrow) pcbqs_gb300_peec();
    if (!h) return pfail(ERR_MEMORY, "peec_create: host allocation");
    PeecOp &op = h->op;
    op.n_ = d->n; op.nb = d->nb; op.ne = d->ne; op.nn = d->nn;
    op.K = csr_of(d->K); op.Kt = csr_of(d->Kt); op.T = csr_of(d->T); op.Tt = csr_of(d->Tt); op.R = csr_of(d->R);
    op.L = d->L; op.ldl = d->ldl; op.P = d->P; op.ldp = d->ldp; op.is_tree = d->is_tree; op.pscale = d->pscale;
    op.Pim = d->nn > 0 ? d->Pim : nullptr;
    op.nsys = d->nsys;
    op.nscaled = d->nscaled > 0 && d->nscaled < d->nb ? d->nscaled : d->nb;
    std::vector<double> w(d->nsys), z(d->nsys), wa(d->nsys), iz(d->nsys), ip(d->nsys, 1.0 / d->pscale);
    for (int s = 0; s < d->nsys; ++s) {
        w[s] = d->omega[s];
        z[s] = d->zscale[s];
        wa[s] = w[s] * z[s] / d->pscale;
        iz[s] = 1.0 / z[s];
    }
    cudaError_t e;
    op.rscale_host.assign(d->nsys, make_double2(1.0, 0.0));
    if (d->rscale)
        for (int s = 0; s < d->nsys; ++s) op.rscale_host[s] = make_double2(d->rscale[2 * s], d->rscale[2 * s + 1]);
    if ((e = dev_alloc(&op.omega, d->nsys)) || (e = dev_alloc(&op.zscale, d->nsys)) ||
        (e = dev_alloc(&op.walpha, d->nsys)) || (e = dev_alloc(&op.inv_z, d->nsys)) ||
        (e = dev_alloc(&op.inv_p, d->nsys)) || (e = dev_alloc(&op.rscale, d->nsys))) {
        delete h;
        return pfail(ERR_MEMORY, "peec_create: %s", cudaGetErrorString(e));
    }
    cudaMemcpy(op.omega, w.data(), sizeof(double) * d->nsys, cudaMemcpyHostToDevice);
    cudaMemcpy(op.zscale, z.data(), sizeof(double) * d->nsys, cudaMemcpyHostToDevice);
    cudaMemcpy(op.walpha, wa.data(), sizeof(double) * d->nsys, cudaMemcpyHostToDevice);
    cudaMemcpy(op.inv_z, iz.data(), sizeof(double) * d->nsys, cudaMemcpyHostToDevice);
    cudaMemcpy(op.inv_p, ip.data(), sizeof(double) * d->nsys, cudaMemcpyHostToDevice);
    cudaMemcpy(op.rscale, op.rscale_host.data(), sizeof(cd) * d->nsys, cudaMemcpyHostToDevice);
    *out = h;
    return OK;
}

void pcbqs_gb300_peec_destroy(pcbqs_gb300_peec *h) { delete h; }

// ERR_TIMEOUT (and the flag cleared) when a tensor-core product of this operator gave up a bounded wait since the
// last check; synchronizes `st`.
static int take_product_timeout(PeecOp &op, cudaStream_t st, const char *what) {
    if (!op.tc_error) return OK;
    int timed_out = 0;
    cudaError_t e = cudaMemcpyAsync(&timed_out, op.tc_error, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    if (!e && timed_out) e = cudaMemsetAsync(op.tc_error, 0, sizeof(int), st);
    if (e) return pfail(cuda_status(e), "%s: %s", what, cudaGetErrorString(e));
    if (timed_out) return pfail(ERR_TIMEOUT, "%s: a bounded wait of a tensor-core product gave up", what);
    return OK;
}

int pcbqs_gb300_peec_apply(pcbqs_gb300_peec *h, int k, const int32_t *sys_host, const double *in, double *out,
                           void *stream) {
    if (!h || k <= 0 || !sys_host || !in || !out) return pfail(ERR_ARGUMENT, "peec_apply: invalid argument");
    for (int s = 0; s < k; ++s)
        if (sys_host[s] < 0 || sys_host[s] >= h->op.nsys) return pfail(ERR_ARGUMENT, "peec_apply: system index");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int *sys = nullptr;
    if (dev_alloc(&sys, k, st)) return pfail(ERR_MEMORY, "peec_apply: allocation");
    cudaMemcpyAsync(sys, sys_host, sizeof(int) * k, cudaMemcpyHostToDevice, st);
    cudaError_t e = h->op.apply(k, sys, reinterpret_cast<const cd *>(in), reinterpret_cast<cd *>(out), st);
    if (!e) e = cudaStreamSynchronize(st);
    dev_free(sys, st);
    if (e) return pfail(cuda_status(e), "peec_apply: %s", cudaGetErrorString(e));
    return take_product_timeout(h->op, st, "peec_apply");
}

static int block_jacobi_impl(pcbqs_gb300_peec *h, int32_t bs, const double *krk, const double *klk_given,
                             const double *tpt_given, void *stream) {
    if (!h || bs <= 0 || bs > 64 || !krk) return pfail(ERR_ARGUMENT, "block_jacobi: invalid argument");
    PeecOp &op = h->op;
    if (!klk_given && (op.compressed || !op.L || (op.nn > 0 && !op.P)))
        return pfail(ERR_ARGUMENT, "block_jacobi: the blocks of a compressed operator are given by the caller");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t nblk = (op.n_ + bs - 1) / bs;
    const size_t bsz = (size_t)nblk * bs * bs;
    double *klk = nullptr, *tpt = nullptr, *tpt_im = nullptr;
    int *singular = nullptr;
    auto *bj = new (std::nothrow) BlockJacobi();
    if (!bj) return pfail(ERR_MEMORY, "block_jacobi: host allocation");
    bj->n = op.n_; bj->nblk = nblk; bj->bs = bs;
    cudaError_t e;
    if ((e = dev_alloc(&klk, bsz, st)) || (e = dev_alloc(&tpt, bsz, st)) || (e = dev_alloc(&singular, 1, st)) ||
        (e = dev_alloc(&bj->inv, (size_t)op.nsys * bsz, st)) || (op.Pim && (e = dev_alloc(&tpt_im, bsz, st)))) {
        dev_free(klk, st); dev_free(tpt, st); dev_free(tpt_im, st); dev_free(singular, st);
        delete bj;
        return pfail(ERR_MEMORY, "block_jacobi: %s", cudaGetErrorString(e));
    }
    cudaMemsetAsync(singular, 0, sizeof(int), st);
    cudaMemsetAsync(tpt, 0, sizeof(double) * bsz, st);
    if (klk_given) {
        cudaMemcpyAsync(klk, klk_given, sizeof(double) * bsz, cudaMemcpyDeviceToDevice, st);
        if (tpt_given) cudaMemcpyAsync(tpt, tpt_given, sizeof(double) * bsz, cudaMemcpyDeviceToDevice, st);
    } else {
        k_block_gather<<<(unsigned)nblk, 256, 0, st>>>(op.n_, bs, op.Kt, op.L, op.ldl, klk);
        if (op.nn > 0) k_block_gather<<<(unsigned)nblk, 256, 0, st>>>(op.n_, bs, op.Tt, op.P, op.ldp, tpt);
        if (op.Pim) {
            k_block_gather<<<(unsigned)nblk, 256, 0, st>>>(op.n_, bs, op.Tt, op.Pim, op.ldp, tpt_im);
            note_launches(1);
        }
    }
    dim3 grid((unsigned)nblk, (unsigned)op.nsys);
    const size_t smem = sizeof(cd) * bs * 2 * bs;
    cudaFuncSetAttribute(k_block_invert, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_block_invert<<<grid, 256, smem, st>>>(op.n_, bs, nblk, krk, klk, tpt, tpt_im, op.is_tree, op.omega,
                                             op.zscale, op.rscale, op.pscale, bj->inv, singular);
    note_launches(op.nn > 0 ? 3 : 2);
    int sing = 0;
    cudaMemcpyAsync(&sing, singular, sizeof(int), cudaMemcpyDeviceToHost, st);
    e = cudaStreamSynchronize(st);
    dev_free(klk, st); dev_free(tpt, st); dev_free(tpt_im, st); dev_free(singular, st);
    if (e) {
        delete bj;
        return pfail(cuda_status(e), "block_jacobi: %s", cudaGetErrorString(e));
    }
    if (sing) {
        delete bj;
        return pfail(ERR_NONFINITE, "block_jacobi: a diagonal block is singular");
    }
    delete h->bj;
    h->bj = bj;
    return OK;
}

int pcbqs_gb300_peec_block_jacobi(pcbqs_gb300_peec *h, int32_t bs, const double *krk, void *stream) {
    return block_jacobi_impl(h, bs, krk, nullptr, nullptr, stream);
}

int pcbqs_gb300_peec_block_jacobi_blocks(pcbqs_gb300_peec *h, int32_t bs, const double *krk, const double *klk,
                                         const double *tpt, void *stream) {
    if (!klk || (h && h->op.nn > 0 && !tpt)) return pfail(ERR_ARGUMENT, "block_jacobi_blocks: blocks missing");
    if (h && h->op.Pim) return pfail(ERR_ARGUMENT, "block_jacobi_blocks: complex P is not supported");
    return block_jacobi_impl(h, bs, krk, klk, tpt, stream);
}

static bool hmat_ok(const pcbqs_gb300_hmat *m) {
    return m && m->n > 0 && m->nblocks >= 0 && m->nslots >= 0 && m->meta && m->slot0 && m->idx && m->row_ptr &&
           m->slots_of_row && m->store && m->max_rank >= 0;
}

static PeecOp::HMat hmat_of(const pcbqs_gb300_hmat &m) {
    PeecOp::HMat h;
    h.n = m.n; h.nblocks = m.nblocks; h.nslots = m.nslots;
    h.meta = m.meta; h.slot0 = m.slot0; h.idx = m.idx; h.row_ptr = m.row_ptr; h.slots_of_row = m.slots_of_row;
    h.store = m.store;
    h.max_rank = m.max_rank;
    return h;
}

int pcbqs_gb300_peec_set_compressed(pcbqs_gb300_peec *h, const pcbqs_gb300_hmat *L, const double *via, int64_t nv,
                                    const pcbqs_gb300_hmat *P, const pcbqs_gb300_csr *W, const pcbqs_gb300_csr *Wt) {
    if (!h || !hmat_ok(L) || nv < 0 || (nv > 0 && !via) || L->n + nv != h->op.ne)
        return pfail(ERR_ARGUMENT, "peec_set_compressed: L's H-matrix rows plus the via rows must be the branch count");
    PeecOp &op = h->op;
    if (op.nn > 0 && (!hmat_ok(P) || !W || !Wt || W->rows != P->n || W->cols != op.nn || Wt->rows != op.nn ||
                      Wt->cols != P->n))
        return pfail(ERR_ARGUMENT, "peec_set_compressed: P's H-matrix (triangles) and W (triangles x nodes) needed");
    if (op.Pim) return pfail(ERR_ARGUMENT, "peec_set_compressed: complex P is not supported");
    op.hl = hmat_of(*L);
    if (op.nn > 0) {
        op.hp = hmat_of(*P);
        op.W = csr_of(*W);
        op.Wt = csr_of(*Wt);
    }
    op.via = via;
    op.nvia = nv;
    op.compressed = true;
    return OK;
}

static int lowrank_of(const pcbqs_gb300_lowrank *lr, int64_t n, int max_rank, PeecOp::HMat &H, const char *what) {
    const bool low = lr && lr->ngroups > 0, dense = lr && lr->dplane && lr->ndgroups > 0;
    if (!lr || (!low && !dense) || !lr->pad_pos || lr->n_pad < n || lr->n_pad % 64 || lr->ndense < 0 ||
        (lr->ndense > 0 && (!lr->meta_dense || !lr->slot0_dense)) || max_rank > 64 ||
        (low && (!lr->lplane || !lr->rplane || !lr->groups || lr->ntiles <= 0 || !lr->tile_group || !lr->tile_m ||
                 lr->rwidth % 64 || lr->lrows < 128)) ||
        (dense && (!lr->dgroups || lr->ndtiles <= 0 || !lr->dtile_group || !lr->dtile_m || lr->dpitch % 64 ||
                   lr->drows < 128)))
        return pfail(ERR_ARGUMENT, "%s: invalid low-rank plan (ranks up to 64)", what);
    if (dense) {
        H.plan.dplane = lr->dplane;
        H.plan.drows = lr->drows;
        H.plan.dpitch = lr->dpitch;
        H.plan.dgroups = static_cast<const LrGroup *>(lr->dgroups);
        H.plan.ndgroups = lr->ndgroups;
        H.plan.dtile_group = lr->dtile_group;
        H.plan.dtile_m = lr->dtile_m;
        H.plan.ndtiles = lr->ndtiles;
    }
    H.plan.lplane = lr->lplane;
    H.plan.lrows = lr->lrows;
    H.plan.rplane = lr->rplane;
    H.plan.rwidth = lr->rwidth;
    H.plan.groups = static_cast<const LrGroup *>(lr->groups);
    H.plan.ngroups = lr->ngroups;
    H.plan.tile_group = lr->tile_group;
    H.plan.tile_m = lr->tile_m;
    H.plan.ntiles = lr->ntiles;
    H.plan.pad_pos = lr->pad_pos;
    H.plan.n = n;
    H.plan.n_pad = lr->n_pad;
    H.meta_dense = lr->meta_dense;
    H.slot0_dense = lr->slot0_dense;
    H.ndense = lr->ndense;
    H.lr = true;
    return OK;
}

int pcbqs_gb300_peec_set_lowrank(pcbqs_gb300_peec *h, int which, const pcbqs_gb300_lowrank *lr) {
    if (!h || !h->op.compressed || (which != 0 && which != 1) || (which == 1 && h->op.nn <= 0))
        return pfail(ERR_ARGUMENT, "peec_set_lowrank: a compressed operator and which 0 (L) or 1 (P)");
    PeecOp::HMat &H = which == 0 ? h->op.hl : h->op.hp;
    return lowrank_of(lr, H.n, H.max_rank, H, "peec_set_lowrank");
}

int pcbqs_gb300_hmatrix_apply_lowrank(const pcbqs_gb300_hmat *Hd, const pcbqs_gb300_lowrank *lr, int k,
                                      const double *x, double *y, void *stream) {
    if (!hmat_ok(Hd) || k <= 0 || k > 128 || !x || !y)
        return pfail(ERR_ARGUMENT, "hmatrix_apply_lowrank: invalid argument (k 1..128)");
    PeecOp op;                  // a carrier for the product's buffers
    op.hl = hmat_of(*Hd);
    if (int status = lowrank_of(lr, Hd->n, Hd->max_rank, op.hl, "hmatrix_apply_lowrank")) return status;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = dev_alloc(&op.hslots, (size_t)std::max<int64_t>(1, Hd->nslots) * k, st);
    if (!e) {
        op.hcap = k;
        e = op.hm_apply(op.hl, true, k, reinterpret_cast<const cd *>(x), reinterpret_cast<cd *>(y), st);
    }
    if (e) return pfail(cuda_status(e), "hmatrix_apply_lowrank: %s", cudaGetErrorString(e));
    return take_product_timeout(op, st, "hmatrix_apply_lowrank");
}

int pcbqs_gb300_peec_potential_gmres(pcbqs_gb300_peec *h, int k, const double *b, double *x, const double *diag,
                                     double tol, int maxiter, int restart, int32_t *iterations, double *residual,
                                     void *stream) {
    if (!h || k <= 0 || !b || !x || !diag || !(tol > 0) || maxiter <= 0 || restart <= 0 || h->op.nn <= 0)
        return pfail(ERR_ARGUMENT, "peec_potential_gmres: invalid argument");
    if (!h->op.compressed && !h->op.P) return pfail(ERR_ARGUMENT, "peec_potential_gmres: no P");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    PotentialView view;
    view.op = &h->op;
    Jacobi J;
    J.n = h->op.nn;
    J.d = const_cast<double *>(diag);
    std::vector<int32_t> sys(k, 0);
    GmresOptions opt;
    opt.tol = tol; opt.maxiter = maxiter; opt.restart = restart;
    GmresReport rep;
    cudaError_t e = gmres_batched(view, &J, k, sys.data(), reinterpret_cast<const cd *>(b), reinterpret_cast<cd *>(x),
                                  opt, rep, st);
    if (e) return pfail(cuda_status(e), "peec_potential_gmres: %s", cudaGetErrorString(e));
    bool ok = true;
    for (int s = 0; s < k; ++s) {
        if (iterations) iterations[s] = rep.iterations[s];
        if (residual) residual[s] = rep.residual[s];
        ok = ok && rep.residual[s] <= tol;
    }
    if (!ok) return pfail(ERR_CONVERGENCE, "peec_potential_gmres: not every column reached the tolerance");
    return OK;
}

int pcbqs_gb300_peec_factor(pcbqs_gb300_peec *h, const pcbqs_gb300_csr *krk, int32_t sys, int math, void *stream) {
    if (!h || !krk || sys < 0 || sys >= h->op.nsys) return pfail(ERR_ARGUMENT, "peec_factor: invalid argument");
    if (math < 0 || math > 5)
        return pfail(ERR_ARGUMENT, "peec_factor: math 0/1 (cuSOLVER getrf, FP32/BF16x9) or 2..5 (blocked: BF16x9, "
                                   "FP32, tcgen05 with 3 or 6 BF16 part products)");
    PeecOp &op = h->op;
    const int64_t n = op.n_;
    if (krk->rows != n || krk->cols != n) return pfail(ERR_ARGUMENT, "peec_factor: K^T R K must be n x n");
    if (op.compressed || !op.L || (op.nn > 0 && !op.P))
        return pfail(ERR_ARGUMENT, "peec_factor: the complex64 factor needs the dense L and P");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    const size_t nn2 = (size_t)n * n;
    // stage times: ev[0] start, ev[1] system assembled, ev[2] factored
    struct Events {
        cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
        ~Events() {
            for (cudaEvent_t x : ev)
                if (x) cudaEventDestroy(x);
        }
    } t;
    for (cudaEvent_t &x : t.ev) cudaEventCreate(&x);
    cudaEventRecord(t.ev[0], st);
    auto stage_times = [&]() {
        float a = 0, b = 0;
        if (cudaEventSynchronize(t.ev[2]) == cudaSuccess && cudaEventElapsedTime(&a, t.ev[0], t.ev[1]) == cudaSuccess &&
            cudaEventElapsedTime(&b, t.ev[1], t.ev[2]) == cudaSuccess) {
            h->assemble_ms = a;
            h->getrf_ms = b;
        }
    };
    if (!h->klk) {
        // K^T L K = K^T (K^T L)^T (L symmetric) and T^T P T likewise: a row combination of L into W = K^T L (n rows),
        // its transpose, and a second row combination; every pass streams whole rows (no gathers).
        double *w = nullptr, *wt = nullptr;
        const int64_t wcols = std::max(op.ne, op.nn);
        if ((e = dev_alloc(&h->klk, nn2, st)) || (e = dev_alloc(&h->tpt, nn2, st)) ||
            (op.Pim && (e = dev_alloc(&h->tpt_im, nn2, st))) ||
            (e = dev_alloc(&w, (size_t)n * wcols, st)) || (e = dev_alloc(&wt, (size_t)n * wcols, st))) {
            dev_free(w, st);
            dev_free(wt, st);
            return pfail(ERR_MEMORY, "peec_factor: dense system blocks: %s", cudaGetErrorString(e));
        }
        const unsigned chunks = 8;
        const dim3 g1 = row_grid(chunks, n);
        auto aligned = [](const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
        auto combine = [&](const Csr &St, const double *M, int64_t ldm, int64_t cols, double *out, int64_t ldo) {
            if (cols % 2 == 0 && ldm % 2 == 0 && ldo % 2 == 0 && aligned(M) && aligned(out))
                k_rows_combine2<<<g1, 256, 0, st>>>(St, M, ldm, cols, out, ldo);
            else
                k_rows_combine<<<g1, 256, 0, st>>>(St, M, ldm, cols, out, ldo);
        };
        auto triple = [&](const Csr &St, const double *M, int64_t ldm, int64_t m, double *out) {
            combine(St, M, ldm, m, w, m);
            dim3 gt((unsigned)((m + 31) / 32), (unsigned)((n + 31) / 32));
            k_transpose<<<gt, dim3(32, 8), 0, st>>>(w, n, m, m, wt, n);
            combine(St, wt, n, n, out, n);
        };
        triple(op.Kt, op.L, op.ldl, op.ne, h->klk);
        if (op.nn > 0) {
            triple(op.Tt, op.P, op.ldp, op.nn, h->tpt);
            if (op.Pim) {
                triple(op.Tt, op.Pim, op.ldp, op.nn, h->tpt_im);
                note_launches(3);
            }
        } else {
            cudaMemsetAsync(h->tpt, 0, sizeof(double) * nn2, st);
        }
        note_launches(op.nn > 0 ? 6 : 3);
        e = cudaStreamSynchronize(st);
        dev_free(w, st);
        dev_free(wt, st);
        if (e) return pfail(cuda_status(e), "peec_factor: %s", cudaGetErrorString(e));
    }
    auto *lu = new (std::nothrow) LuPrecond();
    if (!lu) return pfail(ERR_MEMORY, "peec_factor: host allocation");
    lu->n = n;
    if ((e = dev_alloc(&lu->lu, nn2, st)) || (e = dev_alloc(&lu->ipiv, n, st)) || (e = dev_alloc(&lu->info, 1, st))) {
        delete lu;
        return pfail(ERR_MEMORY, "peec_factor: factor of %lld unknowns: %s", (long long)n, cudaGetErrorString(e));
    }
    double w = 0, zs = 0;
    cudaMemcpy(&w, op.omega + sys, sizeof(double), cudaMemcpyDeviceToHost);
    cudaMemcpy(&zs, op.zscale + sys, sizeof(double), cudaMemcpyDeviceToHost);
    Csr S = csr_of(*krk);
    k_assemble_c64<<<row_grid((unsigned)std::min<int64_t>((n + 255) / 256, 8), n), 256, 0, st>>>(
        n, h->klk, h->tpt, h->tpt_im, op.is_tree, w, zs, op.pscale, lu->lu);
    k_add_krk_c64<<<grid_of(n), 256, 0, st>>>(S, op.is_tree, w, zs, op.pscale, op.rscale_host[sys], lu->lu);
    note_launches(2);
    cudaEventRecord(t.ev[1], st);
    if (cusolverDnCreate(&lu->solver) != CUSOLVER_STATUS_SUCCESS) {
        delete lu;
        return pfail(ERR_CUDA, "peec_factor: cuSOLVER handle");
    }
    cusolverDnSetStream(lu->solver, st);
    if (math >= 2) {
        int singular = 0;
        const int gemm = math == 2 ? LU_GEMM_BF16X9 : math == 3 ? LU_GEMM_FP32 : math == 4 ? LU_GEMM_TC3 : LU_GEMM_TC6;
        e = getrf_blocked(n, lu->lu, lu->ipiv, lu_panel_width(n, gemm), gemm, st, &singular, &h->updates);
        cudaEventRecord(t.ev[2], st);
        if (e || singular) {
            delete lu;
            return pfail(singular ? ERR_NONFINITE : e == cudaErrorLaunchTimeout ? ERR_TIMEOUT : ERR_CUDA,
                         "peec_factor: blocked getrf failed (zero pivot %d, %s)", singular, cudaGetErrorString(e));
        }
        if ((e = lu->tri.prepare(lu->lu, n, lu->ipiv, st))) {
            delete lu;
            return pfail(cuda_status(e), "peec_factor: triangular-solve set-up: %s", cudaGetErrorString(e));
        }
        delete h->lu;
        h->lu = lu;
        stage_times();
        return OK;
    }
    if (math == 1 && cusolverDnSetMathMode(lu->solver, CUSOLVER_FP32_EMULATED_BF16X9_MATH) != CUSOLVER_STATUS_SUCCESS) {
        delete lu;
        return pfail(ERR_CUDA, "peec_factor: BF16x9 emulation unavailable in this cuSOLVER");
    }
    int lwork = 0;
    if (cusolverDnCgetrf_bufferSize(lu->solver, (int)n, (int)n, reinterpret_cast<cuComplex *>(lu->lu), (int)n,
                                    &lwork) != CUSOLVER_STATUS_SUCCESS) {
        delete lu;
        return pfail(ERR_CUDA, "peec_factor: workspace query");
    }
    float2 *ws = nullptr;
    if ((e = dev_alloc(&ws, (size_t)lwork, st))) {
        delete lu;
        return pfail(ERR_MEMORY, "peec_factor: workspace");
    }
    const cusolverStatus_t cs = cusolverDnCgetrf(lu->solver, (int)n, (int)n, reinterpret_cast<cuComplex *>(lu->lu),
                                                 (int)n, reinterpret_cast<cuComplex *>(ws), lu->ipiv, lu->info);
    cudaEventRecord(t.ev[2], st);
    int info = 0;
    cudaMemcpyAsync(&info, lu->info, sizeof(int), cudaMemcpyDeviceToHost, st);
    e = cudaStreamSynchronize(st);
    dev_free(ws, st);
    if (cs != CUSOLVER_STATUS_SUCCESS || e || info != 0) {
        delete lu;
        return pfail(info ? ERR_NONFINITE : ERR_CUDA, "peec_factor: getrf failed (status %d, info %d, %s)", (int)cs,
                     info, cudaGetErrorString(e));
    }
    if ((e = lu->tri.prepare(lu->lu, n, lu->ipiv, st))) {
        delete lu;
        return pfail(cuda_status(e), "peec_factor: triangular-solve set-up: %s", cudaGetErrorString(e));
    }
    delete h->lu;
    h->lu = lu;
    stage_times();
    return OK;
}

// The dense Laplacian: assembled from the branches, factored by getrf_blocked (tcgen05 updates).
static int graph_dense_lap(const pcbqs_gb300_graph *g, const cd *dinv, cudaStream_t st, LapSolver **out) {
    const int64_t nk = g->nkeep;
    const size_t nk2 = (size_t)nk * nk;
    auto *lap = new (std::nothrow) DenseLap();
    if (!lap) return pfail(ERR_MEMORY, "peec_graph: host allocation");
    cudaError_t e;
    if ((e = dev_alloc(&lap->ipiv, nk, st)) || (e = dev_alloc(&lap->G, nk2, st))) {
        delete lap;
        return pfail(ERR_MEMORY, "peec_graph: the dense Laplacian of %lld nodes (%.1f GB): %s", (long long)nk,
                     8e-9 * (double)nk2, cudaGetErrorString(e));
    }
    cudaMemsetAsync(lap->G, 0, sizeof(float2) * nk2, st);
    k_graph_laplacian<<<grid_of(nk), 256, 0, st>>>(nk, g->lap_ptr, g->lap_branch, g->lap_other, dinv, lap->G);
    note_launches(1);
    int singular = 0;
    LuUpdateStats stats;
    e = getrf_blocked(nk, lap->G, lap->ipiv, lu_panel_width(nk, LU_GEMM_TC6), LU_GEMM_TC6, st, &singular, &stats);
    if (e || singular) {
        delete lap;
        return pfail(singular ? ERR_NONFINITE : cuda_status(e), "peec_graph: Laplacian LU failed (zero pivot %d, %s)",
                     singular, cudaGetErrorString(e));
    }
    if ((e = lap->tri.prepare(lap->G, nk, lap->ipiv, st))) {
        delete lap;
        return pfail(cuda_status(e), "peec_graph: triangular-solve set-up: %s", cudaGetErrorString(e));
    }
    *out = lap;
    return OK;
}

// The domain-split Laplacian: each domain's block inverted explicitly, the separator's Schur complement factored.
static int graph_domain_lap(const pcbqs_gb300_graph *g, const cd *dinv, cudaStream_t st, LapSolver **out) {
    const pcbqs_gb300_graph_domains *dm = g->domains;
    const int64_t nk = g->nkeep, parts = dm->parts, n_int = dm->n_int, ns = nk - n_int;
    if (parts < 1 || n_int < 0 || ns < 1 || !dm->dom_ptr || !dm->bnd_ptr || !dm->perm || !dm->pos || !dm->bnd ||
        !dm->bnd_nptr || !dm->bnd_local || !dm->bnd_branch || dm->dom_ptr[0] != 0 || dm->dom_ptr[parts] != n_int ||
        dm->bnd_ptr[0] != 0)
        return pfail(ERR_ARGUMENT, "peec_graph: domain split (%lld parts, %lld interior of %lld kept rows)",
                     (long long)parts, (long long)n_int, (long long)nk);
    auto *lap = new (std::nothrow) DomainLap();
    if (!lap) return pfail(ERR_MEMORY, "peec_graph: host allocation");
    lap->nk = nk;
    lap->n_int = n_int;
    lap->ns = ns;
    lap->parts = parts;
    lap->dom_ptr.assign(dm->dom_ptr, dm->dom_ptr + parts + 1);
    lap->bnd_ptr.assign(dm->bnd_ptr, dm->bnd_ptr + parts + 1);
    lap->perm = dm->perm;
    lap->pos = dm->pos;
    lap->lap_ptr = g->lap_ptr;
    lap->lap_branch = g->lap_branch;
    lap->lap_other = g->lap_other;
    lap->dinv = dinv;
    int64_t total = 0, nmax = 0;
    for (int64_t d = 0; d < parts; ++d) {
        const int64_t nd = lap->dom_ptr[d + 1] - lap->dom_ptr[d];
        if (nd < 0 || lap->bnd_ptr[d + 1] < lap->bnd_ptr[d]) {
            delete lap;
            return pfail(ERR_ARGUMENT, "peec_graph: domain %lld's offsets", (long long)d);
        }
        lap->blk_off.push_back(total);
        total += nd * nd;
        nmax = std::max(nmax, nd);
    }
    if (nmax > 65536) {
        delete lap;
        return pfail(ERR_ARGUMENT, "peec_graph: a domain of %lld rows (at most 65,536)", (long long)nmax);
    }
    cusolverDnHandle_t solver = nullptr;
    float2 *scratch = nullptr, *ws = nullptr;
    int *dpiv = nullptr, *info = nullptr;
    auto cleanup = [&]() {
        dev_free(scratch, st);
        dev_free(ws, st);
        dev_free(dpiv, st);
        dev_free(info, st);
        if (solver) cusolverDnDestroy(solver);
    };
    cudaError_t e;
    int lwork = 0;
    if (cublasCreate(&lap->blas) != CUBLAS_STATUS_SUCCESS || cusolverDnCreate(&solver) != CUSOLVER_STATUS_SUCCESS) {
        cleanup();
        delete lap;
        return pfail(ERR_CUDA, "peec_graph: cuBLAS / cuSOLVER handle");
    }
    cusolverDnSetStream(solver, st);
    if ((e = dev_alloc(&lap->Ainv, (size_t)std::max<int64_t>(total, 1), st)) ||
        (e = dev_alloc(&lap->S, (size_t)ns * ns, st)) || (e = dev_alloc(&lap->ipiv, ns, st)) ||
        (e = dev_alloc(&scratch, (size_t)std::max<int64_t>(nmax * nmax, 1), st)) ||
        (e = dev_alloc(&dpiv, std::max<int64_t>(nmax, 1), st)) || (e = dev_alloc(&info, 2 * parts, st))) {
        cleanup();
        delete lap;
        return pfail(ERR_MEMORY, "peec_graph: domain inverses (%.2f GB) and Schur complement (%.2f GB): %s",
                     8e-9 * (double)total, 8e-9 * (double)ns * (double)ns, cudaGetErrorString(e));
    }
    if (nmax > 0 && cusolverDnCgetrf_bufferSize(solver, (int)nmax, (int)nmax, reinterpret_cast<cuComplex *>(scratch),
                                                (int)nmax, &lwork) != CUSOLVER_STATUS_SUCCESS) {
        cleanup();
        delete lap;
        return pfail(ERR_CUDA, "peec_graph: workspace query");
    }
    if ((e = dev_alloc(&ws, (size_t)std::max(lwork, 1), st))) {
        cleanup();
        delete lap;
        return pfail(ERR_MEMORY, "peec_graph: workspace");
    }
    cudaMemsetAsync(info, 0, sizeof(int) * 2 * parts, st);      // getrf's status per domain, then getrs's
    for (int64_t d = 0; d < parts; ++d) {
        const int64_t off = lap->dom_ptr[d], nd = lap->dom_ptr[d + 1] - off;
        if (!nd) continue;
        float2 *inv = lap->Ainv + lap->blk_off[d];
        cudaMemsetAsync(scratch, 0, sizeof(float2) * nd * nd, st);
        k_domain_block<<<grid_of(nd), 256, 0, st>>>(off, nd, lap->perm, lap->pos, g->lap_ptr, g->lap_branch,
                                                     g->lap_other, dinv, scratch);
        k_identity_c64<<<grid_of(nd * nd), 256, 0, st>>>(nd, inv);
        note_launches(2);
        if (cusolverDnCgetrf(solver, (int)nd, (int)nd, reinterpret_cast<cuComplex *>(scratch), (int)nd,
                             reinterpret_cast<cuComplex *>(ws), dpiv, info + d) != CUSOLVER_STATUS_SUCCESS ||
            cusolverDnCgetrs(solver, CUBLAS_OP_N, (int)nd, (int)nd, reinterpret_cast<const cuComplex *>(scratch),
                             (int)nd, dpiv, reinterpret_cast<cuComplex *>(inv), (int)nd,
                             info + parts + d) != CUSOLVER_STATUS_SUCCESS) {
            cleanup();
            delete lap;
            return pfail(ERR_CUDA, "peec_graph: domain %lld's LU", (long long)d);
        }
    }
    std::vector<int> infos((size_t)(2 * parts));
    cudaMemcpyAsync(infos.data(), info, sizeof(int) * 2 * parts, cudaMemcpyDeviceToHost, st);
    if ((e = cudaStreamSynchronize(st))) {
        cleanup();
        delete lap;
        return pfail(cuda_status(e), "peec_graph: domain inverses: %s", cudaGetErrorString(e));
    }
    for (int64_t d = 0; d < 2 * parts; ++d)
        if (infos[d]) {
            cleanup();
            delete lap;
            return pfail(ERR_NONFINITE, "peec_graph: domain %lld's block: %s info %d", (long long)(d % parts),
                         d < parts ? "getrf" : "getrs", infos[d]);
        }
    // the Schur complement: G_SS, then each domain's term in turn (a fixed order)
    cudaMemsetAsync(lap->S, 0, sizeof(float2) * ns * ns, st);
    k_separator_block<<<grid_of(ns), 256, 0, st>>>(ns, n_int, lap->perm, lap->pos, g->lap_ptr, g->lap_branch,
                                                    g->lap_other, dinv, lap->S);
    note_launches(1);
    for (int64_t d = 0; d < parts; ++d) {
        const int64_t b0 = lap->bnd_ptr[d], mcount = lap->bnd_ptr[d + 1] - b0;
        const int64_t nd = lap->dom_ptr[d + 1] - lap->dom_ptr[d];
        if (!mcount || !nd) continue;
        k_schur_domain<<<grid_of(mcount * mcount), 256, 0, st>>>(mcount, dm->bnd + b0, dm->bnd_nptr + b0,
                                                                  dm->bnd_local, dm->bnd_branch, dinv,
                                                                  lap->Ainv + lap->blk_off[d], nd, lap->S, ns);
        note_launches(1);
    }
    int singular = 0;
    LuUpdateStats stats;
    e = getrf_blocked(ns, lap->S, lap->ipiv, lu_panel_width(ns, LU_GEMM_TC6), LU_GEMM_TC6, st, &singular, &stats);
    cleanup();
    if (e || singular) {
        delete lap;
        return pfail(singular ? ERR_NONFINITE : cuda_status(e), "peec_graph: Schur LU failed (zero pivot %d, %s)",
                     singular, cudaGetErrorString(e));
    }
    if ((e = lap->tri.prepare(lap->S, ns, lap->ipiv, st))) {
        delete lap;
        return pfail(cuda_status(e), "peec_graph: triangular-solve set-up: %s", cudaGetErrorString(e));
    }
    *out = lap;
    return OK;
}

int pcbqs_gb300_peec_graph(pcbqs_gb300_peec *h, const pcbqs_gb300_graph *g, int32_t sys, int refine, void *stream) {
    if (!h || !g || sys < 0 || sys >= h->op.nsys || refine < 0 || refine > 3)
        return pfail(ERR_ARGUMENT, "peec_graph: invalid argument");
    PeecOp &op = h->op;
    const int64_t n = op.n_, nk = g->nkeep;
    if (nk < 1 || g->ncomp < 1 || g->ncomp > nk + 1 || g->ncomp > 65535 || g->nbranch != op.nb)
        return pfail(ERR_ARGUMENT, "peec_graph: %lld kept nodes, %lld components, %lld branches (the operator has %lld)",
                     (long long)nk, (long long)g->ncomp, (long long)g->nbranch, (long long)op.nb);
    if (g->ac.rows != nk || g->ac.cols != n || g->tinv.rows != n || g->tinv.cols != nk || g->tinvt.rows != nk ||
        g->tinvt.cols != n)
        return pfail(ERR_ARGUMENT, "peec_graph: ac (kept x n), tinv (n x kept), tinvt (kept x n) shapes");
    if (!g->ac.ptr || !g->tinv.ptr || !g->tinvt.ptr || !g->lap_ptr || !g->lap_branch || !g->lap_other ||
        !g->branch || !g->loop_ends || !g->comp || !g->member_ptr || !g->members || !g->zdiag || !g->dinv ||
        !g->pinv || !g->total)
        return pfail(ERR_ARGUMENT, "peec_graph: null array");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto *gp = new (std::nothrow) GraphPrecond();
    if (!gp) return pfail(ERR_MEMORY, "peec_graph: host allocation");
    gp->n = n;
    gp->nkeep = nk;
    gp->ncomp = g->ncomp;
    gp->nbranch = g->nbranch;
    gp->ac = csr_of(g->ac);
    gp->tinv = csr_of(g->tinv);
    gp->tinvt = csr_of(g->tinvt);
    gp->K = op.K;
    gp->lap_ptr = g->lap_ptr;
    gp->lap_branch = g->lap_branch;
    gp->lap_other = g->lap_other;
    gp->branch = g->branch;
    gp->loop_ends = g->loop_ends;
    gp->comp = g->comp;
    gp->member_ptr = g->member_ptr;
    gp->members = g->members;
    gp->is_tree = op.is_tree;
    gp->refine = refine;
    gp->ps = op.pscale;
    cudaMemcpy(&gp->zs, op.zscale + sys, sizeof(double), cudaMemcpyDeviceToHost);
    cudaError_t e;
    if ((e = dev_alloc(&gp->zdiag, g->nbranch, st)) || (e = dev_alloc(&gp->dinv, g->nbranch, st)) ||
        (e = dev_alloc(&gp->pinv, nk, st)) || (e = dev_alloc(&gp->rtotal, g->ncomp, st))) {
        delete gp;
        return pfail(ERR_MEMORY, "peec_graph: %s", cudaGetErrorString(e));
    }
    cudaMemcpyAsync(gp->zdiag, g->zdiag, sizeof(cd) * g->nbranch, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(gp->dinv, g->dinv, sizeof(cd) * g->nbranch, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(gp->pinv, g->pinv, sizeof(cd) * nk, cudaMemcpyDeviceToDevice, st);
    // 1 / total per component, on the host (a handful of values)
    std::vector<cd> tot((size_t)g->ncomp);
    cudaMemcpyAsync(tot.data(), g->total, sizeof(cd) * g->ncomp, cudaMemcpyDeviceToHost, st);
    if ((e = cudaStreamSynchronize(st))) {
        delete gp;
        return pfail(cuda_status(e), "peec_graph: %s", cudaGetErrorString(e));
    }
    for (cd &t : tot) {
        const double a = t.x * t.x + t.y * t.y;
        if (!(a > 0) || !std::isfinite(a)) {
            delete gp;
            return pfail(ERR_NONFINITE, "peec_graph: a component's total 1 / P_ii is zero or not finite");
        }
        t = make_double2(t.x / a, -t.y / a);
    }
    cudaMemcpyAsync(gp->rtotal, tot.data(), sizeof(cd) * g->ncomp, cudaMemcpyHostToDevice, st);
    // the long rows of T[keep]^-1, found on the host from its row pointers
    {
        std::vector<int64_t> tptr((size_t)n + 1);
        std::vector<int8_t> tree((size_t)n), flag((size_t)n, 0);
        std::vector<int32_t> rows;
        cudaMemcpyAsync(tptr.data(), g->tinv.ptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(tree.data(), op.is_tree, (size_t)n, cudaMemcpyDeviceToHost, st);
        if ((e = cudaStreamSynchronize(st))) {
            delete gp;
            return pfail(cuda_status(e), "peec_graph: %s", cudaGetErrorString(e));
        }
        for (int64_t j = 0; j < n; ++j)
            if (tree[j] && tptr[j + 1] - tptr[j] > GRAPH_LONG_ROW) {
                rows.push_back((int32_t)j);
                flag[j] = 1;
            }
        gp->nlong = (int64_t)rows.size();
        if ((e = dev_alloc(&gp->long_flag, n, st)) || (e = dev_alloc(&gp->long_rows, std::max<size_t>(rows.size(), 1), st))) {
            delete gp;
            return pfail(ERR_MEMORY, "peec_graph: %s", cudaGetErrorString(e));
        }
        cudaMemcpyAsync(gp->long_flag, flag.data(), (size_t)n, cudaMemcpyHostToDevice, st);
        if (!rows.empty())
            cudaMemcpyAsync(gp->long_rows, rows.data(), sizeof(int32_t) * rows.size(), cudaMemcpyHostToDevice, st);
        if ((e = cudaStreamSynchronize(st))) {          // the host vectors go out of scope here
            delete gp;
            return pfail(cuda_status(e), "peec_graph: %s", cudaGetErrorString(e));
        }
    }
    const int status = g->domains ? graph_domain_lap(g, gp->dinv, st, &gp->lap) : graph_dense_lap(g, gp->dinv, st,
                                                                                                  &gp->lap);
    if (status != OK) {
        delete gp;
        return status;
    }
    delete h->graph;
    h->graph = gp;
    return OK;
}

int pcbqs_gb300_peec_factor_times(const pcbqs_gb300_peec *h, double *assemble_ms, double *getrf_ms) {
    if (!h || !assemble_ms || !getrf_ms) return pfail(ERR_ARGUMENT, "peec_factor_times: invalid argument");
    if (!h->lu) return pfail(ERR_ARGUMENT, "peec_factor_times: no factor set up");
    *assemble_ms = h->assemble_ms;
    *getrf_ms = h->getrf_ms;
    return OK;
}

int pcbqs_gb300_peec_set_captured(pcbqs_gb300_peec *h, int captured) {
    if (!h || (captured != 0 && captured != 1)) return pfail(ERR_ARGUMENT, "peec_set_captured: invalid argument");
    h->captured = captured != 0;
    return OK;
}

int pcbqs_gb300_peec_set_fp64_product(pcbqs_gb300_peec *h, int slices) {
    if (!h || slices < 0 || slices == 1 || slices > 7)
        return pfail(ERR_ARGUMENT, "peec_set_fp64_product: slices 0 or 2..7");
    if (slices != h->op.exact_slices)
        for (bool &p : h->op.xpacked) p = false;
    h->op.exact_slices = slices;
    return OK;
}

int pcbqs_gb300_peec_set_product(pcbqs_gb300_peec *h, int terms) {
    if (!h || (terms != 0 && terms != 3 && terms != 6)) return pfail(ERR_ARGUMENT, "peec_set_product: terms 0, 3 or 6");
    if (terms != h->op.tc_terms) h->op.unpack();
    h->op.tc_terms = terms;
    return OK;
}

int pcbqs_gb300_peec_factor_updates(const pcbqs_gb300_peec *h, double *update_ms, double *update_flops,
                                    int32_t *launches) {
    if (!h || !update_ms || !update_flops || !launches)
        return pfail(ERR_ARGUMENT, "peec_factor_updates: invalid argument");
    *update_ms = h->updates.ms;
    *update_flops = h->updates.flops;
    *launches = h->updates.launches;
    return OK;
}

int pcbqs_gb300_peec_lu_solve(pcbqs_gb300_peec *h, int k, const double *in, double *out, int method,
                              void *stream) {
    if (!h || k <= 0 || !in || !out || method < 0 || method > 3)
        return pfail(ERR_ARGUMENT, "peec_lu_solve: invalid argument");
    if (!h->lu) return pfail(ERR_ARGUMENT, "peec_lu_solve: no factor set up");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const cd *x = reinterpret_cast<const cd *>(in);
    cd *y = reinterpret_cast<cd *>(out);
    cudaError_t e;
    if (method == 1) {
        e = h->lu->apply_library(k, x, y, st);
    } else {
        h->lu->tri.force = method == 2 ? 0 : method == 3 ? 1 : -1;
        e = h->lu->apply(k, nullptr, x, y, st);
        h->lu->tri.force = -1;
    }
    if (!e) e = cudaStreamSynchronize(st);
    if (e) return pfail(cuda_status(e), "peec_lu_solve: %s", cudaGetErrorString(e));
    return OK;
}

int pcbqs_gb300_peec_graph_apply(pcbqs_gb300_peec *h, int k, const double *in, double *out, void *stream) {
    if (!h || k <= 0 || !in || !out) return pfail(ERR_ARGUMENT, "peec_graph_apply: invalid argument");
    if (!h->graph) return pfail(ERR_ARGUMENT, "peec_graph_apply: no graph preconditioner set up");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = h->graph->apply(k, nullptr, reinterpret_cast<const cd *>(in), reinterpret_cast<cd *>(out), st);
    if (!e) e = cudaStreamSynchronize(st);
    if (e) return pfail(cuda_status(e), "peec_graph_apply: %s", cudaGetErrorString(e));
    return OK;
}

int pcbqs_gb300_peec_gmres(pcbqs_gb300_peec *h, int k, const int32_t *sys_host, const double *b, double *x,
                           double tol, int maxiter, int restart, int precondition, int32_t *iterations,
                           double *residual, void *stream) {
    if (!h || k <= 0 || !sys_host || !b || !x || !(tol > 0) || maxiter <= 0 || restart <= 0)
        return pfail(ERR_ARGUMENT, "peec_gmres: invalid argument");
    for (int s = 0; s < k; ++s)
        if (sys_host[s] < 0 || sys_host[s] >= h->op.nsys) return pfail(ERR_ARGUMENT, "peec_gmres: system index");
    if (precondition == 1 && !h->bj) return pfail(ERR_ARGUMENT, "peec_gmres: no block-Jacobi preconditioner set up");
    if (precondition == 2 && !h->lu) return pfail(ERR_ARGUMENT, "peec_gmres: no factor set up");
    if (precondition == 3 && !h->graph) return pfail(ERR_ARGUMENT, "peec_gmres: no graph preconditioner set up");
    if (precondition < 0 || precondition > 3) return pfail(ERR_ARGUMENT, "peec_gmres: preconditioner 0 .. 3");
    GmresOptions opt;
    opt.tol = tol; opt.maxiter = maxiter; opt.restart = restart;
    opt.captured = h->captured;
    GmresReport rep;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Preconditioner *M = precondition == 1   ? static_cast<Preconditioner *>(h->bj)
                        : precondition == 2 ? static_cast<Preconditioner *>(h->lu)
                        : precondition == 3 ? static_cast<Preconditioner *>(h->graph)
                                            : nullptr;
    cudaError_t e = gmres_batched(h->op, M, k, sys_host,
                                  reinterpret_cast<const cd *>(b), reinterpret_cast<cd *>(x), opt, rep, st);
    if (e) return pfail(cuda_status(e), "peec_gmres: %s", cudaGetErrorString(e));
    if (int status = take_product_timeout(h->op, static_cast<cudaStream_t>(stream), "peec_gmres")) return status;
    bool ok = true;
    for (int s = 0; s < k; ++s) {
        if (iterations) iterations[s] = rep.iterations[s];
        if (residual) residual[s] = rep.residual[s];
        ok = ok && rep.residual[s] <= tol;
    }
    if (!ok) return pfail(ERR_CONVERGENCE, "peec_gmres: not every system reached the tolerance");
    return OK;
}

int pcbqs_gb300_dense_apply(int64_t rows, int k, const double *M, int64_t ld, const double *X, double *Y,
                            void *stream) {
    if (rows <= 0 || k <= 0 || !M || ld < rows || !X || !Y) return pfail(ERR_ARGUMENT, "dense_apply: invalid argument");
    cudaError_t e = dense_sym_apply<double, 2>(rows, k, M, ld, reinterpret_cast<const cd *>(X), reinterpret_cast<cd *>(Y),
                                               static_cast<cudaStream_t>(stream));
    if (e) return pfail(cuda_status(e), "dense_apply: %s", cudaGetErrorString(e));
    return OK;
}

int pcbqs_gb300_dense_apply_single(int64_t rows, int k, const float *Mf, int64_t ld, const double *X, double *Y,
                                   void *stream) {
    if (rows <= 0 || k <= 0 || !Mf || ld < rows || !X || !Y)
        return pfail(ERR_ARGUMENT, "dense_apply_single: invalid argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float *xf = nullptr;
    cudaError_t e = dev_alloc(&xf, (size_t)rows * DENSE_NC, st);
    if (e) return pfail(ERR_MEMORY, "dense_apply_single: %s", cudaGetErrorString(e));
    e = dense_sym_apply<float, 4>(rows, k, Mf, ld, reinterpret_cast<const cd *>(X), reinterpret_cast<cd *>(Y), st, xf);
    dev_free(xf, st);
    if (e) return pfail(cuda_status(e), "dense_apply_single: %s", cudaGetErrorString(e));
    return OK;
}

int pcbqs_gb300_dense_apply_tensor(int64_t rows, int k, const float *Mf, int64_t ld, const double *X, double *Y,
                                   int terms, uint64_t wait_cycles, void *stream) {
    if (rows <= 0 || k <= 0 || !Mf || ld < rows || !X || !Y || (terms != 3 && terms != 6) || wait_cycles == 0)
        return pfail(ERR_ARGUMENT, "dense_apply_tensor: invalid argument (terms 3 or 6, ld >= rows, wait_cycles > 0)");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint8_t *plane = nullptr, *scratch = nullptr;
    int *flag = nullptr;
    cudaError_t e;
    if ((e = dev_alloc(&plane, tc_real_plane_bytes(rows, rows, terms), st)) ||
        (e = dev_alloc(&scratch, tc_real_scratch_bytes(rows, k, terms), st)) || (e = dev_alloc(&flag, 1, st))) {
        dev_free(plane, st);
        dev_free(scratch, st);
        return pfail(ERR_MEMORY, "dense_apply_tensor: %s", cudaGetErrorString(e));
    }
    int timed_out = 0;
    if (!(e = cudaMemsetAsync(flag, 0, sizeof(int), st)) && !(e = tc_pack_real(rows, rows, Mf, ld, terms, plane, st)))
        e = tc_real_product(rows, rows, plane, k, reinterpret_cast<const double2 *>(X), k,
                            reinterpret_cast<double2 *>(Y), k, terms, scratch, flag, (unsigned long long)wait_cycles,
                            st);
    if (!e) e = cudaMemcpyAsync(&timed_out, flag, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    dev_free(plane, st);
    dev_free(scratch, st);
    dev_free(flag, st);
    if (e) return pfail(cuda_status(e), "dense_apply_tensor: %s", cudaGetErrorString(e));
    if (timed_out) return pfail(ERR_TIMEOUT, "dense_apply_tensor: a bounded wait of the tensor-core product gave up");
    return OK;
}

int pcbqs_gb300_dense_apply_sliced(int64_t rows, int k, const double *M, int64_t ld, const double *X, double *Y,
                                   int slices, uint64_t wait_cycles, void *stream) {
    if (rows <= 0 || k <= 0 || !M || ld < rows || !X || !Y || slices < 2 || slices > 7 || wait_cycles == 0)
        return pfail(ERR_ARGUMENT, "dense_apply_sliced: invalid argument (slices 2..7, ld >= rows, wait_cycles > 0)");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint8_t *plane = nullptr, *scratch = nullptr;
    int *flag = nullptr;
    cudaError_t e;
    if ((e = dev_alloc(&plane, tc_exact_plane_bytes(rows, rows, slices), st)) ||
        (e = dev_alloc(&scratch, tc_exact_scratch_bytes(rows, k, slices), st)) || (e = dev_alloc(&flag, 1, st))) {
        dev_free(plane, st);
        dev_free(scratch, st);
        return pfail(ERR_MEMORY, "dense_apply_sliced: %s", cudaGetErrorString(e));
    }
    int timed_out = 0;
    if (!(e = cudaMemsetAsync(flag, 0, sizeof(int), st)) && !(e = tc_slice_exact(rows, rows, M, ld, slices, plane, st)))
        e = tc_exact_product(rows, rows, plane, k, reinterpret_cast<const double2 *>(X), k,
                             reinterpret_cast<double2 *>(Y), k, slices, scratch, flag, (unsigned long long)wait_cycles,
                             st);
    if (!e) e = cudaMemcpyAsync(&timed_out, flag, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    dev_free(plane, st);
    dev_free(scratch, st);
    dev_free(flag, st);
    if (e) return pfail(cuda_status(e), "dense_apply_sliced: %s", cudaGetErrorString(e));
    if (timed_out) return pfail(ERR_TIMEOUT, "dense_apply_sliced: a bounded wait of the tensor-core product gave up");
    return OK;
}

int pcbqs_gb300_to_single(const double *in, float *out, int64_t count, void *stream) {
    if (!in || !out || count < 0) return pfail(ERR_ARGUMENT, "to_single: invalid argument");
    if (!count) return OK;
    k_to_f32<<<grid_of(count), 256, 0, static_cast<cudaStream_t>(stream)>>>(count, in, out);
    note_launches(1);
    cudaError_t e = cudaGetLastError();
    return e ? pfail(cuda_status(e), "to_single: %s", cudaGetErrorString(e)) : OK;
}

int pcbqs_gb300_peec_single(pcbqs_gb300_peec *h, const float *Lf, int64_t ldlf, const float *Pf, const float *Pfim,
                            int64_t ldpf) {
    if (!h || !Lf || ldlf < h->op.ne || (h->op.nn > 0 && (!Pf || ldpf < h->op.nn)))
        return pfail(ERR_ARGUMENT, "peec_single: invalid single-precision matrices");
    if (h->op.compressed) return pfail(ERR_ARGUMENT, "peec_single: the compressed operator has no single-precision copy");
    h->op.unpack();
    h->op.Lf = Lf;
    h->op.ldlf = ldlf;
    h->op.Pf = Pf;
    h->op.Pfim = Pfim;
    h->op.ldpf = ldpf;
    if (h->op.Pim && !Pfim) return pfail(ERR_ARGUMENT, "peec_single: P is complex: its FP32 imaginary part is needed");
    return OK;
}

int pcbqs_gb300_peec_solve_mixed(pcbqs_gb300_peec *h, int k, const int32_t *sys_host, const double *b, double *x,
                                 double tol, double inner_tol, int max_outer, int inner_maxiter, int restart,
                                 int precondition, int32_t *iterations, double *residual, int32_t *outer_steps,
                                 void *stream) {
    if (!h || k <= 0 || !sys_host || !b || !x || !(tol > 0) || !(inner_tol > 0) || max_outer < 0 ||
        inner_maxiter <= 0 || restart <= 0)
        return pfail(ERR_ARGUMENT, "peec_solve_mixed: invalid argument");
    if (!h->op.Lf && !h->op.compressed)
        return pfail(ERR_ARGUMENT, "peec_solve_mixed: no single-precision L and P set");
    for (int s = 0; s < k; ++s)
        if (sys_host[s] < 0 || sys_host[s] >= h->op.nsys) return pfail(ERR_ARGUMENT, "peec_solve_mixed: system");
    if (precondition == 1 && !h->bj) return pfail(ERR_ARGUMENT, "peec_solve_mixed: no block-Jacobi set up");
    if (precondition == 2 && !h->lu) return pfail(ERR_ARGUMENT, "peec_solve_mixed: no factor set up");
    if (precondition == 3 && !h->graph) return pfail(ERR_ARGUMENT, "peec_solve_mixed: no graph preconditioner set up");
    if (precondition < 0 || precondition > 3) return pfail(ERR_ARGUMENT, "peec_solve_mixed: preconditioner 0 .. 3");
    Preconditioner *M = precondition == 1   ? static_cast<Preconditioner *>(h->bj)
                        : precondition == 2 ? static_cast<Preconditioner *>(h->lu)
                        : precondition == 3 ? static_cast<Preconditioner *>(h->graph)
                                            : nullptr;
    SingleView single;
    single.op = &h->op;
    RefineOptions opt;
    opt.tol = tol;
    opt.inner_tol = inner_tol;
    opt.max_outer = max_outer;
    opt.inner_maxiter = inner_maxiter;
    opt.restart = restart;
    opt.captured = h->captured;
    GmresReport rep;
    int steps = 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = refine_batched(h->op, single, M, k, sys_host, reinterpret_cast<const cd *>(b),
                                   reinterpret_cast<cd *>(x), opt, rep, steps, st);
    if (e) return pfail(cuda_status(e), "peec_solve_mixed: %s", cudaGetErrorString(e));
    if (int status = take_product_timeout(h->op, st, "peec_solve_mixed")) return status;
    if (outer_steps) *outer_steps = steps;
    bool ok = true;
    for (int s = 0; s < k; ++s) {
        if (iterations) iterations[s] = rep.iterations[s];
        if (residual) residual[s] = rep.residual[s];
        ok = ok && rep.residual[s] <= tol;
    }
    if (!ok) return pfail(ERR_CONVERGENCE, "peec_solve_mixed: not every system reached the tolerance");
    return OK;
}

int pcbqs_gb300_dense_gmres(int64_t n, const double *A, const double *Aim, int64_t lda, int k, const double *b,
                            double *x, double tol, int maxiter, int restart, int precondition, int32_t *iterations,
                            double *residual, void *stream) {
    if (n <= 0 || !A || lda < n || k <= 0 || !b || !x || !(tol > 0) || maxiter <= 0 || restart <= 0 ||
        precondition < 0 || precondition > 2)
        return pfail(ERR_ARGUMENT, "dense_gmres: invalid argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DenseSym op;
    op.n_ = n; op.ld = lda; op.A = A; op.Aim = Aim;
    Jacobi J;
    CholPrecond C;
    Preconditioner *M = nullptr;
    cudaError_t e = cudaSuccess;
    if (precondition == 0) {
        J.n = n;
        if ((e = dev_alloc(&J.d, n, st))) {
            return pfail(ERR_MEMORY, "dense_gmres: allocation");
        }
        k_diag_extract<<<grid_of(n), 256, 0, st>>>(n, A, lda, J.d);
        note_launches(1);
        M = &J;
    } else {
        int info = 0;
        C.library = precondition == 2;
        e = C.factor(n, A, lda, st, info);
        if (e || info) {
            return pfail(info ? ERR_NONFINITE : ERR_CUDA, "dense_gmres: single-precision Cholesky failed (info %d)",
                         info);
        }
        M = &C;
    }
    std::vector<int32_t> sys(k, 0);
    GmresOptions opt;
    opt.tol = tol; opt.maxiter = maxiter; opt.restart = restart;
    GmresReport rep;
    e = gmres_batched(op, M, k, sys.data(), reinterpret_cast<const cd *>(b), reinterpret_cast<cd *>(x), opt, rep, st);
    dev_free(J.d, st);
    if (e) return pfail(cuda_status(e), "dense_gmres: %s", cudaGetErrorString(e));
    bool ok = true;
    for (int s = 0; s < k; ++s) {
        if (iterations) iterations[s] = rep.iterations[s];
        if (residual) residual[s] = rep.residual[s];
        ok = ok && rep.residual[s] <= tol;
    }
    if (!ok) return pfail(ERR_CONVERGENCE, "dense_gmres: not every column reached the tolerance");
    return OK;
}

}  // extern "C"
