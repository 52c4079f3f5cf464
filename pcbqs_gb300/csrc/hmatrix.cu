// H-matrix of the RWG partial inductance on the device: exact entries of edge pairs, dense near leaves, partial-
// pivot ACA of admissible far blocks (one CTA per block), and the compressed product Y = H X.
//
// Reference behaviour (paths within the pcbqs project):
//   entries   core/compressed_kernels.hpp:9-38 (canonical_pair, rwg_entry) and 125-144 (rwg_inductance):
//             L[m,n] = f sum_{i,j} a_mi a_nj [Mrr - v_nj.Mro - v_mi.Mrs + (v_mi.v_nj) M0] over the canonical (min, max)
//             triangle-pair moments of the supports, a = +-1/(2A), f = mu0/4pi
//   ACA       core/hmatrix_build.hpp:143-265 (aca: partial pivoting, a 16-row check set drawn per block from a
//             SplitMix64 stream seeded by the block, a second independent 16-row check before accepting, rank cap
//             min(cap, 0.7 m n / (m + n)), failure -> the host subdivides) and hmatrix.py:103-150
//   product   core/hmatrix_kernels.hpp:1-100 (each block writes its contribution rows into its own slots, then
//             each output row sums its slots in block order: deterministic)
// The cluster tree, admissibility and block packing are host work (pcbqs_gb300/hmatrix.py).
#include <algorithm>
#include <cstdint>

#include <cuda_bf16.h>

#include "../../include/pcbqs_gb300.h"
#include "common.cuh"
#include "hmatrix.cuh"
#include "pairs.cuh"

namespace pq {

struct EdgeSet {
    const int32_t *tri;      // (2, ne) supports T+/T-
    const double *alpha;     // (2, ne) +-1/(2A)
    const double *vertex;    // (2, ne, 2) free vertices (centred coordinates)
    int64_t ne;
};

struct Rule {
    double near;
    int all_near, outer;
};

// Canonical moments of the ordered pair (p, q): integrated as (min, max), Mro/Mrs swapped back when p > q, the
// diagonal's averaged (compressed_kernels.hpp:9-20).
__device__ __forceinline__ void canonical(const Geometry &g, const Rule &r, int p, int q, double *m) {
    const int a = min(p, q), b = max(p, q);
    const double d = g.cls[a].z - g.cls[b].z;
    const int k = classify(g.cls[a], g.cls[b], d, r.near, r.all_near, r.outer);
    pair_moments(g, a, b, d, k, false, m);
    if (p > q) {
        double t = m[1]; m[1] = m[3]; m[3] = t;
        t = m[2]; m[2] = m[4]; m[4] = t;
    } else if (p == q) {
        const double x = (m[1] + m[3]) / 2, y = (m[2] + m[4]) / 2;
        m[1] = m[3] = x;
        m[2] = m[4] = y;
    }
}

__device__ double l_entry(const Geometry &g, const Rule &r, const EdgeSet &e, double factor, int64_t em, int64_t en) {
    double total = 0;
    for (int i = 0; i < 2; ++i) {
        const int p = e.tri[i * e.ne + em];
        const double am = e.alpha[i * e.ne + em];
        const double vpx = e.vertex[2 * (i * e.ne + em)], vpy = e.vertex[2 * (i * e.ne + em) + 1];
        for (int j = 0; j < 2; ++j) {
            const int q = e.tri[j * e.ne + en];
            const double vqx = e.vertex[2 * (j * e.ne + en)], vqy = e.vertex[2 * (j * e.ne + en) + 1];
            double m[6];
            canonical(g, r, p, q, m);
            const double val = m[5] - (vqx * m[1] + vqy * m[2]) - (vpx * m[3] + vpy * m[4]) + (vpx * vqx + vpy * vqy) * m[0];
            total += am * e.alpha[j * e.ne + en] * val;
        }
    }
    return factor * total;
}

// The potential kernel over triangles (PotentialEntries, core/hmatrix_build.hpp:54-67): the canonical pair's M0
// times factor / (A_t A_u), factor = 1 / (4 pi eps0 er).
__device__ double p_entry(const Geometry &g, const Rule &r, double factor, int64_t t, int64_t u) {
    const int a = (int)min(t, u), b = (int)max(t, u);
    const double d = g.cls[a].z - g.cls[b].z;
    const int k = classify(g.cls[a], g.cls[b], d, r.near, r.all_near, r.outer);
    double m[6];
    pair_moments(g, a, b, d, k, true, m);
    return factor * m[0] / (g.far[t].area * g.far[u].area);
}

// kind 0: L over RWG edges; kind 1: the potential kernel over triangles.
__device__ __forceinline__ double hm_entry(int kind, const Geometry &g, const Rule &r, const EdgeSet &e, double factor,
                                           int64_t i, int64_t j) {
    return kind ? p_entry(g, r, factor, i, j) : l_entry(g, r, e, factor, i, j);
}

// Block metadata (host-packed, int64 x 8): a offset, a length, b offset, b length, store offset, rank cap, same,
// and (output of the build) rank: -1 dense leaf / ACA failure, >= 0 low rank.
enum { M_AOFF, M_ALEN, M_BOFF, M_BLEN, M_STORE, M_CAP, M_SAME, M_KIND };

__global__ void k_hm_dense(const int64_t *meta, const int64_t *blocks, int64_t nb, const int64_t *idx, Geometry g,
                           Rule r, EdgeSet e, int kind, double factor, double *store) {
    for (int64_t w = blockIdx.x; w < nb; w += gridDim.x) {
        const int64_t *mt = meta + 8 * blocks[w];
        const int64_t la = mt[M_ALEN], lb = mt[M_BLEN];
        const int64_t *a = idx + mt[M_AOFF], *b = idx + mt[M_BOFF];
        double *out = store + mt[M_STORE];
        for (int64_t t = threadIdx.x; t < la * lb; t += blockDim.x)
            out[t] = hm_entry(kind, g, r, e, factor, a[t / lb], b[t % lb]);
    }
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

constexpr int ACA_THREADS = 256;
constexpr int ACA_CHECK = 16;

// Block-wide sum and arg-max helpers (one value per thread).
__device__ double block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0) {
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
        red[0] = s;
    }
    __syncthreads();
    const double out = red[0];
    __syncthreads();
    return out;
}

__device__ void block_argmax(double v, int64_t i, double *redv, int64_t *redi, double &best, int64_t &at) {
    for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_down_sync(0xffffffffu, v, o);
        const int64_t oi = __shfl_down_sync(0xffffffffu, i, o);
        if (ov > v || (ov == v && oi < i)) { v = ov; i = oi; }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) { redv[wid] = v; redi[wid] = i; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double bv = redv[0];
        int64_t bi = redi[0];
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k)
            if (redv[k] > bv || (redv[k] == bv && redi[k] < bi)) { bv = redv[k]; bi = redi[k]; }
        redv[0] = bv;
        redi[0] = bi;
    }
    __syncthreads();
    best = redv[0];
    at = redi[0];
    __syncthreads();
}

// One CTA per admissible block: U (la x cap) column-major at store, V (cap x lb) row-major after it, then the
// check rows (2 * ACA_CHECK x lb) and their residuals. rank written to meta[M_KIND] (-1: not accepted).
__global__ void __launch_bounds__(ACA_THREADS) k_hm_aca(int64_t *meta, const int64_t *blocks, int64_t nb,
                                                        const int64_t *idx, Geometry g, Rule r, EdgeSet e,
                                                        int kind, double factor, double tol, double *store,
                                                        unsigned char *used_all, int64_t used_stride) {
    __shared__ double redv[32];
    __shared__ int64_t redi[32];
    __shared__ int64_t check[2 * ACA_CHECK];
    __shared__ int s_next;
    for (int64_t w = blockIdx.x; w < nb; w += gridDim.x) {
        int64_t *mt = meta + 8 * blocks[w];
        const int64_t la = mt[M_ALEN], lb = mt[M_BLEN];
        const int64_t *a = idx + mt[M_AOFF], *b = idx + mt[M_BOFF];
        const int cap = (int)mt[M_CAP];
        double *U = store + mt[M_STORE];                 // la x cap, column r at U + r * la
        double *V = U + (int64_t)la * cap;               // cap x lb
        double *ref = V + (int64_t)cap * lb;             // 2*ACA_CHECK x lb reference rows
        unsigned char *used = used_all + w * used_stride;
        for (int64_t t = threadIdx.x; t < la; t += blockDim.x) used[t] = 0;
        // the check rows: distinct, from the block's own SplitMix64 stream
        int nc = (int)(la < ACA_CHECK ? la : ACA_CHECK);
        if (threadIdx.x == 0) {
            uint64_t seed = 0x5DEECE66Dull ^ ((uint64_t)a[0] * 0x100000001B3ull) ^ ((uint64_t)b[0] << 21) ^
                            ((uint64_t)la << 42) ^ (uint64_t)lb;
            int got = 0;
            while (got < nc) {
                const int64_t c = (int64_t)(splitmix64(seed) % (uint64_t)la);
                bool dup = false;
                for (int k = 0; k < got; ++k) dup = dup || check[k] == c;
                if (!dup) check[got++] = c;
            }
        }
        __syncthreads();
        for (int64_t t = threadIdx.x; t < (int64_t)nc * lb; t += blockDim.x)
            ref[t] = hm_entry(kind, g, r, e, factor, a[check[t / lb]], b[t % lb]);
        __syncthreads();
        double refnorm2 = 0;
        for (int64_t t = threadIdx.x; t < (int64_t)nc * lb; t += blockDim.x) refnorm2 += ref[t] * ref[t];
        refnorm2 = block_sum(refnorm2, redv);
        int rank = 0, accepted = 0, second = 0;
        int64_t i = 0;
        for (int step = 0; step < cap; ++step) {
            // row i of the residual, into V[rank]
            double *row = V + (int64_t)rank * lb;
            double bestv = -1;
            int64_t bestj = 0;
            for (int64_t j = threadIdx.x; j < lb; j += blockDim.x) {
                double v = hm_entry(kind, g, r, e, factor, a[i], b[j]);
                for (int k = 0; k < rank; ++k) v -= U[(int64_t)k * la + i] * V[(int64_t)k * lb + j];
                row[j] = v;
                if (fabs(v) > bestv) { bestv = fabs(v); bestj = j; }
            }
            double piv_abs;
            int64_t jp;
            block_argmax(bestv, bestj, redv, redi, piv_abs, jp);
            if (threadIdx.x == 0) used[i] = 1;
            if (piv_abs > 2.2250738585072014e-308) {
                const double pivot = row[jp];
                __syncthreads();
                double *col = U + (int64_t)rank * la;
                for (int64_t t = threadIdx.x; t < la; t += blockDim.x) {
                    double v = hm_entry(kind, g, r, e, factor, a[t], b[jp]);
                    for (int k = 0; k < rank; ++k) v -= U[(int64_t)k * la + t] * V[(int64_t)k * lb + jp];
                    col[t] = v;
                }
                __syncthreads();
                for (int64_t j = threadIdx.x; j < lb; j += blockDim.x) row[j] /= pivot;
                __syncthreads();
                ++rank;
            }
            // residual of the check rows
            double res2 = 0;
            for (int64_t t = threadIdx.x; t < (int64_t)nc * lb; t += blockDim.x) {
                const int64_t c = t / lb, j = t % lb;
                double v = ref[t];
                for (int k = 0; k < rank; ++k) v -= U[(int64_t)k * la + check[c]] * V[(int64_t)k * lb + j];
                res2 += v * v;
            }
            res2 = block_sum(res2, redv);
            if (res2 <= tol * tol * fmax(refnorm2, 1e-300)) {
                if (second || la <= nc) {
                    accepted = 1;
                    break;
                }
                // a second, independent set of check rows before accepting
                const int n2 = (int)(la < ACA_CHECK ? la : ACA_CHECK);
                if (threadIdx.x == 0) {
                    uint64_t seed = 0x243F6A8885A308D3ull ^ ((uint64_t)a[0] << 7) ^ ((uint64_t)b[0] << 29) ^
                                    (uint64_t)la;
                    int got = 0;
                    while (got < n2) {
                        const int64_t c = (int64_t)(splitmix64(seed) % (uint64_t)la);
                        bool dup = false;
                        for (int k = 0; k < nc + got; ++k) dup = dup || check[k] == c;
                        if (!dup) check[nc + got++] = c;
                        if (nc + got >= la) break;
                    }
                    s_next = got;
                }
                __syncthreads();
                const int added = s_next;
                for (int64_t t = threadIdx.x; t < (int64_t)added * lb; t += blockDim.x)
                    ref[(int64_t)nc * lb + t] = hm_entry(kind, g, r, e, factor, a[check[nc + t / lb]], b[t % lb]);
                __syncthreads();
                double e2 = 0, n2s = 0;
                for (int64_t t = threadIdx.x; t < (int64_t)added * lb; t += blockDim.x) {
                    const int64_t c = nc + t / lb, j = t % lb;
                    double v = ref[(int64_t)nc * lb + t];
                    n2s += v * v;
                    for (int k = 0; k < rank; ++k) v -= U[(int64_t)k * la + check[c]] * V[(int64_t)k * lb + j];
                    e2 += v * v;
                }
                e2 = block_sum(e2, redv);
                n2s = block_sum(n2s, redv);
                nc += added;
                refnorm2 += n2s;
                second = 1;
                if (e2 <= tol * tol * fmax(n2s, 1e-300)) {
                    accepted = 1;
                    break;
                }
            }
            // next pivot row: the unused check row with the largest residual, else the unused row with the largest
            // entry of the last column, else stop
            double bv = -1;
            int64_t bi = -1;
            for (int c = threadIdx.x; c < nc; c += blockDim.x) {
                if (used[check[c]]) continue;
                double n2 = 0;
                for (int64_t j = 0; j < lb; ++j) {
                    double v = ref[(int64_t)c * lb + j];
                    for (int k = 0; k < rank; ++k) v -= U[(int64_t)k * la + check[c]] * V[(int64_t)k * lb + j];
                    n2 += v * v;
                }
                if (n2 > bv || (n2 == bv && check[c] < bi)) { bv = n2; bi = check[c]; }
            }
            double gbest;
            int64_t gat;
            block_argmax(bv, bi, redv, redi, gbest, gat);
            if (gbest >= 0 && gat >= 0) {
                i = gat;
            } else {
                double cv = -1;
                int64_t ci = -1;
                for (int64_t t = threadIdx.x; t < la; t += blockDim.x) {
                    if (used[t]) continue;
                    const double v = rank ? fabs(U[(int64_t)(rank - 1) * la + t]) : 0.0;
                    if (v > cv || (v == cv && t < ci)) { cv = v; ci = t; }
                }
                block_argmax(cv, ci, redv, redi, gbest, gat);
                if (gbest < 0 || gat < 0) break;
                i = gat;
            }
        }
        if (threadIdx.x == 0) mt[M_KIND] = accepted ? rank : -1;
        __syncthreads();
    }
}

// Product, phase 1: every block writes its contributions into its slots (forward rows for a, transposed rows for
// b when the block is not a diagonal one). x, y: (n, k) complex128; slot rows are k complex wide.
__global__ void k_hm_apply_blocks(const int64_t *meta, int64_t nb, const int64_t *slot0, const int64_t *idx,
                                  const double *store, int k, const double2 *x, double2 *slots) {
    extern __shared__ double2 tmp[];       // rank x k
    for (int64_t w = blockIdx.x; w < nb; w += gridDim.x) {
        const int64_t *mt = meta + 8 * w;
        const int64_t la = mt[M_ALEN], lb = mt[M_BLEN];
        const int64_t *a = idx + mt[M_AOFF], *b = idx + mt[M_BOFF];
        const int rank = (int)mt[M_KIND];
        const bool same = mt[M_SAME] != 0;
        const double *S = store + mt[M_STORE];
        double2 *fa = slots + slot0[2 * w] * k, *fb = slots + slot0[2 * w + 1] * k;
        if (rank < 0) {        // dense D (la x lb, row-major)
            for (int64_t t = threadIdx.x; t < la * k; t += blockDim.x) {
                const int64_t ia = t / k;
                const int s = (int)(t % k);
                double re = 0, im = 0;
                for (int64_t j = 0; j < lb; ++j) {
                    const double d = S[ia * lb + j];
                    const double2 v = x[b[j] * k + s];
                    re += d * v.x;
                    im += d * v.y;
                }
                fa[t] = make_double2(re, im);
            }
            if (!same)
                for (int64_t t = threadIdx.x; t < lb * k; t += blockDim.x) {
                    const int64_t jb = t / k;
                    const int s = (int)(t % k);
                    double re = 0, im = 0;
                    for (int64_t i2 = 0; i2 < la; ++i2) {
                        const double d = S[i2 * lb + jb];
                        const double2 v = x[a[i2] * k + s];
                        re += d * v.x;
                        im += d * v.y;
                    }
                    fb[t] = make_double2(re, im);
                }
        } else {               // U (la x cap, column-major) V (cap x lb)
            const int cap = (int)mt[M_CAP];
            const double *U = S, *V = S + la * cap;
            // forward: tmp = V x[b]; fa = U tmp
            for (int t = threadIdx.x; t < rank * k; t += blockDim.x) {
                const int q = t / k, s = t % k;
                double re = 0, im = 0;
                for (int64_t j = 0; j < lb; ++j) {
                    const double v = V[(int64_t)q * lb + j];
                    const double2 xv = x[b[j] * k + s];
                    re += v * xv.x;
                    im += v * xv.y;
                }
                tmp[t] = make_double2(re, im);
            }
            __syncthreads();
            for (int64_t t = threadIdx.x; t < la * k; t += blockDim.x) {
                const int64_t ia = t / k;
                const int s = (int)(t % k);
                double re = 0, im = 0;
                for (int q = 0; q < rank; ++q) {
                    const double u = U[(int64_t)q * la + ia];
                    re += u * tmp[q * k + s].x;
                    im += u * tmp[q * k + s].y;
                }
                fa[t] = make_double2(re, im);
            }
            __syncthreads();
            // transposed: tmp = U^T x[a]; fb = V^T tmp
            for (int t = threadIdx.x; t < rank * k; t += blockDim.x) {
                const int q = t / k, s = t % k;
                double re = 0, im = 0;
                for (int64_t i2 = 0; i2 < la; ++i2) {
                    const double u = U[(int64_t)q * la + i2];
                    const double2 xv = x[a[i2] * k + s];
                    re += u * xv.x;
                    im += u * xv.y;
                }
                tmp[t] = make_double2(re, im);
            }
            __syncthreads();
            for (int64_t t = threadIdx.x; t < lb * k; t += blockDim.x) {
                const int64_t jb = t / k;
                const int s = (int)(t % k);
                double re = 0, im = 0;
                for (int q = 0; q < rank; ++q) {
                    const double v = V[(int64_t)q * lb + jb];
                    re += v * tmp[q * k + s].x;
                    im += v * tmp[q * k + s].y;
                }
                fb[t] = make_double2(re, im);
            }
        }
        __syncthreads();
    }
}

// Phase 2: y[row] = sum of the row's slots, in slot order.
__global__ void k_hm_apply_rows(int64_t n, int k, const int64_t *row_ptr, const int64_t *slots_of_row,
                                const double2 *slots, double2 *y) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * k; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = t / k;
        const int s = (int)(t % k);
        double re = 0, im = 0;
        for (int64_t q = row_ptr[row]; q < row_ptr[row + 1]; ++q) {
            const double2 v = slots[slots_of_row[q] * k + s];
            re += v.x;
            im += v.y;
        }
        y[t] = make_double2(re, im);
    }
}

}  // namespace pq

using namespace pq;

// The geometry of a fill context (capi.cu).
const Geometry *pcbqs_gb300_geometry_of(const pcbqs_gb300_ctx *ctx);

extern "C" int pcbqs_gb300_hmatrix_build(const pcbqs_gb300_ctx *ctx, double near, int outer, int kind,
                                         const int32_t *tri, const double *alpha, const double *vertex, int64_t ne,
                                         double factor,
                                         int64_t *meta, const int64_t *dense, int64_t ndense, const int64_t *lowrank,
                                         int64_t nlow, const int64_t *idx, double tol, double *store,
                                         unsigned char *used, int64_t used_stride, void *stream) {
    if (!ctx || kind < 0 || kind > 1 || (kind == 0 && (!tri || !alpha || !vertex || ne <= 0)) || !meta ||
        (ndense && !dense) || (nlow && !lowrank) || !idx ||
        !store || (nlow && !used) || !(tol > 0) || outer < 0 || outer > 2)
        return fail(ERR_ARGUMENT, "hmatrix_build: invalid argument");
    const Geometry *g = pcbqs_gb300_geometry_of(ctx);
    Rule r{near < 0 || std::isinf(near) ? 0.0 : near, near < 0 || std::isinf(near) ? 1 : 0, outer};
    EdgeSet e{tri, alpha, vertex, ne};
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (ndense) {
        k_hm_dense<<<(unsigned)std::min<int64_t>(ndense, (int64_t)sms * 8), 256, 0, st>>>(meta, dense, ndense, idx,
                                                                                          *g, r, e, kind, factor, store);
        note_launches(1);
    }
    if (nlow) {
        k_hm_aca<<<(unsigned)std::min<int64_t>(nlow, (int64_t)sms * 8), ACA_THREADS, 0, st>>>(
            meta, lowrank, nlow, idx, *g, r, e, kind, factor, tol, store, used, used_stride);
        note_launches(1);
    }
    cudaError_t err = cudaGetLastError();
    return err ? fail(ERR_CUDA, "hmatrix_build: %s", cudaGetErrorString(err)) : OK;
}

namespace pq {

cudaError_t hmatrix_blocks(int64_t nb, const int64_t *meta, const int64_t *slot0, const int64_t *idx,
                           const double *store, int max_rank, int k, const double *x, double *slots, cudaStream_t st) {
    if (!nb) return cudaSuccess;
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t smem = sizeof(double2) * (size_t)std::max(1, max_rank) * k;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_hm_apply_blocks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_hm_apply_blocks<<<(unsigned)std::min<int64_t>(nb, (int64_t)sms * 8), 256, smem, st>>>(
        meta, nb, slot0, idx, store, k, reinterpret_cast<const double2 *>(x), reinterpret_cast<double2 *>(slots));
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t hmatrix_rows(int64_t n, const int64_t *row_ptr, const int64_t *slots_of_row, int k, const double *slots,
                         double *y, cudaStream_t st) {
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    k_hm_apply_rows<<<(unsigned)std::min<int64_t>((n * k + 255) / 256, (int64_t)sms * 16), 256, 0, st>>>(
        n, k, row_ptr, slots_of_row, reinterpret_cast<const double2 *>(slots), reinterpret_cast<double2 *>(y));
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t hmatrix_apply(int64_t n, int64_t nb, const int64_t *meta, const int64_t *slot0, const int64_t *idx,
                          const double *store, const int64_t *row_ptr, const int64_t *slots_of_row, int max_rank,
                          int k, const double *x, double *y, double *slots, cudaStream_t st) {
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t smem = sizeof(double2) * (size_t)std::max(1, max_rank) * k;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_hm_apply_blocks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (nb)
        k_hm_apply_blocks<<<(unsigned)std::min<int64_t>(nb, (int64_t)sms * 8), 256, smem, st>>>(
            meta, nb, slot0, idx, store, k, reinterpret_cast<const double2 *>(x), reinterpret_cast<double2 *>(slots));
    k_hm_apply_rows<<<(unsigned)std::min<int64_t>((n * k + 255) / 256, (int64_t)sms * 16), 256, 0, st>>>(
        n, k, row_ptr, slots_of_row, reinterpret_cast<const double2 *>(slots), reinterpret_cast<double2 *>(y));
    note_launches(nb ? 2 : 1);
    return cudaGetLastError();
}

// The BF16 part planes of the tensor-core low-rank product, one thread block per job (a block's factor or dense
// leaf in one direction): job = (base, si, sj, ni, nj, row0, colbase, map_off); for i < ni, j < nj the FP64 entry
// x = store[base + i si + j sj] is rounded to FP32 and split as h = bf16(x), m = bf16(x - h) (both to nearest
// even), written to plane[(row0 + i) pitch + c] and plane[(row0 + i) pitch + off2 + c], c = colbase + map[map_off + j]
// (c = colbase + j when map_off < 0). The jobs' destinations do not overlap.
__global__ void k_pack_parts(const double *store, const int64_t *jobs, const int32_t *map, __nv_bfloat16 *plane,
                             int64_t pitch, int64_t off2) {
    const int64_t *job = jobs + 8 * (int64_t)blockIdx.x;
    const int64_t base = job[0], si = job[1], sj = job[2], ni = job[3], nj = job[4], row0 = job[5], colbase = job[6],
                  map_off = job[7];
    for (int64_t t = threadIdx.x; t < ni * nj; t += blockDim.x) {
        const int64_t i = t / nj, j = t % nj;
        const float x = (float)store[base + i * si + j * sj];
        const __nv_bfloat16 h = __float2bfloat16_rn(x);
        const __nv_bfloat16 m = __float2bfloat16_rn(x - __bfloat162float(h));
        const int64_t c = colbase + (map_off < 0 ? j : (int64_t)map[map_off + j]);
        __nv_bfloat16 *row = plane + (row0 + i) * pitch;
        row[c] = h;
        row[off2 + c] = m;
    }
}

}  // namespace pq

extern "C" int pcbqs_gb300_hmatrix_apply(int64_t n, int64_t nb, const int64_t *meta, const int64_t *slot0,
                                         const int64_t *idx, const double *store, const int64_t *row_ptr,
                                         const int64_t *slots_of_row, int max_rank, int k, const double *x, double *y,
                                         double *slots, void *stream) {
    if (n <= 0 || nb < 0 || !meta || !slot0 || !idx || !store || !row_ptr || !slots_of_row || k <= 0 || !x || !y ||
        !slots || max_rank < 0)
        return pq::fail(pq::ERR_ARGUMENT, "hmatrix_apply: invalid argument");
    const cudaError_t err = pq::hmatrix_apply(n, nb, meta, slot0, idx, store, row_ptr, slots_of_row, max_rank, k, x, y,
                                              slots, static_cast<cudaStream_t>(stream));
    return err ? pq::fail(pq::ERR_CUDA, "hmatrix_apply: %s", cudaGetErrorString(err)) : pq::OK;
}

extern "C" int pcbqs_gb300_pack_bf16_parts(const double *store, const int64_t *jobs, int64_t njobs,
                                           const int32_t *map, void *plane, int64_t pitch, int64_t off2,
                                           void *stream) {
    if (njobs < 0 || njobs > 0x7fffffff || (njobs && (!store || !jobs || !plane)) || pitch <= 0 || off2 < 0)
        return pq::fail(pq::ERR_ARGUMENT, "pack_bf16_parts: invalid argument");
    if (!njobs) return pq::OK;
    pq::k_pack_parts<<<(unsigned)njobs, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        store, jobs, map, static_cast<__nv_bfloat16 *>(plane), pitch, off2);
    pq::note_launches(1);
    const cudaError_t err = cudaGetLastError();
    return err ? pq::fail(pq::ERR_CUDA, "pack_bf16_parts: %s", cudaGetErrorString(err)) : pq::OK;
}
