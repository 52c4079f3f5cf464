// Batched restarted GMRES(m) in complex128 on the device: every column (a frequency and right-hand side) has its
// own Krylov space, but each Arnoldi step applies the operator once to all active columns, so the dense matrices
// are read once per step for the whole batch. Right preconditioning; classical Gram-Schmidt applied twice (CGS2:
// two block passes instead of j dependent ones, orthogonal to working precision like MGS); complex Givens
// rotations and per-column convergence masks; converged columns drop out (compaction) at each restart; the true
// residual |b - A x| / |b| decides convergence. All reductions have a fixed order (two-stage sums over a fixed
// number of row chunks), so results do not depend on scheduling.
//
// Reference behaviour (paths within the pcbqs project): mqs_iterative._lockstep_gmres
// (src/pcbqs/mqs_iterative.py:109-170: per-column Krylov spaces, one product per step, Givens on each column's
// Hessenberg, convergence |g_{j+1}|/|b| <= tol, compaction at restart), and the acceptance rule of
// peec_iterative._gmres (src/pcbqs/peec_iterative.py:100-112).
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "pool.cuh"
#include "solve.cuh"

namespace pq {

constexpr int NCHUNK = 64;       // row chunks of the two-stage reductions
constexpr int RT = 256;          // reduction block size

__device__ __forceinline__ cd cmul(cd a, cd b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ cd cmulc(cd a, cd b) {      // conj(a) * b
    return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ cd cadd(cd a, cd b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ cd csub(cd a, cd b) { return make_double2(a.x - b.x, a.y - b.y); }

// partial[chunk][i][s] = sum over the chunk's rows of conj(V_i[r,s]) w[r,s]   (grid: NCHUNK x jc)
__global__ void __launch_bounds__(RT) k_dots_partial(int64_t n, int k, const cd *V, const cd *w, cd *partial) {
    __shared__ cd acc[RT];
    const int chunk = blockIdx.x, i = blockIdx.y;
    const int64_t r0 = n * chunk / NCHUNK, r1 = n * (chunk + 1) / NCHUNK;
    const cd *Vi = V + (size_t)i * n * k;
    cd *out = partial + ((size_t)chunk * gridDim.y + i) * k;
    if (k <= RT) {
        const int per = RT / k, t = threadIdx.x;
        cd a = make_double2(0, 0);
        if (t < per * k) {
            const int s = t % k, rr = t / k;
            for (int64_t r = r0 + rr; r < r1; r += per) a = cadd(a, cmulc(Vi[r * k + s], w[r * k + s]));
        }
        acc[t] = a;
        __syncthreads();
        if (t < k) {
            cd sum = make_double2(0, 0);
            for (int q = 0; q < per; ++q) sum = cadd(sum, acc[t + q * k]);
            out[t] = sum;
        }
    } else {
        for (int s = threadIdx.x; s < k; s += RT) {
            cd a = make_double2(0, 0);
            for (int64_t r = r0; r < r1; ++r) a = cadd(a, cmulc(Vi[r * k + s], w[r * k + s]));
            out[s] = a;
        }
    }
}

// h[i][s] = sum_chunk partial[chunk][i][s], in chunk order.
__global__ void k_dots_final(int jc, int k, const cd *partial, cd *h) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= jc * k) return;
    cd sum = make_double2(0, 0);
    for (int c = 0; c < NCHUNK; ++c) sum = cadd(sum, partial[(size_t)c * jc * k + idx]);
    h[idx] = sum;
}

// w[r,s] -= sum_{i<jc} V_i[r,s] h[i][s]
__global__ void k_orth_update(int64_t n, int k, int jc, const cd *V, const cd *h, cd *w) {
    const int64_t total = n * k;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(idx % k);
        cd a = w[idx];
        for (int i = 0; i < jc; ++i) a = csub(a, cmul(V[(size_t)i * total + idx], h[i * k + s]));
        w[idx] = a;
    }
}

// Column sums of squares, two stages.
__global__ void __launch_bounds__(RT) k_norm_partial(int64_t n, int k, const cd *x, double *partial) {
    __shared__ double acc[RT];
    const int chunk = blockIdx.x;
    const int64_t r0 = n * chunk / NCHUNK, r1 = n * (chunk + 1) / NCHUNK;
    double *out = partial + (size_t)chunk * k;
    if (k <= RT) {
        const int per = RT / k, t = threadIdx.x;
        double a = 0;
        if (t < per * k) {
            const int s = t % k, rr = t / k;
            for (int64_t r = r0 + rr; r < r1; r += per) {
                const cd v = x[r * k + s];
                a += v.x * v.x + v.y * v.y;
            }
        }
        acc[t] = a;
        __syncthreads();
        if (t < k) {
            double sum = 0;
            for (int q = 0; q < per; ++q) sum += acc[t + q * k];
            out[t] = sum;
        }
    } else {
        for (int s = threadIdx.x; s < k; s += RT) {
            double a = 0;
            for (int64_t r = r0; r < r1; ++r) {
                const cd v = x[r * k + s];
                a += v.x * v.x + v.y * v.y;
            }
            out[s] = a;
        }
    }
}

__global__ void k_norm_final(int k, const double *partial, double *norm) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= k) return;
    double sum = 0;
    for (int c = 0; c < NCHUNK; ++c) sum += partial[(size_t)c * k + s];
    norm[s] = sqrt(sum);
}

// out[:, s] = in[:, s] / norm[s] (norm 0: out = in, a zero column stays zero)
__global__ void k_divide(int64_t n, int k, const cd *in, const double *norm, cd *out) {
    const int64_t total = n * k;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const double d = norm[idx % k];
        const double inv = d > 0 ? 1.0 / d : 1.0;
        out[idx] = make_double2(in[idx].x * inv, in[idx].y * inv);
    }
}

// a[idx] = b[idx] - a[idx]   (residual from a product)
__global__ void k_rsub(int64_t total, const cd *b, cd *a) {
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x)
        a[idx] = csub(b[idx], a[idx]);
}

__global__ void k_add(int64_t total, const cd *b, cd *a) {
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x)
        a[idx] = cadd(a[idx], b[idx]);
}

// Gather / scatter columns between the full batch (k columns) and the active set (ka columns).
__global__ void k_gather_cols(int64_t n, int k, int ka, const int *act, const cd *full, cd *compact) {
    const int64_t total = n * ka;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = idx / ka;
        const int c = (int)(idx % ka);
        compact[idx] = full[r * k + act[c]];
    }
}

__global__ void k_scatter_cols(int64_t n, int k, int ka, const int *act, const cd *compact, cd *full) {
    const int64_t total = n * ka;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = idx / ka;
        const int c = (int)(idx % ka);
        full[r * k + act[c]] = compact[idx];
    }
}

// Start of a cycle: H = 0, g = (beta, 0, ...), done = 0.
__global__ void k_cycle_start(int m, int k, const double *beta, cd *H, cd *g, int *done, int *last) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int hsize = (m + 1) * m * k;
    for (int i = idx; i < hsize; i += gridDim.x * blockDim.x) H[i] = make_double2(0, 0);
    for (int i = idx; i < (m + 1) * k; i += gridDim.x * blockDim.x)
        g[i] = i < k ? make_double2(beta[i], 0) : make_double2(0, 0);
    for (int i = idx; i < k; i += gridDim.x * blockDim.x) {
        done[i] = 0;
        last[i] = m - 1;
    }
}

// Store column j of H: H[i][j] = h1[i] + h2[i] (i <= j), H[j+1][j] = hn.
__global__ void k_store_column(int m, int k, int j, const cd *h1, const cd *h2, const double *hn, cd *H) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < (j + 1) * k) {
        const int i = idx / k, s = idx % k;
        H[((size_t)i * m + j) * k + s] = cadd(h1[idx], h2[idx]);
    }
    if (idx < k) H[((size_t)(j + 1) * m + j) * k + idx] = make_double2(hn[idx], 0);
}

// Givens least squares of step j for every column; convergence |g_{j+1}| / |b| <= tol.
__global__ void k_givens(int m, int k, int j, cd *H, cd *cs, cd *sn, cd *g, const double *bnorm, double tol,
                         int *done, int *last, int *its, int *ndone) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= k) return;
    auto at = [&](int i) -> cd & { return H[((size_t)i * m + j) * k + s]; };
    for (int i = 0; i < j; ++i) {
        const cd a = at(i), b = at(i + 1), c = cs[i * k + s], sv = sn[i * k + s];
        at(i) = cadd(cmulc(c, a), cmulc(sv, b));
        at(i + 1) = csub(cmul(c, b), cmul(sv, a));
    }
    const cd a = at(j), b = at(j + 1);
    double den = sqrt(a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y);
    if (!(den > 0)) den = 1;
    const cd c = make_double2(a.x / den, a.y / den), sv = make_double2(b.x / den, b.y / den);
    cs[j * k + s] = c;
    sn[j * k + s] = sv;
    at(j) = cadd(cmulc(c, a), cmulc(sv, b));
    at(j + 1) = make_double2(0, 0);
    const cd gj = g[j * k + s];
    const cd gn = cmul(sv, gj);
    g[(j + 1) * k + s] = make_double2(-gn.x, -gn.y);
    g[j * k + s] = cmulc(c, gj);
    const bool was = done[s] != 0;
    const double res = sqrt(gn.x * gn.x + gn.y * gn.y) / bnorm[s];
    const bool now = !was && res <= tol;
    if (now) {
        last[s] = j;
        done[s] = 1;
    }
    if (!was) its[s] += 1;
    if (done[s]) atomicAdd(ndone, 1);
}

// Back substitution per column: y = triu(H[:jj,:jj]) \ g[:jj], jj = last + 1 if done else jcur + 1.
__global__ void k_trisolve(int m, int k, int jcur, const cd *H, const cd *g, const int *done, const int *last,
                           cd *y) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= k) return;
    const int jj = done[s] ? last[s] + 1 : jcur + 1;
    for (int i = m - 1; i >= jj; --i) y[i * k + s] = make_double2(0, 0);
    for (int i = jj - 1; i >= 0; --i) {
        cd acc = g[i * k + s];
        for (int l = i + 1; l < jj; ++l) acc = csub(acc, cmul(H[((size_t)i * m + l) * k + s], y[l * k + s]));
        const cd d = H[((size_t)i * m + i) * k + s];
        const double dd = d.x * d.x + d.y * d.y;
        y[i * k + s] = dd > 0 ? make_double2((acc.x * d.x + acc.y * d.y) / dd, (acc.y * d.x - acc.x * d.y) / dd)
                              : make_double2(0, 0);
    }
}

// out[r,s] = sum_{i<jc} V_i[r,s] y[i][s]
__global__ void k_combine(int64_t n, int k, int jc, const cd *V, const cd *y, cd *out) {
    const int64_t total = n * k;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(idx % k);
        cd a = make_double2(0, 0);
        for (int i = 0; i < jc; ++i) a = cadd(a, cmul(V[(size_t)i * total + idx], y[i * k + s]));
        out[idx] = a;
    }
}

// ---- the captured cycle: the same steps with the step index in device memory ------------------------------------
// state[0] = j, the step about to run; state[1] = the cycle's step limit (set before each launch); state[2] = the
// last step run. A conditional WHILE node repeats the step body while k_step_end leaves its condition at 1.

__global__ void k_state_init(int *state) {
    state[0] = 0;
    state[2] = 0;
}

__global__ void k_copy_basis(int64_t n, int k, const cd *V, const int *state, cd *out) {
    const int64_t total = n * k;
    const cd *Vj = V + (size_t)state[0] * total;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x)
        out[idx] = Vj[idx];
}

// k_dots_partial with i < jc = j + 1 (grid NCHUNK x (m + 1): blocks past jc return), partials laid out with a fixed
// stride of m + 1 rows.
__global__ void __launch_bounds__(RT) k_dots_partial_d(int64_t n, int k, const cd *V, const cd *w, cd *partial,
                                                       const int *state) {
    __shared__ cd acc[RT];
    const int chunk = blockIdx.x, i = blockIdx.y;
    if (i > state[0]) return;
    const int64_t r0 = n * chunk / NCHUNK, r1 = n * (chunk + 1) / NCHUNK;
    const cd *Vi = V + (size_t)i * n * k;
    cd *out = partial + ((size_t)chunk * gridDim.y + i) * k;
    if (k <= RT) {
        const int per = RT / k, t = threadIdx.x;
        cd a = make_double2(0, 0);
        if (t < per * k) {
            const int s = t % k, rr = t / k;
            for (int64_t r = r0 + rr; r < r1; r += per) a = cadd(a, cmulc(Vi[r * k + s], w[r * k + s]));
        }
        acc[t] = a;
        __syncthreads();
        if (t < k) {
            cd sum = make_double2(0, 0);
            for (int q = 0; q < per; ++q) sum = cadd(sum, acc[t + q * k]);
            out[t] = sum;
        }
    } else {
        for (int s = threadIdx.x; s < k; s += RT) {
            cd a = make_double2(0, 0);
            for (int64_t r = r0; r < r1; ++r) a = cadd(a, cmulc(Vi[r * k + s], w[r * k + s]));
            out[s] = a;
        }
    }
}

__global__ void k_dots_final_d(int stride, int k, const cd *partial, cd *h, const int *state) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (state[0] + 1) * k) return;
    cd sum = make_double2(0, 0);
    for (int c = 0; c < NCHUNK; ++c) sum = cadd(sum, partial[(size_t)c * stride * k + idx]);
    h[idx] = sum;
}

__global__ void k_orth_update_d(int64_t n, int k, const cd *V, const cd *h, cd *w, const int *state) {
    const int jc = state[0] + 1;
    const int64_t total = n * k;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(idx % k);
        cd a = w[idx];
        for (int i = 0; i < jc; ++i) a = csub(a, cmul(V[(size_t)i * total + idx], h[i * k + s]));
        w[idx] = a;
    }
}

// V_{j+1} = w / |w|
__global__ void k_divide_next(int64_t n, int k, const cd *in, const double *norm, cd *V, const int *state) {
    const int64_t total = n * k;
    cd *out = V + (size_t)(state[0] + 1) * total;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const double d = norm[idx % k];
        const double inv = d > 0 ? 1.0 / d : 1.0;
        out[idx] = make_double2(in[idx].x * inv, in[idx].y * inv);
    }
}

__global__ void k_store_column_d(int m, int k, const cd *h1, const cd *h2, const double *hn, cd *H,
                                 const int *state) {
    const int j = state[0];
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < (j + 1) * k) {
        const int i = idx / k, s = idx % k;
        H[((size_t)i * m + j) * k + s] = cadd(h1[idx], h2[idx]);
    }
    if (idx < k) H[((size_t)(j + 1) * m + j) * k + idx] = make_double2(hn[idx], 0);
}

__global__ void k_givens_d(int m, int k, cd *H, cd *cs, cd *sn, cd *g, const double *bnorm, double tol, int *done,
                           int *last, int *its, int *ndone, const int *state) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= k) return;
    const int j = state[0];
    auto at = [&](int i) -> cd & { return H[((size_t)i * m + j) * k + s]; };
    for (int i = 0; i < j; ++i) {
        const cd a = at(i), b = at(i + 1), c = cs[i * k + s], sv = sn[i * k + s];
        at(i) = cadd(cmulc(c, a), cmulc(sv, b));
        at(i + 1) = csub(cmul(c, b), cmul(sv, a));
    }
    const cd a = at(j), b = at(j + 1);
    double den = sqrt(a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y);
    if (!(den > 0)) den = 1;
    const cd c = make_double2(a.x / den, a.y / den), sv = make_double2(b.x / den, b.y / den);
    cs[j * k + s] = c;
    sn[j * k + s] = sv;
    at(j) = cadd(cmulc(c, a), cmulc(sv, b));
    at(j + 1) = make_double2(0, 0);
    const cd gj = g[j * k + s];
    const cd gn = cmul(sv, gj);
    g[(j + 1) * k + s] = make_double2(-gn.x, -gn.y);
    g[j * k + s] = cmulc(c, gj);
    const bool was = done[s] != 0;
    const double res = sqrt(gn.x * gn.x + gn.y * gn.y) / bnorm[s];
    const bool now = !was && res <= tol;
    if (now) {
        last[s] = j;
        done[s] = 1;
    }
    if (!was) its[s] += 1;
    if (done[s]) atomicAdd(ndone, 1);
}

// End of a step: advance j and leave the WHILE condition at 1 while a column is active and steps remain.
__global__ void k_step_end(int *state, const int *ndone, int k, cudaGraphConditionalHandle handle) {
    if (threadIdx.x || blockIdx.x) return;
    const int j = state[0] + 1;
    state[0] = j;
    state[2] = j - 1;
    cudaGraphSetConditional(handle, (*ndone < k && j < state[1]) ? 1u : 0u);
}

__global__ void k_trisolve_d(int m, int k, const cd *H, const cd *g, const int *done, const int *last, cd *y,
                             const int *state) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= k) return;
    const int jcur = state[2];
    const int jj = done[s] ? last[s] + 1 : jcur + 1;
    for (int i = m - 1; i >= jj; --i) y[i * k + s] = make_double2(0, 0);
    for (int i = jj - 1; i >= 0; --i) {
        cd acc = g[i * k + s];
        for (int l = i + 1; l < jj; ++l) acc = csub(acc, cmul(H[((size_t)i * m + l) * k + s], y[l * k + s]));
        const cd d = H[((size_t)i * m + i) * k + s];
        const double dd = d.x * d.x + d.y * d.y;
        y[i * k + s] = dd > 0 ? make_double2((acc.x * d.x + acc.y * d.y) / dd, (acc.y * d.x - acc.x * d.y) / dd)
                              : make_double2(0, 0);
    }
}

__global__ void k_combine_d(int64_t n, int k, const cd *V, const cd *y, cd *out, const int *state) {
    const int jc = state[2] + 1;
    const int64_t total = n * k;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(idx % k);
        cd a = make_double2(0, 0);
        for (int i = 0; i < jc; ++i) a = cadd(a, cmul(V[(size_t)i * total + idx], y[i * k + s]));
        out[idx] = a;
    }
}

// ---------------------------------------------------------------------------------------------------------------

static int grid_for(int64_t total) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, (int64_t)sms * 16));
}

cudaError_t column_norms(int64_t n, int k, const cd *x, double *out, double *scratch, cudaStream_t s) {
    k_norm_partial<<<NCHUNK, RT, 0, s>>>(n, k, x, scratch);
    k_norm_final<<<(k + 127) / 128, 128, 0, s>>>(k, scratch, out);
    return cudaGetLastError();
}

__global__ void k_scatter_add_cols(int64_t n, int k, int ka, const int *act, const cd *compact, cd *full) {
    const int64_t total = n * ka;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = idx / ka;
        const int c = (int)(idx % ka);
        full[r * k + act[c]] = cadd(full[r * k + act[c]], compact[idx]);
    }
}

cudaError_t gather_columns(int64_t n, int k, int ka, const int *act, const cd *full, cd *compact, cudaStream_t s) {
    k_gather_cols<<<grid_for(n * ka), 256, 0, s>>>(n, k, ka, act, full, compact);
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t scatter_add_columns(int64_t n, int k, int ka, const int *act, const cd *compact, cd *full,
                                cudaStream_t s) {
    k_scatter_add_cols<<<grid_for(n * ka), 256, 0, s>>>(n, k, ka, act, compact, full);
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t subtract_from(int64_t count, const cd *b, cd *a, cudaStream_t s) {
    k_rsub<<<grid_for(count), 256, 0, s>>>(count, b, a);
    note_launches(1);
    return cudaGetLastError();
}


namespace {

// The captured restart cycle: its graph (rebuilt when the active set's size changes) and the buffers it runs on.
struct CycleGraph {
    int ka = -1;
    int kernels = 0;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t capture[2] = {nullptr, nullptr};
    ~CycleGraph() {
        if (exec) cudaGraphExecDestroy(exec);
        for (cudaStream_t s : capture)
            if (s) cudaStreamDestroy(s);
    }
};

struct CycleBuffers {
    int64_t n;
    int k, ka, m;
    double tol;
    cd *V, *r;
    double *norm;
    cd *H, *cs, *sn, *g, *y, *h1, *h2, *dpart;
    double *npart;
    cd *w, *z, *vj, *xc, *x;
    double *bnorm;
    int *done, *last, *its, *ndone, *act_dev, *sys_dev, *state;
};

int grid_of_total(int64_t total) { return (int)std::min<int64_t>(std::max<int64_t>((total + 255) / 256, 1), 4096); }

// Capture one restart cycle on its own streams: the start (V0 = r / |r|, the least-squares state), a conditional
// WHILE node whose body is one Arnoldi step read from and counted in device memory, and the update x += M^-1 V y
// with the active columns scattered back. Same kernels and order as the host-driven cycle, so the same result.
cudaError_t build_cycle_graph(Operator &A, Preconditioner *M, const CycleBuffers &b, CycleGraph &graph) {
    cudaError_t e;
    for (cudaStream_t &s : graph.capture)
        if (!s && (e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking))) return e;
    if (graph.exec) {
        cudaGraphExecDestroy(graph.exec);
        graph.exec = nullptr;
    }
    graph.ka = -1;
    cudaStream_t s0 = graph.capture[0], s1 = graph.capture[1];
    const int64_t n = b.n;
    const int ka = b.ka, m = b.m;
    const int gsz = grid_of_total(n * ka);
    int kernels = 0;
    auto precond = [&](const cd *in, cd *out, cudaStream_t s) -> cudaError_t {
        if (M) return M->apply_deferred(ka, b.sys_dev, in, out, s);
        return cudaMemcpyAsync(out, in, sizeof(cd) * n * ka, cudaMemcpyDeviceToDevice, s);
    };
    cudaGraph_t whole = nullptr;
    auto abandon = [&](cudaError_t err) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(s1, &g);
        if (g) cudaGraphDestroy(g);
        g = nullptr;
        cudaStreamEndCapture(s0, &g);
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return err;
    };
    if ((e = cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal))) return e;
    k_divide<<<gsz, 256, 0, s0>>>(n, ka, b.r, b.norm, b.V);
    k_cycle_start<<<grid_of_total((int64_t)(m + 1) * m * ka), 256, 0, s0>>>(m, ka, b.norm, b.H, b.g, b.done, b.last);
    if ((e = cudaMemsetAsync(b.its, 0, sizeof(int) * ka, s0))) return abandon(e);
    k_state_init<<<1, 1, 0, s0>>>(b.state);
    kernels += 3;
    cudaStreamCaptureStatus status;
    cudaGraph_t captured = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *edges = nullptr;
    size_t ndeps = 0;
    if ((e = cudaStreamGetCaptureInfo(s0, &status, nullptr, &captured, &deps, &edges, &ndeps))) return abandon(e);
    cudaGraphConditionalHandle handle;
    if ((e = cudaGraphConditionalHandleCreate(&handle, captured, 1, cudaGraphCondAssignDefault))) return abandon(e);
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t loop;
    if ((e = cudaGraphAddNode(&loop, captured, deps, edges, ndeps, &cp)) ||
        (e = cudaStreamUpdateCaptureDependencies(s0, &loop, nullptr, 1, cudaStreamSetCaptureDependencies)))
        return abandon(e);
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if ((e = cudaStreamBeginCaptureToGraph(s1, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)))
        return abandon(e);
    {
        // one Arnoldi step (the host-driven cycle's loop body)
        k_copy_basis<<<gsz, 256, 0, s1>>>(n, ka, b.V, b.state, b.vj);
        if ((e = precond(b.vj, b.z, s1)) || (e = A.apply(ka, b.sys_dev, b.z, b.w, s1))) return abandon(e);
        const dim3 dgrid(NCHUNK, m + 1);
        const int hgrid = ((m + 1) * ka + 127) / 128;
        for (cd *h : {b.h1, b.h2}) {
            k_dots_partial_d<<<dgrid, RT, 0, s1>>>(n, ka, b.V, b.w, b.dpart, b.state);
            k_dots_final_d<<<hgrid, 128, 0, s1>>>(m + 1, ka, b.dpart, h, b.state);
            k_orth_update_d<<<gsz, 256, 0, s1>>>(n, ka, b.V, h, b.w, b.state);
        }
        if ((e = column_norms(n, ka, b.w, b.norm, b.npart, s1))) return abandon(e);
        k_divide_next<<<gsz, 256, 0, s1>>>(n, ka, b.w, b.norm, b.V, b.state);
        k_store_column_d<<<hgrid, 128, 0, s1>>>(m, ka, b.h1, b.h2, b.norm, b.H, b.state);
        if ((e = cudaMemsetAsync(b.ndone, 0, sizeof(int), s1))) return abandon(e);
        k_givens_d<<<(ka + 127) / 128, 128, 0, s1>>>(m, ka, b.H, b.cs, b.sn, b.g, b.bnorm, b.tol, b.done, b.last,
                                                     b.its, b.ndone, b.state);
        k_step_end<<<1, 32, 0, s1>>>(b.state, b.ndone, ka, handle);
        kernels += 13;
    }
    if ((e = cudaStreamEndCapture(s1, &body))) return abandon(e);
    // x += M^-1 (V y), the active columns back into x
    k_trisolve_d<<<(ka + 127) / 128, 128, 0, s0>>>(m, ka, b.H, b.g, b.done, b.last, b.y, b.state);
    k_combine_d<<<gsz, 256, 0, s0>>>(n, ka, b.V, b.y, b.w, b.state);
    if ((e = precond(b.w, b.z, s0))) return abandon(e);
    k_add<<<gsz, 256, 0, s0>>>((int64_t)n * ka, b.z, b.xc);
    k_scatter_cols<<<gsz, 256, 0, s0>>>(n, b.k, ka, b.act_dev, b.xc, b.x);
    kernels += 4;
    if ((e = cudaStreamEndCapture(s0, &whole))) return abandon(e);
    e = cudaGraphInstantiate(&graph.exec, whole, 0);
    cudaGraphDestroy(whole);
    if (e) return e;
    graph.ka = ka;
    graph.kernels = kernels;
    return cudaGetLastError();
}

struct Scratch {
    cudaStream_t stream;
    std::vector<void *> blocks;
    cudaError_t err = cudaSuccess;
    explicit Scratch(cudaStream_t s) : stream(s) {}
    template <class T> T *get(size_t count) {
        T *p = nullptr;
        if (err == cudaSuccess) err = pool_alloc_n(&p, count, stream);
        if (err == cudaSuccess) blocks.push_back(p);
        return p;
    }
    ~Scratch() {
        for (void *p : blocks) pool_free(p, stream);
    }
};

}  // namespace

cudaError_t gmres_batched(Operator &A, Preconditioner *M, int k, const int32_t *sys_host, const cd *b, cd *x,
                          const GmresOptions &opt, GmresReport &report, cudaStream_t st) {
    const int64_t n = A.n();
    const int m = std::max(1, std::min(opt.restart, opt.maxiter));
    report.iterations.assign(k, 0);
    report.residual.assign(k, 0.0);
    report.cycles = 0;
    if (k <= 0 || n <= 0) return cudaSuccess;
    Scratch mem(st);
    const size_t nk = (size_t)n * k;
    cd *V = mem.get<cd>((size_t)(m + 1) * nk);
    cd *bc = mem.get<cd>(nk), *xc = mem.get<cd>(nk), *r = mem.get<cd>(nk), *w = mem.get<cd>(nk);
    cd *z = mem.get<cd>(nk);
    cd *H = mem.get<cd>((size_t)(m + 1) * m * k), *cs = mem.get<cd>((size_t)m * k), *sn = mem.get<cd>((size_t)m * k);
    cd *g = mem.get<cd>((size_t)(m + 1) * k), *y = mem.get<cd>((size_t)m * k);
    cd *h1 = mem.get<cd>((size_t)(m + 1) * k), *h2 = mem.get<cd>((size_t)(m + 1) * k);
    cd *dpart = mem.get<cd>((size_t)NCHUNK * (m + 1) * k);
    double *npart = mem.get<double>((size_t)NCHUNK * k), *norm = mem.get<double>(k), *bnorm_all = mem.get<double>(k);
    double *bnorm = mem.get<double>(k);
    int *done = mem.get<int>(k), *last = mem.get<int>(k), *its = mem.get<int>(k), *ndone = mem.get<int>(1);
    int *act_dev = mem.get<int>(k), *sys_dev = mem.get<int>(k);
    cd *vj = opt.captured ? mem.get<cd>(nk) : nullptr;           // the basis vector a captured step works on
    int *state = opt.captured ? mem.get<int>(4) : nullptr;       // the captured cycle's step counters
    if (mem.err != cudaSuccess) return mem.err;
    CycleGraph graph;
    int launches = 0;
    auto apply = [&](int ka, const cd *in, cd *out) { return A.apply(ka, sys_dev, in, out, st); };
    auto precond = [&](int ka, const cd *in, cd *out) -> cudaError_t {
        if (M) return M->apply(ka, sys_dev, in, out, st);
        return cudaMemcpyAsync(out, in, sizeof(cd) * n * ka, cudaMemcpyDeviceToDevice, st);
    };
    cudaError_t err;
    if ((err = column_norms(n, k, b, bnorm_all, npart, st))) return err;
    launches += 2;
    std::vector<double> bn(k), rn(k);
    cudaMemcpyAsync(bn.data(), bnorm_all, sizeof(double) * k, cudaMemcpyDeviceToHost, st);
    if ((err = cudaStreamSynchronize(st))) return err;
    std::vector<int> act(k), its_host(k, 0);
    for (int c = 0; c < k; ++c) act[c] = c;
    // Columns whose right-hand side vanishes are solved by x = 0.
    std::vector<int> keep;
    for (int c : act) {
        if (bn[c] > 0) keep.push_back(c);
        else report.residual[c] = 0.0;
    }
    act.swap(keep);
    std::vector<int> sys_act, its_act;
    bool first = true;
    while (!act.empty()) {
        const int ka = (int)act.size();
        sys_act.resize(ka);
        std::vector<double> bn_act(ka);
        for (int c = 0; c < ka; ++c) {
            sys_act[c] = sys_host[act[c]];
            bn_act[c] = bn[act[c]];
        }
        cudaMemcpyAsync(act_dev, act.data(), sizeof(int) * ka, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(sys_dev, sys_act.data(), sizeof(int) * ka, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(bnorm, bn_act.data(), sizeof(double) * ka, cudaMemcpyHostToDevice, st);
        const int gsz = grid_for((int64_t)n * ka);
        k_gather_cols<<<gsz, 256, 0, st>>>(n, k, ka, act_dev, b, bc);
        k_gather_cols<<<gsz, 256, 0, st>>>(n, k, ka, act_dev, x, xc);
        launches += 2;
        // r = b - A x
        if ((err = apply(ka, xc, r))) return err;
        k_rsub<<<gsz, 256, 0, st>>>((int64_t)n * ka, bc, r);
        if ((err = column_norms(n, ka, r, norm, npart, st))) return err;
        launches += 3;
        cudaMemcpyAsync(rn.data(), norm, sizeof(double) * ka, cudaMemcpyDeviceToHost, st);
        if ((err = cudaStreamSynchronize(st))) return err;
        if (!first) {
            // The true residual after the previous cycle decides which columns stay.
            std::vector<int> next;
            for (int c = 0; c < ka; ++c) {
                const double res = rn[c] / bn_act[c];
                report.residual[act[c]] = res;
                if (res > opt.tol && its_host[act[c]] < opt.maxiter) next.push_back(act[c]);
            }
            if (next.size() != act.size()) {
                act.swap(next);
                continue;      // re-gather the smaller active set
            }
        } else {
            std::vector<int> next;
            for (int c = 0; c < ka; ++c) {
                const double res = rn[c] / bn_act[c];
                report.residual[act[c]] = res;
                if (res > opt.tol) next.push_back(act[c]);
            }
            first = false;
            if (next.size() != act.size()) {
                act.swap(next);
                continue;
            }
        }
        int max_its = 0;
        for (int c : act) max_its = std::max(max_its, its_host[c]);
        const int steps = std::min(m, opt.maxiter - max_its);
        if (steps <= 0) break;
        ++report.cycles;
        if (opt.captured) {
            if (graph.ka != ka) {
                // one uncaptured application of each with ka columns first: work buffers, plans and the product
                // shapes' tuning are set up outside the capture
                if ((err = precond(ka, r, z)) || (err = apply(ka, z, w))) return err;
                CycleBuffers cb{n, k, ka, m, opt.tol, V, r, norm, H, cs, sn, g, y, h1, h2, dpart, npart, w, z, vj,
                                xc, x, bnorm, done, last, its, ndone, act_dev, sys_dev, state};
                if ((err = build_cycle_graph(A, M, cb, graph))) return err;
            }
            if ((err = cudaMemcpyAsync(state + 1, &steps, sizeof(int), cudaMemcpyHostToDevice, st)) ||
                (err = cudaGraphLaunch(graph.exec, st)))
                return err;
            if (M && (err = M->deferred_status(st))) return err;
            launches += graph.kernels;
            its_act.resize(ka);
            cudaMemcpyAsync(its_act.data(), its, sizeof(int) * ka, cudaMemcpyDeviceToHost, st);
            if ((err = cudaStreamSynchronize(st))) return err;
            for (int c = 0; c < ka; ++c) its_host[act[c]] += its_act[c];
            continue;
        }
        // V0 = r / |r|, g = (|r|, 0, ...)
        k_divide<<<gsz, 256, 0, st>>>(n, ka, r, norm, V);
        k_cycle_start<<<grid_for((int64_t)(m + 1) * m * ka), 256, 0, st>>>(m, ka, norm, H, g, done, last);
        cudaMemsetAsync(its, 0, sizeof(int) * ka, st);
        launches += 2;
        int jcur = 0;
        for (int j = 0; j < steps; ++j) {
            jcur = j;
            cd *Vj = V + (size_t)j * n * ka;
            if ((err = precond(ka, Vj, z))) return err;
            if ((err = apply(ka, z, w))) return err;
            const int jc = j + 1;
            dim3 dgrid(NCHUNK, jc);
            k_dots_partial<<<dgrid, RT, 0, st>>>(n, ka, V, w, dpart);
            k_dots_final<<<(jc * ka + 127) / 128, 128, 0, st>>>(jc, ka, dpart, h1);
            k_orth_update<<<gsz, 256, 0, st>>>(n, ka, jc, V, h1, w);
            k_dots_partial<<<dgrid, RT, 0, st>>>(n, ka, V, w, dpart);
            k_dots_final<<<(jc * ka + 127) / 128, 128, 0, st>>>(jc, ka, dpart, h2);
            k_orth_update<<<gsz, 256, 0, st>>>(n, ka, jc, V, h2, w);
            column_norms(n, ka, w, norm, npart, st);
            k_divide<<<gsz, 256, 0, st>>>(n, ka, w, norm, V + (size_t)(j + 1) * n * ka);
            k_store_column<<<((jc + 1) * ka + 127) / 128, 128, 0, st>>>(m, ka, j, h1, h2, norm, H);
            cudaMemsetAsync(ndone, 0, sizeof(int), st);
            k_givens<<<(ka + 127) / 128, 128, 0, st>>>(m, ka, j, H, cs, sn, g, bnorm, opt.tol, done, last, its,
                                                       ndone);
            launches += 10;
            int nd = 0;
            cudaMemcpyAsync(&nd, ndone, sizeof(int), cudaMemcpyDeviceToHost, st);
            if ((err = cudaStreamSynchronize(st))) return err;
            if (nd == ka) break;
        }
        // x += M^-1 (V y)
        k_trisolve<<<(ka + 127) / 128, 128, 0, st>>>(m, ka, jcur, H, g, done, last, y);
        k_combine<<<gsz, 256, 0, st>>>(n, ka, jcur + 1, V, y, w);
        if ((err = precond(ka, w, z))) return err;
        k_add<<<gsz, 256, 0, st>>>((int64_t)n * ka, z, xc);
        k_scatter_cols<<<gsz, 256, 0, st>>>(n, k, ka, act_dev, xc, x);
        launches += 4;
        its_act.resize(ka);
        cudaMemcpyAsync(its_act.data(), its, sizeof(int) * ka, cudaMemcpyDeviceToHost, st);
        if ((err = cudaStreamSynchronize(st))) return err;
        for (int c = 0; c < ka; ++c) its_host[act[c]] += its_act[c];
    }
    report.launches = launches;
    note_launches(launches);
    for (int c = 0; c < k; ++c) report.iterations[c] = its_host[c];
    return cudaGetLastError();
}

cudaError_t refine_batched(Operator &A, Operator &A32, Preconditioner *M, int k, const int32_t *sys_host,
                           const cd *b, cd *x, const RefineOptions &opt, GmresReport &report, int &outer_steps,
                           cudaStream_t st) {
    const int64_t n = A.n();
    report.iterations.assign(k, 0);
    report.residual.assign(k, 0.0);
    outer_steps = 0;
    if (k <= 0 || n <= 0) return cudaSuccess;
    Scratch mem(st);
    cd *r = mem.get<cd>((size_t)n * k), *rc = mem.get<cd>((size_t)n * k), *dc = mem.get<cd>((size_t)n * k);
    double *part = mem.get<double>((size_t)NCHUNK * k), *norm = mem.get<double>(k);
    int *act_dev = mem.get<int>(k), *sys_dev = mem.get<int>(k);
    if (mem.err != cudaSuccess) return mem.err;
    std::vector<int32_t> sys_all(sys_host, sys_host + k);
    cudaMemcpyAsync(sys_dev, sys_all.data(), sizeof(int) * k, cudaMemcpyHostToDevice, st);
    cudaError_t err;
    if ((err = column_norms(n, k, b, norm, part, st))) return err;
    note_launches(2);
    std::vector<double> bn(k), rn(k), xn(k);
    cudaMemcpyAsync(bn.data(), norm, sizeof(double) * k, cudaMemcpyDeviceToHost, st);
    if ((err = cudaStreamSynchronize(st))) return err;
    // a zero initial guess has residual b: the first FP64 product is skipped
    if ((err = column_norms(n, k, x, norm, part, st))) return err;
    note_launches(2);
    cudaMemcpyAsync(xn.data(), norm, sizeof(double) * k, cudaMemcpyDeviceToHost, st);
    if ((err = cudaStreamSynchronize(st))) return err;
    const bool zero_guess = std::all_of(xn.begin(), xn.end(), [](double v) { return v == 0.0; });
    for (int outer = 0; outer <= opt.max_outer; ++outer) {
        // the true residual of every column, with the FP64 operator
        cudaMemcpyAsync(sys_dev, sys_all.data(), sizeof(int) * k, cudaMemcpyHostToDevice, st);
        if (outer == 0 && zero_guess) {
            if ((err = cudaMemcpyAsync(r, b, sizeof(cd) * n * k, cudaMemcpyDeviceToDevice, st))) return err;
        } else {
            if ((err = A.apply(k, sys_dev, x, r, st))) return err;
            if ((err = subtract_from((int64_t)n * k, b, r, st))) return err;
        }
        if ((err = column_norms(n, k, r, norm, part, st))) return err;
        note_launches(2);
        cudaMemcpyAsync(rn.data(), norm, sizeof(double) * k, cudaMemcpyDeviceToHost, st);
        if ((err = cudaStreamSynchronize(st))) return err;
        std::vector<int> act;
        std::vector<int32_t> sys_act;
        for (int c = 0; c < k; ++c) {
            report.residual[c] = bn[c] > 0 ? rn[c] / bn[c] : 0.0;
            if (report.residual[c] > opt.tol) {
                act.push_back(c);
                sys_act.push_back(sys_all[c]);
            }
        }
        if (act.empty() || outer == opt.max_outer) break;
        ++outer_steps;
        const int ka = (int)act.size();
        cudaMemcpyAsync(act_dev, act.data(), sizeof(int) * ka, cudaMemcpyHostToDevice, st);
        if ((err = gather_columns(n, k, ka, act_dev, r, rc, st))) return err;
        cudaMemsetAsync(dc, 0, sizeof(cd) * n * ka, st);
        GmresOptions inner;
        inner.tol = opt.inner_tol;
        inner.maxiter = opt.inner_maxiter;
        inner.restart = opt.restart;
        inner.captured = opt.captured;
        GmresReport rep;
        if ((err = gmres_batched(A32, M, ka, sys_act.data(), rc, dc, inner, rep, st))) return err;
        for (int c = 0; c < ka; ++c) report.iterations[act[c]] += rep.iterations[c];
        cudaMemcpyAsync(act_dev, act.data(), sizeof(int) * ka, cudaMemcpyHostToDevice, st);
        if ((err = scatter_add_columns(n, k, ka, act_dev, dc, x, st))) return err;
    }
    return cudaGetLastError();
}

}  // namespace pq
