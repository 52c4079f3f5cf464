// Triangular solves with the complex64 LU factor of the loop/tree system (trsolve.cuh).
//
// cuSOLVER's getrf leaves M = A^T = P L U column-major; read row-major, row r of that array holds row r of U^T
// (entries 0..r) and row r of L^T (entries r+1..n-1), both contiguous. Solving A x = b = U^T L^T P^T x is a forward
// sweep with U^T, a backward sweep with L^T and a gather. Each sweep walks super-blocks of TRI_BLOCK rows: the
// block's rows left (forward) or right (backward) of its diagonal block are streamed against the solved part of the
// vector, every thread block taking a run of columns of 4 rows (deterministic partial sums, no atomics), then the
// precomputed inverse of the diagonal block is applied. Both sweeps run in one persistent cooperative kernel whose
// thread blocks meet at a grid barrier between the phases (bounded waits: a barrier that does not complete within
// about a second sets a status and every block returns), so the dependency chain of 2 x n / TRI_BLOCK steps costs
// a barrier each rather than a kernel launch. The factor is read once per sweep, 8 right-hand sides at a time.
#include <algorithm>
#include <string>
#include <vector>

#include "common.cuh"
#include "pool.cuh"
#include "tcgemm.cuh"
#include "trsolve.cuh"
#include "tune.cuh"

namespace pq {

namespace {

constexpr int B = TRI_BLOCK;
constexpr int KC = TRI_COLS;
constexpr int PANEL_ROWS = 4;                 // rows per thread block of the panel kernel
constexpr int PANEL_THREADS = 256;
constexpr int MAX_SPLITS = 16;                // column runs per panel row group
constexpr int PANEL_UNROLL = 4;               // columns per thread with loads in flight together
constexpr int SYNC_STRIDE = 32;               // counters 128 B apart: pollers of one do not slow updates of another

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ float2 cdiv(float2 a, float2 b) {
    const float d = b.x * b.x + b.y * b.y;
    return make_float2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

// Inverse of the lower-triangular diagonal block J of U^T: D[a][b] = lu[(J B + a) n + J B + b], b <= a. Thread c
// solves D X[:, c] = e_c down the rows (its own column only, no synchronization), X in shared memory.
__global__ void k_tri_invert_lower(const float2 *lu, int64_t n, float2 *inv) {
    extern __shared__ float2 X[];             // B x B
    const int J = blockIdx.x, c = threadIdx.x;
    const int64_t base = (int64_t)J * B;
    const int m = n - base < B ? (int)(n - base) : B;
    for (int a = 0; a < B; ++a) {
        float2 v = make_float2(0.f, 0.f);
        if (a < m && c < m && c <= a) {
            const float2 *row = lu + (base + a) * n + base;
            float2 s = make_float2(a == c ? 1.f : 0.f, 0.f);
            for (int b = c; b < a; ++b) {
                const float2 t = cmul(__ldg(row + b), X[b * B + c]);
                s.x -= t.x;
                s.y -= t.y;
            }
            v = cdiv(s, __ldg(row + a));
        }
        X[a * B + c] = v;
    }
    float2 *out = inv + (int64_t)J * B * B;
    for (int a = 0; a < B; ++a) out[a * B + c] = X[a * B + c];
}

// Inverse of the unit upper-triangular diagonal block J of L^T: E[a][b] = lu[(J B + a) n + J B + b], b > a.
__global__ void k_tri_invert_upper(const float2 *lu, int64_t n, float2 *inv) {
    extern __shared__ float2 X[];
    const int J = blockIdx.x, c = threadIdx.x;
    const int64_t base = (int64_t)J * B;
    const int m = n - base < B ? (int)(n - base) : B;
    for (int a = B - 1; a >= 0; --a) {
        float2 v = make_float2(0.f, 0.f);
        if (a < m && c < m && a <= c) {
            const float2 *row = lu + (base + a) * n + base;
            float2 s = make_float2(a == c ? 1.f : 0.f, 0.f);
            for (int b = a + 1; b <= c; ++b) {
                const float2 t = cmul(__ldg(row + b), X[b * B + c]);
                s.x -= t.x;
                s.y -= t.y;
            }
            v = s;
        }
        X[a * B + c] = v;
    }
    float2 *out = inv + (int64_t)J * B * B;
    for (int a = 0; a < B; ++a) out[a * B + c] = X[a * B + c];
}

// slot[r][c] = sum over columns i in [i0, i1) of lu[(row0 + r) n + i] x[i][c0 + c], for the 4 rows r of row group
// rg (r < m). Each thread keeps 4 x KC complex sums, so every 8 B of the factor it
// streams meets 8 complex multiply-adds and a vector entry is loaded once for 4 rows; PANEL_UNROLL columns per
// thread have their loads in flight together. x is written during the kernel, so it is read through L2 (ld.cg).
__device__ __forceinline__ void panel_block(const float2 *__restrict__ lu, int64_t n, int64_t row0, int m,
                                            int64_t i0, int64_t i1, const float2 *x, int kpad, int c0, float2 *slot,
                                            int rg) {
    float acc[PANEL_ROWS][KC][2];
#pragma unroll
    for (int r = 0; r < PANEL_ROWS; ++r)
#pragma unroll
        for (int c = 0; c < KC; ++c) acc[r][c][0] = acc[r][c][1] = 0.f;
    const float2 *rows[PANEL_ROWS];
    bool valid[PANEL_ROWS];
#pragma unroll
    for (int r = 0; r < PANEL_ROWS; ++r) {
        const int rr = rg * PANEL_ROWS + r;
        valid[r] = rr < m;
        rows[r] = lu + (row0 + (valid[r] ? rr : 0)) * n;
    }
    for (int64_t base = i0 + threadIdx.x; base < i1; base += (int64_t)PANEL_THREADS * PANEL_UNROLL) {
        float2 xv[PANEL_UNROLL][KC];
        float2 t[PANEL_UNROLL][PANEL_ROWS];
#pragma unroll
        for (int u = 0; u < PANEL_UNROLL; ++u) {
            const int64_t i = base + (int64_t)u * PANEL_THREADS;
            const bool in = i < i1;
            const float4 *xp = reinterpret_cast<const float4 *>(x + (in ? i : i0) * kpad + c0);
#pragma unroll
            for (int q = 0; q < KC / 2; ++q) {
                const float4 v = in ? __ldcg(xp + q) : make_float4(0.f, 0.f, 0.f, 0.f);
                xv[u][2 * q] = make_float2(v.x, v.y);
                xv[u][2 * q + 1] = make_float2(v.z, v.w);
            }
#pragma unroll
            for (int r = 0; r < PANEL_ROWS; ++r)
                t[u][r] = (in && valid[r]) ? __ldg(rows[r] + i) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < PANEL_UNROLL; ++u)
#pragma unroll
            for (int r = 0; r < PANEL_ROWS; ++r)
#pragma unroll
                for (int c = 0; c < KC; ++c) {
                    acc[r][c][0] += t[u][r].x * xv[u][c].x - t[u][r].y * xv[u][c].y;
                    acc[r][c][1] += t[u][r].x * xv[u][c].y + t[u][r].y * xv[u][c].x;
                }
    }
    __shared__ float red[PANEL_THREADS / 32][PANEL_ROWS * KC * 2];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int r = 0; r < PANEL_ROWS; ++r)
#pragma unroll
        for (int c = 0; c < KC; ++c)
#pragma unroll
            for (int p = 0; p < 2; ++p) {
                float v = acc[r][c][p];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
                if (lane == 0) red[warp][(r * KC + c) * 2 + p] = v;
            }
    __syncthreads();
    if (threadIdx.x < PANEL_ROWS * KC * 2) {
        float v = 0.f;
#pragma unroll
        for (int w = 0; w < PANEL_THREADS / 32; ++w) v += red[w][threadIdx.x];
        const int r = threadIdx.x / (KC * 2), c = (threadIdx.x / 2) % KC, p = threadIdx.x & 1;
        const int rr = rg * PANEL_ROWS + r;
        if (rr < m) reinterpret_cast<float *>(slot)[((int64_t)rr * KC + c) * 2 + p] = v;
    }
    __syncthreads();
}

// The diagonal step for rows a of quarter q (32 rows; 256 threads = 32 rows x 8 columns):
// x[row0 + a][c0 + c] = sum_b inv[a][b] (rhs[row0 + b][c0 + c] - sum_s partial[s][b][c]).
// diag_stage loads the quarter's 32 rows of the inverse and the block's right-hand side into shared memory (while
// the panel work of the same step is still running elsewhere: neither depends on it); diag_finish subtracts the
// panel sums once they are complete and applies the inverse. All loads are issued before they are used.
struct DiagSmem {
    float2 acc[B][KC];
    float2 rows[32][B + 1];
};

__device__ __forceinline__ void diag_stage(DiagSmem &sm, const float2 *__restrict__ inv, const float2 *rhs,
                                           int64_t row0, int m, int kpad, int c0, int q) {
    constexpr int ROW_LOADS = 32 * B / PANEL_THREADS, RHS_LOADS = B * KC / PANEL_THREADS;
    float2 v[ROW_LOADS];
#pragma unroll
    for (int it = 0; it < ROW_LOADS; ++it) {
        const int t = threadIdx.x + it * PANEL_THREADS, a = t / B, b = t % B;
        v[it] = (32 * q + a < m && b < m) ? __ldg(inv + (int64_t)(32 * q + a) * B + b) : make_float2(0.f, 0.f);
    }
    float2 r[RHS_LOADS];
#pragma unroll
    for (int it = 0; it < RHS_LOADS; ++it) {
        const int t = threadIdx.x + it * PANEL_THREADS, b = t / KC, c = t % KC;
        r[it] = b < m ? __ldcg(rhs + (row0 + b) * kpad + c0 + c) : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int it = 0; it < ROW_LOADS; ++it) {
        const int t = threadIdx.x + it * PANEL_THREADS;
        sm.rows[t / B][t % B] = v[it];
    }
#pragma unroll
    for (int it = 0; it < RHS_LOADS; ++it) {
        const int t = threadIdx.x + it * PANEL_THREADS;
        sm.acc[t / KC][t % KC] = r[it];
    }
}

__device__ __forceinline__ void diag_finish(DiagSmem &sm, const float2 *partial, int runs, float2 *x, int64_t row0,
                                            int m, int kpad, int c0, int q) {
    constexpr int RHS_LOADS = B * KC / PANEL_THREADS;
    if (runs > 0) {
        float2 sum[RHS_LOADS];
#pragma unroll
        for (int it = 0; it < RHS_LOADS; ++it) sum[it] = make_float2(0.f, 0.f);
        for (int s = 0; s < runs; ++s) {
            float2 p[RHS_LOADS];
#pragma unroll
            for (int it = 0; it < RHS_LOADS; ++it) {
                const int t = threadIdx.x + it * PANEL_THREADS, b = t / KC, c = t % KC;
                p[it] = b < m ? __ldcg(partial + ((int64_t)s * B + b) * KC + c) : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int it = 0; it < RHS_LOADS; ++it) {
                sum[it].x += p[it].x;
                sum[it].y += p[it].y;
            }
        }
#pragma unroll
        for (int it = 0; it < RHS_LOADS; ++it) {
            const int t = threadIdx.x + it * PANEL_THREADS;
            sm.acc[t / KC][t % KC].x -= sum[it].x;
            sm.acc[t / KC][t % KC].y -= sum[it].y;
        }
    }
    __syncthreads();
    const int al = threadIdx.x / KC, c = threadIdx.x % KC, a = 32 * q + al;
    if (a < m) {
        float re = 0.f, im = 0.f;
#pragma unroll 8
        for (int b = 0; b < B; ++b) {
            const float2 t = sm.rows[al][b], v = sm.acc[b][c];
            re += t.x * v.x - t.y * v.y;
            im += t.x * v.y + t.y * v.x;
        }
        x[(row0 + a) * kpad + c0 + c] = make_float2(re, im);
    }
    __syncthreads();
}

// All thread blocks of the (cooperative, co-resident) grid meet here: one arrival counter that only grows, barrier
// number `index` complete when it reaches (index + 1) x blocks; thread 0 arrives with release semantics (covering its
// block's writes through the preceding __syncthreads) and polls with acquire loads. Bounded: after about a second
// of polling (clock64; the library's wait limit) the block records TRI_TIMEOUT in *status and returns false, as do
// blocks that see the status.
constexpr int TRI_TIMEOUT = 1;

__device__ __forceinline__ unsigned load_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ bool grid_barrier(unsigned *count, unsigned index, int *status, long long limit) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        __threadfence();
        atomicAdd(count, 1u);
        const unsigned target = (index + 1) * gridDim.x;
        const long long start = clock64();
        while (load_acquire(count) < target) {
            if (clock64() - start > limit || *(volatile int *)status) {
                atomicExch(status, TRI_TIMEOUT);
                ok = 0;
                break;
            }
        }
    }
    __syncthreads();
    return ok;
}

struct SweepArgs {
    const float2 *lu;
    int64_t n;
    int nblk;
    const float2 *inv_lower, *inv_upper;
    const float2 *b;
    float2 *y, *z;
    int kpad, c0;
    float2 *partial;       // [2][MAX_SPLITS + 1][B][KC]: the panel sums of two consecutive steps
    unsigned *barrier;     // grid barrier arrivals
    unsigned *xready;      // per sweep (stride SYNC_STRIDE): diagonal quarters finished (4 per step)
    unsigned *pdone;       // per sweep and step (stride SYNC_STRIDE): panel items finished
    int *status;
    long long wait;        // limit (SM clocks) of each bounded wait
};

// Bounded wait until *counter >= target (thread 0 polls with acquire loads; the block then proceeds together).
__device__ __forceinline__ bool wait_for(const unsigned *counter, unsigned target, int *status, long long limit) {
    __shared__ int ok;
    if (threadIdx.x == 0) {
        ok = 1;
        const long long start = clock64();
        while (load_acquire(counter) < target) {
            if (clock64() - start > limit || *(volatile int *)status) {
                atomicExch(status, TRI_TIMEOUT);
                ok = 0;
                break;
            }
            __nanosleep(32);       // fewer polls on the counter's cache line while its producers update it
        }
    }
    __syncthreads();
    return ok;
}

// Release this block's writes, then count one more on *counter.
__device__ __forceinline__ void signal(unsigned *counter) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(counter, 1u);
    }
}

// The columns of one step's panel in two parts: the tail (the block solved just before, needed last) and the bulk
// (everything solved earlier, split into runs). Forward step s (block J = s): tail [(s-1)B, sB), bulk [0, (s-1)B);
// backward (block J = nblk-1-s): tail [(J+1)B, (J+2)B), bulk [(J+2)B, n).
struct StepCols {
    int64_t tail0, tail1, bulk0, bulk1;
    int bulk_runs;
};

__device__ __forceinline__ StepCols step_cols(int dir, int step, int nblk, int64_t n, int bulk_workers) {
    StepCols c{0, 0, 0, 0, 0};
    const int groups = (B + PANEL_ROWS - 1) / PANEL_ROWS;
    if (dir == 0) {
        if (step >= 1) { c.tail0 = (int64_t)(step - 1) * B; c.tail1 = (int64_t)step * B; }
        if (step >= 2) { c.bulk0 = 0; c.bulk1 = (int64_t)(step - 1) * B; }
    } else {
        const int J = nblk - 1 - step;
        if (J + 1 < nblk) { c.tail0 = (int64_t)(J + 1) * B; c.tail1 = (int64_t)(J + 2) * B < n ? (int64_t)(J + 2) * B : n; }
        if (J + 2 < nblk) { c.bulk0 = (int64_t)(J + 2) * B; c.bulk1 = n; }
    }
    const int64_t len = c.bulk1 - c.bulk0;
    if (len > 0) {
        int runs = bulk_workers / groups;
        runs = runs < 1 ? 1 : (runs > MAX_SPLITS ? MAX_SPLITS : runs);
        const int64_t by_len = len / 512;
        if (by_len < runs) runs = by_len < 1 ? 1 : (int)by_len;
        c.bulk_runs = runs;
    }
    return c;
}

// Forward sweep b -> y with U^T, then backward sweep y -> z with L^T, for columns c0 .. c0 + 7, with one step of
// lookahead: while the DIAG_BLOCKS diagonal blocks finish step s, BULK workers already stream step s + 1's bulk
// (it only needs blocks solved before s), and TAIL workers wait for block s and add its columns. The diagonal step
// waits for its panel items through a per-step counter and publishes its block through a per-sweep counter, so the
// dependency chain per step is a short tail product and two flag hand-offs instead of two grid barriers.
constexpr int DIAG_BLOCKS = B / 32;
constexpr int TAIL_BLOCKS = (B + PANEL_ROWS - 1) / PANEL_ROWS;     // one per row group of the tail

__global__ void __launch_bounds__(PANEL_THREADS, 1) k_tri_sweeps(SweepArgs a) {
    __shared__ DiagSmem dsm;
    const int role_id = (int)blockIdx.x;
    const bool diag = role_id < DIAG_BLOCKS;
    const bool tail = !diag && role_id < DIAG_BLOCKS + TAIL_BLOCKS;
    const int bulk_workers = (int)gridDim.x - DIAG_BLOCKS - TAIL_BLOCKS;
    const int me = role_id - DIAG_BLOCKS - TAIL_BLOCKS;
    const size_t buf = (size_t)(MAX_SPLITS + 1) * B * KC;
    for (int dir = 0; dir < 2; ++dir) {
        if (dir == 1 && !grid_barrier(a.barrier, 0, a.status, a.wait)) return;      // the backward sweep needs all of y
        const float2 *inv = dir == 0 ? a.inv_lower : a.inv_upper;
        const float2 *rhs = dir == 0 ? a.b : a.y;
        float2 *x = dir == 0 ? a.y : a.z;
        unsigned *xready = a.xready + dir * SYNC_STRIDE, *pdone = a.pdone + (size_t)dir * a.nblk * SYNC_STRIDE;
        // bulk workers start with step 1's bulk (empty) and run one step ahead of the diagonal
        for (int step = 0; step < a.nblk; ++step) {
            const int J = dir == 0 ? step : a.nblk - 1 - step;
            const int64_t row0 = (int64_t)J * B;
            const int m = a.n - row0 < B ? (int)(a.n - row0) : B;
            const StepCols sc = step_cols(dir, step, a.nblk, a.n, bulk_workers);
            float2 *slots = a.partial + (size_t)(step & 1) * buf;
            const int tail_runs = sc.tail1 > sc.tail0 ? 1 : 0;
            if (diag) {
                diag_stage(dsm, inv + (int64_t)J * B * B, rhs, row0, m, a.kpad, a.c0, role_id);
                const unsigned need = (unsigned)(tail_runs * TAIL_BLOCKS + sc.bulk_runs * ((m + PANEL_ROWS - 1) / PANEL_ROWS));
                if (need && !wait_for(pdone + (size_t)step * SYNC_STRIDE, need, a.status, a.wait)) return;
                diag_finish(dsm, slots, tail_runs + sc.bulk_runs, x, row0, m, a.kpad, a.c0, role_id);
                signal(xready);
            } else if (tail) {
                if (tail_runs) {
                    // block `step - 1` of this sweep must be solved: DIAG_BLOCKS quarters per step
                    if (!wait_for(xready, (unsigned)(DIAG_BLOCKS * step), a.status, a.wait)) return;
                    panel_block(a.lu, a.n, row0, m, sc.tail0, sc.tail1, x, a.kpad, a.c0,
                                slots + (size_t)sc.bulk_runs * B * KC, role_id - DIAG_BLOCKS);
                    signal(pdone + (size_t)step * SYNC_STRIDE);
                }
            } else if (step + 1 < a.nblk) {
                // the next step's bulk needs the blocks solved up to this step's predecessor
                const StepCols nx = step_cols(dir, step + 1, a.nblk, a.n, bulk_workers);
                if (nx.bulk_runs) {
                    const int Jn = dir == 0 ? step + 1 : a.nblk - 2 - step;
                    const int64_t rown = (int64_t)Jn * B;
                    const int mn = a.n - rown < B ? (int)(a.n - rown) : B;
                    const int mg = (mn + PANEL_ROWS - 1) / PANEL_ROWS;
                    float2 *nslots = a.partial + (size_t)((step + 1) & 1) * buf;
                    bool waited = false;
                    for (int item = me; item < mg * nx.bulk_runs; item += bulk_workers) {
                        if (!waited) {
                            if (step > 0 && !wait_for(xready, (unsigned)(DIAG_BLOCKS * step), a.status, a.wait)) return;
                            waited = true;
                        }
                        const int s = item / mg;
                        const int64_t len = nx.bulk1 - nx.bulk0;
                        panel_block(a.lu, a.n, rown, mn, nx.bulk0 + len * s / nx.bulk_runs,
                                    nx.bulk0 + len * (s + 1) / nx.bulk_runs, x, a.kpad, a.c0,
                                    nslots + (size_t)s * B * KC, item % mg);
                        signal(pdone + (size_t)(step + 1) * SYNC_STRIDE);
                    }
                }
            }
        }
    }
}

__global__ void k_tri_in(int64_t n, int k, int kpad, const cd *in, float2 *b) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * kpad;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / kpad;
        const int c = (int)(t % kpad);
        const cd v = c < k ? in[i * k + c] : make_double2(0.0, 0.0);
        b[t] = make_float2((float)v.x, (float)v.y);
    }
}

__global__ void k_tri_out(int64_t n, int k, int kpad, const float2 *z, const int32_t *gather, cd *out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * k; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = t / k;
        const int c = (int)(t % k);
        const float2 v = z[(int64_t)gather[j] * kpad + c];
        out[t] = make_double2(v.x, v.y);
    }
}

// barrier, two solved-quarter counters and the status word, then one panel counter per sweep and step
size_t sync_words(int nblk) { return (size_t)(4 + 2 * nblk) * SYNC_STRIDE; }

unsigned blocks_for(int64_t work) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((work + 255) / 256, 152 * 8));
}

}  // namespace

cudaError_t TriSolver::prepare(const float2 *lu_, int64_t n_, const int *ipiv, cudaStream_t s) {
    release();
    lu = lu_;
    n = n_;
    nblk = (int)((n + B - 1) / B);
    const size_t blocks = (size_t)nblk * B * B;
    cudaError_t e;
    if ((e = pool_alloc_n(&inv_lower, blocks, s)) || (e = pool_alloc_n(&inv_upper, blocks, s)) ||
        (e = pool_alloc_n(&gather, (size_t)n, s)))
        return e;
    const int smem = B * B * (int)sizeof(float2);
    if ((e = cudaFuncSetAttribute(k_tri_invert_lower, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) ||
        (e = cudaFuncSetAttribute(k_tri_invert_upper, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)))
        return e;
    k_tri_invert_lower<<<nblk, B, smem, s>>>(lu, n, inv_lower);
    k_tri_invert_upper<<<nblk, B, smem, s>>>(lu, n, inv_upper);
    note_launches(2);
    // the row interchanges (applied last to first) as one gather
    std::vector<int> piv((size_t)n);
    if ((e = cudaMemcpyAsync(piv.data(), ipiv, sizeof(int) * n, cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
        return e;
    std::vector<int32_t> idx((size_t)n);
    for (int64_t i = 0; i < n; ++i) idx[i] = (int32_t)i;
    for (int64_t i = n - 1; i >= 0; --i) {
        const int64_t p = (int64_t)piv[i] - 1;
        if (p < 0 || p >= n) return cudaErrorInvalidValue;
        std::swap(idx[i], idx[p]);
    }
    if ((e = cudaMemcpyAsync(gather, idx.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s)) ||
        (e = cudaStreamSynchronize(s)))
        return e;
    return cudaGetLastError();
}

cudaError_t TriSolver::plan_for(int k, Plan **out) {
    auto it = plans.find(k);
    if (it != plans.end()) {
        *out = &it->second;
        return cudaSuccess;
    }
    Plan p;
    p.kpad = (k + KC - 1) / KC * KC;
    const size_t vec = (size_t)n * p.kpad;
    cudaError_t e;
    if ((e = pool_alloc_n(&p.b, vec, nullptr)) || (e = pool_alloc_n(&p.y, vec, nullptr)) ||
        (e = pool_alloc_n(&p.z, vec, nullptr)) ||
        (e = pool_alloc_n(&p.partial, 2 * (size_t)(MAX_SPLITS + 1) * B * KC, nullptr)) ||
        (e = pool_alloc_n(&p.sync, sync_words(nblk), nullptr)) ||
        (e = cudaMemsetAsync(p.sync, 0, sync_words(nblk) * sizeof(unsigned), nullptr)) ||    // status words start at 0
        (e = cudaStreamSynchronize(nullptr))) {
        for (float2 *q : {p.b, p.y, p.z, p.partial}) pool_free(q, nullptr);
        pool_free(p.sync, nullptr);
        return e;
    }
    auto res = plans.emplace(k, p);
    *out = &res.first->second;
    return cudaSuccess;
}

cudaError_t TriSolver::solve(int k, const cd *in, cd *out, cudaStream_t s, bool deferred) {
    if (!lu || k <= 0) return cudaErrorInvalidValue;
    Plan *p = nullptr;
    cudaError_t e = plan_for(k, &p);
    if (e) return e;
    if (force == 0 || force == 1) {            // a method asked for (validation): not timed, not remembered
        if (force == 0) return solve_streaming(p, k, in, out, s, deferred);
        if ((e = solve_blocked(p, k, in, out, s))) return e;
        return deferred ? cudaGetLastError() : read_status(k, s);
    }
    if (p->method < 0 && p->kpad < 4 * KC) p->method = 0;      // a few columns: the streaming sweeps
    // column counts in one power-of-two bucket share the timing (a GMRES active set shrinks through many counts)
    int bucket = 4 * KC;
    while (bucket < p->kpad) bucket *= 2;
    const std::string key = "trisolve n=" + std::to_string(n) + " columns=" + std::to_string(bucket);
    if (p->method < 0) {
        auto it = method_by_bucket.find(bucket);
        if (it != method_by_bucket.end()) {
            p->method = it->second;
        } else {
            const int known = tune_get(key);        // timed by an earlier factor of this size (or process)
            if (known == 0 || known == 1) p->method = method_by_bucket[bucket] = known;
        }
    }
    if (p->method < 0 && !deferred) {
        // the first call with this many columns: the blocked solve once to set it up, then each method timed once;
        // the faster is kept (its result is the one left in `out`)
        if ((e = solve_blocked(p, k, in, out, s)) || (e = cudaStreamSynchronize(s))) return e;
        cudaEvent_t ev[3];
        for (cudaEvent_t &x : ev)
            if ((e = cudaEventCreate(&x))) return e;
        float streaming = 0, blocked = 0;
        if (!(e = cudaEventRecord(ev[0], s)) && !(e = solve_streaming(p, k, in, out, s, false)) &&
            !(e = cudaEventRecord(ev[1], s)) && !(e = solve_blocked(p, k, in, out, s)) &&
            !(e = cudaEventRecord(ev[2], s)) && !(e = cudaEventSynchronize(ev[2])) &&
            !(e = cudaEventElapsedTime(&streaming, ev[0], ev[1])))
            e = cudaEventElapsedTime(&blocked, ev[1], ev[2]);
        for (cudaEvent_t x : ev) cudaEventDestroy(x);
        if (e) return e;
        p->method = blocked < streaming ? 1 : 0;
        method_by_bucket[bucket] = p->method;
        tune_put(key, p->method);
        return read_status(k, s);
    }
    if (p->method == 1) {
        if ((e = solve_blocked(p, k, in, out, s))) return e;
        return deferred ? cudaGetLastError() : read_status(k, s);
    }
    return solve_streaming(p, k, in, out, s, deferred);
}

int TriSolver::method_for(int k) const {
    auto it = plans.find(k);
    return it == plans.end() ? -1 : it->second.method;
}

// C (R x Cn) = A X (mode 0) or C -= A X (mode 1) for row-major complex64 A (R x Kd, leading dimension lda), X
// (Kd x Cn) and C: the blocked solve's steps inside a diagonal block. 32 x 32 outputs per CTA (each thread one
// column of four rows), K in tiles of 32 staged in shared memory, each tile's partial sums added to the running
// sums (rounding errors grow with the tile count rather than the whole inner dimension).
__global__ void __launch_bounds__(256) k_cgemm_small(int R, int Cn, int Kd, const float2 *A, int64_t lda,
                                                     const float2 *X, int64_t ldx, float2 *C, int64_t ldc, int mode) {
    __shared__ float2 As[32][33], Xs[32][33];
    const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    float2 acc[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) acc[i] = make_float2(0.f, 0.f);
    for (int k0 = 0; k0 < Kd; k0 += 32) {
        for (int i = ty; i < 32; i += 8) {
            As[i][tx] = (r0 + i < R && k0 + tx < Kd) ? A[(int64_t)(r0 + i) * lda + k0 + tx] : make_float2(0.f, 0.f);
            Xs[i][tx] = (k0 + i < Kd && c0 + tx < Cn) ? X[(int64_t)(k0 + i) * ldx + c0 + tx] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        float2 part[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) part[i] = make_float2(0.f, 0.f);
#pragma unroll 8
        for (int j = 0; j < 32; ++j) {
            const float2 v = Xs[j][tx];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float2 a = As[ty + 8 * i][j];
                part[i].x += a.x * v.x - a.y * v.y;
                part[i].y += a.x * v.y + a.y * v.x;
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            acc[i].x += part[i].x;
            acc[i].y += part[i].y;
        }
        __syncthreads();
    }
    const int c = c0 + tx;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = r0 + ty + 8 * i;
        if (r < R && c < Cn) {
            float2 *p = C + (int64_t)r * ldc + c;
            if (mode == 0) {
                *p = acc[i];
            } else {
                float2 v = *p;
                v.x -= acc[i].x;
                v.y -= acc[i].y;
                *p = v;
            }
        }
    }
}

static void launch_cgemm_small(int R, int Cn, int Kd, const float2 *A, int64_t lda, const float2 *X, int64_t ldx,
                               float2 *C, int64_t ldc, int mode, cudaStream_t s) {
    if (R <= 0 || Cn <= 0) return;
    const dim3 grid((unsigned)((Cn + 31) / 32), (unsigned)((R + 31) / 32));
    k_cgemm_small<<<grid, 256, 0, s>>>(R, Cn, Kd, A, lda, X, ldx, C, ldc, mode);
}

// The blocked solve for many right-hand sides. Each TRI_PANEL-row step solves its diagonal block
// (TRI_BLOCK-row sub-blocks in order: x_s = inv_s b_s with the precomputed inverse, then the panel's rows still to
// come lose T[rows, s] x_s; k_cgemm_small) and subtracts the block's product with the off-diagonal panel from the
// rows still to come, on the tcgen05 update
// with `update_terms` BF16 part products (six: FP32's accuracy). With T[r][c] = lu[r n + c] (A = U^T L^T P^T read
// row-major) and the work arrays (n, kpad) row-major, the forward update b_rest -= T[rest, I] y_I and the backward
// y_above -= T[above, I] z_I both take rows of T's column panel I, which is packed once per factor (all n rows) into
// its BF16 part plane: each sweep then reads the factor's planes once for all columns, and packs only the solved
// block of the right-hand sides per step.
cudaError_t TriSolver::solve_blocked(Plan *p, int k, const cd *in, cd *out, cudaStream_t s) {
    cudaError_t e;
    const int kp = p->kpad;
    const int64_t steps = (n + TRI_PANEL - 1) / TRI_PANEL;
    auto panel_width = [&](int64_t I) { return (int)(std::min<int64_t>((I + 1) * TRI_PANEL, n) - I * TRI_PANEL); };
    if (!panel_planes) {
        size_t bytes = 0;
        for (int64_t I = 0; I < steps; ++I) bytes += (size_t)n * tc_rows_row_bytes(panel_width(I), update_terms);
        if ((e = pool_alloc(&panel_planes, bytes, s))) return e;
        uint8_t *at = static_cast<uint8_t *>(panel_planes);
        for (int64_t I = 0; I < steps; ++I) {
            if ((e = tc_pack_rows_c64(n, panel_width(I), lu + I * TRI_PANEL, n, update_terms, at, s))) return e;
            at += (size_t)n * tc_rows_row_bytes(panel_width(I), update_terms);
        }
    }
    if (!p->planes) {
        if ((e = pool_alloc(&p->planes, tc_rows_scratch_bytes(kp, TRI_PANEL, update_terms), s)) ||
            (e = pool_alloc_n(&p->update_error, 1, s)) || (e = cudaMemsetAsync(p->update_error, 0, sizeof(int), s)))
            return e;
    }
    k_tri_in<<<blocks_for(n * kp), 256, 0, s>>>(n, k, kp, in, p->b);
    const unsigned long long wait = wait_cycles();
    int launches = 2;
    std::vector<const uint8_t *> panel((size_t)steps);
    {
        const uint8_t *at = static_cast<const uint8_t *>(panel_planes);
        for (int64_t I = 0; I < steps; ++I) {
            panel[I] = at;
            at += (size_t)n * tc_rows_row_bytes(panel_width(I), update_terms);
        }
    }
    // forward: U^T y = b, block by block; the rest of b then loses T[rest, I] y_I
    for (int64_t I = 0; I < steps; ++I) {
        const int64_t I0 = I * TRI_PANEL, I1 = std::min<int64_t>(I0 + TRI_PANEL, n);
        const int nb = (int)(I1 - I0);
        for (int64_t g0 = I0; g0 < I1; g0 += B) {
            const int rows = (int)std::min<int64_t>(B, I1 - g0);
            launch_cgemm_small(rows, kp, rows, inv_lower + (g0 / B) * B * B, B, p->b + g0 * kp, kp, p->y + g0 * kp, kp,
                               0, s);
            launch_cgemm_small((int)(I1 - g0 - rows), kp, rows, lu + (g0 + rows) * n + g0, n, p->y + g0 * kp, kp,
                               p->b + (g0 + rows) * kp, kp, 1, s);
            launches += 2;
        }
        if (I1 < n && (e = tc_update_rows_c64(n - I1, kp, nb, panel[I] + I1 * tc_rows_row_bytes(nb, update_terms),
                                              p->y + I0 * kp, kp, p->b + I1 * kp, kp, update_terms, p->planes,
                                              p->update_error, wait, s)))
            return e;
    }
    // backward: L^T z = y, last block first; the rows above then lose T[above, I] z_I
    for (int64_t I = steps - 1; I >= 0; --I) {
        const int64_t I0 = I * TRI_PANEL, I1 = std::min<int64_t>(I0 + TRI_PANEL, n);
        const int nb = (int)(I1 - I0);
        for (int64_t g0 = I0 + (nb - 1) / B * B; g0 >= I0; g0 -= B) {
            const int rows = (int)std::min<int64_t>(B, I1 - g0);
            launch_cgemm_small(rows, kp, rows, inv_upper + (g0 / B) * B * B, B, p->y + g0 * kp, kp, p->z + g0 * kp, kp,
                               0, s);
            launch_cgemm_small((int)(g0 - I0), kp, rows, lu + I0 * n + g0, n, p->z + g0 * kp, kp, p->y + I0 * kp, kp,
                               1, s);
            launches += 2;
        }
        if (I0 > 0 && (e = tc_update_rows_c64(I0, kp, nb, panel[I], p->z + I0 * kp, kp, p->y, kp, update_terms,
                                              p->planes, p->update_error, wait, s)))
            return e;
    }
    k_tri_out<<<blocks_for(n * k), 256, 0, s>>>(n, k, kp, p->z, gather, out);
    note_launches(launches);
    return cudaGetLastError();
}

cudaError_t TriSolver::solve_streaming(Plan *p, int k, const cd *in, cd *out, cudaStream_t s, bool deferred) {
    cudaError_t e;
    if (grid <= 0) {
        int device = 0, sms = 0, per_sm = 0, coop = 0;
        if ((e = cudaGetDevice(&device)) ||
            (e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device)) ||
            (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) ||
            (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tri_sweeps, PANEL_THREADS, 0)))
            return e;
        if (!coop || per_sm < 1 || sms * per_sm < DIAG_BLOCKS + TAIL_BLOCKS + 8) return cudaErrorNotSupported;
        grid = sms * per_sm;
    }
    k_tri_in<<<blocks_for(n * p->kpad), 256, 0, s>>>(n, k, p->kpad, in, p->b);
    // a deferred solve keeps the status word of earlier deferred solves (read_status clears it); otherwise every
    // word starts at zero
    if (!deferred && (e = cudaMemsetAsync(p->sync, 0, sync_words(nblk) * sizeof(unsigned), s))) return e;
    for (int c0 = 0; c0 < p->kpad; c0 += KC) {
        // counters restart for every 8 columns; the status word [3] keeps the first failure
        if ((c0 || deferred) && ((e = cudaMemsetAsync(p->sync, 0, 3 * SYNC_STRIDE * sizeof(unsigned), s)) ||
                   (e = cudaMemsetAsync(p->sync + 4 * SYNC_STRIDE, 0,
                                        (sync_words(nblk) - 4 * SYNC_STRIDE) * sizeof(unsigned), s))))
            return e;
        SweepArgs a{lu, n, nblk, inv_lower, inv_upper, p->b, p->y, p->z, p->kpad, c0, p->partial, p->sync,
                    p->sync + SYNC_STRIDE, p->sync + 4 * SYNC_STRIDE,
                    reinterpret_cast<int *>(p->sync + 3 * SYNC_STRIDE), (long long)wait_cycles()};
        void *args[] = {&a};
        if ((e = cudaLaunchCooperativeKernel((const void *)k_tri_sweeps, dim3(grid), dim3(PANEL_THREADS), args, 0,
                                             s)))
            return e;
    }
    k_tri_out<<<blocks_for(n * k), 256, 0, s>>>(n, k, p->kpad, p->z, gather, out);
    note_launches(2 + p->kpad / KC);
    if (deferred) return cudaGetLastError();
    // a barrier that gave up leaves its status; the sweeps are then incomplete
    int status = 0;
    if ((e = cudaMemcpyAsync(&status, p->sync + 3 * SYNC_STRIDE, sizeof(int), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
        return e;
    if (status) return cudaErrorLaunchTimeout;
    return cudaGetLastError();
}

cudaError_t TriSolver::read_status(int k, cudaStream_t s) {
    auto it = plans.find(k);
    if (it == plans.end()) return cudaSuccess;
    Plan &p = it->second;
    int *word = reinterpret_cast<int *>(p.sync + 3 * SYNC_STRIDE);
    int status[2] = {0, 0};
    cudaError_t e;
    if ((e = cudaMemcpyAsync(&status[0], word, sizeof(int), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemsetAsync(word, 0, sizeof(int), s)))
        return e;
    if (p.update_error && ((e = cudaMemcpyAsync(&status[1], p.update_error, sizeof(int), cudaMemcpyDeviceToHost, s)) ||
                           (e = cudaMemsetAsync(p.update_error, 0, sizeof(int), s))))
        return e;
    if ((e = cudaStreamSynchronize(s))) return e;
    return status[0] || status[1] ? cudaErrorLaunchTimeout : cudaSuccess;
}

void TriSolver::release() {
    if (!plans.empty() || inv_lower) cudaDeviceSynchronize();
    for (auto &kv : plans) {
        Plan &p = kv.second;
        for (float2 *q : {p.b, p.y, p.z, p.partial}) pool_free(q, nullptr);
        pool_free(p.sync, nullptr);
        pool_free(p.planes, nullptr);
        pool_free(p.update_error, nullptr);
    }

    plans.clear();
    method_by_bucket.clear();
    pool_free(panel_planes, nullptr);
    panel_planes = nullptr;
    pool_free(inv_lower, nullptr);
    pool_free(inv_upper, nullptr);
    pool_free(gather, nullptr);
    inv_lower = inv_upper = nullptr;
    gather = nullptr;
    lu = nullptr;
}

}  // namespace pq
