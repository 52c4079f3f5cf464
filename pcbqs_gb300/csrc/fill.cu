// Triangle-pair 1/R moments on sm_103a: the far three-point product rule, the analytic near/singular source
// integration, the whole-matrix reciprocal fill (upper tiles, near pairs compacted and integrated separately) and
// the explicit pair-list protocol.
//
// Reference behaviour (paths within the pcbqs project):
//   src/pcbqs/core/static_kernels.hpp:53-106   static_pair       (far_moments, near_moments)
//   src/pcbqs/core/static_kernels.hpp:147-172  static_pairs      (k_pairs)
//   src/pcbqs/core/static_kernels.hpp:184-252  static_fill       (k_fill_tiles + k_fill_near)
//   src/pcbqs/static_cupy_kernels.py:117-157   device row strips (the compaction of near pairs by level)
#include <atomic>
#include <cmath>
#include "common.cuh"
#include "fill.cuh"
#include "pairs.cuh"
#include "tma.cuh"

namespace pq {

// ---------------------------------------------------------------------------------------------------------------
// Explicit pair lists (the plugin's evaluate): kind-sorted so a warp never mixes far and near work.

__global__ void k_kind_count(const int32_t *kind, int64_t n, unsigned long long *count) {
    __shared__ unsigned int local[4];
    if (threadIdx.x < 4) local[threadIdx.x] = 0;
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int k = kind[i];
        if (k >= -1 && k <= 2) atomicAdd(&local[k + 1], 1u);     // invalid kinds are reported by k_pairs
    }
    __syncthreads();
    if (threadIdx.x < 4 && local[threadIdx.x]) atomicAdd(&count[threadIdx.x], (unsigned long long)local[threadIdx.x]);
}

// count[0..3] are the bucket sizes; cursor[0..3] start at the exclusive prefix sums.
__global__ void k_kind_scatter(const int32_t *kind, int64_t n, unsigned long long *cursor, int64_t *order) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int k = kind[i];
        if (k < -1 || k > 2) continue;
        const unsigned long long slot = atomicAdd(&cursor[k + 1], 1ull);
        order[slot] = i;
    }
}

// Positions of pairs with an invalid kind are not in `order`: the tail past the valid buckets is filled with -1
// so k_pairs skips them (and k_pairs flags every invalid pair when it runs in identity order).
__global__ void k_order_tail(int64_t *order, int64_t from, int64_t n) {
    for (int64_t i = from + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        order[i] = -1;
}

__global__ void k_pairs(Geometry g, const int32_t *p, const int32_t *q, const double *d, const int32_t *kind,
                        const int64_t *order, int64_t n, int scalar, double *out, int *nonfinite, int *invalid) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int64_t i = order ? order[t] : t;
    if (i < 0) {                       // a pair whose kind was out of range (dropped by the kind sort)
        *invalid = 1;
        return;
    }
    const int a = p[i], b = q[i], k = kind[i];
    if (a < 0 || a >= g.nt || b < 0 || b >= g.nt || k < -1 || k > 2) {
        *invalid = 1;
        return;
    }
    double m[6];
    pair_moments(g, a, b, d[i], k, scalar, m);
    const int width = scalar ? 1 : 6;
    for (int j = 0; j < width; ++j) out[i * width + j] = m[j];
    if (!finite6(m, scalar)) *nonfinite = 1;
}

// ---------------------------------------------------------------------------------------------------------------
// Whole-matrix fill. Upper tiles of TILE x TILE unordered pairs (p <= q), one CTA per tile, persistent over a
// row-major tile order. Each tile's row and column geometry is staged into shared memory by bulk copies; far
// pairs are integrated at once and written to [p,q] (coalesced rows) and [q,p] (transposed through shared memory);
// near pairs are compacted into per-level lists for k_fill_near.

constexpr int TILE = 32;
constexpr int FILL_THREADS = 256;
constexpr int ROWS_PER_WARP = TILE / (FILL_THREADS / 32);

struct FillSmem {
    FarRec far_r[TILE], far_c[TILE];
    LocalRec loc_r[TILE], loc_c[TILE];
    ClsRec cls_r[TILE], cls_c[TILE];
    float rad_r[TILE], rad_c[TILE];       // radii as floats (mixed precision classification filter)
    double t[4][TILE][TILE + 1];          // transposed staging: [plane][q_local][p_local] (float in mixed)
    unsigned char keep[TILE][TILE];        // [q_local][p_local]: 1 when the reverse entry is written here
    uint64_t bar;
};

__device__ __forceinline__ void tile_of(int64_t t, int nb, int &bp, int &bq) {
    // Row bp of the upper tile triangle starts at off(bp) = bp*nb - bp*(bp-1)/2. The FP32 estimate of the row is
    // corrected exactly in integers below (FP32 here keeps the per-tile index math off the slow FP64 pipe).
    const float b = 2.0f * (float)nb + 1.0f;
    int r = (int)floorf((b - sqrtf(fmaxf(b * b - 8.0f * (float)t, 0.0f))) * 0.5f);
    r = max(0, min(r, nb - 1));
    auto off = [nb](int64_t x) { return x * nb - x * (x - 1) / 2; };
    while (r > 0 && off(r) > t) --r;
    while (r + 1 < nb && off(r + 1) <= t) ++r;
    bp = r;
    bq = r + (int)(t - off(r));
}

// LOCAL = false: the reference's FP64 moments in centred coordinates into FP64 planes (T = double).
// LOCAL = true:  mixed precision -- far pairs as FP32 local moments, planes in FP32 (T = float).
template <class T, bool LOCAL>
__global__ void __launch_bounds__(FILL_THREADS) k_fill_tiles(Geometry g, Planes<T> out, FillRule rule,
                                                             NearLists lists, int *nonfinite, int *status) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    FillSmem &s = *reinterpret_cast<FillSmem *>(smem_raw);
    const int nt = g.nt;
    const int nb = (nt + TILE - 1) / TILE;
    const int64_t ntiles = (int64_t)nb * (nb + 1) / 2;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool scalar = out.scalar;
    if (threadIdx.x == 0) {
        mbar_init(&s.bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    uint32_t phase = 0;
    bool failed = false;
    const float near_f = (float)rule.near;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int bp, bq;
        tile_of(t, nb, bp, bq);
        const int p0 = bp * TILE, q0 = bq * TILE;
        const int np = min(TILE, nt - p0), nqn = min(TILE, nt - q0);
        const bool diagonal = bp == bq;
        if (threadIdx.x == 0) {
            const uint32_t rec = LOCAL ? sizeof(LocalRec) : sizeof(FarRec);
            const uint32_t bytes = (uint32_t)(np + nqn) * (rec + sizeof(ClsRec));
            mbar_arrive_expect_tx(&s.bar, bytes);
            if (LOCAL) {
                bulk_load(s.loc_r, g.local + p0, np * sizeof(LocalRec), &s.bar);
                bulk_load(s.loc_c, g.local + q0, nqn * sizeof(LocalRec), &s.bar);
            } else {
                bulk_load(s.far_r, g.far + p0, np * sizeof(FarRec), &s.bar);
                bulk_load(s.far_c, g.far + q0, nqn * sizeof(FarRec), &s.bar);
            }
            bulk_load(s.cls_r, g.cls + p0, np * sizeof(ClsRec), &s.bar);
            bulk_load(s.cls_c, g.cls + q0, nqn * sizeof(ClsRec), &s.bar);
        }
        if (!mbar_wait_bounded(&s.bar, phase, rule.wait)) failed = true;
        if (__syncthreads_or(failed)) {
            // the tile's copies may still be landing in this block's shared memory: wait for them (they complete
            // by themselves) before the block leaves, so no copy outlives it
            if (threadIdx.x == 0) {
                atomicExch(status, (int)ERR_TIMEOUT);
                mbar_wait_bounded(&s.bar, phase, DRAIN_WAIT_CYCLES);
            }
            __syncthreads();
            break;
        }
        phase ^= 1;
        if (LOCAL) {
            if (threadIdx.x < np) s.rad_r[threadIdx.x] = (float)s.cls_r[threadIdx.x].radius;
            if (threadIdx.x >= 32 && threadIdx.x < 32 + nqn) s.rad_c[threadIdx.x - 32] = (float)s.cls_c[threadIdx.x - 32].radius;
            __syncthreads();
        }
        bool bad = false;
#pragma unroll 1
        for (int i = 0; i < ROWS_PER_WARP; ++i) {
            const int pl = warp + (FILL_THREADS / 32) * i, ql = lane;
            const int p = p0 + pl, q = q0 + ql;
            bool valid = pl < np && ql < nqn && (!diagonal || pl <= ql);
            int k = -2;
            if (valid) {
                if (LOCAL)
                    k = classify_filtered(s.loc_r[pl], s.loc_c[ql], s.rad_r[pl], s.rad_c[ql], s.cls_r[pl], s.cls_c[ql],
                                          near_f, rule.near, rule.all_near, rule.outer);
                else
                    k = classify(s.cls_r[pl], s.cls_c[ql], s.cls_r[pl].z - s.cls_c[ql].z, rule.near, rule.all_near,
                                 rule.outer);
            }
            // Near pairs: warp-aggregated appends to the level's list.
#pragma unroll
            for (int level = 0; level < 2; ++level) {
                const int want = level == 0 ? 0 : rule.outer;
                if (level == 1 && rule.outer == 0) break;
                const bool mine = valid && k == want;
                const unsigned mask = __ballot_sync(0xffffffffu, mine);
                if (mask) {
                    unsigned long long base = 0;
                    const int leader = __ffs(mask) - 1;
                    if (lane == leader) base = atomicAdd(&lists.count[level], (unsigned long long)__popc(mask));
                    base = __shfl_sync(0xffffffffu, base, leader);
                    if (mine) {
                        const unsigned long long slot = base + __popc(mask & ((1u << lane) - 1u));
                        if (slot < lists.capacity) lists.pair[level][slot] = make_int2(p, q);
                    }
                }
            }
            const bool far = valid && k < 0;
            const bool reverse = far && p != q;
            s.keep[ql][pl] = reverse;
            if (LOCAL) {
                // FP32 far moments straight into the FP32 planes and the float staging (no FP64 conversions)
                float m[6] = {0, 0, 0, 0, 0, 0};
                if (far) {
                    far_local(s.loc_r[pl], s.loc_c[ql], scalar, m);
                    bad = bad || !finite6(m, scalar);
                    const size_t pq = (size_t)p * out.ld + q;
                    out.m0[pq] = (T)m[0];
                    if (!scalar) {
                        if (p == q) {
                            out.mx[pq] = (T)((m[1] + m[3]) * 0.5f);
                            out.my[pq] = (T)((m[2] + m[4]) * 0.5f);
                        } else {
                            out.mx[pq] = (T)m[1];
                            out.my[pq] = (T)m[2];
                        }
                        out.mrr[pq] = (T)m[5];
                    }
                }
                if (reverse) {
                    float *tf = reinterpret_cast<float *>(&s.t[0][0][0]);
                    tf[(0 * TILE + ql) * (TILE + 1) + pl] = m[0];
                    tf[(1 * TILE + ql) * (TILE + 1) + pl] = m[3];
                    tf[(2 * TILE + ql) * (TILE + 1) + pl] = m[4];
                    tf[(3 * TILE + ql) * (TILE + 1) + pl] = m[5];
                }
            } else {
                double m[6] = {0, 0, 0, 0, 0, 0};
                if (far) {
                    far_moments(s.far_r[pl], s.far_c[ql], s.cls_r[pl].z - s.cls_c[ql].z, scalar, m);
                    bad = bad || !finite6(m, scalar);
                    const size_t pq = (size_t)p * out.ld + q;
                    out.m0[pq] = (T)m[0];
                    if (!scalar) {
                        if (p == q) {
                            out.mx[pq] = (T)((m[1] + m[3]) / 2);
                            out.my[pq] = (T)((m[2] + m[4]) / 2);
                        } else {
                            out.mx[pq] = (T)m[1];
                            out.my[pq] = (T)m[2];
                        }
                        out.mrr[pq] = (T)m[5];
                    }
                }
                if (reverse) {
                    s.t[0][ql][pl] = m[0];
                    s.t[1][ql][pl] = m[3];
                    s.t[2][ql][pl] = m[4];
                    s.t[3][ql][pl] = m[5];
                }
            }
        }
        __syncthreads();
        // Reverse entries: row q, columns p0.., coalesced along p.
#pragma unroll 1
        for (int i = 0; i < ROWS_PER_WARP; ++i) {
            const int ql = warp + (FILL_THREADS / 32) * i, pl = lane;
            if (ql < nqn && pl < np && s.keep[ql][pl]) {
                const size_t qp = (size_t)(q0 + ql) * out.ld + (p0 + pl);
                if (LOCAL) {
                    const float *tf = reinterpret_cast<const float *>(&s.t[0][0][0]);
                    out.m0[qp] = (T)tf[(0 * TILE + ql) * (TILE + 1) + pl];
                    if (!scalar) {
                        out.mx[qp] = (T)tf[(1 * TILE + ql) * (TILE + 1) + pl];
                        out.my[qp] = (T)tf[(2 * TILE + ql) * (TILE + 1) + pl];
                        out.mrr[qp] = (T)tf[(3 * TILE + ql) * (TILE + 1) + pl];
                    }
                } else {
                    out.m0[qp] = (T)s.t[0][ql][pl];
                    if (!scalar) {
                        out.mx[qp] = (T)s.t[1][ql][pl];
                        out.my[qp] = (T)s.t[2][ql][pl];
                        out.mrr[qp] = (T)s.t[3][ql][pl];
                    }
                }
            }
        }
        if (bad) *nonfinite = 1;
        __syncthreads();
    }
}

// Near pairs of one level, grid-stride over the compacted list; both reciprocal entries written.
template <class T, bool LOCAL>
__global__ void k_fill_near(Geometry g, Planes<T> out, const int2 *list, const unsigned long long *count,
                            unsigned long long capacity, int level, int *nonfinite) {
    const unsigned long long n = min(*count, capacity);
    const bool scalar = out.scalar;
    bool bad = false;
    for (unsigned long long j = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; j < n;
         j += (unsigned long long)gridDim.x * blockDim.x) {
        const int2 pq = list[j];
        const int p = pq.x, q = pq.y;
        const double d = g.cls[p].z - g.cls[q].z;
        double m[6];
        pair_moments(g, p, q, d, level, scalar, m);
        bad = bad || !finite6(m, scalar);
        if (LOCAL && !scalar) to_local(g.cls[p], g.cls[q], m);
        const size_t fwd = (size_t)p * out.ld + q, rev = (size_t)q * out.ld + p;
        out.m0[fwd] = (T)m[0];
        out.m0[rev] = (T)m[0];
        if (!scalar) {
            if (p == q) {
                out.mx[fwd] = (T)((m[1] + m[3]) / 2);
                out.my[fwd] = (T)((m[2] + m[4]) / 2);
            } else {
                out.mx[fwd] = (T)m[1]; out.my[fwd] = (T)m[2];
                out.mx[rev] = (T)m[3]; out.my[rev] = (T)m[4];
            }
            out.mrr[fwd] = (T)m[5];
            out.mrr[rev] = (T)m[5];
        }
    }
    if (bad) *nonfinite = 1;
}

// ---------------------------------------------------------------------------------------------------------------
// Host launchers.

// SM count of the current device, looked up once per device.
constexpr int MAX_DEVICES = 64;
static int sm_count() {
    static std::atomic<int> counts[MAX_DEVICES];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= MAX_DEVICES) dev = 0;
    int count = counts[dev].load(std::memory_order_relaxed);
    if (!count) {
        cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev);
        if (count <= 0) count = 1;
        counts[dev].store(count, std::memory_order_relaxed);
    }
    return count;
}

cudaError_t launch_pairs(const Geometry &g, const int32_t *p, const int32_t *q, const double *d,
                         const int32_t *kind, int64_t n, int scalar, double *out, unsigned long long *count4,
                         int64_t *order, int *nonfinite, int *invalid, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    const int threads = 128;
    const int blocks = (int)std::min<int64_t>((n + threads - 1) / threads, (int64_t)sm_count() * 16);
    const int64_t *ord = nullptr;
    if (order && n > 1) {
        cudaMemsetAsync(count4, 0, 8 * sizeof(unsigned long long), stream);
        k_kind_count<<<blocks, 256, 0, stream>>>(kind, n, count4);
        unsigned long long host[4];
        cudaMemcpyAsync(host, count4, sizeof(host), cudaMemcpyDeviceToHost, stream);
        cudaError_t err = cudaStreamSynchronize(stream);
        if (err != cudaSuccess) return err;
        unsigned long long cursor[4], run = 0;
        for (int b = 0; b < 4; ++b) { cursor[b] = run; run += host[b]; }
        cudaMemcpyAsync(count4 + 4, cursor, sizeof(cursor), cudaMemcpyHostToDevice, stream);
        k_kind_scatter<<<blocks, 256, 0, stream>>>(kind, n, count4 + 4, order);
        if ((int64_t)run < n) {
            k_order_tail<<<blocks, 256, 0, stream>>>(order, (int64_t)run, n);
            note_launches(1);
        }
        note_launches(2);
        err = cudaStreamSynchronize(stream);     // `cursor` lives on this stack frame
        if (err != cudaSuccess) return err;
        ord = order;
    }
    k_pairs<<<(unsigned)((n + threads - 1) / threads), threads, 0, stream>>>(g, p, q, d, kind, ord, n, scalar, out,
                                                                            nonfinite, invalid);
    note_launches(1);
    return cudaGetLastError();
}

size_t fill_smem_bytes() { return sizeof(FillSmem) + 128; }

template <class T, bool LOCAL>
static cudaError_t launch_fill_t(const Geometry &g, const Planes<T> &out, const FillRule &rule,
                                 const NearLists &lists, int *nonfinite, int *status, cudaStream_t stream) {
    const int nb = (g.nt + TILE - 1) / TILE;
    const int64_t ntiles = (int64_t)nb * (nb + 1) / 2;
    const size_t smem = fill_smem_bytes();
    // the dynamic shared-memory limit is a per-device attribute of the kernel: raised once on each device
    static std::atomic<bool> configured[MAX_DEVICES];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= MAX_DEVICES || !configured[dev].load(std::memory_order_relaxed)) {
        const cudaError_t e =
            cudaFuncSetAttribute(k_fill_tiles<T, LOCAL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < MAX_DEVICES) configured[dev].store(true, std::memory_order_relaxed);
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fill_tiles<T, LOCAL>, FILL_THREADS, smem);
    if (per_sm < 1) per_sm = 1;
    const int64_t grid = std::min<int64_t>(ntiles, (int64_t)sm_count() * per_sm);
    cudaMemsetAsync(lists.count, 0, 2 * sizeof(unsigned long long), stream);
    k_fill_tiles<T, LOCAL><<<(unsigned)grid, FILL_THREADS, smem, stream>>>(g, out, rule, lists, nonfinite, status);
    note_launches(1);
    return cudaGetLastError();
}

template <class T, bool LOCAL>
static cudaError_t launch_near_t(const Geometry &g, const Planes<T> &out, const FillRule &rule,
                                 const NearLists &lists, int *nonfinite, cudaStream_t stream) {
    const int threads = 128;
    const int blocks = sm_count() * 8;
    k_fill_near<T, LOCAL><<<blocks, threads, 0, stream>>>(g, out, lists.pair[0], lists.count, lists.capacity, 0,
                                                          nonfinite);
    if (rule.outer > 0)
        k_fill_near<T, LOCAL><<<blocks, threads, 0, stream>>>(g, out, lists.pair[1], lists.count + 1,
                                                              lists.capacity, rule.outer, nonfinite);
    note_launches(rule.outer > 0 ? 2 : 1);
    return cudaGetLastError();
}

cudaError_t launch_fill(const Geometry &g, const FillPlanes &out, const FillRule &rule, const NearLists &lists,
                        int *nonfinite, int *status, cudaStream_t stream) {
    return launch_fill_t<double, false>(g, out, rule, lists, nonfinite, status, stream);
}

cudaError_t launch_fill_near(const Geometry &g, const FillPlanes &out, const FillRule &rule, const NearLists &lists,
                             int *nonfinite, cudaStream_t stream) {
    return launch_near_t<double, false>(g, out, rule, lists, nonfinite, stream);
}

cudaError_t launch_fill_local(const Geometry &g, const Planes<float> &out, const FillRule &rule,
                              const NearLists &lists, int *nonfinite, int *status, cudaStream_t stream) {
    return launch_fill_t<float, true>(g, out, rule, lists, nonfinite, status, stream);
}

cudaError_t launch_fill_near_local(const Geometry &g, const Planes<float> &out, const FillRule &rule,
                                   const NearLists &lists, int *nonfinite, cudaStream_t stream) {
    return launch_near_t<float, true>(g, out, rule, lists, nonfinite, stream);
}

}  // namespace pq
