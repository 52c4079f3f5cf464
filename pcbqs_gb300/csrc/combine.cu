// RWG Galerkin combination of triangle-pair moments into the partial-inductance matrix L, and the
// area-weighted aggregation of M0 into the potential-coefficient matrix P. Both symmetric: upper tiles are
// evaluated once and written to both halves (reverse rows transposed through shared memory).
//
// Reference behaviour (paths within the pcbqs project):
//   src/pcbqs/core/static_kernels.hpp:257-310  static_combine    (k_edge_inductance)
//   src/pcbqs/static.py:103-128                edge_inductance   (factor * diag(s) combine diag(s))
//   src/pcbqs/mqs.py:532-552                   MQS._set_potential (k_potential: W^T M0 W / (4 pi eps0 er))
#include "combine.cuh"

namespace pq {

constexpr int CT = 32;             // tile edge (entries)
constexpr int CT_THREADS = 256;
constexpr int CT_ROWS = CT / (CT_THREADS / 32);

__device__ __forceinline__ void upper_tile(int64_t t, int nb, int &bm, int &bn) {
    // FP32 estimate of the tile row, corrected exactly in integers (keeps the per-tile math off the FP64 pipe)
    const float b = 2.0f * (float)nb + 1.0f;
    int r = (int)floorf((b - sqrtf(fmaxf(b * b - 8.0f * (float)t, 0.0f))) * 0.5f);
    r = max(0, min(r, nb - 1));
    auto off = [nb](int64_t x) { return x * nb - x * (x - 1) / 2; };
    while (r > 0 && off(r) > t) --r;
    while (r + 1 < nb && off(r + 1) <= t) ++r;
    bm = r;
    bn = r + (int)(t - off(r));
}

// L[m,n] = factor s_m s_n sum_{i,j in {+,-}} a_mi a_nj [Mrr(p,q) - v_nj.Mr(p,q) - v_mi.Mr(q,p) + v_mi.v_nj M0(p,q)]
// with p = tri[i][m], q = tri[j][n]; Mr(p,q) = (Mx[p,q], My[p,q]).
__global__ void __launch_bounds__(CT_THREADS) k_edge_inductance(EdgeBasis e, MomentPlanes mo, double factor,
                                                                double *L, int64_t ldl) {
    __shared__ double tr[CT][CT + 1];
    const int64_t ne = e.ne;
    const int nb = (int)((ne + CT - 1) / CT);
    const int64_t ntiles = (int64_t)nb * (nb + 1) / 2;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int bm, bn;
        upper_tile(t, nb, bm, bn);
        const int64_t m0 = (int64_t)bm * CT, n0 = (int64_t)bn * CT;
        const bool diagonal = bm == bn;
        const int64_t n = n0 + lane;
        // The column edge's supports are the same for every row a thread handles.
        int q[2] = {0, 0};
        double an[2] = {0, 0}, vnx[2] = {0, 0}, vny[2] = {0, 0}, sn = 0;
        if (n < ne) {
            for (int j = 0; j < 2; ++j) {
                q[j] = e.tri[j * ne + n];
                an[j] = e.alpha[j * ne + n];
                vnx[j] = e.vertex[2 * (j * ne + n)];
                vny[j] = e.vertex[2 * (j * ne + n) + 1];
            }
            sn = e.scale[n];
        }
#pragma unroll 1
        for (int i = 0; i < CT_ROWS; ++i) {
            const int ml = warp + (CT_THREADS / 32) * i;
            const int64_t m = m0 + ml;
            const bool valid = m < ne && n < ne && (!diagonal || ml <= lane);
            double value = 0;
            if (valid) {
                double sum = 0;
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    const int64_t p = e.tri[a * ne + m];
                    const double am = e.alpha[a * ne + m];
                    const double vmx = e.vertex[2 * (a * ne + m)], vmy = e.vertex[2 * (a * ne + m) + 1];
#pragma unroll
                    for (int b = 0; b < 2; ++b) {
                        const size_t pq = (size_t)p * mo.ld + q[b], qp = (size_t)q[b] * mo.ld + p;
                        sum += am * an[b] *
                               (mo.mrr[pq] - vnx[b] * mo.mx[pq] - vny[b] * mo.my[pq] - vmx * mo.mx[qp] -
                                vmy * mo.my[qp] + (vmx * vnx[b] + vmy * vny[b]) * mo.m0[pq]);
                    }
                }
                value = factor * e.scale[m] * sn * sum;
                L[(size_t)m * ldl + n] = value;
            }
            tr[lane][ml] = valid ? value : 0.0;
        }
        __syncthreads();
        // Reverse half: row n, columns m0.. (skip the diagonal tile's own diagonal and lower part).
#pragma unroll 1
        for (int i = 0; i < CT_ROWS; ++i) {
            const int nl = warp + (CT_THREADS / 32) * i, ml = lane;
            const int64_t nn = n0 + nl, m = m0 + ml;
            if (nn < ne && m < ne && (!diagonal || ml < nl)) L[(size_t)nn * ldl + m] = tr[nl][ml];
        }
        __syncthreads();
    }
}

// Mixed precision: the same combination from moments about each triangle's centroid c (FP32 planes), with the
// supports' offsets a = c_p - v_m, b = c_q - v_n:
//   L[m,n] = factor s_m s_n sum a_mi a_nj [Rr(p,q) + b.Ro(p,q) + a.Ro(q,p) + (a.b) M0(p,q)]
// Every term is of the size of the triangles, so FP32 arithmetic keeps FP32 accuracy. Writes L in FP64 (the outer
// refinement's operator) and its FP32 copy (the inner products).
__global__ void __launch_bounds__(CT_THREADS) k_edge_inductance_local(EdgeBasisF e, MomentPlanesF mo, float factor,
                                                                      double *L, int64_t ldl, float *Lf,
                                                                      int64_t ldlf) {
    __shared__ float tr[CT][CT + 1];
    const int64_t ne = e.ne;
    const int nb = (int)((ne + CT - 1) / CT);
    const int64_t ntiles = (int64_t)nb * (nb + 1) / 2;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int bm, bn;
        upper_tile(t, nb, bm, bn);
        const int64_t m0 = (int64_t)bm * CT, n0 = (int64_t)bn * CT;
        const bool diagonal = bm == bn;
        const int64_t n = n0 + lane;
        int q[2] = {0, 0};
        float an[2] = {0, 0}, bx[2] = {0, 0}, by[2] = {0, 0}, sn = 0;
        if (n < ne) {
            for (int j = 0; j < 2; ++j) {
                q[j] = e.tri[j * ne + n];
                an[j] = e.alpha[j * ne + n];
                bx[j] = e.off[2 * (j * ne + n)];
                by[j] = e.off[2 * (j * ne + n) + 1];
            }
            sn = e.scale[n];
        }
#pragma unroll 1
        for (int i = 0; i < CT_ROWS; ++i) {
            const int ml = warp + (CT_THREADS / 32) * i;
            const int64_t m = m0 + ml;
            const bool valid = m < ne && n < ne && (!diagonal || ml <= lane);
            float value = 0;
            if (valid) {
                float sum = 0;
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    const int64_t p = e.tri[a * ne + m];
                    const float am = e.alpha[a * ne + m];
                    const float ax = e.off[2 * (a * ne + m)], ay = e.off[2 * (a * ne + m) + 1];
#pragma unroll
                    for (int b = 0; b < 2; ++b) {
                        const size_t pq = (size_t)p * mo.ld + q[b], qp = (size_t)q[b] * mo.ld + p;
                        sum += am * an[b] *
                               (mo.mrr[pq] + bx[b] * mo.mx[pq] + by[b] * mo.my[pq] + ax * mo.mx[qp] +
                                ay * mo.my[qp] + (ax * bx[b] + ay * by[b]) * mo.m0[pq]);
                    }
                }
                value = factor * e.scale[m] * sn * sum;
                L[(size_t)m * ldl + n] = value;
                if (Lf) Lf[(size_t)m * ldlf + n] = value;
            }
            tr[lane][ml] = valid ? value : 0.0f;
        }
        __syncthreads();
#pragma unroll 1
        for (int i = 0; i < CT_ROWS; ++i) {
            const int nl = warp + (CT_THREADS / 32) * i, ml = lane;
            const int64_t nn = n0 + nl, m = m0 + ml;
            if (nn < ne && m < ne && (!diagonal || ml < nl)) {
                L[(size_t)nn * ldl + m] = tr[nl][ml];
                if (Lf) Lf[(size_t)nn * ldlf + m] = tr[nl][ml];
            }
        }
        __syncthreads();
    }
}

// P[a,b] = factor * (sum_{t in a} sum_{u in b} M0[t,u]) / (A_a A_b), node members in CSR form; M0 in FP64 or (mixed
// precision) FP32, the sums in FP64; Pf (nullable) receives an FP32 copy.
template <class T>
__global__ void __launch_bounds__(CT_THREADS) k_potential(NodeGroups ng, const T *m0, int64_t ldm, double factor,
                                                          double *P, int64_t ldp, float *Pf) {
    __shared__ double tr[CT][CT + 1];
    const int64_t nn = ng.nn;
    const int nb = (int)((nn + CT - 1) / CT);
    const int64_t ntiles = (int64_t)nb * (nb + 1) / 2;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int ba, bb;
        upper_tile(t, nb, ba, bb);
        const int64_t a0 = (int64_t)ba * CT, b0 = (int64_t)bb * CT;
        const bool diagonal = ba == bb;
        const int64_t b = b0 + lane;
        int64_t bs = 0, be = 0;
        double area_b = 1;
        if (b < nn) { bs = ng.start[b]; be = ng.start[b + 1]; area_b = ng.area[b]; }
#pragma unroll 1
        for (int i = 0; i < CT_ROWS; ++i) {
            const int al = warp + (CT_THREADS / 32) * i;
            const int64_t a = a0 + al;
            const bool valid = a < nn && b < nn && (!diagonal || al <= lane);
            double value = 0;
            if (valid) {
                double s = 0;
                for (int64_t x = ng.start[a]; x < ng.start[a + 1]; ++x) {
                    const size_t row = (size_t)ng.members[x] * ldm;
                    double r = 0;
                    for (int64_t y = bs; y < be; ++y) r += (double)m0[row + ng.members[y]];
                    s += r;
                }
                value = s / (ng.area[a] * area_b) * factor;
                P[(size_t)a * ldp + b] = value;
                if (Pf) Pf[(size_t)a * ldp + b] = (float)value;
            }
            tr[lane][al] = valid ? value : 0.0;
        }
        __syncthreads();
#pragma unroll 1
        for (int i = 0; i < CT_ROWS; ++i) {
            const int bl = warp + (CT_THREADS / 32) * i, al = lane;
            const int64_t bb2 = b0 + bl, a = a0 + al;
            if (bb2 < nn && a < nn && (!diagonal || al < bl)) {
                P[(size_t)bb2 * ldp + a] = tr[bl][al];
                if (Pf) Pf[(size_t)bb2 * ldp + a] = (float)tr[bl][al];
            }
        }
        __syncthreads();
    }
}

static int sms() {
    int dev = 0, count = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev);
    return count > 0 ? count : 1;
}

cudaError_t launch_edge_inductance(const EdgeBasis &e, const MomentPlanes &mo, double factor, double *L,
                                   int64_t ldl, cudaStream_t stream) {
    if (e.ne <= 0) return cudaSuccess;
    const int64_t nb = (e.ne + CT - 1) / CT;
    const int64_t ntiles = nb * (nb + 1) / 2;
    const int64_t grid = std::min<int64_t>(ntiles, (int64_t)sms() * 8);
    k_edge_inductance<<<(unsigned)grid, CT_THREADS, 0, stream>>>(e, mo, factor, L, ldl);
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_potential(const NodeGroups &ng, const double *m0, int64_t ldm, double factor, double *P,
                             int64_t ldp, cudaStream_t stream) {
    if (ng.nn <= 0) return cudaSuccess;
    const int64_t nb = (ng.nn + CT - 1) / CT;
    const int64_t ntiles = nb * (nb + 1) / 2;
    const int64_t grid = std::min<int64_t>(ntiles, (int64_t)sms() * 8);
    k_potential<double><<<(unsigned)grid, CT_THREADS, 0, stream>>>(ng, m0, ldm, factor, P, ldp, nullptr);
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_potential_single(const NodeGroups &ng, const float *m0, int64_t ldm, double factor, double *P,
                                    float *Pf, int64_t ldp, cudaStream_t stream) {
    if (ng.nn <= 0) return cudaSuccess;
    const int64_t nb = (ng.nn + CT - 1) / CT;
    const int64_t ntiles = nb * (nb + 1) / 2;
    const int64_t grid = std::min<int64_t>(ntiles, (int64_t)sms() * 8);
    k_potential<float><<<(unsigned)grid, CT_THREADS, 0, stream>>>(ng, m0, ldm, factor, P, ldp, Pf);
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_edge_inductance_local(const EdgeBasisF &e, const MomentPlanesF &mo, float factor, double *L,
                                         int64_t ldl, float *Lf, int64_t ldlf, cudaStream_t stream) {
    if (e.ne <= 0) return cudaSuccess;
    const int64_t nb = (e.ne + CT - 1) / CT;
    const int64_t ntiles = nb * (nb + 1) / 2;
    const int64_t grid = std::min<int64_t>(ntiles, (int64_t)sms() * 8);
    k_edge_inductance_local<<<(unsigned)grid, CT_THREADS, 0, stream>>>(e, mo, factor, L, ldl, Lf, ldlf);
    note_launches(1);
    return cudaGetLastError();
}

}  // namespace pq
