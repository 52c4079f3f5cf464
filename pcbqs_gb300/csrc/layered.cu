// Layered-dielectric image sums per triangle pair (pcbqs_gb300_layered_device).
//
// value(p, q) = A_p A_q / 9 sum_ij S(|x_i - s_j|)                                 (smooth positive images, spline)
//             + sum_k c_k M0(p, q; d_k)                  for the d_k = 0 images and the close positive images
//             - sum_k c_k A_p A_q / 9 sum_ij 1/sqrt(|x_i - s_j|^2 + d_k^2)          for the close positive images
// with M0(p, q; d) the static scalar moment (3 x 3 product rule when far, analytic when near) at offset d, the
// near/far rule the fill's (FMA-free, identical choices), and the positive images in increasing distance so the
// first far one ends the loop. Follows src/pcbqs/core/layered_kernels.hpp:38-75 (layered_pair) and :19-36
// (spline evaluation). One thread per pair, FP64; the complex result goes to two real planes, both (p, q) and
// (q, p).
#include <algorithm>
#include <cmath>

#include "../../include/pcbqs_gb300.h"
#include "common.cuh"
#include "pairs.cuh"

const pq::Geometry *pcbqs_gb300_geometry_of(const pcbqs_gb300_ctx *ctx);

namespace pq {

namespace {

struct Images {
    const double *dist;      // ascending, zero-distance images first
    const double2 *coef;
    int count;
    const double *x;         // spline breaks x[0..m] (x[0] = 0), or null
    const double2 *c;        // spline coefficients c[4][m] (highest power first)
    int64_t m;
    double rho_max;
};

// The piecewise cubic at r, extrapolated from the end intervals; interval found from the sqrt-uniform grid's
// index estimate, then corrected to the bracketing one.
__device__ __forceinline__ double2 spline_at(const Images &im, double r) {
    const int64_t last = im.m - 1;
    int64_t i = (int64_t)(sqrt(fmax(r, 0.0) / im.rho_max) * (double)im.m);
    i = i < 0 ? 0 : (i > last ? last : i);
    while (i > 0 && r < im.x[i]) --i;
    while (i < last && r >= im.x[i + 1]) ++i;
    const double dx = r - im.x[i];
    double2 v = im.c[i];
    for (int k = 1; k < 4; ++k) {
        const double2 ck = im.c[k * im.m + i];
        v = make_double2(v.x * dx + ck.x, v.y * dx + ck.y);
    }
    return v;
}

__global__ void k_layered(Geometry g, double near, int all_near, int outer, const int32_t *rows, int64_t nrows,
                          const int32_t *cols, int64_t ncols, int same, Images im, double *re, double *imag,
                          int64_t ld, int *flags) {
    const int64_t total = same ? nrows * (nrows + 1) / 2 : nrows * ncols;
    bool bad = false, invalid = false;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t i, j;
        if (same) {        // t -> (i, j), j >= i, row-major over the upper triangle
            const double b = 2.0 * nrows + 1.0;
            i = (int64_t)floor((b - sqrt(b * b - 8.0 * (double)t)) * 0.5);
            i = i < 0 ? 0 : (i >= nrows ? nrows - 1 : i);
            auto off = [nrows](int64_t r) { return r * nrows - r * (r - 1) / 2; };
            while (i > 0 && off(i) > t) --i;
            while (i + 1 < nrows && off(i + 1) <= t) ++i;
            j = i + (t - off(i));
        } else {
            i = t / ncols;
            j = t % ncols;
        }
        const int p = rows[i], q = same ? rows[j] : cols[j];
        if (p < 0 || p >= g.nt || q < 0 || q >= g.nt) {
            invalid = true;
            continue;
        }
        const FarRec &fp = g.far[p], &fq = g.far[q];
        const double A = fp.area * fq.area;
        double quad[9];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                const double dx = fp.p[2 * a] - fq.p[2 * b], dy = fp.p[2 * a + 1] - fq.p[2 * b + 1];
                quad[3 * a + b] = dx * dx + dy * dy;
            }
        double vr = 0, vi = 0;
        const bool smooth = im.m > 0;
        if (smooth) {
            double sr = 0, si = 0;
            for (int k = 0; k < 9; ++k) {
                const double2 s = spline_at(im, sqrt(quad[k]));
                sr += s.x;
                si += s.y;
            }
            vr += sr * (A / 9);
            vi += si * (A / 9);
        }
        const ClsRec cp = g.cls[p], cq = g.cls[q];
        double m[6];
        for (int k = 0; k < im.count; ++k) {
            const double d = im.dist[k];
            const double2 c = im.coef[k];
            const int kind = classify(cp, cq, d, near, all_near, outer);
            if (smooth && d > 0) {
                if (kind < 0) break;            // positive images ascend: the rest are far too
                double approx = 0;
                for (int a = 0; a < 9; ++a) approx += 1 / sqrt(quad[a] + d * d);
                const double w = A * approx / 9;
                vr -= c.x * w;
                vi -= c.y * w;
            }
            if (kind >= 0 || d == 0 || !smooth) {
                if (kind < 0) far_moments(fp, fq, d, true, m);
                else pair_moments(g, p, q, d, kind, true, m);
                vr += c.x * m[0];
                vi += c.y * m[0];
            }
        }
        if (!isfinite(vr) || !isfinite(vi)) bad = true;
        re[(int64_t)p * ld + q] = vr;
        imag[(int64_t)p * ld + q] = vi;
        re[(int64_t)q * ld + p] = vr;
        imag[(int64_t)q * ld + p] = vi;
    }
    if (bad) atomicExch(flags, 1);
    if (invalid) atomicExch(flags + 1, 1);
}

}  // namespace

}  // namespace pq

using namespace pq;

extern "C" int pcbqs_gb300_layered_device(pcbqs_gb300_ctx *ctx, double near, int outer, const int32_t *rows,
                                          int64_t nrows, const int32_t *cols, int64_t ncols, int same,
                                          const double *image_dist, const double *image_coef, int nimages,
                                          const double *spline_x, const double *spline_c, int64_t spline_m,
                                          double rho_max, double *out_re, double *out_im, int64_t ld,
                                          void *stream) {
    if (!ctx || !rows || nrows < 0 || ncols < 0 || (!same && !cols) || nimages < 0 || (nimages && (!image_dist ||
        !image_coef)) || spline_m < 0 || (spline_m && (!spline_x || !spline_c || !(rho_max > 0))) || !out_re ||
        !out_im || outer < 0 || outer > 2)
        return fail(ERR_ARGUMENT, "layered: invalid argument");
    const Geometry &g = *pcbqs_gb300_geometry_of(ctx);
    if (ld < g.nt) return fail(ERR_ARGUMENT, "layered: leading dimension below the triangle count");
    if (g.nq[outer] <= 0) return fail(ERR_ARGUMENT, "layered: outer level %d not prepared", outer);
    const int64_t total = same ? nrows * (nrows + 1) / 2 : nrows * ncols;
    if (total == 0) return OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int *flags = nullptr;
    cudaError_t e = cudaMallocAsync(&flags, 2 * sizeof(int), s);
    if (e) return fail(ERR_MEMORY, "layered: %s", cudaGetErrorString(e));
    cudaMemsetAsync(flags, 0, 2 * sizeof(int), s);
    Images im{image_dist, reinterpret_cast<const double2 *>(image_coef), nimages, spline_x,
              reinterpret_cast<const double2 *>(spline_c), spline_m, rho_max};
    const bool all_near = near < 0;
    const int threads = 128;
    int sms = 0, device = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int64_t blocks = std::min<int64_t>((total + threads - 1) / threads, (int64_t)sms * 16);
    k_layered<<<(unsigned)blocks, threads, 0, s>>>(g, all_near ? 0.0 : near, all_near ? 1 : 0, outer, rows, nrows,
                                                  cols, ncols, same, im, out_re, out_im, ld, flags);
    note_launches(1);
    int host[2] = {0, 0};
    e = cudaGetLastError();
    if (!e) e = cudaMemcpyAsync(host, flags, sizeof host, cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaStreamSynchronize(s);
    cudaFreeAsync(flags, s);
    if (e) return fail(ERR_CUDA, "layered: %s", cudaGetErrorString(e));
    if (host[1]) return fail(ERR_ARGUMENT, "layered: triangle index out of range");
    if (host[0]) return fail(ERR_NONFINITE, "non-finite layered image moments");
    return OK;
}
