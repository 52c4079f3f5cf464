// Biot-Savart near field of RWG sheet currents and straight filaments at observation points.
//
//   H(p) = 1/(4 pi) sum_s w_s J_s x (p - r_s) / |p - r_s|^3,   J = a r + b on each triangle (no z component):
//   H_x = sum wJ_y R_z / r^3,  H_y = -sum wJ_x R_z / r^3,  H_z = sum (wJ_x R_y - wJ_y R_x) / r^3
// over quadrature points r_s (the 6-point rule of each triangle, refined triangles split into midpoint
// sub-triangles), k excitations at once; filaments: H = I / (4 pi d) (cos t1 - cos t2) around each segment.
//
// Reference behaviour (paths within the pcbqs project): biot._h_tris / h_sheets / h_segments
// (src/pcbqs/biot.py:24-105). The host builds the quadrature points and current moments and classifies near
// triangles exactly as h_sheets does (biot.py:54-79); this file does the O(points x sources x excitations) sums.
//
// One thread owns one observation point and keeps its 3 x k complex field in registers; source points are staged
// through shared memory in chunks, so every source is read once per CTA. Geometry and accumulation run in T:
// double for the FP64 path, float for the fast path (positions rounded to float: ~3 nm on a 5 cm board).
#include <algorithm>
#include "common.cuh"

namespace pq {

constexpr int BIOT_THREADS = 128;
constexpr int BIOT_CHUNK = 128;     // source points staged per step
constexpr int BIOT_KMAX = 8;        // excitations per pass (registers); more are done in passes

struct BiotSrc {
    double x, y, z, pad;
};

template <class T>
__global__ void __launch_bounds__(BIOT_THREADS) k_biot_sheets(int64_t npts, const double *pts, int64_t nsrc,
                                                              const BiotSrc *src, const double2 *jx,
                                                              const double2 *jy, int k, int k0, int kn, double2 *H) {
    __shared__ T s_x[BIOT_CHUNK], s_y[BIOT_CHUNK], s_z[BIOT_CHUNK];
    __shared__ double2 s_jx[BIOT_CHUNK][BIOT_KMAX], s_jy[BIOT_CHUNK][BIOT_KMAX];
    const int64_t p = blockIdx.x * (int64_t)BIOT_THREADS + threadIdx.x;
    const bool valid = p < npts;
    T px = 0, py = 0, pz = 0;
    if (valid) {
        px = (T)pts[3 * p];
        py = (T)pts[3 * p + 1];
        pz = (T)pts[3 * p + 2];
    }
    T hx_r[BIOT_KMAX], hx_i[BIOT_KMAX], hy_r[BIOT_KMAX], hy_i[BIOT_KMAX], hz_r[BIOT_KMAX], hz_i[BIOT_KMAX];
#pragma unroll
    for (int e = 0; e < BIOT_KMAX; ++e) hx_r[e] = hx_i[e] = hy_r[e] = hy_i[e] = hz_r[e] = hz_i[e] = 0;
    for (int64_t s0 = 0; s0 < nsrc; s0 += BIOT_CHUNK) {
        const int cn = (int)std::min<int64_t>(BIOT_CHUNK, nsrc - s0);
        __syncthreads();
        for (int t = threadIdx.x; t < cn; t += BIOT_THREADS) {
            const BiotSrc v = src[s0 + t];
            s_x[t] = (T)v.x;
            s_y[t] = (T)v.y;
            s_z[t] = (T)v.z;
        }
        for (int t = threadIdx.x; t < cn * kn; t += BIOT_THREADS) {
            const int j = t / kn, e = t % kn;
            s_jx[j][e] = jx[(s0 + j) * k + k0 + e];
            s_jy[j][e] = jy[(s0 + j) * k + k0 + e];
        }
        __syncthreads();
        if (!valid) continue;
        for (int j = 0; j < cn; ++j) {
            const T rx = px - s_x[j], ry = py - s_y[j], rz = pz - s_z[j];
            const T r2 = rx * rx + ry * ry + rz * rz;
            const T r3 = r2 * sqrt(r2);
            const T inv = r3 > (T)1e-30 ? (T)1 / r3 : (T)0;
            const T ax = rx * inv, ay = ry * inv, az = rz * inv;
#pragma unroll
            for (int e = 0; e < BIOT_KMAX; ++e) {
                if (e >= kn) break;
                const T jxr = (T)s_jx[j][e].x, jxi = (T)s_jx[j][e].y, jyr = (T)s_jy[j][e].x, jyi = (T)s_jy[j][e].y;
                hx_r[e] += az * jyr;
                hx_i[e] += az * jyi;
                hy_r[e] -= az * jxr;
                hy_i[e] -= az * jxi;
                hz_r[e] += ay * jxr - ax * jyr;
                hz_i[e] += ay * jxi - ax * jyi;
            }
        }
    }
    if (!valid) return;
    const double f = 1.0 / (4.0 * 3.14159265358979323846);
    for (int e = 0; e < kn; ++e) {
        double2 *h = H + (p * 3) * k + k0 + e;
        h[0].x += f * (double)hx_r[e];
        h[0].y += f * (double)hx_i[e];
        h[k].x += f * (double)hy_r[e];
        h[k].y += f * (double)hy_i[e];
        h[2 * k].x += f * (double)hz_r[e];
        h[2 * k].y += f * (double)hz_i[e];
    }
}

// Filaments p0 -> p1 carrying I (nseg x k complex); one thread per point, all segments in turn.
__global__ void k_biot_segments(int64_t npts, const double *pts, int64_t nseg, const double *p0, const double *p1,
                                const double2 *I, int k, double2 *H) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const double px = pts[3 * p], py = pts[3 * p + 1], pz = pts[3 * p + 2];
    const double f = 1.0 / (4.0 * 3.14159265358979323846);
    for (int64_t g = 0; g < nseg; ++g) {
        const double lx = p1[3 * g] - p0[3 * g], ly = p1[3 * g + 1] - p0[3 * g + 1], lz = p1[3 * g + 2] - p0[3 * g + 2];
        const double ln = sqrt(lx * lx + ly * ly + lz * lz);
        if (!(ln > 0)) continue;
        const double ux = lx / ln, uy = ly / ln, uz = lz / ln;
        const double rx = px - p0[3 * g], ry = py - p0[3 * g + 1], rz = pz - p0[3 * g + 2];
        const double s = rx * ux + ry * uy + rz * uz;
        const double qx = rx - s * ux, qy = ry - s * uy, qz = rz - s * uz;
        const double d = sqrt(qx * qx + qy * qy + qz * qz);
        if (!(d > 1e-9)) continue;
        const double c1 = s / sqrt(s * s + d * d), c2 = (s - ln) / sqrt((s - ln) * (s - ln) + d * d);
        const double gmag = (c1 - c2) * f / d;
        // direction u x (q / d)
        const double dx = (uy * qz - uz * qy) / d, dy = (uz * qx - ux * qz) / d, dz = (ux * qy - uy * qx) / d;
        for (int e = 0; e < k; ++e) {
            const double2 cur = I[g * k + e];
            double2 *h = H + (p * 3) * k + e;
            h[0].x += dx * gmag * cur.x;
            h[0].y += dx * gmag * cur.y;
            h[k].x += dy * gmag * cur.x;
            h[k].y += dy * gmag * cur.y;
            h[2 * k].x += dz * gmag * cur.x;
            h[2 * k].y += dz * gmag * cur.y;
        }
    }
}

}  // namespace pq

using namespace pq;

extern "C" int pcbqs_gb300_biot_sheets(int64_t npts, const double *pts, int64_t nsrc, const double *src_xyz4,
                                       const double *jx, const double *jy, int k, int single, double *H,
                                       void *stream) {
    if (npts < 0 || nsrc < 0 || k <= 0 || (npts && !pts) || (nsrc && (!src_xyz4 || !jx || !jy)) || !H)
        return fail(ERR_ARGUMENT, "biot_sheets: invalid argument");
    if (!npts || !nsrc) return OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const unsigned blocks = (unsigned)((npts + BIOT_THREADS - 1) / BIOT_THREADS);
    for (int k0 = 0; k0 < k; k0 += BIOT_KMAX) {
        const int kn = std::min(BIOT_KMAX, k - k0);
        if (single)
            k_biot_sheets<float><<<blocks, BIOT_THREADS, 0, st>>>(npts, pts, nsrc,
                                                                reinterpret_cast<const BiotSrc *>(src_xyz4),
                                                                reinterpret_cast<const double2 *>(jx),
                                                                reinterpret_cast<const double2 *>(jy), k, k0, kn,
                                                                reinterpret_cast<double2 *>(H));
        else
            k_biot_sheets<double><<<blocks, BIOT_THREADS, 0, st>>>(npts, pts, nsrc,
                                                                 reinterpret_cast<const BiotSrc *>(src_xyz4),
                                                                 reinterpret_cast<const double2 *>(jx),
                                                                 reinterpret_cast<const double2 *>(jy), k, k0, kn,
                                                                 reinterpret_cast<double2 *>(H));
        note_launches(1);
    }
    cudaError_t e = cudaGetLastError();
    return e ? fail(ERR_CUDA, "biot_sheets: %s", cudaGetErrorString(e)) : OK;
}

extern "C" int pcbqs_gb300_biot_segments(int64_t npts, const double *pts, int64_t nseg, const double *p0,
                                         const double *p1, const double *I, int k, double *H, void *stream) {
    if (npts < 0 || nseg < 0 || k <= 0 || (npts && !pts) || (nseg && (!p0 || !p1 || !I)) || !H)
        return fail(ERR_ARGUMENT, "biot_segments: invalid argument");
    if (!npts || !nseg) return OK;
    k_biot_segments<<<(unsigned)((npts + 127) / 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
        npts, pts, nseg, p0, p1, reinterpret_cast<const double2 *>(I), k, reinterpret_cast<double2 *>(H));
    note_launches(1);
    cudaError_t e = cudaGetLastError();
    return e ? fail(ERR_CUDA, "biot_segments: %s", cudaGetErrorString(e)) : OK;
}

// ---- the FFT near field's source: sheet current deposited on a uniform grid ----------------------------------------
//
// Cloud in cell (src/pcbqs/_numerics/currents.py:28-61, current_deposit): each quadrature point's current moment
// (A m, complex, k excitations) is split onto the four grid points around it with bilinear weights; the grid holds
// the sums (divided by the cell area on the host). One thread per point; FP64 atomics (the sums are order-dependent
// only in their last bits).
namespace {

__global__ void k_current_deposit(int64_t npts, const double *qx, const double *qy, const double2 *mx,
                                  const double2 *my, int k, double x0, double y0, double dx, double dy, int64_t nx,
                                  int64_t ny, double2 *jx, double2 *jy) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < npts; t += (int64_t)gridDim.x * blockDim.x) {
        const double fx = (qx[t] - x0) / dx, fy = (qy[t] - y0) / dy;
        const double fi = floor(fx), fj = floor(fy);
        const int64_t i0 = (int64_t)fi, j0 = (int64_t)fj;
        const double tx = fx - fi, ty = fy - fj;
        const double w[4] = {(1 - tx) * (1 - ty), tx * (1 - ty), (1 - tx) * ty, tx * ty};
        const int di[4] = {0, 1, 0, 1}, dj[4] = {0, 0, 1, 1};
        for (int c = 0; c < 4; ++c) {
            const int64_t ii = i0 + di[c], jj = j0 + dj[c];
            if (ii < 0 || ii >= nx || jj < 0 || jj >= ny) continue;
            for (int s = 0; s < k; ++s) {
                const double2 a = mx[t * k + s], b = my[t * k + s];
                double *gx = reinterpret_cast<double *>(jx + (ii * ny + jj) * k + s);
                double *gy = reinterpret_cast<double *>(jy + (ii * ny + jj) * k + s);
                atomicAdd(gx, a.x * w[c]);
                atomicAdd(gx + 1, a.y * w[c]);
                atomicAdd(gy, b.x * w[c]);
                atomicAdd(gy + 1, b.y * w[c]);
            }
        }
    }
}

}  // namespace

extern "C" int pcbqs_gb300_current_deposit(int64_t npts, const double *qx, const double *qy, const double *mom_x,
                                           const double *mom_y, int k, double x0, double y0, double dx, double dy,
                                           int64_t nx, int64_t ny, double *jx, double *jy, void *stream) {
    if (npts < 0 || k <= 0 || nx <= 0 || ny <= 0 || !(dx > 0) || !(dy > 0) || !jx || !jy ||
        (npts && (!qx || !qy || !mom_x || !mom_y)))
        return fail(ERR_ARGUMENT, "current_deposit: invalid argument");
    if (!npts) return OK;
    const int64_t blocks = std::min<int64_t>((npts + 255) / 256, 152 * 16);
    k_current_deposit<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        npts, qx, qy, reinterpret_cast<const double2 *>(mom_x), reinterpret_cast<const double2 *>(mom_y), k, x0, y0,
        dx, dy, nx, ny, reinterpret_cast<double2 *>(jx), reinterpret_cast<double2 *>(jy));
    note_launches(1);
    cudaError_t e = cudaGetLastError();
    return e ? fail(ERR_CUDA, "current_deposit: %s", cudaGetErrorString(e)) : OK;
}
