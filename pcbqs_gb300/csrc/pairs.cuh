// Triangle-pair moment device functions shared by the fill (fill.cu) and the H-matrix entries (hmatrix.cu).
//
// Reference behaviour (paths within the pcbqs project): static_pair, src/pcbqs/core/static_kernels.hpp:53-106.
#pragma once
#include <cmath>
#include "common.cuh"

namespace pq {

// ---------------------------------------------------------------------------------------------------------------
// Pair moments. m = (M0, Mro_x, Mro_y, Mrs_x, Mrs_y, Mrr) of the ordered pair (observation a, source b).

// Far pairs: g_ij = (A_a A_b / 9) / sqrt(|x_i - s_j|^2 + d^2) over the 3 x 3 rule points; the sums are taken
// per observation point (row sums) so each point multiplies once.
__device__ __forceinline__ void far_moments(const FarRec &a, const FarRec &b, double d, bool scalar, double *m) {
    const double w = a.area * b.area / 9.0;
    const double d2 = d * d;
    double m0 = 0, ro_x = 0, ro_y = 0, rs_x = 0, rs_y = 0, rr = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double x = a.p[2 * i], y = a.p[2 * i + 1];
        double g_sum = 0, gsx = 0, gsy = 0;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const double sx = b.p[2 * j], sy = b.p[2 * j + 1];
            const double dx = x - sx, dy = y - sy;
            const double g = w * rsqrt(dx * dx + dy * dy + d2);
            g_sum += g;
            if (!scalar) { gsx += g * sx; gsy += g * sy; }
        }
        m0 += g_sum;
        if (!scalar) {
            ro_x += g_sum * x; ro_y += g_sum * y;
            rs_x += gsx; rs_y += gsy;
            rr += x * gsx + y * gsy;
        }
    }
    m[0] = m0; m[1] = ro_x; m[2] = ro_y; m[3] = rs_x; m[4] = rs_y; m[5] = rr;
}

// asinh(s+/r0) - asinh(s-/r0) with s+ = s- + L, r-+ = sqrt(r0^2 + s-+^2), as one logarithm. From
// asinh(s/r0) = sign(s) log((|s| + r)/r0): both ends on one side of the foot point give a ratio of two sums of
// positive terms, straddling ends a product over r0^2 -- no term cancels, where the difference of two inverse
// hyperbolic sines loses the leading digits when s- and s+ are large and close.
__device__ __forceinline__ double asinh_difference(double sm, double sp, double rm, double rp, double r02) {
    if (sm >= 0) return log((sp + rp) / (sm + rm));
    if (sp <= 0) return log((rm - sm) / (rp - sp));
    return log((sp + rp) * (rm - sm) / r02);
}

// atan2(t0 s+, r0^2 + |d| r+) - atan2(t0 s-, r0^2 + |d| r-) as one arctangent: both denominators are positive,
// so each angle lies in (-pi/2, pi/2) and the difference is atan2(y1 x2 - y2 x1, x1 x2 + y1 y2) with no wrap. The
// cross term y1 x2 - y2 x1 = t0 (L r0^2 + |d| (s+ r- - s- r+)) is formed without cancellation: for ends on one
// side, s+ r- - s- r+ = r0^2 L (s+ + s-) / (s+ r- + s- r+); for straddling ends both of its terms are positive.
__device__ __forceinline__ double atan2_difference(double t0, double sm, double sp, double rm, double rp,
                                                   double r02, double ad, double le) {
    const double cross = (sm >= 0 || sp <= 0) ? r02 * le * (sp + sm) / (sp * rm + sm * rp) : sp * rm - sm * rp;
    const double x1 = r02 + ad * rp, x2 = r02 + ad * rm;
    return atan2(t0 * (le * r02 + ad * cross), x1 * x2 + t0 * t0 * sp * sm);
}

// Near pairs: for each observation point x_j of triangle a (level-k rule) and each edge e of source triangle b,
// the closed-form inner integrals of 1/R and of the edge term over b at height offset d:
//   s- = (V_e - x).tau_e, s+ = s- + L_e, t0 = (V_e - x).u_e, r0 = sqrt(t0^2 + d^2), r-+ = sqrt(r0^2 + s-+^2)
//   lg = asinh(s+/r0) - asinh(s-/r0)  (0 when r0 <= 1e-14 L_e)
//   I1 += t0 lg - |d| (atan2(t0 s+, r0^2 + |d| r+) - atan2(t0 s-, r0^2 + |d| r-))
//   IR += 1/2 (r0^2 lg + s+ r+ - s- r-) u_e
// accumulated with weights A_a w_j into M0 = sum w I1, Mro = sum w x I1, Mrs = sum w (IR + x I1),
// Mrr = sum w x.(IR + x I1).
__device__ __forceinline__ void near_moments(const double *obs, const double *wts, int nq, double area_a,
                                             const SrcRec &b, double d, bool scalar, double *m) {
    const double ad = fabs(d);
    const double d2 = d * d;
    double m0 = 0, ro_x = 0, ro_y = 0, rs_x = 0, rs_y = 0, rr = 0;
    for (int j = 0; j < nq; ++j) {
        const double x = obs[2 * j], y = obs[2 * j + 1];
        double i1 = 0, irx = 0, iry = 0;
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            const double vx = b.v[2 * e] - x, vy = b.v[2 * e + 1] - y;
            const double le = b.len[e];
            const double sm = vx * b.tau[2 * e] + vy * b.tau[2 * e + 1];
            const double sp = sm + le;
            const double t0 = vx * b.un[2 * e] + vy * b.un[2 * e + 1];
            const double r02 = t0 * t0 + d2, r0 = sqrt(r02);
            const double rm = sqrt(r02 + sm * sm), rp = sqrt(r02 + sp * sp);
            const double lg = r0 > 1e-14 * le ? asinh_difference(sm, sp, rm, rp, r02) : 0.0;
            double inner = t0 * lg;
            if (ad > 0) inner -= ad * atan2_difference(t0, sm, sp, rm, rp, r02, ad, le);
            i1 += inner;
            if (!scalar) {
                const double er = 0.5 * (r02 * lg + sp * rp - sm * rm);
                irx += er * b.un[2 * e];
                iry += er * b.un[2 * e + 1];
            }
        }
        const double w = area_a * wts[j];
        m0 += w * i1;
        if (!scalar) {
            const double sx = irx + x * i1, sy = iry + y * i1;
            ro_x += w * x * i1; ro_y += w * y * i1;
            rs_x += w * sx; rs_y += w * sy;
            rr += w * (x * sx + y * sy);
        }
    }
    m[0] = m0; m[1] = ro_x; m[2] = ro_y; m[3] = rs_x; m[4] = rs_y; m[5] = rr;
}

__device__ __forceinline__ void pair_moments(const Geometry &g, int a, int b, double d, int k, bool scalar,
                                             double *m) {
    if (k < 0) {
        far_moments(g.far[a], g.far[b], d, scalar, m);
    } else {
        const int nq = g.nq[k];
        near_moments(g.obs[k] + 2 * (size_t)a * nq, g.w[k], nq, g.far[a].area, g.src[b], d, scalar, m);
    }
}

// Mixed precision, far pairs: moments about each triangle's own centroid (local coordinates), in FP32.
//   M0 = sum g, Ro = sum g (x_i - c_a), Rs = sum g (s_j - c_b), Rr = sum g (x_i - c_a).(s_j - c_b)
// with g = (A_a A_b / 9) / |x_i - s_j| and x_i - s_j = (c_a - c_b) + (u_i - v_j): the centroid difference from a
// two-float split of the centroids, the rule points as small offsets u, v. Every term stays of the size of the
// triangles, so the RWG combine of these moments has no cancellation (the centred-coordinate form cancels by
// about (board / edge)^2 and cannot be used in FP32).
__device__ __forceinline__ void far_local(const LocalRec &a, const LocalRec &b, bool scalar, float *m) {
    const float dcx = (a.chi[0] - b.chi[0]) + (a.clo[0] - b.clo[0]);
    const float dcy = (a.chi[1] - b.chi[1]) + (a.clo[1] - b.clo[1]);
    const float dz = a.z - b.z, d2 = dz * dz;
    const float w = a.area * b.area / 9.0f;
    float m0 = 0, ro_x = 0, ro_y = 0, rs_x = 0, rs_y = 0, rr = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float ux = a.u[2 * i], uy = a.u[2 * i + 1];
        float g_sum = 0, gvx = 0, gvy = 0;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const float vx = b.u[2 * j], vy = b.u[2 * j + 1];
            const float rx = dcx + (ux - vx), ry = dcy + (uy - vy);
            const float g = w * rsqrtf(rx * rx + ry * ry + d2);
            g_sum += g;
            if (!scalar) { gvx += g * vx; gvy += g * vy; }
        }
        m0 += g_sum;
        if (!scalar) {
            ro_x += g_sum * ux; ro_y += g_sum * uy;
            rs_x += gvx; rs_y += gvy;
            rr += ux * gvx + uy * gvy;
        }
    }
    m[0] = m0; m[1] = ro_x; m[2] = ro_y; m[3] = rs_x; m[4] = rs_y; m[5] = rr;
}

// Centred-coordinate moments (FP64) to moments about the two triangles' centroids c_a, c_b.
__device__ __forceinline__ void to_local(const ClsRec &ca, const ClsRec &cb, double *m) {
    const double m0 = m[0], ox = m[1], oy = m[2], sx = m[3], sy = m[4], rr = m[5];
    m[1] = ox - ca.cx * m0;
    m[2] = oy - ca.cy * m0;
    m[3] = sx - cb.cx * m0;
    m[4] = sy - cb.cy * m0;
    m[5] = rr - (ca.cx * sx + ca.cy * sy) - (cb.cx * ox + cb.cy * oy) + (ca.cx * cb.cx + ca.cy * cb.cy) * m0;
}

template <class V> __device__ __forceinline__ bool finite6(const V *m, bool scalar) {
    bool ok = isfinite(m[0]);
    if (!scalar)
        for (int j = 1; j < 6; ++j) ok = ok && isfinite(m[j]);
    return ok;
}

// The near/far rule of classify() decided in FP32 from the centroid split (chi + clo) and float radii whenever the
// FP32 distance clears a threshold by a relative margin of 1e-5 (far above FP32's rounding of these few
// operations, so the FP64 rule necessarily agrees); only pairs within the margin of a threshold are classified by
// the exact FP64 rule. Keeps the mixed tile kernel off the FP64 pipe for all but a sliver of pairs.
__device__ __forceinline__ int classify_filtered(const LocalRec &a, const LocalRec &b, float ra, float rb,
                                                 const ClsRec &ca, const ClsRec &cb, float near_f, double near,
                                                 int all_near, int outer) {
    const float dcx = (a.chi[0] - b.chi[0]) + (a.clo[0] - b.clo[0]);
    const float dcy = (a.chi[1] - b.chi[1]) + (a.clo[1] - b.clo[1]);
    const float dz = a.z - b.z;
    const float dist2 = dcx * dcx + dcy * dcy + dz * dz;
    const float size = ra + rb;
    constexpr float lo = 1.0f - 1e-5f, hi = 1.0f + 1e-5f;
    bool exact = false;
    if (!all_near) {
        const float t = near_f * size, t2 = t * t;
        if (dist2 > t2 * hi) return -1;
        exact = !(dist2 < t2 * lo);
    }
    if (!exact) {
        const float s2 = size * size;
        if (dist2 > s2 * hi) return 0;
        if (dist2 < s2 * lo) return outer;
    }
    return classify(ca, cb, ca.z - cb.z, near, all_near, outer);
}

}  // namespace pq
