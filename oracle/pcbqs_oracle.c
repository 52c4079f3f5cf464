/*
 * CPU oracle for the pcbqs static fill: a plain-C restatement of the reference's triangle-pair 1/R moments,
 * near/far classification, whole-matrix reciprocal fill, RWG combine and area-weighted potential aggregation.
 *
 * TEST INFRASTRUCTURE ONLY. Nothing in the product links or calls this file: only the tests, the smoke check and
 * the CPU-baseline leg of bench.py load it, as the oracle and as the timed CPU restatement of the reference's
 * compiled core. Parity is pinned against the reference itself (see tests/golden/make_golden.py: vectors produced
 * by the reference's own NumPy and compiled paths, and tests/test_oracle_golden.py).
 *
 * Built with -ffp-contract=off: every product is rounded before use, as the reference's x86 build does.
 * Reference files (paths within the pcbqs project):
 *   src/pcbqs/core/static_kernels.hpp:53-106   static_pair        -> og_pair
 *   src/pcbqs/core/static_kernels.hpp:111-136  rmul / pair_kind   -> og_kind
 *   src/pcbqs/core/static_kernels.hpp:147-172  static_pairs       -> og_pairs
 *   src/pcbqs/core/static_kernels.hpp:184-252  static_fill        -> og_fill
 *   src/pcbqs/core/static_kernels.hpp:257-310  static_combine     -> og_combine
 *   src/pcbqs/mqs.py:532-552                   MQS._set_potential -> og_potential
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* Triangle geometry, the reference's FillGeometry arrays (static_backends.py:104-130, sing.py:56-69):
 * v (nt,3,2) vertices; len (nt,3) edge lengths; tau/un (nt,3,2) unit tangent and outward normal per edge;
 * area (nt); p3 (nt,3,2) three-point rule points; qp[k] (nt,nq[k],2) and qw[k] (nq[k]) the observation rule of
 * refinement level k. */
typedef struct {
    int nt;
    const double *v, *len, *tau, *un, *area, *p3;
    const double *qp[3], *qw[3];
    int nq[3];
} og_geometry;

/* Moments M0, Mro_x, Mro_y, Mrs_x, Mrs_y, Mrr of the ordered pair (p observation, q source) at height offset d.
 * k < 0: far three-point product rule; k = 0/1/2: analytic source integration with the level-k observation
 * rule. Follows static_kernels.hpp:53-106 term by term. */
void og_pair(const og_geometry *g, int p, int q, double d, int k, int scalar_only, double *m) {
    const double ad = fabs(d);
    for (int j = 0; j < 6; ++j) m[j] = 0;
    if (k < 0) {
        const double w = g->area[p] * g->area[q] / 9;
        for (int ip = 0; ip < 3; ++ip) {
            const double x = g->p3[6 * (size_t)p + 2 * ip], y = g->p3[6 * (size_t)p + 2 * ip + 1];
            for (int iq = 0; iq < 3; ++iq) {
                const double sx = g->p3[6 * (size_t)q + 2 * iq], sy = g->p3[6 * (size_t)q + 2 * iq + 1];
                const double dx = x - sx, dy = y - sy;
                const double gg = w / sqrt(dx * dx + dy * dy + d * d);
                m[0] += gg;
                if (!scalar_only) {
                    m[1] += gg * x; m[2] += gg * y; m[3] += gg * sx; m[4] += gg * sy;
                    m[5] += gg * (x * sx + y * sy);
                }
            }
        }
        return;
    }
    const double *qp = g->qp[k], *qw = g->qw[k];
    const int nq = g->nq[k];
    for (int j = 0; j < nq; ++j) {
        const double x = qp[2 * ((size_t)p * nq + j)], y = qp[2 * ((size_t)p * nq + j) + 1];
        double i1 = 0, irx = 0, iry = 0;
        for (int e = 0; e < 3; ++e) {
            const size_t ve = 6 * (size_t)q + 2 * e;
            const double le = g->len[3 * (size_t)q + e];
            const double vx = g->v[ve] - x, vy = g->v[ve + 1] - y;
            const double sm = vx * g->tau[ve] + vy * g->tau[ve + 1];
            const double sp = sm + le;
            const double t0 = vx * g->un[ve] + vy * g->un[ve + 1];
            const double r02 = t0 * t0 + d * d, r0 = sqrt(r02);
            const double rm = sqrt(r02 + sm * sm), rp = sqrt(r02 + sp * sp);
            const double lg = r0 > 1e-14 * le ? asinh(sp / r0) - asinh(sm / r0) : 0;
            double inner = t0 * lg;
            if (ad > 0) inner -= ad * (atan2(t0 * sp, r02 + ad * rp) - atan2(t0 * sm, r02 + ad * rm));
            i1 += inner;
            if (!scalar_only) {
                const double er = .5 * (r02 * lg + sp * rp - sm * rm);
                irx += er * g->un[ve]; iry += er * g->un[ve + 1];
            }
        }
        const double w = g->area[p] * qw[j];
        m[0] += w * i1;
        if (!scalar_only) {
            const double sx = irx + x * i1, sy = iry + y * i1;
            m[1] += w * x * i1; m[2] += w * y * i1;
            m[3] += w * sx; m[4] += w * sy; m[5] += w * (x * sx + y * sy);
        }
    }
}

/* Near/far rule, static_kernels.hpp:130-136 (and FillEngine.kinds, static_backends.py:288-298): -1 far,
 * `outer` when the centroid distance is within the radii sum, else 0. Products rounded (no contraction). */
int og_kind(const double *cent, const double *radius, int p, int q, double d, double near, int all_near,
            int outer) {
    const double dx = cent[2 * p] - cent[2 * q], dy = cent[2 * p + 1] - cent[2 * q + 1];
    const double distance = sqrt((dx * dx + dy * dy) + d * d);
    const double size = radius[p] + radius[q];
    if (!all_near && !(distance <= near * size)) return -1;
    return distance <= size ? outer : 0;
}

/* Explicit pair list (static_kernels.hpp:147-172): out (n, 1|6). Returns 0, or -1 on an invalid index/kind. */
int og_pairs(const og_geometry *g, long n, const int32_t *p, const int32_t *q, const double *d,
             const int32_t *kind, int scalar_only, double *out, int threads) {
    const int width = scalar_only ? 1 : 6;
    for (long i = 0; i < n; ++i)
        if (p[i] < 0 || p[i] >= g->nt || q[i] < 0 || q[i] >= g->nt || kind[i] < -1 || kind[i] > 2 ||
            !isfinite(d[i]))
            return -1;
#pragma omp parallel for num_threads(threads) schedule(guided) if (threads > 1)
    for (long i = 0; i < n; ++i) {
        double m[6];
        og_pair(g, p[i], q[i], d[i], kind[i], scalar_only, m);
        for (int j = 0; j < width; ++j) out[(size_t)i * width + j] = m[j];
    }
    return 0;
}

/* Whole reciprocal moment matrices (static_kernels.hpp:184-252): planes M0, Mx, My, Mrr (nt x nt, row-major),
 * each unordered pair (p <= q) integrated once at d = z[p] - z[q] and written to [p,q] (Mro) and [q,p] (Mrs);
 * the diagonal's Mx/My average Mro and Mrs. Returns 0, or 1 if a moment was not finite. *analytic receives the
 * number of unordered pairs that were not far. */
int og_fill(const og_geometry *g, const double *cent, const double *radius, const double *z, double near,
            int all_near, int outer, int scalar_only, int threads, double *m0, double *mx, double *my,
            double *mrr, int64_t *analytic) {
    const int nt = g->nt;
    long long count = 0;
    int finite = 1;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1) reduction(+ : count) reduction(&& : finite) \
    if (threads > 1)
    for (int p = 0; p < nt; ++p) {
        for (int q = p; q < nt; ++q) {
            const double d = z[p] - z[q];
            const int k = og_kind(cent, radius, p, q, d, near, all_near, outer);
            double m[6];
            count += k >= 0;
            og_pair(g, p, q, d, k, scalar_only, m);
            for (int j = 0; j < (scalar_only ? 1 : 6); ++j) finite = finite && isfinite(m[j]);
            const size_t pq = (size_t)p * nt + q, qp = (size_t)q * nt + p;
            m0[pq] = m0[qp] = m[0];
            if (scalar_only) continue;
            if (p == q) {
                mx[pq] = (m[1] + m[3]) / 2; my[pq] = (m[2] + m[4]) / 2;
            } else {
                mx[pq] = m[1]; my[pq] = m[2];
                mx[qp] = m[3]; my[qp] = m[4];
            }
            mrr[pq] = mrr[qp] = m[5];
        }
    }
    *analytic = count;
    return finite ? 0 : 1;
}

/* RWG Galerkin combination (static_kernels.hpp:257-310):
 * L[m,n] = factor s_m s_n sum_{i,j} a_mi a_nj [Mrr(p,q) - v_nj.Mr(p,q) - v_mi.Mr(q,p) + v_mi.v_nj M0(p,q)],
 * p = tri[i][m], q = tri[j][n]; tri (2,ne), alpha (2,ne), vertex (2,ne,2) for the T+ and T- supports.
 * Upper triangle evaluated, written symmetrically. */
void og_combine(long ne, long nt, const int32_t *tri, const double *alpha, const double *vertex,
                const double *scale, double factor, const double *rr, const double *mx, const double *my,
                const double *m0, double *out, int threads) {
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1) if (threads > 1)
    for (long m = 0; m < ne; ++m) {
        for (long n = m; n < ne; ++n) {
            double sum = 0;
            for (int i = 0; i < 2; ++i) {
                const size_t p = (size_t)tri[i * ne + m];
                const double am = alpha[i * ne + m], vmx = vertex[2 * (i * ne + m)], vmy = vertex[2 * (i * ne + m) + 1];
                for (int j = 0; j < 2; ++j) {
                    const size_t q = (size_t)tri[j * ne + n];
                    const double vnx = vertex[2 * (j * ne + n)], vny = vertex[2 * (j * ne + n) + 1];
                    const size_t pq = p * nt + q, qp = q * nt + p;
                    sum += am * alpha[j * ne + n] *
                           (rr[pq] - vnx * mx[pq] - vny * my[pq] - vmx * mx[qp] - vmy * my[qp] +
                            (vmx * vnx + vmy * vny) * m0[pq]);
                }
            }
            const double value = factor * scale[m] * scale[n] * sum;
            out[(size_t)m * ne + n] = value;
            out[(size_t)n * ne + m] = value;
        }
    }
}

/* Area-weighted potential coefficients (mqs.py:532-552): P = W^T M0 W * factor with W[t, node] = 1/A_node,
 * A_node the summed area of the node's triangles. node_of (nt) maps triangles to nodes 0..nn-1; the node's
 * triangles are listed in CSR form (start (nn+1), members (nt)). */
void og_potential(long nt, long nn, const int64_t *start, const int32_t *members, const double *node_area,
                  const double *m0, double factor, double *out, int threads) {
#pragma omp parallel for num_threads(threads) schedule(dynamic, 4) if (threads > 1)
    for (long a = 0; a < nn; ++a) {
        for (long b = a; b < nn; ++b) {
            double s = 0;
            for (int64_t i = start[a]; i < start[a + 1]; ++i) {
                const size_t t = (size_t)members[i];
                double row = 0;
                for (int64_t j = start[b]; j < start[b + 1]; ++j) row += m0[t * nt + members[j]];
                s += row;
            }
            const double value = s / (node_area[a] * node_area[b]) * factor;
            out[(size_t)a * nn + b] = value;
            out[(size_t)b * nn + a] = value;
        }
    }
}
