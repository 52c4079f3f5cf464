"""CPU restatement of the reference's dense PEEC solve -- TEST INFRASTRUCTURE ONLY (the benchmark's reference arm and
the CPU tests; nothing in the package imports it).

The reference solves the PEEC charge system by LU, one factorization per frequency shared by every drive:
  peec.prepare (src/pcbqs/peec.py:164-208): loop/tree basis K = [cycles, tree branches], T = A K_tree, the dense
      projections R = K^T R_branch K, L = K^T L_edge K, electro = T^T P T / pscale;
  peec.solve (peec.py:211-292): per frequency the scaled system of kernels.peec_system (src/pcbqs/kernels.py:67-81:
      Z = R + jw L, zscale = max |Z|, loop columns Z / zscale, tree columns jw Z / pscale, electro added to the tree
      block), factored by lu_factor_rows -- MixedLU (kernels.py:125-181: LAPACK cgetrf of the complex64 copy, each
      solve refined with the double system until the residual is 1e-12 of b) for 4,000 unknowns or more -- and
      each drive's right-hand side from the tree part of the excitation (baseline currents through the tree).
This module restates those steps with NumPy/SciPy on the host (every BLAS thread), on the moments and matrices the C
oracle (oracle.py) fills; the loop basis is oracle.graph's restatement of the reference's spanning forest. The
sheet resistance restates MQS._sheet_resistance (src/pcbqs/mqs.py:478-515): the Gram matrix of the RWG functions
with the 3-point rule at each triangle's DC sheet resistance, in total edge currents.

`lu_seconds` times LAPACK's complex64 getrf on a bounded sample, as a cross-check of the full factorization's time.
"""
import time

import numpy as np
import scipy.linalg as sl
from scipy.sparse import coo_matrix, csr_matrix, diags, eye, hstack
from scipy.sparse.csgraph import connected_components
from scipy.sparse.linalg import splu

from . import graph

BAR3 = np.array([[2 / 3, 1 / 6, 1 / 6], [1 / 6, 2 / 3, 1 / 6], [1 / 6, 1 / 6, 2 / 3]])
W3 = np.full(3, 1 / 3)


def lu_seconds(n, sample=3072, repeats=2, seed=0):
    """Estimated seconds of a complex64 LU of an n x n matrix, from a timed `sample`-sized one."""
    rng = np.random.default_rng(seed)
    a = (rng.standard_normal((sample, sample)) + 1j * rng.standard_normal((sample, sample))).astype(np.complex64)
    a += sample * np.eye(sample, dtype=np.complex64)
    best = np.inf
    for _ in range(repeats):
        m = a.copy(order='F')
        t = time.perf_counter()
        sl.lu_factor(m, overwrite_a=True, check_finite=False)
        best = min(best, time.perf_counter() - t)
    return best * (n / sample) ** 3, best


def _qform(S1, M, S2):
    """S1^T M S2 for sparse S1, S2 and dense M, without a dense copy of either sparse factor."""
    return np.asarray((S2.T @ np.asarray(S1.T @ M).T).T)


def sheet_resistance(rwg, sigma, thickness):
    """R (ne x ne sparse) in total edge currents: diag(1/l) G diag(1/l), G the Gram matrix of the RWG functions
    f = alpha (r - v) over each triangle with the 3-point rule, weighted by the sheet resistance 1/(sigma t)."""
    nt, ne = len(rwg.tris), rwg.Ne
    tri = np.r_[rwg.tp, rwg.tm]
    alpha = np.r_[rwg.l / (2 * rwg.area[rwg.tp]), -rwg.l / (2 * rwg.area[rwg.tm])]
    v = np.r_[rwg.vp, rwg.vm]
    col = np.r_[np.arange(ne), np.arange(ne)]
    pts = np.einsum('qk,tkc->tqc', BAR3, rwg.nodes[rwg.tris])            # (nt, 3, 2)
    rs = rwg.area / (sigma * np.broadcast_to(thickness, (nt,)))
    # each triangle's (up to 3) RWG sides in a padded table, then every pair of sides on one triangle:
    # integral over triangle t of f_a . f_b = alpha_a alpha_b A_t sum_q w_q (p_q - v_a) . (p_q - v_b)
    order = np.argsort(tri, kind='stable')
    start = np.searchsorted(tri[order], np.arange(nt))
    count = np.bincount(tri, minlength=nt)
    slot = np.arange(2 * ne) - start[tri[order]]
    table = np.full((nt, 3), -1)
    table[tri[order], slot] = order
    ta, tb = np.meshgrid(np.arange(3), np.arange(3), indexing='ij')
    t_idx = np.repeat(np.arange(nt), 9)
    a = table[t_idx, np.tile(ta.ravel(), nt)]
    b = table[t_idx, np.tile(tb.ravel(), nt)]
    ok = (a >= 0) & (b >= 0)
    t_idx, a, b = t_idx[ok], a[ok], b[ok]
    p = pts[t_idx]                                                       # (pairs, 3, 2)
    dot = (((p - v[a][:, None]) * (p - v[b][:, None])).sum(-1) * W3).sum(1)
    vals = rs[t_idx] * alpha[a] * alpha[b] * dot
    assert count.max() <= 3
    G = coo_matrix((vals, (col[a], col[b])), shape=(ne, ne)).tocsr()
    s = diags(1.0 / rwg.l)
    return (s @ G @ s).tocsr()


class DenseSolve:
    """The reference's dense PEEC charge solve of one board, prepared once (topology and projections) and solved per
    frequency for every port drive (Z[i, j]: voltage of port i for 1 A in port j)."""

    def __init__(self, board, rwg, L_edge, P, timings=None):
        t = time.perf_counter()
        node_of, nn, ne = board.node_of, board.n_nodes, rwg.Ne
        if board.nv:
            raise ValueError('the CPU dense solve restates boards without plated via segments')
        ends = np.r_[np.c_[node_of[rwg.tp], node_of[rwg.tm]],
                     np.array([(board.term_node(a), board.term_node(c)) for _, a, c in board.ports], np.int64)]
        nb = len(ends)
        is_src = np.r_[np.zeros(ne, bool), np.ones(len(board.ports), bool)]
        C, src_cols, tree, _ = graph.loop_basis(nn, [tuple(e) for e in ends], is_src, ne)
        ea, eb = ends.T
        br = np.arange(nb)
        A = coo_matrix((np.r_[np.ones(nb), -np.ones(nb)], (np.r_[ea, eb], np.r_[br, br])), shape=(nn, nb)).tocsc()
        passive, sources = np.flatnonzero(~is_src), np.flatnonzero(is_src)
        cycles = [k for k in range(C.shape[1]) if k not in src_cols.values()]
        K = hstack([C[passive][:, cycles], eye(nb, format='csc')[passive][:, np.flatnonzero(tree)]], format='csc')
        self.nl = nl = len(cycles)
        T = (A[:, passive] @ K[:, nl:]).tocsc()
        self.pscale = pscale = float(np.max(np.abs(P)))
        self.electro = _qform(T, P, T) / pscale
        R_branch = sheet_resistance(rwg, board.sigma, board.thickness)
        self.R = (K.T @ R_branch @ K).toarray()
        self.L = _qform(K, L_edge, K)
        self.PT = np.asarray((T.T @ P).T) if T.shape[1] else np.zeros((nn, 0))
        graph_nodes = coo_matrix((np.ones(len(passive)), (ea[passive], eb[passive])), shape=(nn, nn))
        nc, labels = connected_components(graph_nodes, directed=False)
        roots = np.unique(labels, return_index=True)[1]
        keep = np.ones(nn, bool)
        keep[roots] = False
        self.tree_lu = splu(T[keep].astype(complex).tocsc())
        self.keep, self.As = keep, A[:, sources]
        self.B = np.eye(nc)[labels]                                   # node -> its passive component
        self.source_components = np.asarray(self.As.T @ self.B)       # (sources, components)
        self.P = P
        self.PinvB = None
        self.n = K.shape[1]
        if timings is not None:
            timings['prepare_s'] = round(time.perf_counter() - t, 3)

    def solve(self, freq, timings=None, mixed=None):
        """Port impedance matrix at `freq` (Hz): the system assembled, factored once (MixedLU for 4,000 unknowns or
        more, else a double LU; `mixed` True/False chooses) and solved for every drive."""
        n, nl = self.n, self.nl
        w = 2 * np.pi * freq
        jw = 1j * w
        t0 = time.perf_counter()
        Z = np.empty((n, n), complex)                     # R + jw L in one matrix (no temporaries of its size)
        Z.real, Z.imag = self.R, self.L
        Z.imag *= w
        zscale = max(float(np.max(np.abs(Z))), np.finfo(float).tiny)
        system = Z
        system[:, :nl] /= zscale
        system[:, nl:] *= jw / self.pscale
        system[nl:, nl:] += self.electro
        t1 = time.perf_counter()
        mixed = n >= 4000 if mixed is None else bool(mixed)
        # lu_factor_rows: LAPACK's LU of the row-major system's transpose (its own memory read by columns), solved
        # transposed, so that no column-major copy of the system is made
        if mixed:
            lu = sl.lu_factor(system.astype(np.complex64).T, overwrite_a=True, check_finite=False)
        else:
            lu = sl.lu_factor(system.T, check_finite=False)
        t2 = time.perf_counter()
        # right-hand sides: a source between two components first charges them to their equilibrium (the
        # components' capacitance, P^-1 B solved once by Cholesky), then each drive's tree currents (baseline) give
        # the system's scaled excitation
        drives = np.eye(self.As.shape[1])
        drive = np.asarray(self.As @ drives)
        totals = self.source_components.T @ drives                   # (components, drives)
        qpart = np.zeros((len(self.keep), drives.shape[1]))
        vpart = np.zeros((self.B.shape[1], drives.shape[1]))
        if np.any(totals):
            if self.PinvB is None:
                self.PinvB = sl.cho_solve(sl.cho_factor(self.P, lower=True, check_finite=False), self.B,
                                          check_finite=False)
                self.component_lu = sl.lu_factor(self.B.T @ self.PinvB)
            vpart = sl.lu_solve(self.component_lu, -totals)
            qpart = self.PinvB @ vpart
        source_voltage = -self.source_components @ vpart
        y0 = self.tree_lu.solve((-drive - qpart)[self.keep].astype(complex))
        baseline = np.r_[np.zeros((nl, drive.shape[1]), complex), y0]
        rmul = lambda G, v: G @ v.real + 1j * (G @ v.imag)         # (no complex copy of the real matrix)
        rhs = -(rmul(self.R, baseline) + jw * rmul(self.L, baseline)) / zscale
        x = self._solve(system, lu, rhs, mixed)
        alpha = zscale / self.pscale
        volt = source_voltage / jw + alpha * (self.As.T @ (self.PT @ x[nl:]))
        t3 = time.perf_counter()
        if timings is not None:
            timings.update(assemble_s=round(t1 - t0, 3), lu_s=round(t2 - t1, 3), solves_s=round(t3 - t2, 3),
                           lu='complex64 getrf (MixedLU)' if mixed else 'complex128 getrf')
        return np.asarray(volt)

    @staticmethod
    def _solve(a, lu, b, mixed, tol=1e-12, steps=12):
        """MixedLU.solve: the single-precision solution refined with the double system until ||r|| <= tol ||b||
        (at most `steps`, stopping when a step no longer halves the residual); a double LU when that stalls above
        1e-10. Without mixed precision, the double factor's solve."""
        if not mixed:
            return sl.lu_solve(lu, b, trans=1, check_finite=False)
        one = lambda r: sl.lu_solve(lu, r.astype(np.complex64), trans=1, check_finite=False).astype(complex)
        x = one(b)
        nb = max(float(np.linalg.norm(b)), 1e-300)
        last = np.inf
        for _ in range(steps):
            r = b - a @ x
            res = float(np.linalg.norm(r)) / nb
            if res <= tol:
                return x
            if res > 0.5 * last:
                break
            last = res
            x = x + one(r)
        if last <= 1e-10:
            return x
        return sl.lu_solve(sl.lu_factor(a.T, check_finite=False), b, trans=1, check_finite=False)
