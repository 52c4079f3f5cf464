"""PEEC port impedances on one GB300: device-resident L and P, the loop/tree operator and batched GMRES.

    model = PeecModel(Board.load('planes'))
    result = model.solve([1e6])                 # all ports driven one at a time: Z (nf, np, np)

Host bookkeeping (sparse topology) restates the reference:
  spanning_tree, loops   src/pcbqs/mqs.py:48-130, 592-637 (breadth-first forest from central roots, parts join
                         islands; fundamental cycles of the cotree; ideal terminals) -- native, loop_basis()
  sheet_resistance       src/pcbqs/mqs.py:478-515  (Gram matrix of the RWG functions at DC sheet resistance)
  prepare / solve        src/pcbqs/peec_iterative.py:127-161, 229-346 (loop/tree basis K, T = A K_tree,
                         components and equilibrium charge, scaled operator, currents, charges, source voltages)
Device work (C ABI): the fill of L and P (homogeneous, or the layered stack's images), the operator products, the
block-Jacobi blocks and their inverses, the complex64 factor and its streaming triangular solves, the batched
GMRES and the mixed-precision refinement; P^-1 B for the equilibrium split by the dense GMRES. The loop basis is
native host code in the same library.
"""
import concurrent.futures
import ctypes
import time
import warnings

import numpy as np
import torch
from scipy.sparse import block_diag, coo_matrix, csr_matrix, diags, eye, hstack
from scipy.sparse.csgraph import connected_components
from scipy.sparse.linalg import splu

from . import _lib
from .fill import MU0, DeviceFill, EPS0
from .geometry import BAR3, W3


# ---- graph: spanning forest and loop basis --------------------------------------------------------------------

def loop_basis(n_nodes, ends, is_src, n_rwg, ideal_terminals=True):
    """(C (nb x ncol) csc, src_cols {branch: col}, tree, col_branch): each non-tree branch's fundamental cycle,
    oriented with the branch (col_branch[c] is column c's branch); copper edges inside one node are no loop (ideal
    terminals); branches whose ends lie on islands joined only through them have none. The spanning forest (the
    first `n_rwg` branches as a breadth-first forest from each island's most central node, the other non-source
    branches joining islands) and the cycle walk run natively (pcbqs_gb300_loop_basis; src/pcbqs/mqs.py:48-130,
    :592-637)."""
    lib = _lib.load()
    ends = np.asarray(ends, np.int32).reshape(-1, 2)
    nb = len(ends)
    ea, eb = np.ascontiguousarray(ends[:, 0]), np.ascontiguousarray(ends[:, 1])
    src = np.ascontiguousarray(is_src, np.uint8)
    tree = np.zeros(nb, np.uint8)
    col_branch = np.zeros(max(nb, 1), np.int32)
    nnz, ncol = ctypes.c_int64(), ctypes.c_int64()
    capacity = max(64 * nb, 1024)
    while True:
        rows, cols, vals = np.empty(capacity, np.int32), np.empty(capacity, np.int32), np.empty(capacity)
        status = lib.pcbqs_gb300_loop_basis(n_nodes, nb, _lib.ptr(ea, ctypes.c_int32), _lib.ptr(eb, ctypes.c_int32),
                                            _lib.ptr(src, ctypes.c_uint8), n_rwg, int(ideal_terminals),
                                            _lib.ptr(tree, ctypes.c_uint8), capacity, _lib.ptr(rows, ctypes.c_int32),
                                            _lib.ptr(cols, ctypes.c_int32), _lib.ptr(vals), ctypes.byref(nnz),
                                            _lib.ptr(col_branch, ctypes.c_int32), ctypes.byref(ncol))
        if status == 0:
            break
        if nnz.value <= capacity:
            _lib.check(status, lib)
        capacity = nnz.value
    m, c = nnz.value, ncol.value
    C = coo_matrix((vals[:m], (rows[:m], cols[:m])), shape=(nb, c)).tocsc()
    col_branch = col_branch[:c].astype(np.int64)
    src_cols = {int(k): j for j, k in enumerate(col_branch) if is_src[k]}
    return C, src_cols, tree.astype(bool), col_branch


# ---- resistance: Gram matrix of the RWG functions ---------------------------------------------------------------

def rwg_sparse(rwg, nt):
    """The RWG functions' sparse triangle maps (A_alpha, B_x, B_y): alpha, alpha v_x, alpha v_y on (T+/-, edge)."""
    ne = rwg.Ne
    alpha = np.concatenate([rwg.l / (2 * rwg.area[rwg.tp]), -rwg.l / (2 * rwg.area[rwg.tm])])
    vv = np.vstack([rwg.vp, rwg.vm])
    rows = np.r_[rwg.tp, rwg.tm]
    cols = np.r_[np.arange(ne), np.arange(ne)]
    sp = lambda values: csr_matrix((values, (rows, cols)), shape=(nt, ne))
    return sp(alpha), sp(alpha * vv[:, 0]), sp(alpha * vv[:, 1])


def qform(S1, M, S2):
    return (S2.T @ (S1.T @ M).T).T


def sheet_resistance(rwg, sigma, thickness):
    """R (ne x ne, sparse) of total edge currents: diag(1/l) Gram diag(1/l), Gram the integral of f_m . f_n times
    each triangle's DC sheet resistance 1/(sigma t), with the 3-point rule (mqs.py:478-515)."""
    nt = len(rwg.tris)
    A, Bx, By = rwg_sparse(rwg, nt)
    Ar = rwg.area
    Pq = np.einsum('qk,tkc->tqc', BAR3, rwg.nodes[rwg.tris])
    rs = 1.0 / (sigma * np.broadcast_to(thickness, (nt,)))
    m = lambda v: diags(Ar * rs * (W3[None, :] * v).sum(1))
    Mrr, Mrx, Mry, M0 = m((Pq ** 2).sum(-1)), m(Pq[..., 0]), m(Pq[..., 1]), diags(Ar * rs)
    G = (qform(A, Mrr, A) - qform(A, Mrx, Bx) - qform(A, Mry, By) - qform(Bx, Mrx.T, A) - qform(By, Mry.T, A)
         + qform(Bx, M0, Bx) + qform(By, M0, By))
    scale = diags(1.0 / rwg.l)
    return (scale @ G @ scale).tocsr()


# ---- plated vias: filament segments along z ----------------------------------------------------------------------

def via_resistance(seg, sigma, plating):
    """DC resistance (ohm) of each via segment's plated barrel, seg rows (x, y, r, z0, z1) m: length over sigma
    times the plated ring's area (src/pcbqs/mqs.py:132-137)."""
    v = np.asarray(seg, float).reshape(-1, 5)
    outer = v[:, 2]
    inner = np.maximum(outer - plating, 0.0)
    return (v[:, 4] - v[:, 3]) / (sigma * np.pi * (outer ** 2 - inner ** 2))


def via_inductance(seg, out, device):
    """The via segments' partial inductance matrix written into `out` (a (nv, nv) FP64 CUDA view, any row stride)
    by the device kernel (pcbqs_gb300_via_inductance: filaments along z, Grover's formula)."""
    v = torch.as_tensor(np.ascontiguousarray(seg, float).reshape(-1, 5), device=device)
    lib = _lib.load()
    _lib.check(lib.pcbqs_gb300_via_inductance(len(v), v.data_ptr(), MU0 / (4 * np.pi), out.data_ptr(), out.stride(0),
                                              ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)), lib)
    return out


def with_vias(board, L, Lf=None):
    """The inductance of every branch with impedance, the edges' L and the via segments' as one block-diagonal
    matrix (edges first): the reference couples neither to the other (MQS._loops keeps them as separate blocks,
    src/pcbqs/mqs.py:655-662). L, Lf unchanged for a board without vias; Lf (FP32 copy) optional."""
    nv = board.nv
    if not nv:
        return L, Lf
    ne = L.shape[0]
    full = torch.zeros((ne + nv, ne + nv), dtype=L.dtype, device=L.device)
    full[:ne, :ne] = L
    via_inductance(board.via_seg, full[ne:, ne:], L.device)
    fullf = None
    if Lf is not None:
        fullf = torch.zeros((ne + nv, ne + nv), dtype=torch.float32, device=L.device)
        fullf[:ne, :ne] = Lf
        fullf[ne:, ne:] = full[ne:, ne:]
    return full, fullf


# ---- ordering for block-Jacobi -----------------------------------------------------------------------------------

def cluster_order(points, bs):
    """Recursive coordinate bisection of points (n, d) into leaves of exactly `bs` points (the last may be
    shorter): returns the permutation that makes each leaf a contiguous run."""
    order = []

    def split(idx):
        if len(idx) <= bs:
            order.extend(idx.tolist())
            return
        pts = points[idx]
        axis = int(np.argmax(pts.max(0) - pts.min(0)))
        half = bs * int(np.ceil(len(idx) / bs / 2))
        srt = idx[np.argsort(pts[:, axis], kind='stable')]
        split(srt[:half])
        split(srt[half:])
    split(np.arange(len(points)))
    return np.asarray(order, np.int64)


def _host_csr(S):
    """The arrays a device CSR takes (int64 row pointers, int32 sorted column indices, FP64 values, shape)."""
    S = csr_matrix(S)
    S.sum_duplicates()
    return (S.indptr.astype(np.int64), S.indices.astype(np.int32), S.data.astype(np.float64), S.shape)


def _dev_csr(S, device):
    ptr, idx, val, shape = S if isinstance(S, tuple) else _host_csr(S)
    return (torch.as_tensor(ptr, device=device), torch.as_tensor(idx, device=device),
            torch.as_tensor(val, device=device), shape)


def _csr_struct(t):
    ptr, idx, val, shape = t
    c = _lib.CsrDesc()
    c.rows, c.cols = shape
    c.ptr, c.idx, c.val = ptr.data_ptr(), idx.data_ptr(), val.data_ptr()
    return c


class PeecResult:
    def __init__(self, freqs, names, Z, currents, iterations, residual, timings):
        self.frequencies, self.names, self.impedance = freqs, names, Z
        self.currents, self.iterations, self.residual, self.timings = currents, iterations, residual, timings


class PeecTopology:
    """Host side of the PEEC model (peec_iterative.prepare): branches, loop/tree basis K, T = A K_tree, node
    incidence A, components B and the equilibrium tree factor, the sheet resistance R, and the clustered order of
    the unknowns. `rwg` is the RWG basis on the centred mesh nodes."""

    def __init__(self, board, rwg, block_size=32, log=None):
        self.board, self.rwg, self.bs = board, rwg, block_size
        self.log = log or (lambda *a: None)
        self._topology()

    def _topology(self):
        b, r = self.board, self.rwg
        node_of = b.node_of
        nn = b.n_nodes
        self.ne = ne = r.Ne
        self.nv = nv = b.nv
        self.ni = ne + nv                 # branches with impedance: RWG edges, then plated via segments
        self.names = [p for p, _, _ in b.ports]
        ends = np.r_[np.c_[node_of[r.tp], node_of[r.tm]], b.via_ends(),
                     np.array([(b.term_node(a), b.term_node(c)) for _, a, c in b.ports], np.int64).reshape(-1, 2)]
        nb = len(ends)
        is_src = np.r_[np.zeros(ne + nv, bool), np.ones(len(b.ports), bool)]
        C, src_cols, tree, col_branch = loop_basis(nn, ends, is_src, ne)
        ea, eb = np.asarray(ends).T
        branch = np.arange(nb)
        A = coo_matrix((np.r_[np.ones(nb), -np.ones(nb)], (np.r_[ea, eb], np.r_[branch, branch])),
                       shape=(nn, nb)).tocsc()
        sources, passive = np.flatnonzero(is_src), np.flatnonzero(~is_src)
        if not np.array_equal(passive, np.arange(ne + nv)):
            raise ValueError('only copper edges and via segments may be passive branches (no lumped parts)')
        cycles = np.setdiff1d(np.arange(C.shape[1]), np.fromiter(src_cols.values(), np.int64, len(src_cols)))
        K = hstack((C[:, cycles], eye(nb, format='csc')[:, np.flatnonzero(tree)]), format='csc')
        nl = len(cycles)
        T = (A @ K[:, nl:]).tocsc()
        graph = coo_matrix((np.ones(len(passive)), (ea[passive], eb[passive])), shape=(nn, nn))
        nc, labels = connected_components(graph, directed=False)
        B = coo_matrix((np.ones(nn), (np.arange(nn), labels)), shape=(nn, nc)).tocsc()
        roots = np.unique(labels, return_index=True)[1]
        keep = np.ones(nn, bool)
        keep[roots] = False
        self.tree_lu = splu(T[keep].astype(complex).tocsc()) if T.shape[1] else None
        self.A, self.K, self.T, self.B, self.keep, self.nl = A, K, T, B, keep, nl
        self.ends, self.labels, self.tree = np.asarray(ends, np.int64).reshape(-1, 2), labels, tree
        self.sources, self.passive, self.nn, self.nb = sources, passive, nn, nb
        self.source_components = np.asarray((A[:, sources].T @ B).todense())
        self.R = sheet_resistance(r, b.sigma, b.thickness)
        if nv:
            self.R = block_diag((self.R, diags(via_resistance(b.via_seg, b.sigma, b.plating))), format='csr')
        # K-space unknowns ordered into geometric blocks: a cycle at its defining (cotree) branch, a tree unknown
        # at its branch; branch positions are RWG edge midpoints at their sheet's height, via segments their axis
        # at mid height.
        n = K.shape[1]
        pos_branch = np.c_[r.mid, 1e3 * b.z[r.tp]]      # sheets far apart in the ordering
        if nv:
            v = np.asarray(b.via_seg)
            pos_branch = np.r_[pos_branch, np.c_[v[:, :2], 1e3 * (v[:, 3] + v[:, 4]) / 2]]
        own = np.r_[col_branch[cycles], np.flatnonzero(tree)]
        assert len(own) == n and own.max() < ne + nv
        self.own = own
        self.order = cluster_order(pos_branch[own], self.bs)
        self.Kp = K[passive][:, self.order].tocsc()           # passive rows, clustered columns
        Tfull = hstack((csr_matrix((nn, nl)), T), format='csc')     # loop columns carry no charge
        self.Tp = Tfull[:, self.order].tocsc()
        self.is_tree = np.r_[np.zeros(nl, np.int8), np.ones(n - nl, np.int8)][self.order]
        self.n = n
        # the operator's sparse matrices and K^T R K in device-ready form (host work, done here once)
        self.host_csr = dict(K=_host_csr(self.Kp), Kt=_host_csr(self.Kp.T), T=_host_csr(self.Tp),
                             Tt=_host_csr(self.Tp.T), R=_host_csr(self.R))
        self.log(f'peec: {nn:,} nodes, {ne:,} edges, {n:,} unknowns ({nl:,} loops), {nc} components')

    def graph_structure(self):
        """The frequency-independent arrays of the graph preconditioner (src/pcbqs/peec_iterative.py:44-84, boards
        without face-sheet pairs), indexed by the clustered unknowns, made once per topology (host arrays):

        kept (nn) / keep_row (nn): each node's row among the kept nodes, -1 at each component's grounded node (whose
        equation T[keep] drops; the reference drops the lowest-numbered node, peec_iterative.py:150, here the tree's
        centre, see below); ac (nkeep x n): each loop's defining (cotree) branch's
        incidence, +1 at its first end and -1 at its second (Ap on the loops' trial currents); lap_ptr / lap_branch /
        lap_other: each kept node's passive branches and their other ends' rows (-1 at a root), the graph Laplacian
        Ap Dinv Ap^T [keep][:, keep] by its edges; tinv (n x nkeep, rows of the tree unknowns) = T[keep]^-1 and tinvt
        its transpose, explicit: T[keep] is the incidence of the spanning forest without its roots, so with the
        forest rooted there the current in tree branch e is A[c, e] times the sum of the right-hand side over the
        nodes below e (c the lower end of e), and a node's potential is the signed sum of the right-hand side over
        the branches of its path to the root (nonzeros: the sum of the nodes' depths); branch (n): each unknown's
        branch (a loop's defining branch, a tree unknown's own); loop_ends (n x 2): a loop's defining branch's ends
        as kept rows; comp (nkeep), member_ptr / members: the kept nodes of each component."""
        g = self.__dict__.get('_graph')
        if g is not None:
            return g
        from scipy.sparse.csgraph import breadth_first_order
        nn, n, ni = self.nn, self.n, self.ni
        ea, eb = self.ends[:, 0], self.ends[:, 1]
        tb = np.flatnonzero(self.tree)
        adj = csr_matrix((np.r_[tb, tb] + 1.0, (np.r_[ea[tb], eb[tb]], np.r_[eb[tb], ea[tb]])), shape=(nn, nn))
        # The grounded node of each component: the preconditioner's output does not depend on it (a constant added
        # to the node potentials cancels in the branch drops and in the charges, whose sum over a component is
        # zero, so the dropped node's equation holds by itself), so each tree is rooted at its centre, the middle
        # of a longest path (two breadth-first sweeps), rather than at the reference's lowest-numbered node: half
        # the depth, half the entries of T[keep]^-1.
        keep = np.ones(nn, bool)
        for first in np.unique(self.labels, return_index=True)[1]:
            reached = breadth_first_order(adj, int(first), directed=False, return_predecessors=False)
            far, pred = breadth_first_order(adj, int(reached[-1]), directed=False, return_predecessors=True)
            path = [int(far[-1])]
            while pred[path[-1]] >= 0:
                path.append(int(pred[path[-1]]))
            keep[path[len(path) // 2]] = False
        nkeep = int(keep.sum())
        kidx = np.full(nn, -1, np.int64)
        kidx[keep] = np.arange(nkeep)
        branch = np.asarray(self.own)[self.order]
        is_tree = self.is_tree.astype(bool)
        if int(is_tree.sum()) != nkeep:
            raise ValueError('graph preconditioner: the spanning forest does not span the components')
        loops = np.flatnonzero(~is_tree)
        la, lb = kidx[ea[branch[loops]]], kidx[eb[branch[loops]]]
        rows, cols = np.r_[la, lb], np.r_[loops, loops]
        vals = np.r_[np.ones(len(loops)), -np.ones(len(loops))]
        ok = rows >= 0
        ac = csr_matrix((vals[ok], (rows[ok], cols[ok])), shape=(nkeep, n))
        ac.sum_duplicates()
        ac.eliminate_zeros()
        loop_ends = np.full((n, 2), -1, np.int32)
        loop_ends[loops, 0], loop_ends[loops, 1] = la, lb
        # the Laplacian's edges at each kept node, in branch order
        p = np.flatnonzero(ea[:ni] != eb[:ni])
        r = np.r_[kidx[ea[p]], kidx[eb[p]]]
        br = np.r_[p, p]
        oth = np.r_[kidx[eb[p]], kidx[ea[p]]]
        ok = r >= 0
        r, br, oth = r[ok], br[ok], oth[ok]
        o = np.lexsort((br, r))
        r, br, oth = r[o], br[o], oth[o]
        lap_ptr = np.r_[0, np.cumsum(np.bincount(r, minlength=nkeep))].astype(np.int64)
        # the spanning forest rooted at the dropped nodes: each node's parent and the branch to it
        parent = np.full(nn, -1, np.int64)
        for root in np.flatnonzero(~keep):
            reached, pred = breadth_first_order(adj, int(root), directed=False, return_predecessors=True)
            below = reached[1:]
            parent[below] = pred[below]
        if (parent[keep] < 0).any():
            raise ValueError('graph preconditioner: a node is not reached by the spanning forest')
        up = np.flatnonzero(keep)
        pbranch = np.full(nn, -1, np.int64)
        pbranch[up] = np.asarray(adj[up, parent[up]]).ravel().astype(np.int64) - 1
        tpos = np.full(self.nb, -1, np.int64)
        tpos[branch[is_tree]] = np.flatnonzero(is_tree)
        # T[keep]^-T row by row: each kept node's row holds the branches of its path to the root, nearest first
        # (level l of the walk is entry l of the row), so its CSR is filled in place; T[keep]^-1 is its transpose
        levels = []
        depth = np.zeros(nkeep, np.int64)
        cur, start = up.copy(), kidx[up]
        while cur.size:
            e = pbranch[cur]
            levels.append((start, tpos[e].astype(np.int32), np.where(ea[e] == cur, 1.0, -1.0)))
            depth[start] += 1
            cur = parent[cur]
            more = keep[cur]
            cur, start = cur[more], start[more]
        tptr = np.r_[0, np.cumsum(depth)].astype(np.int64)
        tidx = np.empty(int(tptr[-1]), np.int32)
        tval = np.empty(int(tptr[-1]))
        for level, (rows_l, cols_l, vals_l) in enumerate(levels):
            at = tptr[rows_l] + level
            tidx[at] = cols_l
            tval[at] = vals_l
        del levels
        tinvt = (tptr, tidx, tval, (nkeep, n))
        tinv_csc = csr_matrix((tval, tidx, tptr), shape=(nkeep, n)).tocsc()
        tinv = (tinv_csc.indptr.astype(np.int64), tinv_csc.indices.astype(np.int32), tinv_csc.data, (n, nkeep))
        del tinv_csc
        comp = np.asarray(self.labels)[keep].astype(np.int32)
        nc = int(self.B.shape[1])
        members = np.argsort(comp, kind='stable').astype(np.int32)
        member_ptr = np.r_[0, np.cumsum(np.bincount(comp, minlength=nc))].astype(np.int64)
        g = dict(nkeep=nkeep, ncomp=nc, kept=keep, keep_row=kidx, ac=_host_csr(ac), lap_ptr=lap_ptr,
                 lap_branch=br.astype(np.int32), lap_other=oth.astype(np.int32), tinv=tinv,
                 tinvt=tinvt, branch=branch.astype(np.int32), loop_ends=loop_ends, comp=comp,
                 member_ptr=member_ptr, members=members)
        self._graph = g
        return g

    GRAPH_DENSE_BYTES = 16e9     # the graph Laplacian dense up to this size (about 44,700 kept nodes)
    GRAPH_DOMAIN_ROWS = 1500     # above it, domains of about this many rows

    def _graph_parts(self, parts):
        """0 (the dense Laplacian) or the domain count: `parts` if given, else by the Laplacian's size."""
        if parts is not None:
            if parts != 0 and (parts < 2 or parts & (parts - 1)):
                raise ValueError('graph_parts must be 0 (dense) or a power of two >= 2')
            return int(parts)
        nk = self.graph_structure()['nkeep']
        if 8.0 * nk * nk <= self.GRAPH_DENSE_BYTES:
            return 0
        return 2 ** max(1, int(round(np.log2(nk / self.GRAPH_DOMAIN_ROWS))))

    def graph_domains(self, parts):
        """A nested-dissection-style split of the graph Laplacian's kept nodes for boards whose Laplacian is too large
        to factor dense (made once per topology and part count; host arrays): the nodes (triangle centroids, averaged
        over merged triangles) are cut by recursive coordinate bisection in the board's plane into `parts` (a power of
        two) parts; the node of each Laplacian edge between two parts that lies in the higher-numbered part joins the
        separator, so no edge joins two parts' interiors. New order: the parts' interiors one after another
        (dom_ptr), then the separator; perm[p] the kept row at new position p, pos its inverse. For the Schur
        complement, each part's boundary (the separator nodes next to its interior, bnd_ptr / bnd as separator
        positions) with each boundary node's interior neighbours (bnd_nptr / bnd_local / bnd_branch: local row in the
        part, and the branch)."""
        cache = self.__dict__.setdefault('_graph_domain_cache', {})
        if parts in cache:
            return cache[parts]
        if parts < 2 or parts & (parts - 1):
            raise ValueError('graph domains: the part count must be a power of two >= 2')
        g = self.graph_structure()
        nk = g['nkeep']
        b = self.board
        nn = self.nn
        cent = np.asarray(b.nodes)[np.asarray(b.tris)].mean(axis=1)
        node_of = np.asarray(b.node_of)
        cnt = np.maximum(np.bincount(node_of, minlength=nn), 1)
        xy = np.c_[np.bincount(node_of, cent[:, 0], minlength=nn), np.bincount(node_of, cent[:, 1], minlength=nn)]
        xy = (xy / cnt[:, None])[np.flatnonzero(g['kept'])]
        part = np.zeros(nk, np.int64)
        groups = [np.arange(nk)]
        while len(groups) < parts:
            nxt = []
            for idx in groups:
                ext = xy[idx].max(axis=0) - xy[idx].min(axis=0) if len(idx) else np.zeros(2)
                o = idx[np.argsort(xy[idx, int(np.argmax(ext))], kind='stable')]
                nxt += [o[:len(o) // 2], o[len(o) // 2:]]
            groups = nxt
        for d, idx in enumerate(groups):
            part[idx] = d
        rows = np.repeat(np.arange(nk), np.diff(g['lap_ptr']))
        oth = g['lap_other'].astype(np.int64)
        cut = (oth >= 0) & (part[rows] != part[np.maximum(oth, 0)])
        sep = np.zeros(nk, bool)
        r, o = rows[cut], oth[cut]
        sep[np.where(part[r] > part[o], r, o)] = True
        interior = [np.sort(idx[~sep[idx]]) for idx in groups]
        perm = np.concatenate(interior + [np.flatnonzero(sep)]).astype(np.int64)
        pos = np.empty(nk, np.int64)
        pos[perm] = np.arange(nk)
        dom_ptr = np.r_[0, np.cumsum([len(i) for i in interior])].astype(np.int64)
        n_int = int(dom_ptr[-1])
        # each part's boundary: interior row r of part d next to separator node s, through branch br
        m = (oth >= 0) & ~sep[rows] & sep[np.maximum(oth, 0)]
        r, s_, br = rows[m], oth[m], g['lap_branch'][m]
        d = part[r]
        sl = pos[s_] - n_int
        il = pos[r] - dom_ptr[d]
        o = np.lexsort((il, sl, d))
        d, sl, il, br = d[o], sl[o], il[o], br[o]
        first = np.r_[True, (d[1:] != d[:-1]) | (sl[1:] != sl[:-1])] if len(d) else np.zeros(0, bool)
        entry = np.cumsum(first) - 1
        nent = int(first.sum())
        bnd = sl[first].astype(np.int32)
        bnd_ptr = np.r_[0, np.cumsum(np.bincount(d[first], minlength=parts))].astype(np.int64)
        bnd_nptr = np.r_[0, np.cumsum(np.bincount(entry, minlength=nent))].astype(np.int64)
        out = dict(parts=parts, perm=perm, pos=pos, dom_ptr=dom_ptr, n_int=n_int, n_sep=nk - n_int, bnd_ptr=bnd_ptr,
                   bnd=bnd, bnd_nptr=bnd_nptr, bnd_local=il.astype(np.int32), bnd_branch=br.astype(np.int32))
        cache[parts] = out
        return out



_HOST_POOL = None


def _host_pool():
    """One helper thread for host-side preparation that overlaps device work."""
    global _HOST_POOL
    if _HOST_POOL is None:
        _HOST_POOL = concurrent.futures.ThreadPoolExecutor(max_workers=1, thread_name_prefix='pcbqs-host')
    return _HOST_POOL


class PeecModel(PeecTopology):
    """A board's surface-charge PEEC model, every port a 1 A current source from its first to its second terminal
    (MQS.source), solved on the device. The dielectric is homogeneous (board.er) unless `stack` (a
    layered.DielectricStack) is given: then P comes from the stack's electrostatic images and is complex for a lossy
    stack (MQS dielectric='stack', src/pcbqs/mqs.py:555-563)."""

    def __init__(self, board, near=3.0, outer_levels=1, device=0, block_size=32, tol=1e-8, maxiter=2000,
                 restart=100, log=None, inner_tol=1e-4, conductor_loss='dc', conductor_faces=2, stack=None,
                 matrix='dense', hmatrix=None):
        """matrix='hierarchical': L and P as device H-matrices (DeviceHMatrix; `hmatrix` overrides their options,
        default tol 1e-6, leaf 256, eta 1, rank 32) instead of dense matrices, as the reference's
        matrix_backend='hierarchical' (src/pcbqs/mqs.py:452-455): every product of the solve goes through them, in
        FP64, and block-Jacobi takes its blocks from exact entries; solve(mixed=True) runs the inner GMRES with the
        low-rank blocks' products in BF16 on the tensor cores (stacked U (V^T X), FP32 accumulation) under FP64 outer
        residuals. The complex64 factor ('lu32') needs the dense matrices."""
        if conductor_loss not in ('dc', 'slab') or conductor_faces not in (1, 2):
            raise ValueError('conductor_loss must be dc or slab; conductor_faces must be 1 or 2')
        if matrix not in ('dense', 'hierarchical'):
            raise ValueError("matrix must be 'dense' or 'hierarchical'")
        if not 1e-5 <= inner_tol < 1:
            # the inner products are BF16 parts or FP32: a tighter inner tolerance is out of their reach, and every
            # inner solve would then run to maxiter
            raise ValueError('inner_tol must lie in [1e-5, 1)')
        if matrix == 'hierarchical' and stack is not None:
            raise ValueError('the compressed operator takes a homogeneous dielectric')
        self.matrix = matrix
        self.hmatrix_options = dict(tol=1e-6, leaf=256, eta=1.0, rank=32)
        self.hmatrix_options.update(hmatrix or {})
        self.HL = self.HP = None
        self.tol, self.maxiter, self.restart, self.inner_tol = tol, maxiter, restart, inner_tol
        self.conductor_loss, self.conductor_faces = conductor_loss, conductor_faces
        self.stack = stack
        self.Pim = self.Pfim = None
        self.device = torch.device('cuda', device)
        self.timings = {}
        self.board = board
        self.fill = DeviceFill(board.nodes, board.tris, board.z, outer_levels, near, device)
        self.L = self.P = self.Lf = self.Pf = None
        # the host topology (loop basis, incidences, sheet resistance, ordering) needs no device: it is built on a
        # helper thread while the caller's first assemble() fills L and P; the first use of one of its attributes
        # waits for it (__getattr__) and raises its error, if any
        rwg = self.fill.rwg

        def topology():
            t0 = time.perf_counter()
            PeecTopology.__init__(self, board, rwg, block_size, log)
            self.timings['host_topology_s'] = time.perf_counter() - t0
        self._topology_job = _host_pool().submit(topology)

    def __getattr__(self, name):
        job = self.__dict__.get('_topology_job')
        if job is None:
            raise AttributeError(name)
        job.result()                        # the topology's error, raised at every use until it is fixed
        self.__dict__['_topology_job'] = None
        return getattr(self, name)

    # -- device matrices --
    def assemble(self, mixed=False):
        """Fill L and P on the device (moments, combine, aggregation); frees the moment planes. mixed=True: far
        pairs in FP32 local coordinates (near pairs FP64), FP32 combine; L and P kept in FP64 and FP32.
        matrix='hierarchical': build the H-matrices of L's edges and of the triangle potential instead."""
        if self.matrix == 'hierarchical':
            self._nearblk = self._papply = None
            return self._assemble_compressed(mixed)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        self.L = self.P = self.Lf = self.Pf = self.Pim = self.Pfim = None
        ev[0].record()
        if mixed:
            planes, analytic = self.fill.moments_local()
            ev[1].record()
            self.L, self.Lf = with_vias(self.board, *self.fill.inductance_local(planes))
            ev[2].record()
            if self.stack is None:
                self.P, self.Pf = self.fill.potential_single(planes[0], self.board.node_of, self.board.er)
        else:
            planes, analytic = self.fill.moments()
            ev[1].record()
            self.L, _ = with_vias(self.board, self.fill.inductance(planes))
            ev[2].record()
            if self.stack is None:
                self.P = self.fill.potential(planes[0], self.board.node_of, self.board.er)
        del planes
        if self.stack is not None:
            from .layered import LayeredPotential
            lp = LayeredPotential(self.fill, self.stack, self.board.layer)
            self.P, Pim = lp.potential_parts(self.board.node_of)
            self.Pim = Pim if bool(Pim.any()) else None
            if mixed:
                self.Pf = self.P.float()
                self.Pfim = self.Pim.float() if self.Pim is not None else None
        ev[3].record()
        torch.cuda.synchronize()
        self.mixed_fill = mixed
        self.analytic = analytic
        self.timings.update(fill_ms=ev[0].elapsed_time(ev[1]), combine_ms=ev[1].elapsed_time(ev[2]),
                            potential_ms=ev[2].elapsed_time(ev[3]))
        pdiag = torch.diagonal(self.P) if self.Pim is None else torch.complex(torch.diagonal(self.P),
                                                                               torch.diagonal(self.Pim))
        self.pscale = float(pdiag.abs().max())
        self.pdiag_host = pdiag.cpu().numpy()
        self.ldiag = torch.diagonal(self.L).cpu().numpy()
        self._pinvb = None
        return self

    def _krk_device(self):
        """K^T R K (frequency independent) as a device CSR, made once per model by two sparse products on the
        device (cuSPARSE through torch; the same on the host took 0.2 s for the plane pair)."""
        if getattr(self, '_krk', None) is None:
            dev = self.device

            def csr(key):
                ptr, idx, val, shape = self.host_csr[key]
                return torch.sparse_csr_tensor(torch.as_tensor(ptr, device=dev),
                                               torch.as_tensor(idx.astype(np.int64), device=dev),
                                               torch.as_tensor(val, device=dev), size=shape)
            with warnings.catch_warnings():
                warnings.simplefilter('ignore', UserWarning)         # torch: sparse CSR support is beta
                M = torch.sparse.mm(torch.sparse.mm(csr('Kt'), csr('R')), csr('K'))
            self._krk = (M.crow_indices().to(torch.int64).contiguous(), M.col_indices().to(torch.int32).contiguous(),
                         M.values().to(torch.float64).contiguous(), tuple(M.shape))
        return self._krk

    def _operator(self, omegas):
        dev = self.device
        R = self.R
        ratio = self.resistance_ratio(omegas / (2 * np.pi))
        zscale = np.array([max(float(np.max(np.abs(ratio[i] * R.diagonal() + 1j * w * self.ldiag))),
                               np.finfo(float).tiny) for i, w in enumerate(omegas)])
        if getattr(self, '_dev', None) is None:      # the topology's sparse matrices, uploaded once per model
            h = self.host_csr
            self._dev = dict(K=_dev_csr(h['K'], dev), Kt=_dev_csr(h['Kt'], dev), T=_dev_csr(h['T'], dev),
                             Tt=_dev_csr(h['Tt'], dev), R=_dev_csr(h['R'], dev),
                             is_tree=torch.as_tensor(self.is_tree, device=dev))
        d = _lib.PeecDesc()
        d.n, d.nb, d.ne, d.nn = self.n, len(self.passive), self.ni, self.nn
        for name in ('K', 'Kt', 'T', 'Tt', 'R'):
            setattr(d, name, _csr_struct(self._dev[name]))
        if self.matrix == 'hierarchical':
            d.L, d.ldl, d.P, d.ldp = None, 0, None, 0
        else:
            d.L, d.ldl, d.P, d.ldp = self.L.data_ptr(), self.L.stride(0), self.P.data_ptr(), self.P.stride(0)
        d.is_tree = self._dev['is_tree'].data_ptr()
        d.pscale = self.pscale
        d.Pim = self.Pim.data_ptr() if self.Pim is not None else None
        d.nscaled = self.ne                 # the sheets' rows: via barrels keep their DC resistance
        d.nsys = len(omegas)
        self._omega = np.ascontiguousarray(omegas, float)
        self._zscale = np.ascontiguousarray(zscale, float)
        d.omega, d.zscale = _lib.ptr(self._omega), _lib.ptr(self._zscale)
        self._rscale = np.ascontiguousarray(np.c_[ratio.real, ratio.imag].ravel())
        d.rscale = _lib.ptr(self._rscale)
        lib = _lib.load()
        handle = ctypes.c_void_p()
        _lib.check(lib.pcbqs_gb300_peec_create(ctypes.byref(d), ctypes.byref(handle)), lib)
        if self.matrix == 'hierarchical':
            hl, hp = self.HL.desc(), self.HP.desc()
            w, wt = _csr_struct(self._Wdev), _csr_struct(self._Wtdev)
            status = lib.pcbqs_gb300_peec_set_compressed(handle, ctypes.byref(hl), self.Lvia.data_ptr(),
                                                          self.board.nv, ctypes.byref(hp), ctypes.byref(w),
                                                          ctypes.byref(wt))
            if status:
                lib.pcbqs_gb300_peec_destroy(handle)
                _lib.check(status, lib)
        self._live_handle = handle
        return handle, zscale

    def _assemble_compressed(self, mixed):
        """The H-matrices (the same for mixed=True: its inner products then take their low-rank blocks in BF16)."""
        from .hmatrix import DeviceHMatrix
        t0 = time.perf_counter()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        self.L = self.P = self.Lf = self.Pf = self.Pim = self.Pfim = None
        ev[0].record()
        self.HL = DeviceHMatrix(self.fill, kernel='inductance', **self.hmatrix_options)
        ev[1].record()
        self.HP = DeviceHMatrix(self.fill, kernel='potential', er=self.board.er, **self.hmatrix_options)
        ev[2].record()
        dev = self.device
        nv = self.board.nv
        self.Lvia = torch.zeros((max(nv, 1), max(nv, 1)), dtype=torch.float64, device=dev)
        if nv:
            via_inductance(self.board.via_seg, self.Lvia, dev)
        # W[t, node] = A_t / A_node and its transpose, device CSR
        node_of = np.asarray(self.board.node_of)
        nt, nn = len(node_of), self.nn
        area_t = np.asarray(self.fill.geometry.area)
        area_n = np.bincount(node_of, weights=area_t, minlength=nn)
        self._w = area_t / area_n[node_of]
        W = csr_matrix((self._w, (np.arange(nt), node_of)), shape=(nt, nn))
        self._Wdev, self._Wtdev = _dev_csr(W, dev), _dev_csr(W.T.tocsr(), dev)
        self._tris_of = np.split(np.argsort(node_of, kind='stable'), np.cumsum(np.bincount(node_of, minlength=nn))[:-1])
        # diagonals: L's edges and vias, P's nodes (exact entries)
        ne = self.ne
        ld = self.HL.dense_entries([(np.array([e]), np.array([e])) for e in range(ne)], host=True)
        ldiag = np.array([m[0, 0] for m in ld])
        if nv:
            ldiag = np.r_[ldiag, torch.diagonal(self.Lvia).cpu().numpy()]
        pdiag = self._node_blocks([np.array([i]) for i in range(nn)])
        self.pdiag = torch.as_tensor(np.array([b[0, 0] for b in pdiag]), device=dev)
        torch.cuda.synchronize()
        self.ldiag = ldiag
        self.pscale = float(self.pdiag.abs().max())
        self.pdiag_host = self.pdiag.cpu().numpy()
        self._pinvb = None
        self.mixed_fill = False
        self.analytic = None
        self.timings.update(fill_ms=ev[0].elapsed_time(ev[1]), combine_ms=0.0, potential_ms=ev[1].elapsed_time(ev[2]),
                            hmatrix_s=time.perf_counter() - t0, hmatrix_L=self.HL.info, hmatrix_P=self.HP.info)
        return self

    def _node_blocks(self, groups):
        """P[N, N] = W_N^T H[T, T] W_N for each node set N (T: its triangles), from exact triangle entries; host
        arrays."""
        tris = [np.concatenate([self._tris_of[i] for i in g]) for g in groups]
        blocks = self.HP.dense_entries([(t, t) for t in tris], host=True)
        node_of = np.asarray(self.board.node_of)
        out = []
        for g, t, H in zip(groups, tris, blocks):
            pos = {int(i): k for k, i in enumerate(g)}
            Wb = np.zeros((len(t), len(g)))
            Wb[np.arange(len(t)), [pos[int(node_of[x])] for x in t]] = self._w[t]
            out.append(Wb.T @ H @ Wb)
        return out

    def _near_blocks(self):
        """The diagonal blocks of K^T L K and T^T P T for block-Jacobi from exact entries (the compressed
        operator has no dense L and P to gather from): (nblk, bs, bs) device arrays."""
        bs, n, ne = self.bs, self.n, self.ne
        Kt = csr_matrix(self.Kp.T)
        Tt = csr_matrix(self.Tp.T)
        nblk = (n + bs - 1) // bs
        klk = np.zeros((nblk, bs, bs))
        tpt = np.zeros((nblk, bs, bs))
        spans = [(b * bs, min(n, (b + 1) * bs)) for b in range(nblk)]
        ksub = [Kt[a:z] for a, z in spans]
        branches = [np.unique(s.indices) for s in ksub]
        edges = [br[br < ne] for br in branches]
        Le = self.HL.dense_entries([(e, e) for e in edges], host=True)
        Lvia = self.Lvia.cpu().numpy()
        tsub = [Tt[a:z] for a, z in spans]
        nodes = [np.unique(s.indices) for s in tsub]
        Pn = self._node_blocks(nodes) if self.nn else [np.zeros((0, 0))] * nblk
        for b, ((a, z), ks, br, e, ts, nd) in enumerate(zip(spans, ksub, branches, edges, tsub, nodes)):
            Lb = np.zeros((len(br), len(br)))
            m = len(e)
            Lb[:m, :m] = Le[b]
            v = br[m:] - ne
            Lb[m:, m:] = Lvia[np.ix_(v, v)]
            Kb = ks[:, br].toarray()
            klk[b, :z - a, :z - a] = Kb @ Lb @ Kb.T
            if self.nn:
                Tb = ts[:, nd].toarray()
                tpt[b, :z - a, :z - a] = Tb @ Pn[b] @ Tb.T
        dev = self.device
        return torch.as_tensor(klk, device=dev), torch.as_tensor(tpt, device=dev)

    def _krk_blocks(self):
        bs, n = self.bs, self.n
        ptr, idx, val, shape = (v.cpu().numpy() if torch.is_tensor(v) else v for v in self._krk_device())
        M = csr_matrix((val, idx, ptr), shape=shape).tocoo()
        same = (M.row // bs) == (M.col // bs)
        nblk = (n + bs - 1) // bs
        out = np.zeros((nblk, bs, bs))
        out[M.row[same] // bs, M.row[same] % bs, M.col[same] % bs] = M.data[same]
        return torch.as_tensor(out, device=self.device)

    def _equilibrium(self, excitation, beside=False):
        """Baseline tree currents and the equilibrium charge of each drive (peec_iterative.solve:240-251).
        beside=True: a factorization is in flight on another stream, so P's solves must not use the cooperative
        triangular sweeps (they need the device to themselves)."""
        A, B = self.A, self.B
        sources = self.sources
        drive = np.asarray(A[:, sources] @ excitation)                 # (nn, ndrive)
        totals = self.source_components.T @ excitation                 # (nc, ndrive)
        qpart = np.zeros((self.nn, excitation.shape[1]), complex)
        vpart = np.zeros((B.shape[1], excitation.shape[1]), complex)
        if np.any(totals):
            if self._pinvb is None:
                t0 = time.perf_counter()
                self._pinvb = self._potential_solve(B.toarray(), precondition=2 if beside else 1)
                self._component = np.asarray(B.T @ self._pinvb)
                self.timings['potential_solve_s'] = time.perf_counter() - t0
            vpart = np.linalg.solve(self._component, -totals)
            qpart = self._pinvb @ vpart
        y0 = np.zeros((self.K.shape[1] - self.nl, excitation.shape[1]), complex)
        if self.tree_lu is not None:
            for c in range(excitation.shape[1]):
                y0[:, c] = self.tree_lu.solve((-drive[:, c] - qpart[:, c])[self.keep])
        baseline = np.asarray(self.K[:, self.nl:] @ y0)               # (nb, ndrive)
        source_voltage = -self.source_components @ vpart                # (nsrc, ndrive)
        return baseline, qpart, vpart, source_voltage

    def _potential_solve(self, rhs, precondition=1):
        """P^-1 rhs on the device (dense GMRES preconditioned by P's single-precision Cholesky factor, its solves by
        the streaming sweeps (1) or cuBLAS (2)), rhs (nn, k) real."""
        k = rhs.shape[1]
        b = torch.as_tensor(np.ascontiguousarray(rhs.astype(complex)), device=self.device)
        x = torch.zeros_like(b)
        its = np.zeros(k, np.int32)
        res = np.zeros(k)
        lib = _lib.load()
        if self.matrix == 'hierarchical':
            # Jacobi-preconditioned GMRES on the compressed P, through the live operator
            _lib.check(lib.pcbqs_gb300_peec_potential_gmres(
                self._live_handle, k, b.data_ptr(), x.data_ptr(), self.pdiag.data_ptr(), self.tol * 1e-2, 4000,
                self.restart, _lib.ptr(its, ctypes.c_int32), _lib.ptr(res),
                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), lib)
            self.timings['potential_solve_iterations'] = its.tolist()
            return x.cpu().numpy()
        Pim = self.Pim.data_ptr() if self.Pim is not None else None
        _lib.check(lib.pcbqs_gb300_dense_gmres(self.nn, self.P.data_ptr(), Pim, self.P.stride(0), k, b.data_ptr(),
                                               x.data_ptr(), self.tol * 1e-2, 4000, self.restart, precondition,
                                               _lib.ptr(its, ctypes.c_int32), _lib.ptr(res),
                                               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), lib)
        self.timings['potential_solve_iterations'] = its.tolist()
        return x.cpu().numpy()

    HM_COLUMNS = 64     # columns per compressed FP64 product (its blocks stage rank x columns in shared memory)

    def _mv_L(self, X):
        """L X for complex branch vectors X (ne, k), FP64 on the device (pcbqs_gb300_dense_apply, or the compressed
        product)."""
        if self.matrix == 'hierarchical':
            Xt = torch.as_tensor(np.ascontiguousarray(X, complex), device=self.device).reshape(self.ni, -1)
            Y = torch.empty_like(Xt)
            for c in range(0, Xt.shape[1], self.HM_COLUMNS):
                part = slice(c, c + self.HM_COLUMNS)
                Y[:self.ne, part] = self.HL.matmat(Xt[:self.ne, part])
            if self.board.nv:
                Y[self.ne:] = self.Lvia.to(torch.complex128) @ Xt[self.ne:]
            return Y.cpu().numpy().reshape(np.shape(X))
        return self._dense(self.L, X)

    def _mv_P(self, X):
        if self.matrix == 'hierarchical':
            Xt = torch.as_tensor(np.ascontiguousarray(X, complex), device=self.device).reshape(self.nn, -1)
            if getattr(self, '_papply', None) is None:
                self._papply = self.HP.potential_operator(self.board.node_of)
            Y = torch.cat([self._papply(Xt[:, c:c + self.HM_COLUMNS].contiguous())
                           for c in range(0, Xt.shape[1], self.HM_COLUMNS)], dim=1)
            return Y.cpu().numpy().reshape(np.shape(X))
        Y = self._dense(self.P, X)
        return Y if self.Pim is None else Y + 1j * self._dense(self.Pim, X)

    def _dense(self, M, X):
        """M X in FP64's accuracy: on the FP64 pipe below 4 columns, else from integer slices on the tensor cores
        (pcbqs_gb300_dense_apply_sliced, six slices)."""
        Xt = torch.as_tensor(np.ascontiguousarray(X, complex), device=self.device)
        shape = Xt.shape
        Xt = Xt.reshape(shape[0], -1)
        Y = torch.empty_like(Xt)
        lib = _lib.load()
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        if Xt.shape[1] >= 4:
            _lib.check(lib.pcbqs_gb300_dense_apply_sliced(M.shape[0], Xt.shape[1], M.data_ptr(), M.stride(0),
                                                          Xt.data_ptr(), Y.data_ptr(), 6, 1 << 31, stream), lib)
        else:
            _lib.check(lib.pcbqs_gb300_dense_apply(M.shape[0], Xt.shape[1], M.data_ptr(), M.stride(0), Xt.data_ptr(),
                                                   Y.data_ptr(), stream), lib)
        return Y.cpu().numpy().reshape(shape)

    PRECONDITIONERS = {'none': 0, 'block_jacobi': 1, 'lu32': 2, 'graph': 3}

    def resistance_ratio(self, freqs):
        """R(f) / R_dc per frequency: 1 for conductor_loss='dc'; for 'slab' the finite-thickness sheet impedance
        Zs(f) sigma t of the copper (current entering from one or both faces), so R(f) = ratio R_dc for the
        single-sheet model (MQS._resistance_delta, src/pcbqs/mqs.py:517-530; surface_impedance,
        src/pcbqs/conductor.py:12-26)."""
        f = np.atleast_1d(np.asarray(freqs, float))
        if self.conductor_loss == 'dc':
            return np.ones(len(f), complex)
        sigma, t = float(self.board.sigma), float(self.board.thickness)
        u = np.sqrt(2j * np.pi * f * MU0 * sigma) * t / self.conductor_faces
        small = np.abs(u) < 1e-3
        safe = np.where(small, 1.0, u)
        return np.where(small, 1 + u * u / 3 - u ** 4 / 45, safe / np.tanh(safe)).astype(complex)

    def _factor_async(self, handle, sys_index, math):
        """Start pcbqs_gb300_peec_factor for system `sys_index` on a side stream from a helper thread; the returned
        future yields its device time (ms) or raises its error. L, P and the handle's operator must be complete."""
        lib = _lib.load()
        if getattr(self, '_side', None) is None:
            self._side = torch.cuda.Stream(self.device)
            self._pool = concurrent.futures.ThreadPoolExecutor(max_workers=1, thread_name_prefix='pcbqs-factor')
        side = self._side
        desc = _csr_struct(self._krk_device())
        torch.cuda.current_stream(self.device).synchronize()

        def work():
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(side)
            status = lib.pcbqs_gb300_peec_factor(handle, ctypes.byref(desc), sys_index, math,
                                                 ctypes.c_void_p(side.cuda_stream))
            e1.record(side)
            side.synchronize()
            _lib.check(status, lib)
            return e0.elapsed_time(e1)
        return self._pool.submit(work)

    FACTOR_MATH = {'fp32': 0, 'bf16x9': 1, 'bf16x9-blocked': 2, 'fp32-blocked': 3, 'tc3-blocked': 4,
                   'tc6-blocked': 5}

    PRODUCT = {'fp32': 0, 'tc3': 3, 'tc6': 6}
    FP64_PRODUCT = {'fp64': 0, 'sliced5': 5, 'sliced6': 6, 'sliced7': 7}

    def _graph_device(self):
        """The graph preconditioner's structure (graph_structure) on the device, uploaded once per model."""
        gd = self.__dict__.get('_graph_dev')
        if gd is None:
            g, dev = self.graph_structure(), self.device
            up = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
            gd = dict(ac=_dev_csr(g['ac'], dev), tinv=_dev_csr(g['tinv'], dev), tinvt=_dev_csr(g['tinvt'], dev),
                      **{name: up(g[name]) for name in ('lap_ptr', 'lap_branch', 'lap_other', 'branch', 'loop_ends',
                                                        'comp', 'member_ptr', 'members')})
            self._graph_dev = gd
        return gd

    def _graph_domains_device(self, parts):
        """The domain split (graph_domains) as its C struct over device arrays, uploaded once per part count."""
        cache = self.__dict__.setdefault('_graph_dom_dev', {})
        if parts not in cache:
            dm = self.graph_domains(parts)
            up = lambda a: torch.as_tensor(np.ascontiguousarray(a if len(a) else np.zeros(1, a.dtype)),
                                           device=self.device)
            arrays = {name: up(dm[name]) for name in ('perm', 'pos', 'bnd', 'bnd_nptr', 'bnd_local', 'bnd_branch')}
            host = {name: np.ascontiguousarray(dm[name], np.int64) for name in ('dom_ptr', 'bnd_ptr')}
            desc = _lib.GraphDomainsDesc()
            desc.parts, desc.n_int = dm['parts'], dm['n_int']
            for name, t in arrays.items():
                setattr(desc, name, t.data_ptr())
            for name, a in host.items():
                setattr(desc, name, a.ctypes.data)
            cache[parts] = (desc, arrays, host)
        return cache[parts][0]

    def _graph_precondition(self, handle, sys_index, freq, refine, stream, parts=0):
        """Set up the graph preconditioner of system sys_index (frequency freq) in the live operator: the branches'
        own impedance d = r(f) R_ii + j w L_ii (the via barrels at their DC resistance, as in the operator), 1/d with
        |d| raised to 1e-12 zscale where smaller (peec_iterative.py:52), and 1/P_ii with its per-component sums
        (peec_iterative.py:29-30)."""
        g, gd = self.graph_structure(), self._graph_device()
        lib = _lib.load()
        zs = float(self._zscale[sys_index])
        rd = np.asarray(self.R.diagonal(), complex)
        rd[:self.ne] *= self.resistance_ratio([freq])[0]
        zdiag = rd + 1j * 2 * np.pi * freq * np.asarray(self.ldiag[:self.ni], float)
        d = zdiag.copy()
        d[np.abs(d) < zs * 1e-12] = zs * 1e-12
        pinv = 1 / np.asarray(self.pdiag_host, complex)
        total = (np.bincount(self.labels, pinv.real, minlength=g['ncomp']) +
                 1j * np.bincount(self.labels, pinv.imag, minlength=g['ncomp']))
        vals = {name: torch.as_tensor(np.ascontiguousarray(a, complex), device=self.device)
                for name, a in (('zdiag', zdiag), ('dinv', 1 / d), ('pinv', pinv[g['kept']]), ('total', total))}
        desc = _lib.GraphDesc()
        desc.nkeep, desc.ncomp, desc.nbranch = g['nkeep'], g['ncomp'], self.ni
        for name in ('ac', 'tinv', 'tinvt'):
            setattr(desc, name, _csr_struct(gd[name]))
        for name in ('lap_ptr', 'lap_branch', 'lap_other', 'branch', 'loop_ends', 'comp', 'member_ptr', 'members'):
            setattr(desc, name, gd[name].data_ptr())
        for name, t in vals.items():
            setattr(desc, name, t.data_ptr())
        desc.domains = ctypes.pointer(self._graph_domains_device(parts)) if parts else None
        _lib.check(lib.pcbqs_gb300_peec_graph(handle, ctypes.byref(desc), int(sys_index), int(refine), stream), lib)

    @classmethod
    def solve_options(cls, matrix, freqs, precondition, mixed, factor_math, anchors, captured, product, fp64_product,
                      graph_parts, graph_refine):
        """The checks of solve's options, made before any device work: (frequencies, preconditioner mode, anchors,
        fp64_product) with the defaults filled in; ValueError for an invalid one."""
        f = np.atleast_1d(np.asarray(freqs, float))
        if f.ndim != 1 or not len(f) or not np.isfinite(f).all() or (f <= 0).any():
            raise ValueError('frequencies must be finite and positive')
        if precondition not in cls.PRECONDITIONERS:
            raise ValueError(f'precondition must be one of {sorted(cls.PRECONDITIONERS)}')
        if factor_math not in cls.FACTOR_MATH:
            raise ValueError(f'factor_math must be one of {sorted(cls.FACTOR_MATH)}')
        if product not in cls.PRODUCT:
            raise ValueError(f'product must be one of {sorted(cls.PRODUCT)}')
        if fp64_product is None:
            fp64_product = 'sliced6' if mixed else 'fp64'
        if fp64_product not in cls.FP64_PRODUCT:
            raise ValueError(f'fp64_product must be one of {sorted(cls.FP64_PRODUCT)}')
        if matrix == 'hierarchical' and precondition == 'lu32':
            raise ValueError("the compressed operator solves with precondition 'block_jacobi', 'graph' or 'none'")
        if anchors is None:
            anchors = len(f)
        if not isinstance(anchors, (int, np.integer)) or isinstance(anchors, bool) or not 1 <= anchors <= len(f):
            raise ValueError('anchors must be an integer between 1 and the number of frequencies')
        if graph_parts is not None and (not isinstance(graph_parts, (int, np.integer)) or isinstance(graph_parts, bool)
                                        or (graph_parts != 0 and (graph_parts < 2 or graph_parts & (graph_parts - 1)))):
            raise ValueError('graph_parts must be 0 (dense) or a power of two >= 2')
        if graph_refine is not None and (not isinstance(graph_refine, (int, np.integer))
                                         or isinstance(graph_refine, bool) or not 0 <= graph_refine <= 3):
            raise ValueError('graph_refine must be an integer in 0..3')
        if captured and graph_parts and precondition == 'graph':
            raise ValueError('captured GMRES cycles need the dense graph Laplacian (graph_parts=0)')
        return f, cls.PRECONDITIONERS[precondition], int(anchors), fp64_product

    def solve(self, freqs, precondition='block_jacobi', mixed=False, factor_math='tc6-blocked', anchors=None,
              captured=False, product='tc3', fp64_product=None, graph_parts=None, graph_refine=None):
        """Port impedance matrix (nf, np, np): column j drives port j with 1 A (the others 0).

        precondition: 'block_jacobi' (geometric blocks of the loop/tree unknowns), 'lu32' (the complex64 LU of the
        dense loop/tree system), 'graph' (the reference's graph preconditioner, peec_iterative.py:44-84: loop
        currents from the branches' graph Laplacian, factored on the device in complex64: dense up to about 44,700
        nodes, else (or graph_parts, a power of two) split into domains with explicit inverses and a dense Schur
        complement on their separator; graph_refine FP64 corrections of each Laplacian solve (default 1 dense, 2
        split); tree charges through the spanning forest's explicit inverse; dense or compressed operator), or
        'none'. mixed=False: FP64 GMRES on the FP64 operator;
        mixed=True: FP64 iterative refinement (true residuals with the FP64 operator) around an inner GMRES whose
        dense products run in single precision, both to the same 1e-8 relative residual. factor_math: arithmetic of the 'lu32'
        factorization: 'fp32' or 'bf16x9' (FP32 emulated on the tensor cores, same accuracy) through cuSOLVER's getrf;
        through this library's blocked LU (2048-column panels factored ahead of the trailing updates) 'fp32-blocked'
        or 'bf16x9-blocked' with cuBLAS trailing GEMMs, or 'tc6-blocked' (the default) / 'tc3-blocked' with this
        library's tcgen05 update on six / three BF16 part products (six: FP32's accuracy; three: about 16 bits, a
        weaker preconditioner that costs GMRES steps). anchors ('lu32'
        and 'graph'): how many factorizations a sweep shares; the frequencies, in increasing order, are split into that
        many runs and every run is solved as one batch of (frequency, port) columns preconditioned by the factor
        at its middle frequency (default: one factor per frequency). Every column still reaches the tolerance of
        its own frequency's FP64 system; farther from the anchor it takes more iterations. captured=True: each GMRES
        restart cycle is one CUDA graph launch (its Arnoldi steps in a device-controlled conditional loop, no host
        synchronization between steps; pcbqs_gb300_peec_set_captured), with the same results. product (mixed only):
        the inner dense products over 16 or more columns on the tensor cores with three ('tc3', the default) or six
        ('tc6') BF16 part products, or 'fp32' on the CUDA cores throughout (pcbqs_gb300_peec_set_product); the FP64
        refinement holds the answer to the same tolerance either way. fp64_product: the FP64 operator's dense
        products over 4 or more columns (the mixed solve's outer residuals, the FP64 GMRES): 'fp64' on the FP64 pipe,
        or 'sliced6' (5, 7) on the tensor cores from integer slices at FP64's accuracy
        (pcbqs_gb300_peec_set_fp64_product); default 'sliced6' for mixed=True, 'fp64' (the plain path) otherwise."""
        f, mode, anchors, fp64_product = self.solve_options(self.matrix, freqs, precondition, mixed, factor_math,
                                                            anchors, captured, product, fp64_product, graph_parts,
                                                            graph_refine)
        if self.L is None and self.HL is None:
            self.assemble()
        nf = len(f)
        parts = self._graph_parts(graph_parts) if mode == 3 else 0
        refine = (2 if parts else 1) if graph_refine is None else int(graph_refine)
        if parts and captured:
            raise ValueError('captured GMRES cycles need the dense graph Laplacian (graph_parts=0)')
        t0 = time.perf_counter()
        npo = len(self.names)
        excitation = np.eye(npo, dtype=complex)
        omegas = 2 * np.pi * f
        handle, zscale = self._operator(omegas)
        if mode in (2, 3):
            runs = np.array_split(np.argsort(f, kind='stable'), anchors)
            groups = [(int(run[len(run) // 2]), run) for run in runs]
        else:
            groups = [(None, np.arange(nf))]
        lib = _lib.load()
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        timed = lambda: (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        precondition_ms = gmres_ms = 0.0
        stage_ms = np.zeros(2)             # the factorizations' assembly and LU times
        updates = np.zeros(3)              # their tcgen05 trailing updates: ms, complex flops, launches
        outer_total = 0
        factored = None

        def factor_stages():
            a, b = ctypes.c_double(), ctypes.c_double()
            _lib.check(lib.pcbqs_gb300_peec_factor_times(handle, ctypes.byref(a), ctypes.byref(b)), lib)
            stage_ms[:] += (a.value, b.value)
            c = ctypes.c_int32()
            _lib.check(lib.pcbqs_gb300_peec_factor_updates(handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
                       lib)
            updates[:] += (a.value, b.value, c.value)
        try:
            _lib.check(lib.pcbqs_gb300_peec_set_captured(handle, int(bool(captured))), lib)
            _lib.check(lib.pcbqs_gb300_peec_set_product(handle, self.PRODUCT[product]), lib)
            _lib.check(lib.pcbqs_gb300_peec_set_fp64_product(handle, self.FP64_PRODUCT[fp64_product]), lib)
            t1 = time.perf_counter()
            if mode == 2:
                # the first complex64 factorization depends only on L, P and the frequency: it runs on a side
                # stream from a helper thread while this thread solves for the equilibrium charge and forms the
                # right-hand sides and the single-precision copies (the ctypes calls release the interpreter lock).
                # Meanwhile nothing here may launch the cooperative triangular sweeps: the equilibrium solve uses
                # cuBLAS triangular solves instead.
                factored = self._factor_async(handle, groups[0][0], self.FACTOR_MATH[factor_math])
            if mode == 2:
                # at the device's highest priority, so its short dependent kernels are not queued behind the
                # factorization's GEMMs
                if getattr(self, '_urgent', None) is None:
                    self._urgent = torch.cuda.Stream(self.device, priority=-1)
                self._urgent.wait_stream(torch.cuda.current_stream(self.device))
                with torch.cuda.stream(self._urgent):
                    baseline, qpart, vpart, source_voltage = self._equilibrium(excitation, beside=True)
                torch.cuda.current_stream(self.device).wait_stream(self._urgent)
            else:
                baseline, qpart, vpart, source_voltage = self._equilibrium(excitation)
            t2 = time.perf_counter()
            self.timings.update(equilibrium_s=t2 - t1, operator_setup_s=t1 - t0)
            # rhs = -K^T (R + j w L) baseline / zscale, per (frequency, port) column, in the clustered order.
            Lb = self._mv_L(baseline[:self.ni])
            Rb = self.R @ baseline[:self.ni]
            Rv = np.zeros_like(Rb)             # the via barrels' part keeps its DC value
            Rv[self.ne:] = Rb[self.ne:]
            Rb[self.ne:] = 0
            Kpt = self.Kp.T
            ratio = self.resistance_ratio(f)
            cols = [-(Kpt @ (ratio[fi] * Rb + Rv + 1j * w * Lb)) / zscale[fi] for fi, w in enumerate(omegas)]
            rhs = np.ascontiguousarray(np.concatenate(cols, axis=1))      # (n, nf * np), column fi * np + port
            self.timings['rhs_s'] = time.perf_counter() - t2
            b_all = torch.as_tensor(rhs, device=self.device)
            x_all = torch.zeros_like(b_all)
            k_all = rhs.shape[1]
            its, res = np.zeros(k_all, np.int32), np.zeros(k_all)
            if mode == 1:
                e0, e1 = timed()
                e0.record()
                if self.matrix == 'hierarchical':
                    if getattr(self, '_nearblk', None) is None:
                        self._nearblk = self._near_blocks()
                    klk, tpt = self._nearblk
                    _lib.check(lib.pcbqs_gb300_peec_block_jacobi_blocks(handle, self.bs, self._krk_blocks().data_ptr(),
                                                                        klk.data_ptr(), tpt.data_ptr(), stream), lib)
                else:
                    _lib.check(lib.pcbqs_gb300_peec_block_jacobi(handle, self.bs, self._krk_blocks().data_ptr(),
                                                                 stream), lib)
                e1.record()
                torch.cuda.synchronize()
                precondition_ms += e0.elapsed_time(e1)
            if mode == 3:
                # the graph preconditioner's host structure and its upload: once per model (and part count)
                t3 = time.perf_counter()
                self._graph_device()
                if parts:
                    self._graph_domains_device(parts)
                self.timings['graph_host_s'] = time.perf_counter() - t3
            if mixed and self.matrix == 'hierarchical':
                # the inner products: the H-matrices' blocks, low rank and dense, in BF16 on the tensor cores
                t3 = time.perf_counter()
                for which, H in ((0, self.HL), (1, self.HP)):
                    plans = H.__dict__.setdefault('_plans', {})
                    if True not in plans:
                        plans[True] = H.lowrank_plan(dense=True)
                    if plans[True] is not None:
                        _lib.check(lib.pcbqs_gb300_peec_set_lowrank(handle, which, ctypes.byref(plans[True][1])), lib)
                self.timings['lowrank_plan_s'] = time.perf_counter() - t3
            elif mixed:
                # single-precision copies of L and P for the inner products; FP64 outer residuals
                Lf, Pf = self.Lf, self.Pf
                if Lf is None:
                    Lf = torch.empty(self.L.shape, dtype=torch.float32, device=self.device)
                    Pf = torch.empty(self.P.shape, dtype=torch.float32, device=self.device)
                    _lib.check(lib.pcbqs_gb300_to_single(self.L.data_ptr(), Lf.data_ptr(), self.L.numel(), stream),
                               lib)
                    _lib.check(lib.pcbqs_gb300_to_single(self.P.data_ptr(), Pf.data_ptr(), self.P.numel(), stream),
                               lib)
                if self.Pim is not None and self.Pfim is None:
                    self.Pfim = torch.empty(self.Pim.shape, dtype=torch.float32, device=self.device)
                    _lib.check(lib.pcbqs_gb300_to_single(self.Pim.data_ptr(), self.Pfim.data_ptr(), self.Pim.numel(),
                                                         stream), lib)
            if factored is not None:
                precondition_ms += factored.result()
                factored = None
                factor_stages()
            if mixed and self.matrix != 'hierarchical':
                Pfim = self.Pfim.data_ptr() if self.Pfim is not None else None
                _lib.check(lib.pcbqs_gb300_peec_single(handle, Lf.data_ptr(), Lf.stride(0), Pf.data_ptr(), Pfim,
                                                       Pf.stride(0)), lib)
            converged = True
            for g, (anchor, members) in enumerate(groups):
                if mode == 3:
                    e0, e1 = timed()
                    e0.record()
                    self._graph_precondition(handle, anchor, f[anchor], refine, stream, parts)
                    e1.record()
                    torch.cuda.synchronize()
                    precondition_ms += e0.elapsed_time(e1)
                if mode == 2 and g > 0:
                    e0, e1 = timed()
                    e0.record()
                    desc = _csr_struct(self._krk_device())
                    _lib.check(lib.pcbqs_gb300_peec_factor(handle, ctypes.byref(desc), anchor,
                                                           self.FACTOR_MATH[factor_math], stream), lib)
                    e1.record()
                    torch.cuda.synchronize()
                    precondition_ms += e0.elapsed_time(e1)
                    factor_stages()
                sel = (np.asarray(members)[:, None] * npo + np.arange(npo)).ravel()
                whole = len(sel) == k_all
                b = b_all if whole else b_all[:, torch.as_tensor(sel, device=self.device)].contiguous()
                x = x_all if whole else torch.zeros_like(b)
                k = len(sel)
                sys = np.ascontiguousarray(np.repeat(np.asarray(members), npo), np.int32)
                its_g, res_g = np.zeros(k, np.int32), np.zeros(k)
                e0, e1 = timed()
                e0.record()
                if mixed:
                    outer = ctypes.c_int32()
                    status = lib.pcbqs_gb300_peec_solve_mixed(handle, k, _lib.ptr(sys, ctypes.c_int32), b.data_ptr(),
                                                              x.data_ptr(), self.tol, self.inner_tol, 12,
                                                              self.maxiter, self.restart, mode,
                                                              _lib.ptr(its_g, ctypes.c_int32), _lib.ptr(res_g),
                                                              ctypes.byref(outer), stream)
                    outer_total = max(outer_total, int(outer.value))
                else:
                    status = lib.pcbqs_gb300_peec_gmres(handle, k, _lib.ptr(sys, ctypes.c_int32), b.data_ptr(),
                                                        x.data_ptr(), self.tol, self.maxiter, self.restart, mode,
                                                        _lib.ptr(its_g, ctypes.c_int32), _lib.ptr(res_g), stream)
                e1.record()
                torch.cuda.synchronize()
                gmres_ms += e0.elapsed_time(e1)
                if status not in (0, 5):
                    _lib.check(status, lib)
                converged = converged and status == 0
                if not whole:
                    x_all[:, torch.as_tensor(sel, device=self.device)] = x
                its[sel], res[sel] = its_g, res_g
            self.timings.update(precondition_ms=precondition_ms, gmres_ms=gmres_ms, gmres_iterations=its.tolist(),
                                factorizations=len(groups) if mode in (2, 3) else 0, factor_assemble_ms=stage_ms[0],
                                factor_lu_ms=stage_ms[1], factor_update_ms=updates[0],
                                factor_update_flops=updates[1], factor_update_launches=int(updates[2]))
            if mixed:
                self.timings['outer_steps'] = outer_total
            X = x_all.cpu().numpy()
        finally:
            if factored is not None:        # an error above: let the factorization finish before the handle goes
                try:
                    factored.result()
                except Exception:  # noqa: BLE001 -- the first error is the one raised
                    pass
            lib.pcbqs_gb300_peec_destroy(handle)
        # back to the unclustered order, then currents, charges and source voltages (peec_iterative.py:331-341), for
        # every (frequency, port) column at once: one P product over all of them
        t4 = time.perf_counter()
        Xo = np.empty_like(X)
        Xo[self.order] = X
        Z = np.zeros((len(f), npo, npo), complex)
        currents = np.zeros((len(f), self.nb, npo), complex)
        Kc, Kt = self.K[:, :self.nl], self.K[:, self.nl:]
        correction = Xo[self.nl:] * np.repeat(zscale / self.pscale, npo)[None]
        pcorrection = self._mv_P(np.asarray(self.T @ correction))
        voltages = np.asarray(self.A[:, self.sources].T @ pcorrection)
        loop_part = np.asarray(Kc @ Xo[:self.nl])
        tree_part = np.asarray(Kt @ correction)
        for fi, w in enumerate(omegas):
            cols = slice(fi * npo, (fi + 1) * npo)
            currents[fi] = baseline + loop_part[:, cols] + 1j * w * tree_part[:, cols]
            currents[fi][self.sources] = excitation
            Z[fi] = source_voltage / (1j * w) + voltages[:, cols]
        self.timings['post_s'] = time.perf_counter() - t4
        self.timings['solve_s'] = time.perf_counter() - t0
        if not converged:
            raise RuntimeError(f'GMRES did not reach {self.tol:g}: residuals {res.max():.3g}, iterations {its.max()}')
        return PeecResult(f, self.names, Z, currents, its, res, dict(self.timings))
