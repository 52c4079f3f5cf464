"""Pure-Python restatement of the PEEC spanning forest and loop basis, the oracle the tests hold the native
pcbqs_gb300_loop_basis to, and of the graph preconditioner, the oracle for pcbqs_gb300_peec_graph (test
infrastructure only: nothing in the package imports this module).

Follows src/pcbqs/mqs.py:48-130 (spanning_tree: breadth-first forest from each island's most central node, other
branches only joining islands), src/pcbqs/mqs.py:592-637 (_loops: each non-tree branch's fundamental cycle) and
src/pcbqs/peec_iterative.py:19-84 (_tree_preconditioner, _graph_preconditioner; boards without face-sheet pairs).
"""
import collections

import numpy as np
from scipy.sparse import coo_matrix, diags
from scipy.sparse.linalg import splu


def spanning_tree(n_nodes, ends, is_src, first=None):
    """(tree, comp, up, upb, ups, depth) of the branches `ends` excluding sources: the first `first` branches
    (copper) as a breadth-first forest from each island's most central node (the middle of a double sweep's
    longest path), the remaining non-source branches only joining islands the copper leaves apart."""
    nb = len(ends)
    first = nb if first is None else first
    adj = [[] for _ in range(n_nodes)]
    for k in range(first):
        a, b = ends[k]
        if not is_src[k] and a != b:
            adj[a].append((b, k))
            adj[b].append((a, k))
    tree = np.zeros(nb, bool)

    def sweep(root):
        dist = {root: 0}
        queue = collections.deque([root])
        order = [root]
        while queue:
            u = queue.popleft()
            for v, _ in adj[u]:
                if v not in dist:
                    dist[v] = dist[u] + 1
                    queue.append(v)
                    order.append(v)
        return order, dist
    seen = np.zeros(n_nodes, bool)
    for s in range(n_nodes):
        if seen[s]:
            continue
        order, _ = sweep(s)
        seen[order] = True
        root = s
        if len(order) > 2:
            _, d1 = sweep(order[-1])
            _, d2 = sweep(max(d1, key=d1.get))
            root = min(order, key=lambda v: max(d1[v], d2[v]))
        mark = {root}
        queue = collections.deque([root])
        while queue:
            u = queue.popleft()
            for v, k in adj[u]:
                if v not in mark:
                    mark.add(v)
                    tree[k] = True
                    queue.append(v)
    parent = list(range(n_nodes))

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a
    for k in np.flatnonzero(tree):
        a, b = ends[k]
        parent[find(b)] = find(a)
    for k in range(first, nb):
        a, b = ends[k]
        if not is_src[k] and find(a) != find(b):
            parent[find(b)] = find(a)
            tree[k] = True
    tadj = [[] for _ in range(n_nodes)]
    for k in np.flatnonzero(tree):
        a, b = ends[k]
        tadj[a].append((b, k))
        tadj[b].append((a, k))
    up = np.full(n_nodes, -1)
    upb = np.full(n_nodes, -1)
    ups = np.zeros(n_nodes, int)
    depth = np.full(n_nodes, -1)
    comp = np.full(n_nodes, -1)
    for root in range(n_nodes):
        if depth[root] >= 0:
            continue
        depth[root] = 0
        comp[root] = root
        stack = [root]
        while stack:
            u = stack.pop()
            for v, k in tadj[u]:
                if depth[v] < 0:
                    depth[v], up[v], upb[v], comp[v] = depth[u] + 1, u, k, root
                    ups[v] = 1 if ends[k][0] == u else -1
                    stack.append(v)
    return tree, comp, up, upb, ups, depth


def loop_basis(n_nodes, ends, is_src, n_rwg, ideal_terminals=True):
    """(C (nb x ncol) csc, src_cols {branch: col}, tree, col_branch): each non-tree branch's fundamental cycle,
    oriented with the branch (col_branch[c] is column c's branch); copper edges inside one node are no loop (ideal
    terminals); branches whose ends lie on islands joined only through them have none."""
    nb = len(ends)
    tree, comp, up, upb, ups, depth = spanning_tree(n_nodes, ends, is_src, n_rwg)
    rows, cols, vals, src_cols, col_branch = [], [], [], {}, []
    col = 0
    for k in np.flatnonzero(~tree):
        a, b = ends[k]
        if a == b and k < n_rwg and ideal_terminals:
            continue
        if comp[a] != comp[b]:
            continue
        u, v = b, a
        pu, pv = [], []
        while depth[u] > depth[v]:
            pu.append((upb[u], -ups[u]))
            u = up[u]
        while depth[v] > depth[u]:
            pv.append((upb[v], ups[v]))
            v = up[v]
        while u != v:
            pu.append((upb[u], -ups[u]))
            u = up[u]
            pv.append((upb[v], ups[v]))
            v = up[v]
        rows.append(k)
        cols.append(col)
        vals.append(1.0)
        for kb, sg in pu + pv[::-1]:
            rows.append(kb)
            cols.append(col)
            vals.append(float(sg))
        if is_src[k]:
            src_cols[k] = col
        col_branch.append(int(k))
        col += 1
    C = coo_matrix((vals, (rows, cols)), shape=(nb, col)).tocsc()
    return C, src_cols, tree, np.asarray(col_branch, np.int64)


def graph_preconditioner(K, A, T, B, nl, keep, passive, cotree, diagonal, zscale, pscale, pdiag):
    """apply(y) of the reference's graph preconditioner in its own unknown order (the nl loops, then the tree
    branches), with exact sparse LU factors (SuperLU) where the reference takes an incomplete LU of the Laplacian
    with drop tolerance 1e-6: K (branches x unknowns) the loop/tree basis, A (nodes x branches) the incidence,
    T = A K[:, nl:], B (nodes x components) the component indicator, keep the non-root nodes, passive the passive
    branches, cotree each loop's defining branch, diagonal (branches) each branch's own impedance, zscale / pscale
    the system's scales, pdiag P's diagonal. peec_iterative.py:44-84 (the loop part) over :19-42 (the charge tree)."""
    Kc, Kt = K[:, :nl], K[:, nl:]
    position = np.full(A.shape[1], -1)
    position[passive] = np.arange(len(passive))
    d = np.asarray(diagonal)[passive].astype(complex)
    d[np.abs(d) < zscale * 1e-12] = zscale * 1e-12
    Ap = A[:, passive]
    Dinv = diags(1 / d).tocsr()
    Zb = diags(np.asarray(diagonal, complex)).tocsc()
    laplacian = splu((Ap @ Dinv @ Ap.T).tocsc()[keep][:, keep].tocsc())
    tree_lu = splu(T[keep].astype(complex).tocsc())
    inverse = 1 / np.asarray(pdiag, complex)
    total = np.asarray(B.T @ inverse).ravel()

    def apply(y):
        force = np.zeros(A.shape[1], complex)
        force[cotree] = zscale * y[:nl]
        trial = Dinv @ force[passive]
        voltage = np.zeros(A.shape[0], complex)
        voltage[keep] = laplacian.solve(np.asarray(Ap @ trial).ravel()[keep])
        loop = (trial - Dinv @ (Ap.T @ voltage))[position[cotree]]
        rhs = np.array(y, complex)
        rhs[nl:] -= np.asarray(Kt.T @ (Zb @ (Kc @ loop))).ravel() / zscale
        v = np.zeros(T.shape[0], complex)
        v[keep] = tree_lu.solve(rhs[nl:], trans='T')
        common = np.asarray(B.T @ (inverse * v)).ravel() / total
        charge = inverse * (v - B @ common)
        out = np.empty(K.shape[1], complex)
        out[nl:] = pscale * tree_lu.solve(charge[keep])
        out[:nl] = loop
        return out
    return apply
