"""The graph preconditioner's host-built structure (PeecTopology.graph_structure: kept-node rows, the loops' node
incidence, the Laplacian's edge lists, the spanning forest's explicit inverse, the components) against the
oracle's restatement of the reference's graph preconditioner (oracle/graph.py, src/pcbqs/peec_iterative.py:19-84),
on the CPU: the device kernels' steps replayed in numpy from the structure give the reference's output to rounding,
and the explicit inverse is T[keep]^-1."""
import numpy as np
import pytest
from scipy.sparse import csr_matrix


def _topology(board):
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecTopology
    from pcbqs_gb300.rwg import RWG
    b = Board.load(board)
    return PeecTopology(b, RWG(b.nodes, b.tris))


def _csr(h):
    ptr, idx, val, shape = h
    return csr_matrix((val, idx, ptr), shape=shape)


def _kernel_steps(t, g, zdiag, dinv, zs, ps, pinv_keep, total, y):
    """The steps of the device preconditioner (k_graph_* in csrc/peec_op.cu) in numpy, the Laplacian solved
    densely."""
    is_tree = t.is_tree.astype(bool)
    br, nk = g['branch'], g['nkeep']
    ac, tinv, tinvt = _csr(g['ac']), _csr(g['tinv']), _csr(g['tinvt'])
    tw = np.where(is_tree, 0, zs * dinv[br])
    rhs = ac @ (tw * y)
    rows = np.repeat(np.arange(nk), np.diff(g['lap_ptr']))
    w = dinv[g['lap_branch']]
    G = csr_matrix((w, (rows, rows)), shape=(nk, nk)).toarray()
    m = g['lap_other'] >= 0
    G -= csr_matrix((w[m], (rows[m], g['lap_other'][m])), shape=(nk, nk)).toarray()
    v = np.linalg.solve(G, rhs)
    out = np.zeros(t.n, complex)
    loops = ~is_tree
    ka, kb = g['loop_ends'][:, 0], g['loop_ends'][:, 1]
    va = np.where(ka >= 0, v[np.maximum(ka, 0)], 0)
    vb = np.where(kb >= 0, v[np.maximum(kb, 0)], 0)
    out[loops] = (tw * y - dinv[br] * (va - vb))[loops]
    current = t.Kp.tocsr()[:, loops] @ out[loops]
    rt = np.zeros(t.n, complex)
    rt[is_tree] = (y - zdiag[br] / zs * current[br])[is_tree]
    v2 = tinvt @ rt
    mp, mem = g['member_ptr'], g['members']
    common = np.array([np.sum(pinv_keep[mem[mp[c]:mp[c + 1]]] * v2[mem[mp[c]:mp[c + 1]]])
                       for c in range(g['ncomp'])]) / total
    charge = pinv_keep * (v2 - common[g['comp']])
    out[is_tree] = ps * (tinv @ charge)[is_tree]
    return out


@pytest.mark.parametrize('board', ['tiny', 'strip', 'viapair'])
def test_graph_structure_replays_the_reference_preconditioner(board):
    import oracle.graph as G
    t = _topology(board)
    g = t.graph_structure()
    rng = np.random.default_rng(7)
    ni = t.ni
    diagonal = np.r_[rng.uniform(0.5, 2, ni) + 1j * rng.uniform(0.1, 5, ni), np.zeros(t.nb - ni)]
    zs, ps = float(np.abs(diagonal).max()), 3.7
    pdiag = rng.uniform(1, 2, t.nn)
    apply = G.graph_preconditioner(t.K, t.A, t.T, t.B, t.nl, t.keep, t.passive, t.own[:t.nl], diagonal, zs, ps, pdiag)
    d = diagonal[:ni].copy()
    d[np.abs(d) < zs * 1e-12] = zs * 1e-12
    pinv = 1 / pdiag
    total = np.bincount(t.labels, pinv, minlength=g['ncomp']).astype(complex)
    for _ in range(2):
        y = rng.standard_normal(t.n) + 1j * rng.standard_normal(t.n)
        ref = apply(y)
        got = _kernel_steps(t, g, diagonal[:ni], 1 / d, zs, ps, pinv[g['kept']], total, y[t.order])
        assert np.abs(got - ref[t.order]).max() <= 1e-11 * np.abs(ref).max()


@pytest.mark.parametrize('board', ['tiny', 'viapair'])
def test_explicit_tree_inverse_is_the_inverse(board):
    t = _topology(board)
    g = t.graph_structure()
    is_tree = t.is_tree.astype(bool)
    Tk = t.Tp.tocsr()[g['kept']][:, np.flatnonzero(is_tree)]       # kept nodes x tree unknowns (clustered)
    tinv = _csr(g['tinv'])[np.flatnonzero(is_tree)]
    eye = (tinv @ Tk).toarray()
    assert np.array_equal(eye, np.eye(g['nkeep']))
    assert np.array_equal(_csr(g['tinvt']).toarray()[:, is_tree], tinv.T.toarray())
    assert g['member_ptr'][-1] == g['nkeep'] and len(g['comp']) == g['nkeep']
    assert (g['keep_row'] >= 0).sum() == g['nkeep']


@pytest.mark.parametrize('board,parts', [('tiny', 4), ('strip', 8), ('viapair', 4)])
def test_domain_split_solves_the_laplacian(board, parts):
    """PeecTopology.graph_domains: no Laplacian edge joins two domains' interiors; the Schur complement built from
    the boundary lists as k_schur_domain builds it equals G_SS - G_SI A_I^-1 G_IS; and the two-stage solve
    (y_I = A_I^-1 r_I, x_S = S^-1 (r_S - G_SI y_I), x_I = y_I - A_I^-1 G_IS x_S) is G^-1 r."""
    t = _topology(board)
    g = t.graph_structure()
    dm = t.graph_domains(parts)
    nk, ni_, ns = g['nkeep'], dm['n_int'], dm['n_sep']
    rng = np.random.default_rng(5)
    dinv = rng.uniform(0.5, 2, t.ni) + 1j * rng.uniform(-3, -0.1, t.ni)
    rows = np.repeat(np.arange(nk), np.diff(g['lap_ptr']))
    w = dinv[g['lap_branch']]
    G = csr_matrix((w, (rows, rows)), shape=(nk, nk)).toarray()
    m = g['lap_other'] >= 0
    G -= csr_matrix((w[m], (rows[m], g['lap_other'][m])), shape=(nk, nk)).toarray()
    perm, dp = dm['perm'], dm['dom_ptr']
    Gn = G[perm][:, perm]
    part_of = np.full(nk, parts)
    for d in range(parts):
        part_of[dp[d]:dp[d + 1]] = d
    inner = np.nonzero(Gn[:ni_, :ni_])
    assert (part_of[inner[0]] == part_of[inner[1]]).all()
    inv = [np.linalg.inv(Gn[dp[d]:dp[d + 1], dp[d]:dp[d + 1]]) for d in range(parts)]
    S = Gn[ni_:, ni_:].copy()
    bp, bn = dm['bnd_ptr'], dm['bnd_nptr']
    for d in range(parts):
        for p in range(bp[d], bp[d + 1]):
            for q in range(bp[d], bp[d + 1]):
                val = 0
                for a in range(bn[p], bn[p + 1]):
                    for b_ in range(bn[q], bn[q + 1]):
                        val += dinv[dm['bnd_branch'][a]] * inv[d][dm['bnd_local'][a], dm['bnd_local'][b_]] * \
                            dinv[dm['bnd_branch'][b_]]
                S[dm['bnd'][p], dm['bnd'][q]] -= val
    AI = np.zeros((ni_, ni_), complex)
    for d in range(parts):
        AI[dp[d]:dp[d + 1], dp[d]:dp[d + 1]] = inv[d]
    Sref = Gn[ni_:, ni_:] - Gn[ni_:, :ni_] @ AI @ Gn[:ni_, ni_:]
    assert np.abs(S - Sref).max() <= 1e-12 * np.abs(Sref).max()
    r = rng.standard_normal((nk, 2)) + 1j * rng.standard_normal((nk, 2))
    rn = r[perm]
    yI = AI @ rn[:ni_]
    xS = np.linalg.solve(S, rn[ni_:] - Gn[ni_:, :ni_] @ yI)
    xI = yI - AI @ (Gn[:ni_, ni_:] @ xS)
    x = np.empty_like(r)
    x[perm] = np.r_[xI, xS]
    ref = np.linalg.solve(G, r)
    assert np.abs(x - ref).max() <= 1e-9 * np.abs(ref).max()
    assert ns == nk - ni_ and ns > 0


def test_part_count_and_split_at_full_size():
    """The Laplacian's form by its size: dense for the plane pair (22,224 kept nodes, 4 GB as complex64), split for
    the C5-shaped board (210,072 kept nodes, 353 GB dense) into 128 domains of about 1,500 rows; the split leaves no
    Laplacian edge between two domains' interiors, and every boundary entry's neighbours lie in its own domain."""
    for board, want in (('planes', 0), ('c5', 128)):
        t = _topology(board)
        parts = t._graph_parts(None)
        assert parts == want, (board, parts)
        if not parts:
            continue
        g = t.graph_structure()
        dm = t.graph_domains(parts)
        nk, n_int, dp = g['nkeep'], dm['n_int'], dm['dom_ptr']
        assert len(dp) == parts + 1 and dp[-1] == n_int and 0 < dm['n_sep'] < nk // 10
        assert np.array_equal(np.sort(dm['perm']), np.arange(nk)) and np.array_equal(dm['pos'][dm['perm']],
                                                                                        np.arange(nk))
        dom = np.searchsorted(dp, np.arange(nk), side='right') - 1          # the domain of each new position
        dom[n_int:] = -1
        rows = np.repeat(np.arange(nk), np.diff(g['lap_ptr']))
        m = g['lap_other'] >= 0
        a, b = dm['pos'][rows[m]], dm['pos'][g['lap_other'][m]]
        inner = (a < n_int) & (b < n_int)
        assert (dom[a[inner]] == dom[b[inner]]).all()
        sizes = np.diff(dp)
        assert sizes.max() <= 2 * 1500 and sizes.min() > 0
        bp, bn = dm['bnd_ptr'], dm['bnd_nptr']
        assert bp[-1] == len(dm['bnd']) and bn[-1] == len(dm['bnd_local'])
        ent_dom = np.repeat(np.arange(parts), np.diff(bp))
        nb_dom = np.repeat(ent_dom, np.diff(bn))
        assert (dm['bnd_local'] < sizes[nb_dom]).all() and (dm['bnd'] < dm['n_sep']).all()
