"""The native loop basis (pcbqs_gb300_loop_basis, host code in the C-ABI library) against the pure-Python
restatement of the reference's spanning_tree and _loops (oracle/graph.py) on the committed boards: the same
forest, the same cycles in the same order with the same signs. No GPU needed."""
import numpy as np
import pytest

from oracle import graph as G


@pytest.fixture(scope='module')
def lib():
    from pcbqs_gb300 import build
    build.build()
    from pcbqs_gb300 import _lib
    return _lib.load()


@pytest.mark.parametrize('board', ['tiny', 'strip', 'planes', 'viapair'])
def test_native_loop_basis_matches_restatement(lib, board):
    """The via pair adds its plated via segments as branches after the RWG edges (non-source branches that join
    the two sheets' islands), as MQS does."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.geometry import prepare
    from pcbqs_gb300.peec import loop_basis
    from pcbqs_gb300.rwg import RWG
    b = Board.load(board)
    g = prepare(b.nodes, b.tris, b.z, 1)
    r = RWG(g.nodes, g.tris)
    of = b.node_of
    ends = [(int(of[a]), int(of[c])) for a, c in zip(r.tp, r.tm)]
    ends += [tuple(int(v) for v in e) for e in b.via_ends()]
    ends += [(b.term_node(a), b.term_node(c)) for _, a, c in b.ports]
    is_src = np.r_[np.zeros(r.Ne + b.nv, bool), np.ones(len(b.ports), bool)]
    C, src, tree, col_branch = loop_basis(b.n_nodes, ends, is_src, r.Ne)
    Co, srco, treeo, col_brancho = G.loop_basis(b.n_nodes, ends, is_src, r.Ne)
    assert np.array_equal(tree, treeo)
    assert np.array_equal(col_branch, col_brancho)
    assert src == srco
    assert C.shape == Co.shape and (C != Co).nnz == 0


def test_loop_basis_reports_short_capacity(lib):
    import ctypes
    from pcbqs_gb300 import _lib
    ea = np.array([0, 1, 2, 0], np.int32)           # a triangle of branches plus a parallel branch
    eb = np.array([1, 2, 0, 1], np.int32)
    src = np.zeros(4, np.uint8)
    tree = np.zeros(4, np.uint8)
    rows, cols, vals = np.zeros(1, np.int32), np.zeros(1, np.int32), np.zeros(1)
    cb = np.zeros(4, np.int32)
    nnz, ncol = ctypes.c_int64(), ctypes.c_int64()
    status = lib.pcbqs_gb300_loop_basis(3, 4, _lib.ptr(ea, ctypes.c_int32), _lib.ptr(eb, ctypes.c_int32),
                                        _lib.ptr(src, ctypes.c_uint8), 4, 1, _lib.ptr(tree, ctypes.c_uint8), 1,
                                        _lib.ptr(rows, ctypes.c_int32), _lib.ptr(cols, ctypes.c_int32),
                                        _lib.ptr(vals), ctypes.byref(nnz), _lib.ptr(cb, ctypes.c_int32),
                                        ctypes.byref(ncol))
    assert status == 1 and nnz.value == 5 and ncol.value == 2 and tree.sum() == 2
