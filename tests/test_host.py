"""Host logic of the backend: mesh preparation, RWG order, node merging, plugin contract without a device."""
import sys

import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as O


@pytest.mark.parametrize('board', ['tiny', 'strip'])
def test_prepare_is_bit_identical_to_reference(board):
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.geometry import prepare
    b = Board.load(board)
    gold = load_golden(board)
    g = prepare(b.nodes, b.tris, b.z, 1)
    np.testing.assert_array_equal(g.cent, gold['cent'])
    np.testing.assert_array_equal(g.radius, gold['radius'])
    np.testing.assert_array_equal(g.nodes, gold['centred'])
    og = O.Geometry(b.nodes, b.tris, b.z, 1)
    for level in (0, 1):
        for a, c in zip(g.levels[level], og.levels[level]):
            np.testing.assert_array_equal(a, c)
    np.testing.assert_array_equal(g.points, og.points)


@pytest.mark.parametrize('board', ['tiny', 'strip', 'planes'])
def test_rwg_order_and_nodes_match_reference(board):
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.geometry import prepare
    from pcbqs_gb300.rwg import RWG
    b = Board.load(board)
    gold = load_golden(board)
    g = prepare(b.nodes, b.tris, b.z, 1)
    r = RWG(g.nodes, g.tris)
    assert r.Ne == int(gold['ne'])
    np.testing.assert_array_equal(r.tp, gold['tp'])
    np.testing.assert_array_equal(r.tm, gold['tm'])
    np.testing.assert_array_equal(b.node_of, gold['node_of'])


def test_prepare_validation():
    from pcbqs_gb300.geometry import prepare
    nodes = np.array([[0, 0], [1, 0], [0, 1.]])
    with pytest.raises(ValueError, match='counter-clockwise'):
        prepare(nodes, np.array([[0, 2, 1]]), np.zeros(1))
    with pytest.raises(ValueError, match='finite planar'):
        prepare(nodes, np.array([[0, 1, 3]]), np.zeros(1))
    with pytest.raises(ValueError, match='outer_levels'):
        prepare(nodes, np.array([[0, 1, 2]]), np.zeros(1), 3)


def test_missing_gpu_does_not_fall_back_to_cpu(tiny8):
    import torch
    if torch.cuda.is_available():
        pytest.skip('a device is present')
    from pcbqs_gb300.backend import factory
    from pcbqs_gb300.geometry import prepare
    g = prepare(tiny8['nodes'], tiny8['tris'], tiny8['z'], 1)
    with pytest.raises(RuntimeError, match='GB300 fill unavailable'):
        factory(g, 1, 16384, None)


def test_entry_point_is_declared():
    import tomllib
    from pathlib import Path
    meta = tomllib.loads((Path(__file__).resolve().parents[1] / 'pyproject.toml').read_text())
    group = meta['project']['entry-points']['pcbqs.static_backends']
    assert group == {'gb300': 'pcbqs_gb300.backend:factory'}


def test_reference_engine_selects_the_plugin_and_raises_without_device(tiny8, monkeypatch):
    """Through the reference's own FillEngine (where its checkout is present): the entry point is loaded only when
    `gb300` is selected, and without a device the selection fails loudly instead of falling back."""
    from oracle import reference
    if not reference.available():
        pytest.skip('reference checkout not present')
    import torch
    pcbqs = reference.load_reference()
    import pcbqs.static_backends as backends
    from types import SimpleNamespace
    monkeypatch.setattr(backends, '_FACTORIES', dict(backends._FACTORIES))
    loaded = []

    def load():
        loaded.append(True)
        from pcbqs_gb300.backend import factory
        return factory
    monkeypatch.setattr(backends.metadata, 'entry_points',
                        lambda **kw: [SimpleNamespace(name='gb300', load=load)])
    backends.FillEngine(tiny8['nodes'], tiny8['tris'], tiny8['z'], backend='numpy')
    assert loaded == []
    if torch.cuda.is_available():
        e = backends.FillEngine(tiny8['nodes'], tiny8['tris'], tiny8['z'], backend='gb300')
        assert loaded == [True] and e.info['backend'] == 'gb300'
    else:
        with pytest.raises(RuntimeError, match='GB300 fill unavailable'):
            backends.FillEngine(tiny8['nodes'], tiny8['tris'], tiny8['z'], backend='gb300')
        assert loaded == [True]


@pytest.mark.parametrize('board', ['tiny', 'strip'])
def test_cluster_tree_partition_covers_each_entry_once(board):
    """The H-matrix block structure: every (row, column) of the symmetric matrix lies in exactly one stored block
    or in the transpose of one (diagonal blocks only once), and every compressed block is admissible."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.geometry import prepare
    from pcbqs_gb300.hmatrix import ClusterTree
    from pcbqs_gb300.rwg import RWG
    b = Board.load(board)
    g = prepare(b.nodes, b.tris, b.z, 1)
    r = RWG(g.nodes, g.tris)
    v = g.nodes[g.tris]
    lo_t, hi_t = np.c_[v.min(1), g.z], np.c_[v.max(1), g.z]
    support = np.stack((r.tp, r.tm), axis=1)
    lo, hi = lo_t[support].min(1), hi_t[support].max(1)
    tree = ClusterTree(lo, hi, 16)
    leaves = np.concatenate([tree.ids(k) for k in range(len(tree.start)) if tree.leaf(k)])
    np.testing.assert_array_equal(np.sort(leaves), np.arange(r.Ne))
    assert all(tree.size(k) <= 16 for k in range(len(tree.start)) if tree.leaf(k))
    count = np.zeros((r.Ne, r.Ne), np.int32)
    level, far = [(0, 0)], 0
    while level:
        deeper = []
        for i, j in level:
            if tree.separated(i, j, 1.0):
                far += 1
            elif not (tree.leaf(i) and tree.leaf(j)):
                deeper += tree.refine(i, j)
                continue
            a, c = tree.ids(i), tree.ids(j)
            count[np.ix_(a, c)] += 1
            if i != j:
                count[np.ix_(c, a)] += 1
        level = deeper
    assert far > 0
    np.testing.assert_array_equal(count, 1)


def test_peec_model_rejects_bad_options_before_touching_the_device():
    """Option checks of PeecModel run before any device work (no GPU needed): the inner tolerance must lie within
    the inner products' reach, and the compressed operator takes a homogeneous dielectric."""
    import pytest
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    b = Board.load('tiny')
    with pytest.raises(ValueError, match='inner_tol'):
        PeecModel(b, inner_tol=1e-7)
    with pytest.raises(ValueError, match='inner_tol'):
        PeecModel(b, inner_tol=1.0)
    with pytest.raises(ValueError, match="'dense' or 'hierarchical'"):
        PeecModel(b, matrix='sparse')
    with pytest.raises(ValueError, match='homogeneous'):
        PeecModel(b, matrix='hierarchical', stack=object())


def test_solve_options_are_checked_before_device_work():
    """PeecModel.solve_options (run first in solve, no GPU needed): frequencies, preconditioner names, the graph
    preconditioner's part count (0 or a power of two), its refinement count (0..3), captured cycles only with the
    dense Laplacian, and the complex64 factor only for the dense operator."""
    import numpy as np
    import pytest
    from pcbqs_gb300.peec import PeecModel
    base = dict(matrix='dense', freqs=[1e6], precondition='graph', mixed=False, factor_math='tc6-blocked',
                anchors=None, captured=False, product='tc3', fp64_product=None, graph_parts=None, graph_refine=None)

    def check(**kw):
        return PeecModel.solve_options(**{**base, **kw})
    f, mode, anchors, fp64 = check()
    assert mode == 3 and anchors == 1 and fp64 == 'fp64' and np.array_equal(f, [1e6])
    assert check(mixed=True)[3] == 'sliced6'
    assert check(graph_parts=0, captured=True)[1] == 3
    assert check(graph_parts=16, graph_refine=0)[1] == 3
    for kw, match in ((dict(freqs=[0.0]), 'frequencies'), (dict(freqs=[]), 'frequencies'),
                      (dict(freqs=[np.inf]), 'frequencies'), (dict(precondition='ilu'), 'precondition'),
                      (dict(graph_parts=3), 'graph_parts'), (dict(graph_parts=1), 'graph_parts'),
                      (dict(graph_parts=True), 'graph_parts'), (dict(graph_refine=4), 'graph_refine'),
                      (dict(graph_refine=-1), 'graph_refine'), (dict(graph_refine=1.5), 'graph_refine'),
                      (dict(graph_parts=8, captured=True), 'captured'),
                      (dict(matrix='hierarchical', precondition='lu32'), 'compressed'),
                      (dict(anchors=2), 'anchors'), (dict(product='bf16'), 'product'),
                      (dict(fp64_product='sliced9'), 'fp64_product'), (dict(factor_math='fp16'), 'factor_math')):
        with pytest.raises(ValueError, match=match):
            check(**kw)


def test_graph_entries_reject_bad_arguments_without_a_device():
    """The graph preconditioner's and the plane packer's C entries check their arguments before any CUDA call."""
    import ctypes
    from pcbqs_gb300 import _lib, build
    build.build()
    lib = _lib.load()
    g = _lib.GraphDesc()
    assert lib.pcbqs_gb300_peec_graph(None, ctypes.byref(g), 0, 1, None) == 1
    assert lib.pcbqs_gb300_peec_graph_apply(None, 1, None, None, None) == 1
    assert lib.pcbqs_gb300_pack_bf16_parts(None, None, -1, None, None, 64, 0, None) == 1
    assert lib.pcbqs_gb300_pack_bf16_parts(None, None, 1, None, None, 64, 0, None) == 1     # null arrays
    assert lib.pcbqs_gb300_pack_bf16_parts(None, None, 0, None, None, 64, 0, None) == 0     # nothing to pack
    assert b'invalid argument' in lib.pcbqs_gb300_last_error()
