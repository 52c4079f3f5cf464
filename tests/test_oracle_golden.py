"""The CPU oracle pinned against the reference's own outputs (tests/golden/, made by make_golden.py)."""
import platform
from pathlib import Path

import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as O

NAMES = ('m0', 'mx', 'my', 'mrr')
X86 = platform.machine() in ('x86_64', 'AMD64')


def geo8(g, level):
    return O.Geometry(g['nodes'], g['tris'], g['z'], level)


@pytest.mark.parametrize('level', [0, 1, 2])
@pytest.mark.parametrize('scalar', [False, True])
def test_oracle_fill_matches_reference(tiny8, level, scalar):
    mats, analytic = O.fill(geo8(tiny8, level), 3.0, level, scalar, nthreads=2)
    tag = f'l{level}_{"s" if scalar else "f"}'
    for name, m in zip(NAMES, mats):
        assert m == pytest.approx(tiny8[f'numpy_{tag}_{name}'], rel=2e-11, abs=1e-27)
        if X86:     # the reference's compiled core on the same ISA, products rounded: bit for bit
            np.testing.assert_array_equal(m, tiny8[f'openmp_{tag}_{name}'])
    assert analytic == int(tiny8[f'numpy_{tag}_analytic'])
    again, _ = O.fill(geo8(tiny8, level), 3.0, level, scalar, nthreads=1)
    assert all(np.array_equal(a, b) for a, b in zip(mats, again))


def test_oracle_all_analytic_path(tiny8):
    mats, analytic = O.fill(geo8(tiny8, 1), np.inf, 1, False)
    for name, m in zip(NAMES, mats):
        assert m == pytest.approx(tiny8[f'allnear_{name}'], rel=2e-11, abs=1e-27)
    assert analytic == 36


@pytest.mark.parametrize('near', [0., .5, 3., np.inf])
@pytest.mark.parametrize('level', [0, 1, 2])
def test_oracle_kinds(tiny8, near, level):
    g = geo8(tiny8, level)
    n = g.nt
    p, q = np.meshgrid(np.arange(n), np.arange(n), indexing='ij')
    p, q = p.ravel(), q.ravel()
    d = g.z[p] - g.z[q]
    expected = tiny8[f'kinds_{near}_{level}']
    np.testing.assert_array_equal(O.kinds(g, p, q, d, near, level), expected)
    lib = O.lib()
    c = np.array([lib.og_kind(g.cent.ctypes.data, g.radius.ctypes.data, int(a), int(b), float(dd),
                              0.0 if np.isinf(near) else near, int(np.isinf(near)), level)
                  for a, b, dd in zip(p, q, d)])
    np.testing.assert_array_equal(c, expected)


@pytest.mark.parametrize('level', [0, 1, 2])
@pytest.mark.parametrize('scalar', [False, True])
def test_oracle_pair_protocol(tiny8, level, scalar):
    g = geo8(tiny8, level)
    p, q = tiny8['pair_p'], tiny8['pair_q']
    tag = f'l{level}_{"s" if scalar else "f"}'
    out = O.pairs(g, p, q, g.z[p] - g.z[q], tiny8[f'pairs_{tag}_kind'], scalar)
    assert out == pytest.approx(tiny8[f'pairs_{tag}'], rel=1e-12, abs=1e-27)


def test_oracle_rejects_invalid_pairs(tiny8):
    g = geo8(tiny8, 1)
    with pytest.raises(ValueError):
        O.pairs(g, [8], [0], [0.0], [-1])
    with pytest.raises(ValueError):
        O.pairs(g, [0], [0], [np.nan], [0])
    with pytest.raises(ValueError):
        O.pairs(g, [0], [0], [0.0], [3])


def test_oracle_combine_matches_reference(tiny8):
    g = geo8(tiny8, 1)
    mats, _ = O.fill(g, 3.0, 1, False)
    rwg = O.RWG(g.nodes, g.tris)
    L = O.combine(rwg, mats)
    ref = tiny8['L']
    assert L == pytest.approx(ref, rel=1e-12, abs=1e-12 * np.abs(ref).max())
    assert np.array_equal(L, L.T)
    np.testing.assert_array_equal(g.nodes, tiny8['centred'])


@pytest.mark.parametrize('board', ['tiny', 'strip'])
def test_oracle_on_boards(board):
    from pcbqs_gb300.board import Board
    b = Board.load(board)
    gold = load_golden(board)
    g = O.Geometry(b.nodes, b.tris, b.z, 1)
    np.testing.assert_array_equal(g.cent, gold['cent'])
    np.testing.assert_array_equal(g.radius, gold['radius'])
    np.testing.assert_array_equal(g.nodes, gold['centred'])
    mats, analytic = O.fill(g, 3.0, 1, False)
    assert analytic == int(gold['analytic'])
    rows = gold['rows']
    for name, m in zip(NAMES, mats):
        assert m[rows] == pytest.approx(gold[f'{name}_rows'], rel=1e-13, abs=1e-30)
        i, j = gold[f'{name}_at']
        assert m[i, j] == pytest.approx(gold[f'{name}_val'], rel=1e-13, abs=1e-30)
        assert np.abs(m).sum() == pytest.approx(gold[f'{name}_sum'][1], rel=1e-12)
    rwg = O.RWG(g.nodes, g.tris)
    np.testing.assert_array_equal(rwg.tp, gold['tp'])
    np.testing.assert_array_equal(rwg.tm, gold['tm'])
    L = O.combine(rwg, mats)
    scale = np.abs(gold['L_rows']).max()
    assert L[gold['edge_rows']] == pytest.approx(gold['L_rows'], rel=1e-10, abs=1e-13 * scale)
    i, j = gold['L_at']
    assert L[i, j] == pytest.approx(gold['L_val'], rel=1e-10, abs=1e-13 * scale)
    np.testing.assert_array_equal(b.node_of, gold['node_of'])
    P = O.potential(mats[0], rwg.area, b.node_of, b.er)
    assert P[gold['node_rows']] == pytest.approx(gold['P_rows'], rel=1e-12)
    i, j = gold['P_at']
    assert P[i, j] == pytest.approx(gold['P_val'], rel=1e-12)


@pytest.mark.parametrize('board,mixed', [('tiny', False), ('strip', False), ('strip', True)])
def test_cpu_dense_solve_matches_reference(board, mixed):
    """The CPU restatement of the reference's dense PEEC solve (the benchmark's reference arm) against the
    reference's own port impedances: the C oracle's fill, combine and aggregation, then topology, projections, the
    scaled system, LU (double, or MixedLU's complex64 factor with refinement) and every drive."""
    from oracle import peec_cpu
    from pcbqs_gb300.board import Board
    b = Board.load(board)
    g = O.Geometry(b.nodes, b.tris, b.z, 1)
    mats, _ = O.fill(g, 3.0, 1, False)
    rwg = O.RWG(g.nodes, g.tris)
    L = O.combine(rwg, mats)
    P = O.potential(mats[0], g.area, b.node_of, b.er)
    solver = peec_cpu.DenseSolve(b, rwg, L, P)
    with np.load(Path(__file__).parent / 'golden' / f'peec_{board}.npz') as ref:
        for f, Zref in zip(ref['freqs'], ref['Z']):
            Z = solver.solve(float(f), mixed=mixed)
            assert np.abs(Z - Zref).max() / np.abs(Zref).max() < 1e-8
