"""Device fill parity through the C ABI: the sm_103a kernels against the reference's golden vectors and the CPU
oracle. Tolerances: the reference holds its own device path to rel 2e-10 on moments
(tests/test_static_backends.py:197); classification must be bit-exact (identical analytic-pair counts)."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu
NAMES = ('m0', 'mx', 'my', 'mrr')


def device_geometry(nodes, tris, z, level):
    from pcbqs_gb300.geometry import DeviceGeometry, prepare
    g = prepare(nodes, tris, z, level)
    return g, DeviceGeometry(g, 0)


def host_fill(dev, nt, near, level, scalar):
    from pcbqs_gb300 import _lib
    mats = [np.full((nt, nt), np.nan) for _ in range(1 if scalar else 4)]
    planes = (ctypes.c_void_p * 4)(*[m.ctypes.data for m in mats], *([None] * (4 - len(mats))))
    analytic = ctypes.c_uint64()
    _lib.check(dev.lib.pcbqs_gb300_fill(dev.handle, -1.0 if np.isinf(near) else near, level, int(scalar), planes,
                                        ctypes.byref(analytic)))
    return mats, int(analytic.value)


@pytest.mark.parametrize('level', [0, 1, 2])
@pytest.mark.parametrize('scalar', [False, True])
def test_device_fill_matches_reference(device_library, tiny8, level, scalar):
    g, dev = device_geometry(tiny8['nodes'], tiny8['tris'], tiny8['z'], level)
    mats, analytic = host_fill(dev, 8, 3.0, level, scalar)
    tag = f'l{level}_{"s" if scalar else "f"}'
    for name, m in zip(NAMES, mats):
        assert m == pytest.approx(tiny8[f'numpy_{tag}_{name}'], rel=2e-10, abs=1e-26)
    assert analytic == int(tiny8[f'numpy_{tag}_analytic'])
    again, _ = host_fill(dev, 8, 3.0, level, scalar)
    assert all(np.array_equal(a, b) for a, b in zip(mats, again))
    assert np.array_equal(mats[0], mats[0].T)
    if not scalar:
        assert np.array_equal(mats[3], mats[3].T)


def test_device_all_analytic(device_library, tiny8):
    g, dev = device_geometry(tiny8['nodes'], tiny8['tris'], tiny8['z'], 1)
    mats, analytic = host_fill(dev, 8, np.inf, 1, False)
    for name, m in zip(NAMES, mats):
        assert m == pytest.approx(tiny8[f'allnear_{name}'], rel=2e-10, abs=1e-26)
    assert analytic == 36


@pytest.mark.parametrize('level', [0, 1, 2])
@pytest.mark.parametrize('scalar', [False, True])
def test_device_pair_protocol(device_library, tiny8, level, scalar):
    from pcbqs_gb300.backend import Gb300Backend
    from pcbqs_gb300.geometry import prepare
    g = prepare(tiny8['nodes'], tiny8['tris'], tiny8['z'], level)
    backend = Gb300Backend(g, 1, 16384, 0)
    p, q = tiny8['pair_p'].astype(np.int32), tiny8['pair_q'].astype(np.int32)
    tag = f'l{level}_{"s" if scalar else "f"}'
    kind = tiny8[f'pairs_{tag}_kind'].astype(np.int32)
    out = backend.evaluate(p, q, g.z[p] - g.z[q], kind, scalar)
    assert out.dtype == np.float64 and out.shape == (7, 1 if scalar else 6)
    assert out == pytest.approx(tiny8[f'pairs_{tag}'], rel=2e-10, abs=1e-26)
    # kind-sorted order does not change any result: every pair against the oracle one by one
    og = O.Geometry(tiny8['nodes'], tiny8['tris'], tiny8['z'], level)
    assert out == pytest.approx(O.pairs(og, p, q, g.z[p] - g.z[q], kind, scalar), rel=2e-10, abs=1e-26)


def test_device_pair_protocol_errors(device_library, tiny8):
    from pcbqs_gb300.backend import Gb300Backend
    from pcbqs_gb300.geometry import prepare
    g = prepare(tiny8['nodes'], tiny8['tris'], tiny8['z'], 1)
    backend = Gb300Backend(g, 1, 16384, 0)
    with pytest.raises(ValueError, match='out of range'):
        backend.evaluate(np.array([8]), np.array([0]), np.zeros(1), np.array([-1]), False)
    with pytest.raises(ValueError, match='non-finite offset'):
        backend.evaluate(np.array([0]), np.array([0]), np.array([np.nan]), np.array([0]), False)
    with pytest.raises(ValueError, match='prepared analytic level'):
        backend.evaluate(np.array([0]), np.array([0]), np.zeros(1), np.array([2]), False)
    assert backend.evaluate(np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0), np.zeros(0, np.int32),
                            True).shape == (0, 1)


@pytest.mark.parametrize('board', ['tiny', 'strip'])
def test_device_fill_combine_potential_vs_oracle(device_library, board):
    import torch
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.fill import DeviceFill
    b = Board.load(board)
    gold = load_golden(board)
    f = DeviceFill(b.nodes, b.tris, b.z, outer_levels=1, near=3.0)
    planes, analytic = f.moments()
    assert analytic == int(gold['analytic'])
    og = O.Geometry(b.nodes, b.tris, b.z, 1)
    mats, oracle_analytic = O.fill(og, 3.0, 1, False)
    assert analytic == oracle_analytic
    for k, (name, m) in enumerate(zip(NAMES, mats)):
        dev = planes[k].cpu().numpy()
        scale = np.abs(m).max()
        assert dev == pytest.approx(m, rel=1e-10, abs=1e-14 * scale), name
    L = f.inductance(planes).cpu().numpy()
    Lo = O.combine(O.RWG(og.nodes, og.tris), mats)
    assert np.array_equal(L, L.T)
    assert L == pytest.approx(Lo, rel=1e-10, abs=1e-12 * np.abs(Lo).max())
    P = f.potential(planes[0], b.node_of, b.er).cpu().numpy()
    Po = O.potential(mats[0], og.area, b.node_of, b.er)
    assert np.array_equal(P, P.T)
    assert P == pytest.approx(Po, rel=1e-12)
    torch.cuda.synchronize()


def test_device_fill_planes_board(device_library):
    """The 22,554-triangle plane pair: classification count exact, samples and checksums against the reference."""
    import torch
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.fill import DeviceFill
    b = Board.load('planes')
    gold = load_golden('planes')
    f = DeviceFill(b.nodes, b.tris, b.z, outer_levels=1, near=3.0)
    planes, analytic = f.moments()
    assert analytic == int(gold['analytic'])
    for k, name in enumerate(NAMES):
        m = planes[k]
        i, j = (torch.as_tensor(a, device=m.device) for a in gold[f'{name}_at'])
        scale = float(gold[f'{name}_sum'][3])
        assert m[i, j].cpu().numpy() == pytest.approx(gold[f'{name}_val'], rel=1e-10, abs=1e-14 * scale)
        rows = m[torch.as_tensor(gold['rows'], device=m.device)].cpu().numpy()
        assert rows == pytest.approx(gold[f'{name}_rows'], rel=1e-10, abs=1e-14 * scale)
        assert float(m.abs().sum()) == pytest.approx(float(gold[f'{name}_sum'][1]), rel=1e-11)
    L = f.inductance(planes)
    i, j = (torch.as_tensor(a, device=L.device) for a in gold['L_at'])
    scale = float(gold['L_sum'][3])
    assert L[i, j].cpu().numpy() == pytest.approx(gold['L_val'], rel=1e-10, abs=1e-12 * scale)
    assert torch.diagonal(L).cpu().numpy() == pytest.approx(gold['L_diag'], rel=1e-10)
    assert float(L.abs().sum()) == pytest.approx(float(gold['L_sum'][1]), rel=1e-10)
    del L
    P = f.potential(planes[0], b.node_of, b.er)
    i, j = (torch.as_tensor(a, device=P.device) for a in gold['P_at'])
    assert P[i, j].cpu().numpy() == pytest.approx(gold['P_val'], rel=1e-11)
    assert torch.diagonal(P).cpu().numpy() == pytest.approx(gold['P_diag'], rel=1e-11)


@pytest.mark.parametrize('board', ['tiny', 'strip'])
def test_mixed_fill_against_fp64_oracle(device_library, board):
    """The mixed fill (far pairs in FP32 local coordinates, near pairs FP64, FP32 combine): L and P against the FP64
    oracle. Stated errors: max |dL| / max |L| < 2e-6 and max |dP| / max |P| < 2e-6; the near-field (diagonal) entries,
    dominated by the FP64 near pairs, within 1e-5 relative each."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.fill import DeviceFill
    b = Board.load(board)
    f = DeviceFill(b.nodes, b.tris, b.z, outer_levels=1, near=3.0)
    planes, analytic = f.moments_local()
    og = O.Geometry(b.nodes, b.tris, b.z, 1)
    mats, oracle_analytic = O.fill(og, 3.0, 1, False)
    assert analytic == oracle_analytic
    L, Lf = f.inductance_local(planes)
    L, Lf = L.cpu().numpy(), Lf.cpu().numpy()
    Lo = O.combine(O.RWG(og.nodes, og.tris), mats)
    assert np.array_equal(L, L.T) and np.array_equal(Lf.astype(np.float64), L)
    assert np.abs(L - Lo).max() / np.abs(Lo).max() < 2e-6
    assert np.diag(L) == pytest.approx(np.diag(Lo), rel=1e-5)
    P, Pf = f.potential_single(planes[0], b.node_of, b.er)
    Po = O.potential(mats[0], og.area, b.node_of, b.er)
    P = P.cpu().numpy()
    assert np.abs(P - Po).max() / np.abs(Po).max() < 2e-6


def test_mixed_fill_planes_against_reference_rows(device_library):
    """The mixed fill on the benchmarked board (22,554 triangles, 33,368 edges): L and P at the reference's sampled
    rows (golden_planes.npz: the reference's FP64 static_combine and _set_potential) within 2e-6 of their largest
    entry, the diagonals within 1e-5 relative, and the analytic pair count exact."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.fill import DeviceFill
    gold = load_golden('planes')
    b = Board.load('planes')
    f = DeviceFill(b.nodes, b.tris, b.z, outer_levels=1, near=3.0)
    planes, analytic = f.moments_local()
    assert analytic == int(gold['analytic'])
    L, Lf = f.inductance_local(planes)
    rows = torch_rows(L, gold['edge_rows'])
    scale = np.abs(gold['L_rows']).max()
    errL = np.abs(rows - gold['L_rows']).max() / scale
    assert errL < 2e-6, errL
    assert torch_diag(L) == pytest.approx(gold['L_diag'], rel=1e-5)
    del L, Lf
    P, Pf = f.potential_single(planes[0], b.node_of, b.er)
    prow = torch_rows(P, gold['node_rows'])
    errP = np.abs(prow - gold['P_rows']).max() / np.abs(gold['P_rows']).max()
    assert errP < 2e-6, errP
    assert torch_diag(P) == pytest.approx(gold['P_diag'], rel=1e-5)
    print(f'planes mixed fill: L error {errL:.2e}, P error {errP:.2e} of the largest sampled entry')


def torch_rows(M, rows):
    import torch
    return M[torch.as_tensor(np.asarray(rows), device=M.device)].cpu().numpy()


def torch_diag(M):
    import torch
    return torch.diagonal(M).cpu().numpy()
