"""Biot-Savart near field on the device against the reference's own h_sheets / h_segments (tests/golden/biot_*.npz,
made by make_biot_golden.py): FP64 sums within 1e-10 of the largest field, FP32 sums within 2e-5; filaments 1e-12."""
import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def golden(name):
    with np.load(GOLDEN / f'biot_{name}.npz') as d:
        return {k: d[k] for k in d.files}


@pytest.mark.parametrize('board', ['tiny', 'strip'])
@pytest.mark.parametrize('precision,tol', [('f64', 1e-10), ('f32', 2e-5)])
def test_sheet_field_matches_reference(device_library, board, precision, tol):
    from pcbqs_gb300.biot import h_sheets, rwg_currents
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.rwg import RWG
    g = golden(board)
    b = Board.load(board)
    r = RWG(b.nodes, b.tris)
    a, bb = rwg_currents(r, g['I'])
    sheets = []
    for layer in np.unique(b.layer):
        idx = np.flatnonzero(b.layer == layer)
        sheets.append((b.nodes, b.tris[idx], a[idx], bb[idx], float(b.z[idx[0]])))
    H = h_sheets(sheets, g['pts'], precision=precision)
    assert H.shape == g['H'].shape
    assert np.abs(H - g['H']).max() <= tol * np.abs(g['H']).max()
    # one excitation at a time gives the same columns
    a0, b0 = rwg_currents(r, g['I'][:, 0])
    H0 = h_sheets([(n, t, a0[np.isin(np.arange(len(b.tris)), np.flatnonzero(b.layer == l))],
                    b0[np.flatnonzero(b.layer == l)], z) for (n, t, _, _, z), l in zip(sheets, np.unique(b.layer))],
                  g['pts'], precision=precision)
    assert np.abs(H0 - H[..., 0]).max() <= tol * np.abs(g['H']).max()


def test_filament_field_matches_reference(device_library):
    from pcbqs_gb300.biot import h_segments
    g = golden('strip')
    H = h_segments(g['p0'], g['p1'], g['Iseg'], g['pts'])
    assert np.abs(H - g['Hseg']).max() <= 1e-12 * np.abs(g['Hseg']).max()
