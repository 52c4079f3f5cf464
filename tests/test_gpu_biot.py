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


def test_fft_grid_field_matches_reference(device_library):
    """h_grid on the device (cloud-in-cell deposit kernel, zero-padded FFT convolution) against the reference's own
    h_grid for the same branch currents on the tiny two-layer board, refine 2, above and below the copper; FP64
    throughout (the FFTs' rounding differs: 1e-9 of the field's largest value)."""
    import numpy as np
    from pcbqs_gb300.biot import h_grid
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.rwg import RWG
    g = np.load(GOLDEN / 'hgrid_tiny.npz')
    b = Board.load('tiny')
    r = RWG(b.nodes, b.tris)
    layer_tris = {int(k): np.flatnonzero(b.layer == k) for k in np.unique(b.layer)}
    I = (g['i'] / r.l[None, :]).T                     # RWG amplitudes (ne, 2)
    H = h_grid(r, layer_tris, b.z, I, g['x'], g['y'], g['heights'], refine=int(g['refine']))
    Hr = g['H']
    assert H.shape == Hr.shape
    assert np.abs(H - Hr).max() <= 1e-9 * np.abs(Hr).max()
    one = h_grid(r, layer_tris, b.z, I[:, 1], g['x'], g['y'], g['heights'], refine=int(g['refine']))
    assert np.abs(one - Hr[..., 1]).max() <= 1e-9 * np.abs(Hr).max()
