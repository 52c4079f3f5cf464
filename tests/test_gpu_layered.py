"""The layered-dielectric potential on the device (csrc/layered.cu) against the reference's own potential_moments
run through its compiled layered_pairs kernel (tests/golden/make_layered_golden.py): the tiny two-layer board in a
lossy FR-4 slab. FP64 throughout, so the bar is the FP64 fill's: 1e-10 relative on entries and checksums."""
import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def golden():
    with np.load(GOLDEN / 'layered_tiny.npz') as d:
        return {k: d[k] for k in d.files}


def test_layered_moments_and_potential_match_reference(device_library):
    import torch
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.fill import DeviceFill
    from pcbqs_gb300.layered import DielectricStack, LayeredPotential
    g = golden()
    b = Board.load('tiny')
    z0, z1, er, tand = g['slab']
    fill = DeviceFill(b.nodes, b.tris, b.z, int(g['outer']), float(g['near']))
    lp = LayeredPotential(fill, DielectricStack.slab(z0, z1, er, tand), b.layer)
    re, im = lp.moments()
    M = (re + 1j * im).cpu().numpy()
    assert lp.info['image_terms'] == int(g['image_terms'])
    scale = np.abs(g['M_rows']).max()
    assert M[g['rows']] == pytest.approx(g['M_rows'], rel=1e-10, abs=1e-12 * scale)
    assert np.diag(M) == pytest.approx(g['M_diag'], rel=1e-10)
    assert np.abs(M).sum() == pytest.approx(float(g['M_abs_sum']), rel=1e-10)
    assert M.sum() == pytest.approx(complex(g['M_sum']), rel=1e-10)
    assert np.array_equal(M, M.T)
    P = lp.potential(b.node_of, (re, im)).cpu().numpy()
    pscale = np.abs(g['P_rows']).max()
    assert P[g['rows']] == pytest.approx(g['P_rows'], rel=1e-10, abs=1e-12 * pscale)
    assert np.diag(P) == pytest.approx(g['P_diag'], rel=1e-10)
    assert np.abs(P).sum() == pytest.approx(float(g['P_abs_sum']), rel=1e-10)
    # a lossy dielectric, eps = er (1 - j tand): the potential coefficients go as 1/eps, so their imaginary part is
    # positive
    assert (np.diag(P).imag > 0).all() and (np.diag(P).real > 0).all()
    torch.cuda.synchronize()


def test_uniform_stack_reduces_to_homogeneous_potential(device_library):
    """A stack with the same medium everywhere has only the direct image (coefficient 1/er): M = M0 / er, the
    homogeneous fill's scalar moments (the check of tests/test_electrostatic.py:56-68)."""
    import torch
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.fill import DeviceFill
    from pcbqs_gb300.layered import DielectricStack, LayeredPotential
    b = Board.load('tiny')
    er = 4.3
    fill = DeviceFill(b.nodes, b.tris, b.z, 1, 3.0)
    lp = LayeredPotential(fill, DielectricStack([0.0, 0.2e-3], [er, er, er]), b.layer)
    re, im = lp.moments()
    planes, _ = fill.moments(scalar_only=True)
    M0 = planes[0].cpu().numpy()
    assert re.cpu().numpy() == pytest.approx(M0 / er, rel=1e-12, abs=1e-14 * np.abs(M0).max())
    assert not im.cpu().numpy().any()
    torch.cuda.synchronize()
