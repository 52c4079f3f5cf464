"""The device copper-port reduction (pcbqs_gb300.ports: FP64 fill of L, loop matrices on the device, direct
elimination of the free loops) against the reference's own CopperPorts on the strip (tests/golden/ports_strip.npz,
made by make_ports_golden.py), DC included, for DC and slab sheet resistance; and the device MixedLU."""
import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def golden():
    with np.load(GOLDEN / 'ports_strip.npz') as d:
        return {k: d[k] for k in d.files}


@pytest.mark.parametrize('loss', ['dc', 'slab'])
def test_copper_ports_match_reference(device_library, loss):
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.ports import CopperPorts, MagneticModel
    g = golden()
    r = CopperPorts(MagneticModel(Board.load('strip'), conductor_loss=loss)).extract(g['freqs'])
    assert list(r.names) == [str(n) for n in g['ports']]
    Z, Zr = r.impedance, g[f'Z_{loss}']
    for fi in range(len(g['freqs'])):
        assert np.abs(Z[fi] - Zr[fi]).max() <= 1e-8 * np.abs(Zr[fi]).max(), fi
    I, Ir = r.currents, g[f'currents_{loss}']
    assert I.shape == Ir.shape
    assert np.abs(I - Ir).max() <= 1e-8 * np.abs(Ir).max()
    assert np.abs(Z - Z.transpose(0, 2, 1)).max() <= 1e-9 * np.abs(Z).max()      # reciprocity
    assert (np.abs(I[:, -len(r.names):]) == 0).all()                             # port connectors carry none


def test_copper_ports_need_a_loop(device_library):
    """The tiny board's ports join two islands (a plane pair): no magnetic loop, as the reference reports."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.ports import MagneticModel
    with pytest.raises(ValueError, match='island'):
        MagneticModel(Board.load('tiny'))


def test_device_mixed_lu_refines_to_double(device_library):
    """DeviceMixedLU (complex64 blocked LU + FP64 refinement) on 4,500 unknowns: the residual reaches 1e-12 and the
    solution matches the FP64 solve; lu_factor_rows picks it at and above 4,000 unknowns, as the reference."""
    import torch
    from pcbqs_gb300.mixedlu import DeviceMixedLU, lu_factor_rows, lu_solve_rows
    n = 4500
    g = torch.Generator(device='cuda').manual_seed(3)
    A = torch.complex(torch.randn(n, n, device='cuda', dtype=torch.float64, generator=g),
                      torch.randn(n, n, device='cuda', dtype=torch.float64, generator=g))
    A += 4 * np.sqrt(n) * torch.eye(n, device='cuda', dtype=torch.complex128)
    b = torch.complex(torch.randn(n, 3, device='cuda', dtype=torch.float64, generator=g),
                      torch.randn(n, 3, device='cuda', dtype=torch.float64, generator=g))
    lu = lu_factor_rows(A)
    assert isinstance(lu, DeviceMixedLU)
    x = lu_solve_rows(lu, b)
    assert lu.double is None                                  # refined, not refactored in double
    assert (torch.linalg.norm(b - A @ x) / torch.linalg.norm(b)).item() <= 1e-12
    ref = torch.linalg.solve(A, b)
    assert (torch.linalg.norm(x - ref) / torch.linalg.norm(ref)).item() <= 1e-11
    x1 = lu_solve_rows(lu, b[:, 0])
    assert x1.shape == (n,)
    small = lu_factor_rows(A[:100, :100])
    assert not isinstance(small, DeviceMixedLU)


def test_copper_ports_by_pencil_match_reference(device_library):
    """The whole sweep from one generalized eigendecomposition (method='pencil') gives the reference's direct
    reduction too; it refuses a frequency-dependent resistance."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.ports import CopperPorts, MagneticModel
    g = golden()
    r = CopperPorts(MagneticModel(Board.load('strip'))).extract(g['freqs'], method='pencil')
    for fi in range(len(g['freqs'])):
        assert np.abs(r.impedance[fi] - g['Z_dc'][fi]).max() <= 1e-8 * np.abs(g['Z_dc'][fi]).max(), fi
    assert np.abs(r.currents - g['currents_dc']).max() <= 1e-8 * np.abs(g['currents_dc']).max()
    with pytest.raises(ValueError, match='pencil'):
        CopperPorts(MagneticModel(Board.load('strip'), conductor_loss='slab')).extract(g['freqs'], method='pencil')


def via_golden():
    with np.load(GOLDEN / 'ports_viapair.npz') as d:
        return {k: d[k] for k in d.files}


def test_via_filaments_match_reference(device_library):
    """Via segments' R (host) and L (device filament kernel, pcbqs_gb300_via_inductance) against the reference's
    via_resistance / via_inductance of the via pair's segments."""
    import torch
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import via_inductance, via_resistance
    g, b = via_golden(), Board.load('viapair')
    np.testing.assert_allclose(via_resistance(b.via_seg, b.sigma, b.plating), g['via_R'], rtol=1e-14)
    out = torch.full((b.nv + 3, b.nv + 5), float('nan'), dtype=torch.float64, device='cuda')
    via_inductance(b.via_seg, out[1:1 + b.nv, 2:2 + b.nv], out.device)
    L = out[1:1 + b.nv, 2:2 + b.nv].cpu().numpy()
    np.testing.assert_allclose(L, g['via_L'], rtol=1e-13)
    assert torch.isnan(out[0]).all() and torch.isnan(out[1 + b.nv:]).all()      # writes stay in the view


@pytest.mark.parametrize('loss', ['dc', 'slab'])
def test_copper_ports_through_vias_match_reference(device_library, loss):
    """The via pair's loop closes through its two plated vias: port Z and branch currents (via segments included)
    against the reference's CopperPorts; the barrels keep their DC resistance under slab loss."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.ports import CopperPorts, MagneticModel
    g = via_golden()
    r = CopperPorts(MagneticModel(Board.load('viapair'), conductor_loss=loss)).extract(g['freqs'])
    for fi in range(len(g['freqs'])):
        assert np.abs(r.impedance[fi] - g[f'Z_{loss}'][fi]).max() <= 1e-8 * np.abs(g[f'Z_{loss}'][fi]).max(), fi
    assert np.abs(r.currents - g[f'currents_{loss}']).max() <= 1e-8 * np.abs(g[f'currents_{loss}']).max()


def test_field_of_port_currents_through_vias_matches_reference(device_library):
    """H of the via pair's currents (1 A per port, slab loss, 1 MHz): the sheets by Biot-Savart and the via
    segments as filaments (pcbqs_gb300.biot.h_field), against the reference's MQS.h_field of its own response."""
    from pcbqs_gb300.biot import h_field
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.ports import CopperPorts, MagneticModel
    g = via_golden()
    b = Board.load('viapair')
    r = CopperPorts(MagneticModel(b, conductor_loss='slab')).extract(g['freqs'])
    res = r.drive(np.ones((len(g['freqs']), len(r.names))))
    H = h_field(b, res.i[int(g['field_fi'])], g['field_pts'])
    assert H.shape == g['field_H'].shape
    assert np.abs(H - g['field_H']).max() <= 1e-7 * np.abs(g['field_H']).max()
    Hk = h_field(b, res.i[[int(g['field_fi'])]].T, g['field_pts'])          # (n, 3, k) form
    assert np.allclose(Hk[..., 0], H, rtol=0, atol=1e-12 * np.abs(H).max())
