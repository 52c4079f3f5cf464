"""The batched GMRES with each restart cycle captured as one CUDA graph launch (PeecModel.solve(captured=True):
the Arnoldi steps in a conditional WHILE node controlled on the device, per-column convergence masks, no host
synchronization between steps) against the host-driven cycle, and the batched sweep of the 16-port plane pair
(64 log-spaced frequencies from 1 kHz to 100 MHz x 16 ports = 1,024 columns, 8 shared complex64 factors) against
the reference's own dense solve (tests/golden/peec_planes16.npz, pcbqs.peec.solve at two of the sweep's
frequencies). Reference behaviour: mqs_iterative.port_matrix / _lockstep_gmres (src/pcbqs/mqs_iterative.py:109-170,
:298-367): every column to the relative residual 1e-8."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('board,precondition,mixed,restart,anchors', [
    ('tiny', 'block_jacobi', False, 20, None),     # many restart cycles: the active set shrinks, graphs rebuilt
    ('tiny', 'lu32', False, 100, 1),               # one factor shared by three frequencies
    ('strip', 'lu32', True, 100, 1),               # the mixed refinement's inner GMRES captured
])
def test_captured_cycles_match_host_driven(device_library, board, precondition, mixed, restart, anchors):
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    model = PeecModel(Board.load(board), restart=restart)
    model.assemble(mixed=mixed)
    freqs = [1e5, 1e6, 1e7]
    host = model.solve(freqs, precondition=precondition, mixed=mixed, anchors=anchors)
    graph = model.solve(freqs, precondition=precondition, mixed=mixed, anchors=anchors, captured=True)
    assert np.array_equal(graph.iterations, host.iterations)
    assert np.array_equal(graph.impedance, host.impedance)
    assert (graph.residual <= 1e-8).all()
    if precondition == 'block_jacobi':
        assert host.iterations.max() > restart       # the case really restarts


def test_sweep_16_ports_64_frequencies_matches_reference(device_library):
    from conftest import GOLDEN
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    freqs = np.geomspace(1e3, 1e8, 64)
    model = PeecModel(Board.load('planes16'))
    model.assemble(mixed=True)
    res = model.solve(freqs, precondition='lu32', mixed=True, anchors=8, captured=True)
    assert res.impedance.shape == (64, 16, 16)
    assert (res.residual <= 1e-8).all(), res.residual.max()
    with np.load(GOLDEN / 'peec_planes16.npz') as g:
        for f, Zr in zip(g['freqs'], g['Z']):
            fi = int(np.argmin(np.abs(freqs - f)))
            assert abs(freqs[fi] / f - 1) < 1e-12
            err = np.abs(res.impedance[fi] - Zr).max() / np.abs(Zr).max()
            print(f'{f:.4g} Hz: port Z error {err:.2e}')
            assert err < 1e-6, err


def test_tensor_core_inner_products_match_the_fp32_ones(device_library):
    """Nine frequencies x 2 ports = 18 columns in one batch: the mixed refinement's inner products run on the
    tensor cores (16 or more columns). With three or six BF16 parts or the FP32 CUDA-core product, and with the
    outer FP64 residuals on the FP64 pipe or from integer slices on the tensor cores, every column reaches 1e-8 on
    its FP64 system and the port impedances agree with each other and with the reference at its three frequencies;
    the captured cycles repeat the host-driven ones bit for bit on the tensor-core path too."""
    from conftest import GOLDEN
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    freqs = np.geomspace(1e5, 1e7, 9)
    model = PeecModel(Board.load('strip'))
    model.assemble(mixed=True)
    runs = {p: model.solve(freqs, precondition='lu32', mixed=True, anchors=1, product=p, fp64_product='fp64')
            for p in ('fp32', 'tc3', 'tc6')}
    runs['tc3+sliced6'] = model.solve(freqs, precondition='lu32', mixed=True, anchors=1, product='tc3',
                                      fp64_product='sliced6')
    graph = model.solve(freqs, precondition='lu32', mixed=True, anchors=1, product='tc3', fp64_product='fp64',
                        captured=True)
    assert np.array_equal(graph.impedance, runs['tc3'].impedance)
    assert np.array_equal(graph.iterations, runs['tc3'].iterations)
    Zf = runs['fp32'].impedance
    with np.load(GOLDEN / 'peec_strip.npz') as g:
        Zr = g['Z']
    for p, res in runs.items():
        assert (res.residual <= 1e-8).all(), (p, res.residual.max())
        assert np.abs(res.impedance - Zf).max() / np.abs(Zf).max() < 1e-7, p
        err = np.abs(res.impedance[::4] - Zr).max() / np.abs(Zr).max()
        print(f'{p}: inner iterations {res.iterations.max()}, outer {res.timings.get("outer_steps")}, '
              f'error vs reference {err:.2e}')
        assert err < 1e-6, (p, err)
