"""The graph preconditioner on the device (pcbqs_gb300_peec_graph: the reference's _graph_preconditioner,
src/pcbqs/peec_iterative.py:19-84, its Laplacian factored dense in complex64) against the oracle's restatement of the
reference (oracle/graph.py, exact SuperLU factors), and the GMRES it preconditions against the reference's own
iterative solve with it (tests/golden/graph_<board>.npz: the reference's port impedances and GMRES steps)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _apply_on_device(model, freq, refine, y, parts=0):
    import torch
    from pcbqs_gb300 import _lib
    lib = _lib.load()
    handle, zscale = model._operator(np.array([2 * np.pi * freq]))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    try:
        model._graph_precondition(handle, 0, freq, refine, stream, parts)
        x = torch.as_tensor(np.ascontiguousarray(y), device='cuda')
        out = torch.empty_like(x)
        _lib.check(lib.pcbqs_gb300_peec_graph_apply(handle, y.shape[1], x.data_ptr(), out.data_ptr(), stream), lib)
        return out.cpu().numpy(), float(zscale[0])
    finally:
        lib.pcbqs_gb300_peec_destroy(handle)


@pytest.mark.parametrize('board,parts', [('tiny', 0), ('strip', 0), ('viapair', 0), ('tiny', 4), ('strip', 8)])
def test_graph_preconditioner_matches_oracle(device_library, board, parts):
    """Three random columns through the device preconditioner and through the restatement, at 1 MHz: within 1e-5
    of the largest output with FP64 corrections of the Laplacian solves (one for the dense Laplacian, two for the
    domain split), within 1e-2 without (the complex64 factors alone). parts > 0: the Laplacian split into domains
    (explicit block inverses, Schur complement on the separator)."""
    import oracle.graph as G
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    model = PeecModel(Board.load(board)).assemble()
    freq = 1e6
    rng = np.random.default_rng(3)
    y = rng.standard_normal((model.n, 3)) + 1j * rng.standard_normal((model.n, 3))
    errs = []
    for refine, bound in ((2 if parts else 1, 1e-5), (0, 1e-2)):
        got, zs = _apply_on_device(model, freq, refine, y, parts)
        diagonal = np.zeros(model.nb, complex)
        rd = np.asarray(model.R.diagonal(), complex)
        rd[:model.ne] *= model.resistance_ratio([freq])[0]
        diagonal[:model.ni] = rd + 2j * np.pi * freq * model.ldiag[:model.ni]
        apply = G.graph_preconditioner(model.K, model.A, model.T, model.B, model.nl, model.keep, model.passive,
                                       model.own[:model.nl], diagonal, zs, model.pscale, model.pdiag_host)
        for c in range(y.shape[1]):
            yref = np.empty(model.n, complex)
            yref[model.order] = y[:, c]
            ref = apply(yref)[model.order]
            err = np.abs(got[:, c] - ref).max() / np.abs(ref).max()
            errs.append(err)
            assert err < bound, (refine, err)
    print(f'{board} (parts {parts}): device graph preconditioner against the restatement: {max(errs[:3]):.2e} '
          f'(FP64 corrections), {max(errs[3:]):.2e} (complex64 factors alone)')


@pytest.mark.parametrize('board,parts', [('tiny', 0), ('strip', 0), ('viapair', 0), ('strip', 8)])
def test_graph_gmres_matches_reference_iterative_solve(device_library, board, parts):
    """GMRES to 1e-8 with the device graph preconditioner against the reference's GMRES with its own: the port
    impedances within 1e-5 (the reference's solve is on its compressed operator) and about the reference's step
    counts (at most 1.5 times + 5); the captured restart cycles (the preconditioner inside the CUDA graph) reach
    the same tolerance and impedances."""
    from conftest import GOLDEN
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    with np.load(GOLDEN / f'graph_{board}.npz') as g:
        freqs, its_ref, Zg = g['freqs'], g['iterations'], g['Z']
    model = PeecModel(Board.load(board))
    res = model.solve(freqs, precondition='graph', graph_parts=parts)
    its = res.iterations.reshape(len(freqs), -1)
    err = np.abs(res.impedance - Zg).max() / np.abs(Zg).max()
    print(f'{board} graph (parts {parts}): GMRES steps {its.max(axis=1).tolist()} (reference {its_ref.max(axis=1).tolist()}), '
          f'port Z against the reference iterative solve {err:.2e}, set-up {model.timings["precondition_ms"]:.1f} ms')
    assert (res.residual <= 1e-8).all()
    assert err < 1e-5, err
    assert (its.max(axis=1) <= 1.5 * its_ref.max(axis=1) + 5).all()
    if parts:
        with pytest.raises(ValueError, match='captured'):
            model.solve(freqs, precondition='graph', graph_parts=parts, captured=True)
        return
    cap = model.solve(freqs, precondition='graph', captured=True)
    assert (cap.residual <= 1e-8).all()
    assert np.abs(cap.impedance - res.impedance).max() <= 1e-9 * np.abs(res.impedance).max()


def test_graph_preconditions_the_compressed_plane_pair(device_library):
    """The 22,554-triangle plane pair with the compressed operator (H-matrices at their default tolerance 1e-6),
    which block-Jacobi does not bring to 1e-8 within 2,000 steps: the graph preconditioner does, for the FP64 GMRES
    and for the mixed solve (BF16 low-rank inner products), with the dense Laplacian and split into 16 domains, and
    the port impedances agree with the reference's dense
    solve (tests/golden/peec_planes.npz) within 1e-4 of the largest."""
    from conftest import GOLDEN
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    with np.load(GOLDEN / 'peec_planes.npz') as g:
        f, Zr = float(g['freqs'][0]), g['Z'][0]
    model = PeecModel(Board.load('planes'), matrix='hierarchical').assemble()
    for mixed, parts in ((False, 0), (True, 0), (True, 16)):
        res = model.solve([f], precondition='graph', mixed=mixed, graph_parts=parts)
        err = np.abs(res.impedance[0] - Zr).max() / np.abs(Zr).max()
        t = model.timings
        print(f'planes compressed, graph (parts {parts}), mixed={mixed}: GMRES steps {res.iterations.max()}, port Z error {err:.2e}, '
              f'preconditioner {t["precondition_ms"]:.0f} ms, GMRES {t["gmres_ms"]:.0f} ms')
        assert (res.residual <= 1e-8).all()
        assert err < 1e-4, err


def test_graph_on_the_dense_plane_pair(device_library):
    """The dense plane pair with the graph preconditioner beside the complex64 factor of the whole system: both
    reach 1e-8 and the same port impedances (1e-7); the graph preconditioner takes more steps from a smaller factor
    (the Laplacian's 22,224 nodes against 32,990 unknowns)."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    model = PeecModel(Board.load('planes')).assemble()
    f = 1e6
    graph = model.solve([f], precondition='graph')
    tg = dict(model.timings)
    lu = model.solve([f], precondition='lu32')
    err = np.abs(graph.impedance - lu.impedance).max() / np.abs(lu.impedance).max()
    print(f'planes dense: graph {graph.iterations.max()} steps ({tg["precondition_ms"]:.0f} + {tg["gmres_ms"]:.0f} '
          f'ms), lu32 {lu.iterations.max()} steps ({model.timings["precondition_ms"]:.0f} + '
          f'{model.timings["gmres_ms"]:.0f} ms), port Z {err:.2e}')
    assert (graph.residual <= 1e-8).all()
    assert err < 1e-7, err
