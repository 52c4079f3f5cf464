"""The device PEEC solve (fill -> L, P -> loop/tree operator -> block-Jacobi GMRES) against the reference's own
dense PEEC solve (tests/golden/peec_*.npz, made by make_peec_golden.py) on the same boards. Port impedances
within 1e-6 relative (GMRES to a 1e-8 relative residual per column); the resistive part within 1e-4 of itself."""
import ctypes

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def golden(name):
    with np.load(GOLDEN / f'peec_{name}.npz') as d:
        return {k: d[k] for k in d.files}


@pytest.mark.parametrize('board', ['tiny', 'strip'])
@pytest.mark.parametrize('precondition', ['block_jacobi', 'lu32'])
def test_port_impedance_matches_reference(device_library, board, precondition):
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    g = golden(board)
    model = PeecModel(Board.load(board))
    res = model.solve(g['freqs'], precondition=precondition)
    assert list(res.names) == [str(p) for p in g['ports']]
    Z, Zr = res.impedance, g['Z']
    err = np.abs(Z - Zr).max() / np.abs(Zr).max()
    assert err < 1e-6, err
    assert np.abs(Z.real - Zr.real).max() <= 1e-4 * np.abs(Zr.real).max() + 1e-9 * np.abs(Zr).max()
    assert (res.residual <= 1e-8).all() and (res.iterations > 0).all()
    # reciprocity of the port matrix
    assert np.abs(Z - Z.transpose(0, 2, 1)).max() <= 1e-6 * np.abs(Z).max()
    if precondition == 'lu32':      # a single-precision factor leaves a handful of FP64 GMRES steps
        assert res.iterations.max() <= 20


def test_operator_product_matches_host_algebra(device_library):
    """pcbqs_gb300_peec_apply against K^T (R + j w L) K D y / zscale + T^T P T y / pscale on the host."""
    import torch
    from pcbqs_gb300 import _lib
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    model = PeecModel(Board.load('tiny')).assemble()
    omegas = np.array([2e5 * np.pi, 2e7 * np.pi])
    handle, zscale = model._operator(omegas)
    lib = _lib.load()
    try:
        rng = np.random.default_rng(0)
        n, k = model.n, 3
        y = rng.standard_normal((n, k)) + 1j * rng.standard_normal((n, k))
        sys = np.array([0, 1, 1], np.int32)
        yin = torch.as_tensor(y, device='cuda')
        out = torch.zeros_like(yin)
        _lib.check(lib.pcbqs_gb300_peec_apply(handle, k, _lib.ptr(sys, ctypes.c_int32), yin.data_ptr(), out.data_ptr(),
                                              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), lib)
        got = out.cpu().numpy()
    finally:
        lib.pcbqs_gb300_peec_destroy(handle)
    L, P = model.L.cpu().numpy(), model.P.cpu().numpy()
    K, T, R = model.Kp, model.Tp, model.R
    for c in range(k):
        w, zs = omegas[sys[c]], zscale[sys[c]]
        d = np.where(model.is_tree == 1, 1j * w * zs / model.pscale, 1.0)
        branch = K @ (d * y[:, c])
        v = R @ branch + 1j * w * (L @ branch)
        expect = K.T @ v / zs + T.T @ (P @ (T @ y[:, c])) / model.pscale
        assert np.abs(got[:, c] - expect).max() <= 1e-12 * np.abs(expect).max()


@pytest.mark.parametrize('board', ['tiny', 'strip'])
def test_mixed_precision_solve_matches_reference(device_library, board):
    """FP64 refinement around a single-precision inner GMRES reaches the same 1e-8 FP64 residual and port Z."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    g = golden(board)
    model = PeecModel(Board.load(board))
    res = model.solve(g['freqs'], precondition='lu32', mixed=True)
    Z, Zr = res.impedance, g['Z']
    assert np.abs(Z - Zr).max() / np.abs(Zr).max() < 1e-6
    assert (res.residual <= 1e-8).all()
    assert model.timings['outer_steps'] >= 1


@pytest.mark.parametrize('factor_math', ['bf16x9-blocked', 'tc6-blocked', 'tc3-blocked'])
def test_planes_solves_match_reference(device_library, factor_math):
    """The benchmarked board, the 22,554-triangle plane pair (32,990 unknowns, 8 ports) at 1 MHz, against the
    reference's own dense solve of it (tests/golden/peec_planes.npz: pcbqs.peec.solve through MQS, LAPACK's double
    LU): the FP64 path (FP64 fill and operator) and the mixed path (FP32 far pairs and inner products under FP64
    refinement), both with the complex64-factor preconditioner of each trailing-update arithmetic, reach a 1e-8
    relative residual and match every port impedance to 1e-6 of the largest. The part of Z that differs between
    ports (Z minus its mean entry: the inductive and resistive coupling under the common plane capacitance) to 1e-3
    of its own largest entry. The matrix is reciprocal, with non-negative loss on the diagonal."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    from conftest import GOLDEN
    with np.load(GOLDEN / 'peec_planes.npz') as g:
        f, Zr = float(g['freqs'][0]), g['Z'][0]
    model = PeecModel(Board.load('planes'))
    fp64 = model.solve([f], precondition='lu32', factor_math=factor_math)
    model.assemble(mixed=True)
    mixed = model.solve([f], precondition='lu32', mixed=True, factor_math=factor_math)
    Z64, Zm = fp64.impedance[0], mixed.impedance[0]
    assert (fp64.residual <= 1e-8).all() and (mixed.residual <= 1e-8).all()
    scale, Dr = np.abs(Zr).max(), Zr - Zr.mean()
    for Z in (Z64, Zm):
        err, derr = np.abs(Z - Zr).max() / scale, np.abs((Z - Z.mean()) - Dr).max() / np.abs(Dr).max()
        print(f'{factor_math}: port Z error {err:.2e} of max |Z|, coupling error {derr:.2e}; GMRES '
              f'{fp64.iterations.max()} / {mixed.iterations.max()} steps')
        assert err < 1e-6 and derr < 1e-3, (err, derr)
    assert np.abs(Z64 - Z64.T).max() <= 1e-6 * np.abs(Z64).max()
    assert (np.diag(Z64).real > 0).all() and (np.diag(Z64).imag < 0).all()     # capacitive plane pair at 1 MHz


@pytest.mark.parametrize('board,k,math', [('tiny', 3, 0), ('strip', 8, 0), ('strip', 11, 0), ('strip', 8, 2),
                                          ('strip', 11, 3)])
def test_streaming_triangular_solves_match_getrs(device_library, board, k, math):
    """The library's streaming solve with the complex64 factor (super-block panels, inverted diagonal blocks, one
    gather for the row interchanges) against cuSOLVER getrs on the same factor; k = 11 exercises a padded second
    sweep of 8 columns. math 2 and 3 factor with the library's blocked LU (two 2048-column panels on the strip),
    so getrs on its output also checks that it keeps getrf's layout and pivots. Both are FP32 solves in a different order, so they differ by FP32 rounding amplified by
    the factor's conditioning; the bar is the quantity GMRES cares about, the residual of the FP64 system, which
    over the batch must be no worse than getrs's (within 50 %)."""
    import torch
    from pcbqs_gb300 import _lib
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel, _csr_struct
    model = PeecModel(Board.load(board)).assemble()
    handle, _ = model._operator(np.array([2e6 * np.pi]))
    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    sys = np.zeros(k, np.int32)
    try:
        desc = _csr_struct(model._krk_device())
        _lib.check(lib.pcbqs_gb300_peec_factor(handle, ctypes.byref(desc), 0, math, stream), lib)
        rng = np.random.default_rng(k)
        b = torch.as_tensor(rng.standard_normal((model.n, k)) + 1j * rng.standard_normal((model.n, k)), device='cuda')
        outs, residuals = [], []
        for method in (0, 1, 0):
            x = torch.full_like(b, complex('nan'))
            _lib.check(lib.pcbqs_gb300_peec_lu_solve(handle, k, b.data_ptr(), x.data_ptr(), method, stream), lib)
            ax = torch.empty_like(b)
            _lib.check(lib.pcbqs_gb300_peec_apply(handle, k, _lib.ptr(sys, ctypes.c_int32), x.data_ptr(),
                                                  ax.data_ptr(), stream), lib)
            outs.append(x.cpu().numpy())
            residuals.append((torch.linalg.norm(ax - b, dim=0) / torch.linalg.norm(b, dim=0)).cpu().numpy())
    finally:
        lib.pcbqs_gb300_peec_destroy(handle)
    ours, getrs, again = outs
    assert np.isfinite(ours).all()
    assert np.array_equal(ours, again)                  # the captured sweep replays deterministically
    # column by column the two FP32 rounding patterns scatter; over the batch ours is no worse
    assert residuals[0].max() <= 1.5 * residuals[1].max() + 1e-6, (residuals[0], residuals[1])
    assert residuals[0].mean() <= 1.5 * residuals[1].mean() + 1e-6, (residuals[0], residuals[1])
    assert np.linalg.norm(ours - getrs) <= 1e-2 * np.linalg.norm(getrs)


@pytest.mark.parametrize('board,k', [('tiny', 40), ('strip', 40), ('strip', 128), ('planes', 128)])
def test_blocked_triangular_solve_matches_getrs(device_library, board, k):
    """The blocked solve for many right-hand sides (1024-row steps: the diagonal block in 128-row sub-blocks with
    their precomputed inverses, the off-diagonal products on the tcgen05 update with six part products; the
    factor read once for all columns) against the streaming sweeps and cuSOLVER
    getrs on the same complex64 factor (method 3, 2, 1 of pcbqs_gb300_peec_lu_solve). All three are FP32 solves
    with different rounding orders on an ill-conditioned factor (getrs's own residuals reach 1e-2 on the strip), so
    they scatter column by column: the FP64 system's residual over the batch no worse than getrs's within 50 % on
    average and 2x on the worst column, and the solutions within 1 % of each other; the automatic choice
    (method 0) is one of the two."""
    import torch
    from pcbqs_gb300 import _lib
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel, _csr_struct
    model = PeecModel(Board.load(board)).assemble()
    handle, _ = model._operator(np.array([2e6 * np.pi]))
    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    sys = np.zeros(k, np.int32)
    try:
        desc = _csr_struct(model._krk_device())
        _lib.check(lib.pcbqs_gb300_peec_factor(handle, ctypes.byref(desc), 0, 5, stream), lib)
        rng = np.random.default_rng(k)
        b = torch.as_tensor(rng.standard_normal((model.n, k)) + 1j * rng.standard_normal((model.n, k)), device='cuda')
        outs, residuals = {}, {}
        for method in (3, 2, 1, 0):
            x = torch.full_like(b, complex('nan'))
            _lib.check(lib.pcbqs_gb300_peec_lu_solve(handle, k, b.data_ptr(), x.data_ptr(), method, stream), lib)
            ax = torch.empty_like(b)
            _lib.check(lib.pcbqs_gb300_peec_apply(handle, k, _lib.ptr(sys, ctypes.c_int32), x.data_ptr(),
                                                  ax.data_ptr(), stream), lib)
            outs[method] = x.cpu().numpy()
            residuals[method] = (torch.linalg.norm(ax - b, dim=0) / torch.linalg.norm(b, dim=0)).cpu().numpy()
    finally:
        lib.pcbqs_gb300_peec_destroy(handle)
    blocked, streaming, getrs = outs[3], outs[2], outs[1]
    print(f'{board} k={k}: residual blocked {residuals[3].max():.2e}, streaming {residuals[2].max():.2e}, '
          f'getrs {residuals[1].max():.2e}')
    assert np.isfinite(blocked).all()
    assert residuals[3].mean() <= 1.5 * residuals[1].mean() + 1e-6, (residuals[3], residuals[1])
    assert residuals[3].max() <= 2.0 * residuals[1].max() + 1e-6, (residuals[3], residuals[1])
    assert np.linalg.norm(blocked - getrs) <= 1e-2 * np.linalg.norm(getrs)
    assert np.linalg.norm(blocked - streaming) <= 1e-2 * np.linalg.norm(streaming)
    assert np.array_equal(outs[0], blocked) or np.array_equal(outs[0], streaming)


@pytest.mark.parametrize('board', ['tiny', 'strip'])
def test_sweep_sharing_one_factor_matches_reference(device_library, board):
    """A three-decade sweep (1e5, 1e6, 1e7 Hz) solved as one batch of (frequency, port) columns, all preconditioned by
    the complex64 factor at the middle frequency: every column still reaches 1e-8 on its own FP64 system and the
    port impedances match the reference's dense solve; the anchor's own columns need the fewest iterations."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    g = golden(board)
    model = PeecModel(Board.load(board))
    res = model.solve(g['freqs'], precondition='lu32', mixed=True, anchors=1)
    assert res.timings['factorizations'] == 1
    Z, Zr = res.impedance, g['Z']
    assert np.abs(Z - Zr).max() / np.abs(Zr).max() < 1e-6
    assert (res.residual <= 1e-8).all()
    its = res.iterations.reshape(len(g['freqs']), -1)
    assert its[1].max() <= its.max()


@pytest.mark.parametrize('board', ['tiny', 'strip'])
@pytest.mark.parametrize('mixed', [False, True])
def test_slab_conductor_loss_matches_reference(device_library, board, mixed):
    """conductor_loss='slab': R(f) = Zs(f) sigma t R_dc per frequency (finite-thickness sheet impedance) in the
    operator, the factor and the right-hand side; port impedances against the reference's dense solve with the same
    loss model, and the resistive part against itself."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    g = golden(f'{board}_slab')
    assert str(g['conductor_loss']) == 'slab'
    model = PeecModel(Board.load(board), conductor_loss='slab')
    res = model.solve(g['freqs'], precondition='lu32', mixed=mixed)
    Z, Zr = res.impedance, g['Z']
    assert np.abs(Z - Zr).max() / np.abs(Zr).max() < 1e-6
    assert np.abs(Z.real - Zr.real).max() <= 1e-4 * np.abs(Zr.real).max() + 1e-9 * np.abs(Zr).max()
    assert (res.residual <= 1e-8).all()
    ratio = model.resistance_ratio(g['freqs'])
    assert ratio.real[-1] > ratio.real[0] >= 1.0         # skin effect raises the resistance with frequency


@pytest.mark.parametrize('mixed', [False, True])
def test_lossy_stack_dielectric_matches_reference(device_library, mixed):
    """dielectric='stack': P from the electrostatic images of a lossy FR-4 slab (complex), through the operator, the
    complex64 factor, the equilibrium solve (GMRES on the complex P preconditioned by Re P's Cholesky) and the
    charge correction; port impedances against the reference's dense solve with the same stack, and the loss tangent
    visible as Re Z / -Im Z."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.layered import DielectricStack
    from pcbqs_gb300.peec import PeecModel
    g = golden('tiny_stack')
    z0, z1, er, tand = g['slab']
    model = PeecModel(Board.load('tiny'), stack=DielectricStack.slab(z0, z1, er, tand))
    res = model.solve(g['freqs'], precondition='lu32', mixed=mixed)
    Z, Zr = res.impedance, g['Z']
    assert np.abs(Z - Zr).max() / np.abs(Zr).max() < 1e-6
    assert np.abs(Z.real - Zr.real).max() <= 1e-4 * np.abs(Zr.real).max() + 1e-9 * np.abs(Zr).max()
    assert (res.residual <= 1e-8).all()
    assert model.Pim is not None
    ratio = Z[1, 0, 0].real / -Z[1, 0, 0].imag
    assert 0.5 * tand < ratio < 2 * tand


@pytest.mark.parametrize('n,k', [(1000, 3), (2500, 8), (700, 11)])
def test_dense_products_match_host(device_library, n, k):
    """pcbqs_gb300_dense_apply (FP64) and _dense_apply_single (FP32, autotuned shape) against NumPy for a random
    symmetric matrix and complex columns, including a column count that takes two passes of 16 real columns."""
    import torch
    from pcbqs_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(n + k)
    M = rng.standard_normal((n, n))
    M = (M + M.T) / 2
    X = rng.standard_normal((n, k)) + 1j * rng.standard_normal((n, k))
    ref = M @ X
    Md, Mf = torch.as_tensor(M, device='cuda'), torch.as_tensor(M.astype(np.float32), device='cuda')
    Xd = torch.as_tensor(X, device='cuda')
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    Y = torch.empty_like(Xd)
    _lib.check(lib.pcbqs_gb300_dense_apply(n, k, Md.data_ptr(), n, Xd.data_ptr(), Y.data_ptr(), stream), lib)
    torch.cuda.synchronize()
    assert np.abs(Y.cpu().numpy() - ref).max() <= 1e-12 * np.abs(ref).max() + 1e-12 * np.sqrt(n)
    Yf = torch.empty_like(Xd)
    for _ in range(2):              # first call tunes the shape, the second uses the cached choice
        _lib.check(lib.pcbqs_gb300_dense_apply_single(n, k, Mf.data_ptr(), n, Xd.data_ptr(), Yf.data_ptr(), stream),
                   lib)
        torch.cuda.synchronize()
        assert np.abs(Yf.cpu().numpy() - ref).max() <= 1e-4 * np.abs(ref).max()


@pytest.mark.parametrize('precondition,mixed,loss', [('block_jacobi', False, 'dc'), ('lu32', False, 'dc'),
                                                     ('lu32', True, 'dc'), ('lu32', False, 'slab'),
                                                     ('block_jacobi', False, 'slab')])
def test_port_impedance_through_vias_matches_reference(device_library, precondition, mixed, loss):
    """The via pair (a strip over its return, joined by two plated vias) with capacitance: the via segments are
    branches with their barrel's R and filament L, the port impedance against the reference's dense PEEC solve; under
    slab loss the sheets' R follows the frequency and the barrels keep their DC resistance (the preconditioners
    scale both, which only costs iterations)."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    g = golden('viapair' if loss == 'dc' else 'viapair_slab')
    model = PeecModel(Board.load('viapair'), conductor_loss=loss).assemble(mixed=mixed)
    res = model.solve(g['freqs'], precondition=precondition, mixed=mixed)
    assert model.n == int(g['unknowns']) and model.nl == int(g['loops'])
    err = np.abs(res.impedance - g['Z']).max() / np.abs(g['Z']).max()
    assert err < 1e-6, err
    assert (res.residual <= 1e-8).all()


@pytest.mark.parametrize('board', ['tiny', 'strip', 'viapair'])
def test_preconditioners_against_the_reference_graph_preconditioner(device_library, board):
    """The reference's own iterative solve with its graph preconditioner (tests/golden/graph_<board>.npz:
    peec_iterative.solve on its compressed model, solver_preconditioner='graph', SciPy GMRES restart 100 to 1e-8,
    every port driven alone) beside this library's preconditioners on the same board and frequencies: the port
    impedances agree within the compression tolerance (1e-6 relative), and the GMRES step counts are reported per
    preconditioner (printed: block-Jacobi, the complex64 factor, the reference's graph ILU)."""
    from conftest import GOLDEN
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    with np.load(GOLDEN / f'graph_{board}.npz') as g:
        freqs, its_graph, Zg = g['freqs'], g['iterations'], g['Z']
    model = PeecModel(Board.load(board))
    for precondition in ('block_jacobi', 'lu32'):
        res = model.solve(freqs, precondition=precondition)
        its = res.iterations.reshape(len(freqs), -1)
        err = np.abs(res.impedance - Zg).max() / np.abs(Zg).max()
        print(f'{board} {precondition}: GMRES steps {its.max(axis=1).tolist()} (reference graph ILU '
              f'{its_graph.max(axis=1).tolist()}), port Z against the reference iterative solve {err:.2e}')
        assert (res.residual <= 1e-8).all()
        assert err < 1e-5, err
