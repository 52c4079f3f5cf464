"""The compressed PEEC operator (PeecModel(matrix='hierarchical')): L's edges and the triangle potential as device
H-matrices, the via segments as their dense block, every product of the FP64 GMRES through them, block-Jacobi from
exact entries and the equilibrium charge by GMRES on the compressed P. Reference behaviour: matrix_backend=
'hierarchical' (src/pcbqs/mqs.py:452-455) with the products of peec_iterative.py:267-278 through
HMatrix._native_matmat and compressed.PotentialOperator (compressed.py:194-204): its port impedances within the
compression tolerance of the dense solve, here against the reference's own dense solve (tests/golden/peec_*.npz)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _golden(board):
    from conftest import GOLDEN
    with np.load(GOLDEN / f'peec_{board}.npz') as g:
        return {k: g[k] for k in g.files}


@pytest.mark.parametrize('board', ['tiny', 'strip', 'viapair'])
def test_compressed_solve_matches_reference(device_library, board):
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    g = _golden(board)
    model = PeecModel(Board.load(board), matrix='hierarchical', hmatrix=dict(tol=1e-9, leaf=64))
    model.assemble()
    info = model.timings['hmatrix_L']
    res = model.solve(g['freqs'], precondition='block_jacobi')
    Z, Zr = res.impedance, g['Z']
    err = np.abs(Z - Zr).max() / np.abs(Zr).max()
    print(f'{board}: L {info["blocks"]} blocks ({info["low_rank_blocks"]} low rank, {info["bytes"] / 1e6:.1f} MB '
          f'of {info["dense_bytes"] / 1e6:.1f} MB dense), GMRES steps {res.iterations.max()}, port Z error {err:.2e}')
    assert (res.residual <= 1e-8).all()
    assert err < 1e-6, err


def test_compressed_operator_matches_dense(device_library):
    """The operator's product on random columns, compressed against dense: the blocks' ACA tolerance (1e-10 of each
    block) carried through the operator's sums (its L and P terms partly cancel), about 1e-8 of its norm."""
    import torch
    from pcbqs_gb300 import _lib
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    board = Board.load('viapair')
    freqs = np.array([1e5, 1e7])
    dense = PeecModel(board).assemble()
    comp = PeecModel(board, matrix='hierarchical', hmatrix=dict(tol=1e-10, leaf=64)).assemble()
    lib = device_library
    g = torch.Generator(device='cuda').manual_seed(11)
    k = 6
    x = torch.complex(torch.randn(dense.n, k, device='cuda', generator=g, dtype=torch.float64),
                      torch.randn(dense.n, k, device='cuda', generator=g, dtype=torch.float64))
    sys = np.array([0, 1, 0, 1, 0, 1], np.int32)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = []
    for m in (dense, comp):
        h, _ = m._operator(2 * np.pi * freqs)
        y = torch.empty_like(x)
        try:
            _lib.check(lib.pcbqs_gb300_peec_apply(h, k, _lib.ptr(sys, ctypes.c_int32), x.data_ptr(), y.data_ptr(),
                                                  stream), lib)
        finally:
            lib.pcbqs_gb300_peec_destroy(h)
        out.append(y)
    err = (torch.linalg.norm(out[1] - out[0]) / torch.linalg.norm(out[0])).item()
    print(f'compressed operator against dense: {err:.2e}')
    assert err < 1e-7, err
    assert np.abs(comp.ldiag - dense.ldiag).max() <= 1e-12 * np.abs(dense.ldiag).max()
    assert abs(comp.pscale / dense.pscale - 1) < 1e-12


def test_compressed_rejects_what_needs_dense_matrices(device_library):
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    model = PeecModel(Board.load('tiny'), matrix='hierarchical', hmatrix=dict(leaf=64))
    model.assemble()
    with pytest.raises(ValueError, match='block_jacobi'):
        model.solve([1e6], precondition='lu32')


@pytest.mark.parametrize('dense', [False, True])
@pytest.mark.parametrize('kernel,k', [('inductance', 16), ('inductance', 128), ('potential', 40)])
def test_lowrank_product_on_tensor_cores(device_library, kernel, k, dense):
    """The H-matrix product with its low-rank blocks (and, dense=True, its dense leaves) in BF16 three-part products
    on the tensor cores against the FP64 product: the difference stays at BF16x3's level (about 2^-16 of the part
    on the tensor cores)."""
    import torch
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.fill import DeviceFill
    from pcbqs_gb300.hmatrix import DeviceHMatrix
    b = Board.load('strip')
    fill = DeviceFill(b.nodes, b.tris, b.z, 1, 3.0)
    H = DeviceHMatrix(fill, tol=1e-8, leaf=64, kernel=kernel)
    assert H.low_rank > 0
    g = torch.Generator(device='cuda').manual_seed(5)
    X = torch.complex(torch.randn(H.n, k, device='cuda', generator=g, dtype=torch.float64),
                      torch.randn(H.n, k, device='cuda', generator=g, dtype=torch.float64))
    ref = H.matmat(X)
    ours = H.matmat_lowrank(X, dense=dense)
    err = (torch.linalg.norm(ours - ref) / torch.linalg.norm(ref)).item()
    print(f'{kernel} k={k} dense={dense}: {H.low_rank} low-rank blocks, BF16 product against FP64 {err:.2e}')
    assert err < (1e-4 if dense else 1e-5), err
    again = H.matmat_lowrank(X, dense=dense)
    assert torch.equal(again, ours)               # deterministic (slot rows summed in block order)


@pytest.mark.parametrize('kernel', ['inductance', 'potential'])
def test_plane_packing_kernel_matches_restatement(device_library, monkeypatch, kernel):
    """The tensor-core planes of the low-rank plan (left, right and dense-leaf planes) as k_pack_parts writes them
    equal, bit for bit, the same plan packed by the kernel's restatement (tests/test_lowrank_host.py)."""
    import torch
    import pcbqs_gb300.hmatrix as hm
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.fill import DeviceFill
    from test_lowrank_host import emulate_pack_parts
    b = Board.load('strip')
    fill = DeviceFill(b.nodes, b.tris, b.z, 1, 3.0)
    H = hm.DeviceHMatrix(fill, tol=1e-8, leaf=64, kernel=kernel, er=b.er)
    keep, _ = H.lowrank_plan(dense=True)
    monkeypatch.setattr(hm, '_pack_launch', emulate_pack_parts)
    ref, _ = H.lowrank_plan(dense=True)
    for name in ('lplane', 'rplane', 'dplane'):
        assert torch.equal(keep[name].view(torch.int16), ref[name].view(torch.int16)), name
    assert int((keep['lplane'] != 0).sum()) > 0 and int((keep['dplane'] != 0).sum()) > 0


@pytest.mark.parametrize('board', ['strip', 'viapair'])
def test_compressed_mixed_solve_matches_reference(device_library, board):
    """The mixed compressed solve: inner GMRES with the low-rank blocks in BF16 on the tensor cores, FP64 outer
    residuals through the FP64 H-matrix products; every column to 1e-8 and the port impedances to the reference."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    g = _golden(board)
    model = PeecModel(Board.load(board), matrix='hierarchical', hmatrix=dict(tol=1e-9, leaf=64))
    model.assemble(mixed=True)
    res = model.solve(g['freqs'], precondition='block_jacobi', mixed=True)
    err = np.abs(res.impedance - g['Z']).max() / np.abs(g['Z']).max()
    print(f'{board} mixed compressed: GMRES steps {res.iterations.max()}, outer {res.timings.get("outer_steps")}, '
          f'port Z error {err:.2e}')
    assert (res.residual <= 1e-8).all()
    assert err < 1e-6, err
