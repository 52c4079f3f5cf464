"""Device H-matrix of L (device ACA and dense leaves, device product) against the reference's own HMatrix product and
its dense L (tests/golden/hmatrix_strip.npz, made by make_hmatrix_golden.py): the reference's tests hold two builds
within 50 x tol of each other (tests/test_compressed.py:316-320)."""
import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('rank', [32, 128])
def test_hmatrix_product_matches_reference(device_library, rank):
    import torch
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.fill import DeviceFill
    from pcbqs_gb300.hmatrix import DeviceHMatrix
    with np.load(GOLDEN / 'hmatrix_strip.npz') as d:
        g = {k: d[k] for k in d.files}
    b = Board.load('strip')
    fill = DeviceFill(b.nodes, b.tris, b.z, outer_levels=1, near=3.0)
    H = DeviceHMatrix(fill, tol=float(g['tol']), leaf=int(g['leaf']), eta=float(g['eta']), rank=rank)
    X = torch.as_tensor(g['X'], device='cuda')
    Y = H.matmat(X).cpu().numpy()
    scale = np.abs(g['Y_dense']).max()
    assert np.abs(Y - g['Y_dense']).max() <= 50 * float(g['tol']) * scale
    assert np.abs(Y - g['Y_h']).max() <= 50 * float(g['tol']) * scale
    assert H.info['low_rank_blocks'] > 0 and H.info['bytes'] < 0.5 * H.info['dense_bytes']
    assert H.info['max_rank'] <= rank
    # the product is deterministic
    assert np.array_equal(Y, H.matmat(X).cpu().numpy())


def test_compressed_potential_matches_dense(device_library):
    """W^T H W with H the compressed triangle kernel M0 / (A A 4 pi eps0 er) against the dense device P (itself
    pinned to the reference), within 50 x tol."""
    import torch
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.fill import DeviceFill
    from pcbqs_gb300.hmatrix import DeviceHMatrix
    b = Board.load('strip')
    fill = DeviceFill(b.nodes, b.tris, b.z, outer_levels=1, near=3.0)
    H = DeviceHMatrix(fill, tol=1e-6, leaf=64, eta=1.0, rank=32, kernel='potential', er=b.er)
    apply = H.potential_operator(b.node_of)
    planes, _ = fill.moments(scalar_only=True)
    P = fill.potential(planes[0], b.node_of, b.er)
    rng = np.random.default_rng(1)
    nn = P.shape[0]
    X = torch.as_tensor(rng.standard_normal((nn, 2)) + 1j * rng.standard_normal((nn, 2)), device='cuda')
    Y = apply(X).cpu().numpy()
    Yd = (P.to(torch.complex128) @ X).cpu().numpy()
    assert np.abs(Y - Yd).max() <= 50 * 1e-6 * np.abs(Yd).max()
    assert H.info['low_rank_blocks'] > 0


@pytest.mark.parametrize('kernel', ['inductance', 'potential'])
def test_hmatrix_pickle_round_trip(device_library, kernel):
    """A pickled and reloaded operator (the operator cache of HMatrix.__getstate__/__setstate__,
    src/pcbqs/hmatrix.py:308-316) applies bit for bit as the original; it keeps no fill (no exact entries)."""
    import pickle
    import torch
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.fill import DeviceFill
    from pcbqs_gb300.hmatrix import DeviceHMatrix
    b = Board.load('strip')
    fill = DeviceFill(b.nodes, b.tris, b.z, outer_levels=1, near=3.0)
    H = DeviceHMatrix(fill, tol=1e-6, leaf=64, eta=1.0, rank=32, kernel=kernel, er=b.er)
    blob = pickle.dumps(H)
    G = pickle.loads(blob)
    assert G.fill is None and G.info == H.info
    rng = np.random.default_rng(5)
    X = torch.as_tensor(rng.standard_normal((H.n, 3)) + 1j * rng.standard_normal((H.n, 3)), device='cuda')
    assert torch.equal(H.matmat(X), G.matmat(X))
    if kernel == 'potential':
        nn = int(b.node_of.max()) + 1
        Xn = X[:nn].contiguous()
        Yh, Yg = H.potential_operator(b.node_of)(Xn), G.potential_operator(b.node_of)(Xn)
        assert torch.allclose(Yh, Yg, rtol=1e-13, atol=1e-13 * Yh.abs().max().item())   # sparse W products
