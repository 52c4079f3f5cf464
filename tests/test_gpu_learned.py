"""The learned block preconditioner's device kernels against the CPU restatement (oracle/learned.py), its training
on the GPU, and what the trained network (pcbqs_gb300/learned_params.npz, trained on the seeded random boards
train_*) gains over block-Jacobi on held-out boards."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def random_system(n=150, bs=16, seed=0):
    import torch
    from pcbqs_gb300.learned import block_system
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A = A * np.exp(-np.abs(np.subtract.outer(np.arange(n), np.arange(n))) / 20) + 5 * np.sqrt(n) * np.eye(n)
    return A, block_system(torch.as_tensor(A, device='cuda'), rng.random(n) < 0.4, 1e6, bs=bs, per_block=4)


def test_kernels_match_oracle(device_library):
    import torch
    from oracle import learned as lo
    from pcbqs_gb300 import learned as L
    A, s = random_system()
    rng = np.random.default_rng(3)
    params = torch.as_tensor(0.4 * rng.standard_normal(L.NPARAMS), device='cuda')
    hidden, gains = L.forward(s, params)
    h_ref, g_ref = lo.forward(s.phi.cpu().numpy(), params.cpu().numpy(), L.NHIDDEN)
    np.testing.assert_allclose(gains.cpu().numpy(), g_ref, rtol=1e-12, atol=1e-13)
    Z = L.probes(s, 5, 7)
    X, U = L.apply(s, gains, Z, corrections=True)
    args = (len(A), s.bs, s.eptr.cpu().numpy(), s.ecol.cpu().numpy(), s.dinv.cpu().numpy(), s.E.cpu().numpy())
    X_ref, U_ref = lo.apply(*args, g_ref, Z.cpu().numpy())
    assert np.abs(X.cpu().numpy() - X_ref).max() <= 1e-12 * np.abs(X_ref).max()
    assert np.abs(U.cpu().numpy() - U_ref).max() <= 1e-12 * np.abs(U_ref).max()
    loss, grad = L.loss_and_gradient(s, params, Z)
    loss_ref, dg_ref = lo.loss_and_gains_gradient(A, *args[1:], g_ref, Z.cpu().numpy())
    grad_ref = lo.backward(s.phi.cpu().numpy(), params.cpu().numpy(), L.NHIDDEN, h_ref, dg_ref)
    assert abs(loss - loss_ref) <= 1e-10 * loss_ref
    np.testing.assert_allclose(grad.cpu().numpy(), grad_ref, rtol=1e-9, atol=1e-12 * np.abs(grad_ref).max())
    # block-Jacobi alone: zero gains give the same as no gains
    Y0 = L.apply(s, None, Z)
    Yz = L.apply(s, torch.zeros_like(gains), Z)
    assert torch.equal(Y0, Yz)


def test_training_lowers_the_preconditioned_residual(device_library):
    from pcbqs_gb300 import learned as L
    systems = [random_system(seed=i)[1] for i in range(2)]
    params, history = L.train(systems, steps=40, lr=0.05)
    assert history[0] == pytest.approx(1.0, abs=1e-12)          # it starts at block-Jacobi
    assert history[-1] < 0.9 * history[0]


def _held_out_steps(name, params):
    import torch
    from pcbqs_gb300 import learned as L
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    model = PeecModel(Board.load(name)).assemble()
    total_bj = total_l = 0
    for f in (3e5, 3e6):
        s = L.block_system_of(model, f)
        Z = L.probes(s, 8, 11)
        base = L.loss_and_gradient(s, torch.zeros_like(params), Z)[0]
        learned = L.loss_and_gradient(s, params, Z)[0]
        assert learned < base, (name, f, learned, base)
        its_bj, its_l, res = L.compare(s, params)
        assert (res <= 1e-8).all()
        total_bj += int(its_bj.sum())
        total_l += int(its_l.sum())
    return total_bj, total_l


@pytest.mark.parametrize('name', ['viapair', 'tiny'])
def test_trained_network_beats_block_jacobi_on_held_out_boards(device_library, name):
    """On each board outside the training set (the strip pair joined by vias, the tiny plane pair), at frequencies
    of the training range, the trained gains lower the preconditioned residual of fresh probes and the GMRES steps
    to 1e-8 (every column still converges: the learned preconditioner is only an accelerator)."""
    from pcbqs_gb300 import learned as L
    total_bj, total_l = _held_out_steps(name, L.load())
    assert total_l < total_bj, (name, total_l, total_bj)


@pytest.mark.xfail(strict=True, reason='the one-layer strip, a geometry outside the training set, converges more '
                                       'slowly with the learned gains than with block-Jacobi alone')
def test_trained_network_on_the_one_layer_strip(device_library):
    from pcbqs_gb300 import learned as L
    total_bj, total_l = _held_out_steps('strip', L.load())
    assert total_l < total_bj, ('strip', total_l, total_bj)
