"""The learned block preconditioner's CPU restatement (oracle/learned.py) against finite differences, and the block
and edge bookkeeping of pcbqs_gb300.learned.block_system on a CPU tensor: the checks its device kernels are held to."""
import numpy as np


def random_system(n=70, bs=8, per=3, seed=0):
    import torch
    from pcbqs_gb300.learned import block_system
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A = A * np.exp(-np.abs(np.subtract.outer(np.arange(n), np.arange(n))) / 12) + 4 * np.sqrt(n) * np.eye(n)
    s = block_system(torch.as_tensor(A), rng.random(n) < 0.4, 1e6, bs=bs, per_block=per)
    return A, s


def test_block_system_bookkeeping():
    A, s = random_system()
    nblk, bs = s.nblk, s.bs
    assert s.eptr[0] == 0 and s.eptr[-1] == s.nedge and (np.diff(s.eptr.numpy()) <= 3).all()
    for b in range(nblk):
        cols = s.ecol[s.eptr[b]:s.eptr[b + 1]].numpy()
        assert (np.diff(cols) > 0).all() and b not in cols
        for e, c in zip(range(int(s.eptr[b]), int(s.eptr[b + 1])), cols):
            r0, c0 = b * bs, c * bs
            blk = np.zeros((bs, bs), complex)
            sub = A[r0:r0 + bs, c0:c0 + bs]
            blk[:sub.shape[0], :sub.shape[1]] = sub
            assert np.array_equal(s.E[e].numpy(), blk)
    assert np.isfinite(s.phi.numpy()).all() and s.phi.shape == (s.nedge, 6)
    last = s.dinv[-1].numpy() @ np.pad(A[(nblk - 1) * bs:, (nblk - 1) * bs:], ((0, nblk * bs - len(A)),) * 2)
    assert np.allclose(last[:len(A) - (nblk - 1) * bs, :len(A) - (nblk - 1) * bs], np.eye(len(A) - (nblk - 1) * bs))


def test_oracle_gradients_match_finite_differences():
    from oracle import learned as lo
    A, s = random_system(seed=1)
    args = (A, s.bs, s.eptr.numpy(), s.ecol.numpy(), s.dinv.numpy(), s.E.numpy())
    rng = np.random.default_rng(2)
    Z = rng.standard_normal((len(A), 3)) + 1j * rng.standard_normal((len(A), 3))
    g = 0.3 * rng.standard_normal(s.nedge)
    loss, dg = lo.loss_and_gains_gradient(*args, g, Z)
    for e in (0, s.nedge // 2, s.nedge - 1):
        h = 1e-6
        gp, gm = g.copy(), g.copy()
        gp[e] += h
        gm[e] -= h
        fd = (lo.loss_and_gains_gradient(*args, gp, Z)[0] - lo.loss_and_gains_gradient(*args, gm, Z)[0]) / (2 * h)
        assert abs(fd - dg[e]) <= 1e-6 * max(abs(fd), 1e-8), (e, fd, dg[e])
    phi = s.phi.numpy()
    params = 0.4 * rng.standard_normal(16 * 6 + 33)
    w = rng.standard_normal(s.nedge)
    f = lambda p: float(lo.forward(phi, p, 16)[1] @ w)
    hidden, _ = lo.forward(phi, params, 16)
    grad = lo.backward(phi, params, 16, hidden, w)
    for q in (0, 50, 96, 100, 120, 128):
        h = 1e-6
        pp, pm = params.copy(), params.copy()
        pp[q] += h
        pm[q] -= h
        fd = (f(pp) - f(pm)) / (2 * h)
        assert abs(fd - grad[q]) <= 1e-6 * max(abs(fd), 1e-8), (q, fd, grad[q])
