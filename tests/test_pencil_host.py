"""The pencil solve (pcbqs_gb300.mixedlu.DevicePencil, the reference's Pencil, src/pcbqs/kernels.py:205-245)
against a direct solve of (R + s L + P^T diag(z) P) x = b: its algebra is plain torch linear algebra, so it is
checked here on CPU tensors (on the GPU through the copper-port sweep)."""
import numpy as np
import pytest


@pytest.mark.parametrize('with_parts', [False, True])
def test_pencil_matches_direct_solve(with_parts):
    import torch
    from pcbqs_gb300.mixedlu import DevicePencil
    rng = np.random.default_rng(2)
    n, k = 120, 3
    M = rng.standard_normal((n, n))
    R = M @ M.T / n + 0.1 * np.eye(n)
    N = rng.standard_normal((n, n))
    L = 1e-9 * (N @ N.T / n + np.eye(n))
    P = np.zeros((k, n))
    P[np.arange(k), rng.choice(n, k, replace=False)] = 1.0
    pencil = DevicePencil(torch.as_tensor(R), torch.as_tensor(L), torch.as_tensor(P) if with_parts else None)
    b = rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2))
    for f in (0.0, 1e3, 1e6, 1e8):
        s = 2j * np.pi * f
        z = np.array([1.0 + 1e-9 * s, 5.0, 0.5 + 2e-9 * s]) if with_parts else None
        A = R + s * L + (P.T @ np.diag(z) @ P if with_parts else 0)
        x = pencil.solve(s, z, torch.as_tensor(b)).numpy()
        ref = np.linalg.solve(A, b)
        assert np.abs(x - ref).max() <= 1e-10 * np.abs(ref).max(), f
        assert pencil.solve(s, z, torch.as_tensor(b[:, 0])).shape == (n,)


def test_pencil_pays_rule():
    from pcbqs_gb300.mixedlu import pencil_lus, pencil_pays
    assert not pencil_pays(150, 1000)                       # too small
    n = 2000
    need = 1.25 * pencil_lus(n) + 1
    assert not pencil_pays(n, int(need) - 1) and pencil_pays(n, int(np.ceil(need)))
