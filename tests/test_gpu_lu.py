"""pcbqs_gb300_lu_factor_c64, the blocked complex64 LU (panels factored one step ahead of the trailing GEMMs),
against the definition P A = L U and against cuSOLVER's own getrf (torch.linalg.lu_factor) on the same matrix.
Both are FP32 factorizations, so the bar is the backward error: ours no worse than 4x the library's, and a
solve through the standard getrs convention (torch.linalg.lu_solve with our factor and pivots) at FP32 accuracy."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _factor(lib, A, block, math):
    """Our factor of the complex64 (n, n) torch matrix A: (LU as the matrix (n, n), 1-based pivots)."""
    import torch
    from pcbqs_gb300 import _lib
    n = A.shape[0]
    F = A.T.contiguous()                 # row-major A^T = column-major A, what getrf takes
    piv = torch.zeros(n, dtype=torch.int32, device=A.device)
    singular = ctypes.c_int32(-1)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.pcbqs_gb300_lu_factor_c64(n, F.data_ptr(), piv.data_ptr(), block, math, ctypes.byref(singular),
                                             stream), lib)
    assert singular.value == 0
    return F.T.contiguous(), piv


def _backward_error(A, LU, piv):
    import torch
    n = A.shape[0]
    L = torch.tril(LU, -1).to(torch.complex128) + torch.eye(n, dtype=torch.complex128, device=A.device)
    U = torch.triu(LU).to(torch.complex128)
    perm = list(range(n))
    for i, p in enumerate(piv.cpu().tolist()):
        perm[i], perm[p - 1] = perm[p - 1], perm[i]
    PA = A.to(torch.complex128)[torch.as_tensor(perm, device=A.device)]
    return (torch.linalg.norm(PA - L @ U) / torch.linalg.norm(A.to(torch.complex128))).item()


@pytest.mark.parametrize('n,block,math', [(300, 64, 0), (1000, 128, 1), (1000, 1000, 1), (2100, 256, 1),
                                          (2100, 1024, 0), (4097, 512, 1), (4500, 2048, 1), (6000, 4096, 1),
                                          (300, 64, 3), (1000, 128, 3), (2100, 256, 3), (4097, 512, 3),
                                          (4500, 2048, 3), (6000, 4096, 3)])
def test_blocked_lu_matches_getrf(device_library, n, block, math):
    import torch
    g = torch.Generator(device='cuda').manual_seed(n + block)
    A = torch.complex(torch.randn(n, n, device='cuda', generator=g), torch.randn(n, n, device='cuda', generator=g))
    LU, piv = _factor(device_library, A, block, math)
    p = piv.cpu().numpy()
    assert torch.isfinite(torch.view_as_real(LU)).all()
    assert ((p >= np.arange(1, n + 1)) & (p <= n)).all()          # pivot rows at or below their step
    ours = _backward_error(A, LU, piv)
    LUr, pivr = torch.linalg.lu_factor(A)
    theirs = _backward_error(A, LUr, pivr)
    assert ours <= 4 * theirs + 1e-7, (ours, theirs)
    b = torch.complex(torch.randn(n, 3, device='cuda', generator=g), torch.randn(n, 3, device='cuda', generator=g))
    x = torch.linalg.lu_solve(LU, piv, b)
    xr = torch.linalg.lu_solve(LUr, pivr, b)
    res = (torch.linalg.norm(A @ x - b) / torch.linalg.norm(b)).item()
    resr = (torch.linalg.norm(A @ xr - b) / torch.linalg.norm(b)).item()
    assert res <= 4 * resr + 1e-6, (res, resr)


def test_blocked_lu_is_deterministic(device_library):
    import torch
    g = torch.Generator(device='cuda').manual_seed(7)
    n = 1500
    A = torch.complex(torch.randn(n, n, device='cuda', generator=g), torch.randn(n, n, device='cuda', generator=g))
    LU1, p1 = _factor(device_library, A, 256, 1)
    LU2, p2 = _factor(device_library, A, 256, 1)
    assert torch.equal(p1, p2)
    assert torch.equal(torch.view_as_real(LU1), torch.view_as_real(LU2))


def test_blocked_lu_rejects_bad_block(device_library):
    import torch
    from pcbqs_gb300 import _lib
    A = torch.eye(64, dtype=torch.complex64, device='cuda')
    piv = torch.zeros(64, dtype=torch.int32, device='cuda')
    singular = ctypes.c_int32(0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for block in (16, 8192):
        status = device_library.pcbqs_gb300_lu_factor_c64(64, A.data_ptr(), piv.data_ptr(), block, 1,
                                                          ctypes.byref(singular), stream)
        assert status == 1
        with pytest.raises(ValueError, match='block'):
            _lib.check(status, device_library)


def _cholesky(lib, A, block, math, pad=0):
    """Our Cholesky of A, its column-major copy stored with leading dimension n + pad."""
    import torch
    from pcbqs_gb300 import _lib
    n = A.shape[0]
    F = torch.zeros(n, n + pad, dtype=A.dtype, device=A.device)     # row r of F = column r of the matrix
    F[:, :n] = A.T
    info = ctypes.c_int32(-1)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.pcbqs_gb300_cholesky_f32(n, F.data_ptr(), n + pad, block, math, ctypes.byref(info), stream), lib)
    return torch.tril(F[:, :n].T), info.value


@pytest.mark.parametrize('n,block,math,pad', [(300, 64, 1, 0), (2100, 512, 1, 0), (2100, 1024, 0, 12),
                                              (4097, 1024, 1, 31)])
def test_blocked_cholesky_matches_potrf(device_library, n, block, math, pad):
    """pcbqs_gb300_cholesky_f32 against A = L L^T, no worse than 4x cuSOLVER's own FP32 potrf (torch.cholesky)."""
    import torch
    g = torch.Generator(device='cuda').manual_seed(n + block)
    M = torch.randn(n, n, device='cuda', generator=g)
    A = M @ M.T / n + 0.05 * torch.eye(n, device='cuda')
    L, info = _cholesky(device_library, A, block, math, pad)
    assert info == 0
    assert torch.isfinite(L).all() and (torch.diagonal(L) > 0).all()
    A64 = A.double()
    ours = (torch.linalg.norm(A64 - L.double() @ L.double().T) / torch.linalg.norm(A64)).item()
    Lr = torch.linalg.cholesky(A)
    theirs = (torch.linalg.norm(A64 - Lr.double() @ Lr.double().T) / torch.linalg.norm(A64)).item()
    assert ours <= 4 * theirs + 1e-7, (ours, theirs)


def test_blocked_cholesky_reports_indefinite(device_library):
    """A matrix whose 70th leading minor is not positive definite: info = 70 (found by the second 64-column
    block's own potrf), as potrf reports it."""
    import torch
    n = 200
    A = torch.eye(n, device='cuda')
    A[69, 69] = -1.0
    _, info = _cholesky(device_library, A, 64, 1)
    assert info == 70


@pytest.mark.parametrize('precondition', [0, 1, 2])
@pytest.mark.parametrize('lossy', [False, True])
def test_dense_gmres_solves_potential_systems(device_library, precondition, lossy):
    """pcbqs_gb300_dense_gmres (the equilibrium charge's P^-1 B) with the diagonal (0) or the FP32 Cholesky factor,
    its solves by the streaming sweeps (1) or by cuBLAS (2), on a symmetric positive definite A (+ j A_im for a
    lossy dielectric): every column to 1e-10, and x against the FP64 direct solve."""
    import torch
    from pcbqs_gb300 import _lib
    n, k = 1500, 3
    g = torch.Generator(device='cuda').manual_seed(11)
    M = torch.randn(n, n, device='cuda', dtype=torch.float64, generator=g)
    A = M @ M.T / n + torch.eye(n, device='cuda', dtype=torch.float64)
    Aim = (0.02 * A).contiguous() if lossy else None
    b = torch.complex(torch.randn(n, k, device='cuda', dtype=torch.float64, generator=g),
                      torch.randn(n, k, device='cuda', dtype=torch.float64, generator=g))
    x = torch.zeros_like(b)
    its, res = np.zeros(k, np.int32), np.zeros(k)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(device_library.pcbqs_gb300_dense_gmres(n, A.data_ptr(), Aim.data_ptr() if lossy else None, n, k,
                                                      b.data_ptr(), x.data_ptr(), 1e-10, 2000, 100, precondition,
                                                      _lib.ptr(its, ctypes.c_int32), _lib.ptr(res), stream),
               device_library)
    assert (res <= 1e-10).all()
    Ac = torch.complex(A, Aim if lossy else torch.zeros_like(A))
    ref = torch.linalg.solve(Ac, b)
    assert (torch.linalg.norm(x - ref) / torch.linalg.norm(ref)).item() < 1e-8
    if precondition:
        assert its.max() <= (8 if lossy else 4), its


@pytest.mark.parametrize('n,block', [(1000, 128), (4500, 2048)])
def test_blocked_lu_three_term_update(device_library, n, block):
    """math 2: the tcgen05 trailing update with three BF16 part products (about 16 correct bits per product): on
    these random matrices a factor with a backward error of a few 1e-4 rather than FP32's 1e-6, which still brings a
    solve close enough for iterative refinement (one refinement step with the factor halves the residual)."""
    import torch
    g = torch.Generator(device='cuda').manual_seed(n + block + 2)
    A = torch.complex(torch.randn(n, n, device='cuda', generator=g), torch.randn(n, n, device='cuda', generator=g))
    LU, piv = _factor(device_library, A, block, 2)
    assert torch.isfinite(torch.view_as_real(LU)).all()
    ours = _backward_error(A, LU, piv)
    assert ours < 2e-3, ours
    b = torch.complex(torch.randn(n, 2, device='cuda', generator=g), torch.randn(n, 2, device='cuda', generator=g))
    x = torch.linalg.lu_solve(LU, piv, b)
    r = b - A @ x
    res0 = (torch.linalg.norm(r) / torch.linalg.norm(b)).item()
    x = x + torch.linalg.lu_solve(LU, piv, r)
    res1 = (torch.linalg.norm(b - A @ x) / torch.linalg.norm(b)).item()
    assert res1 < 0.5 * res0, (res0, res1)
