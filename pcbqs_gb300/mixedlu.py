"""Dense complex LU solves on the device: MixedLU and lu_factor_rows / lu_solve_rows of the reference
(src/pcbqs/kernels.py:122-181, :266-294), with this library's blocked complex64 LU (pcbqs_gb300_lu_factor_c64) as
the single-precision factor.

    lu = lu_factor_rows(A)          # A: (n, n) complex128 CUDA tensor, row-major
    X = lu_solve_rows(lu, B)        # B: (n,) or (n, k)

A complex system of MIXED_MIN unknowns or more is factored in single precision and refined with FP64 residuals
until |b - A x| <= 1e-12 |b| (at most 12 steps; a stalled refinement that is at 1e-10 or better is accepted,
anything else is factored in double, once); a smaller or real one is factored in double. The solves with the
complex64 factor go through cuSOLVER getrs (torch.linalg.lu_solve), whose layout and pivots the factor keeps.
"""
import ctypes

import numpy as np
import torch

from . import _lib

MIXED_MIN = 4000       # the reference's threshold (kernels.py:122): smaller systems are factored in double
BLOCK = 2048           # panel width of the blocked complex64 LU


class DeviceMixedLU:
    """The complex64 LU of a complex128 device matrix, refined to double's accuracy (MixedLU, kernels.py:125-181).
    The FP64 matrix is kept for the residuals."""

    TOL, STEPS = 1e-12, 12

    def __init__(self, a):
        if a.dim() != 2 or a.shape[0] != a.shape[1] or not a.is_cuda:
            raise ValueError('DeviceMixedLU needs a square CUDA matrix')
        self.a = a.to(torch.complex128)
        n = a.shape[0]
        lib = _lib.load()
        factor = self.a.T.to(torch.complex64).contiguous()        # row-major a^T = column-major a
        piv = torch.empty(n, dtype=torch.int32, device=a.device)
        singular = ctypes.c_int32(0)
        stream = ctypes.c_void_p(torch.cuda.current_stream(a.device).cuda_stream)
        _lib.check(lib.pcbqs_gb300_lu_factor_c64(n, factor.data_ptr(), piv.data_ptr(), min(BLOCK, max(32, n)), 1,
                                                 ctypes.byref(singular), stream), lib)
        self.lu = (factor.T, piv) if singular.value == 0 else None       # the factor as a matrix (a view)
        self.double = None
        if self.lu is None:                       # an exactly zero single-precision pivot: double from the start
            self._double()

    def _double(self):
        if self.double is None:
            self.lu = None
            self.double = torch.linalg.lu_factor(self.a)
        return self.double

    def solve(self, b):
        b = b.to(torch.complex128)
        one_column = b.dim() == 1
        B = b.reshape(b.shape[0], -1)
        X = self._solve(B)
        return X[:, 0] if one_column else X

    def _solve(self, b):
        if self.double is not None:
            return torch.linalg.lu_solve(*self.double, b)
        one = lambda r: torch.linalg.lu_solve(self.lu[0], self.lu[1], r.to(torch.complex64)).to(torch.complex128)
        x = one(b)
        nb = max(float(torch.linalg.norm(b)), 1e-300)
        last = np.inf
        for _ in range(self.STEPS):
            r = b - self.a @ x
            res = float(torch.linalg.norm(r)) / nb
            if res <= self.TOL:
                return x
            if res > 0.5 * last:                  # no longer converging
                break
            last = res
            x = x + one(r)
        if last <= 1e-10:                         # stalled at a double solve's own level
            return x
        return torch.linalg.lu_solve(*self._double(), b)


def lu_factor_rows(a, mixed='auto'):
    """The LU of the square device matrix `a`: DeviceMixedLU for a complex one of MIXED_MIN unknowns or more
    (mixed='auto'), else the FP64 LU (cuSOLVER getrf through torch)."""
    if mixed == 'auto':
        mixed = a.is_complex() and a.shape[0] >= MIXED_MIN
    if mixed:
        return DeviceMixedLU(a)
    return torch.linalg.lu_factor(a)


def lu_solve_rows(lu, b):
    """x of a x = b for lu = lu_factor_rows(a)."""
    if isinstance(lu, DeviceMixedLU):
        return lu.solve(b)
    one_column = b.dim() == 1
    x = torch.linalg.lu_solve(lu[0], lu[1], b.reshape(b.shape[0], -1).to(lu[0].dtype))
    return x[:, 0] if one_column else x


class DevicePencil:
    """(R + s L + P^T diag(z) P)^-1 for any s from one generalized eigendecomposition, on the device (the
    reference's Pencil, src/pcbqs/kernels.py:205-245): R, L real symmetric (n, n) with R positive definite, P an
    optional dense (k, n) incidence of k parts of impedance z(s). With R = C C^T and C^-1 L C^-T = W diag(lam) W^T,
    G = C^-T W gives (R + s L)^-1 = G diag(1 / (1 + s lam)) G^T, and the parts enter by Woodbury (a k x k solve).
    FP64 throughout (cuSOLVER potrf and syevd, cuBLAS); torch.linalg.LinAlgError where R is not positive definite."""

    def __init__(self, R, L, P=None):
        R = R.to(torch.float64)
        L = L.to(torch.float64)
        c = torch.linalg.cholesky(R)
        X = torch.linalg.solve_triangular(c, L, upper=False)
        X = torch.linalg.solve_triangular(c, X.T.contiguous(), upper=False)
        X = (X + X.T) / 2
        self.lam, W = torch.linalg.eigh(X)
        del X
        self.G = torch.linalg.solve_triangular(c.T, W, upper=True)
        self.P = None if P is None or P.shape[0] == 0 else P.to(torch.float64)
        self.PG = None if self.P is None else self.P @ self.G

    def _real_times(self, M, v):
        """M v for a real M and a complex v without a complex copy of M."""
        return torch.complex(M @ v.real.contiguous(), M @ v.imag.contiguous())

    def solve(self, s, z, b):
        """x of (R + s L + P^T diag(z) P) x = b, b (n,) or (n, m) (complex)."""
        b = b.to(torch.complex128)
        one_column = b.dim() == 1
        B = b.reshape(b.shape[0], -1)
        d = 1 / (1 + complex(s) * self.lam.to(torch.complex128))
        u = d[:, None] * self._real_times(self.G.T, B)
        x = self._real_times(self.G, u)
        if self.PG is not None and z is not None and bool(torch.as_tensor(z).abs().gt(0).any()):
            z = torch.as_tensor(np.asarray(z, complex), device=B.device)
            PGc = self.PG.to(torch.complex128)
            S = (PGc * d[None, :]) @ PGc.T                            # P Z0^-1 P^T
            k = len(z)
            t = torch.linalg.solve(torch.eye(k, dtype=torch.complex128, device=B.device) + z[:, None] * S,
                                   z[:, None] * (PGc @ u))
            x = x - self._real_times(self.G, d[:, None] * (PGc.T @ t))
        return x[:, 0] if one_column else x


def pencil_lus(n):
    """About how many complex LUs of n unknowns a pencil's eigendecomposition costs (the reference's CPU estimate,
    kernels.py:248-251)."""
    return 4.0 + 1.6 * n / 1000


def pencil_pays(n, frequencies):
    """Whether a sweep of `frequencies` on n loops is quicker by one pencil than by an LU each (kernels.py:254-263,
    without its host-memory probe: the device holds the four n x n matrices)."""
    return n >= 200 and frequencies >= 1.25 * pencil_lus(n) + 1
