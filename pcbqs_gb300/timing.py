"""Kernel timing on one GPU, for profiling the hot kernels on cases small enough for a full ncu capture.

    python -m pcbqs_gb300.timing fill <board> [triangles]   # mixed and FP64 fill of the first N triangles
    python -m pcbqs_gb300.timing lu <board> [k ...]          # the complex64 factor's triangular solves, k columns
    python -m pcbqs_gb300.timing dense <n> [k]               # FP64 and FP32 symmetric dense products, n x n, k columns
    python -m pcbqs_gb300.timing getrf <n> [block ...]       # the blocked complex64 LU of a random n x n matrix
    python -m pcbqs_gb300.timing potrf <n> [block ...]       # the blocked FP32 Cholesky of a random SPD matrix

Times are CUDA-event times after a warm-up call; boards are the npz meshes of tests/golden (planes, strip, tiny).
"""
import ctypes
import sys

import numpy as np
import torch


def _event_ms(fn):
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    out = fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), out


def fill(board, triangles=None):
    from .board import Board
    from .fill import DeviceFill
    b = Board.load(board)
    nt = len(b.tris) if triangles is None else int(triangles)
    tris = b.tris[:nt]
    used = np.unique(tris)
    remap = np.full(len(b.nodes), -1)
    remap[used] = np.arange(len(used))
    f = DeviceFill(b.nodes[used], remap[tris], b.z[:nt], 1, 3.0)
    for mode in ('mixed', 'fp64'):
        for _ in range(3):
            ms, (planes, analytic) = _event_ms(f.moments_local if mode == 'mixed' else f.moments)
            del planes
            print(f'fill {mode} {nt} triangles: {ms:.2f} ms, {analytic} analytic pairs', flush=True)


def lu(board, ks=(8,)):
    from . import _lib
    from .board import Board
    from .peec import PeecModel, _csr_struct
    m = PeecModel(Board.load(board))
    m.assemble(mixed=True)
    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    handle, _ = m._operator(np.array([2 * np.pi * 1e6]))
    try:
        desc = _csr_struct(m._krk_device())
        for math in (1, 2, 3):
            ms, _ = _event_ms(lambda: _lib.check(lib.pcbqs_gb300_peec_factor(handle, ctypes.byref(desc), 0, math,
                                                                             stream), lib))
            print(f'factor n={m.n} math {math}: {ms:.1f} ms', flush=True)
        for k in ks:
            x = torch.randn(m.n, k, dtype=torch.complex128, device='cuda')
            y = torch.empty_like(x)
            for _ in range(3):
                ms, _ = _event_ms(lambda: _lib.check(lib.pcbqs_gb300_peec_lu_solve(handle, k, x.data_ptr(),
                                                                                   y.data_ptr(), 0, stream), lib))
                print(f'lu_solve k={k}: {ms:.2f} ms', flush=True)
    finally:
        lib.pcbqs_gb300_peec_destroy(handle)


def getrf(n, blocks=(1024,)):
    """The blocked complex64 LU of a random n x n matrix with each panel width, BF16x9 and FP32 GEMMs."""
    from . import _lib
    n = int(n)
    lib = _lib.load()
    g = torch.Generator(device='cuda').manual_seed(1)
    A = torch.complex(torch.randn(n, n, device='cuda', generator=g), torch.randn(n, n, device='cuda', generator=g))
    F = torch.empty_like(A)
    piv = torch.zeros(n, dtype=torch.int32, device='cuda')
    singular = ctypes.c_int32(0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    flops = 8 / 3 * n ** 3
    for block in blocks:
        for math in (1, 0):
            for _ in range(2):
                F.copy_(A)
                ms, status = _event_ms(lambda: lib.pcbqs_gb300_lu_factor_c64(n, F.data_ptr(), piv.data_ptr(), block,
                                                                             math, ctypes.byref(singular), stream))
                _lib.check(status, lib)
                print(f'getrf n={n} block {block} math {math}: {ms:.1f} ms, {flops / ms / 1e9:.1f} TFLOP/s',
                      flush=True)


def potrf(n, blocks=(1024,)):
    """The blocked FP32 Cholesky of a random n x n positive definite matrix, against cuSOLVER's potrf."""
    from . import _lib
    n = int(n)
    lib = _lib.load()
    g = torch.Generator(device='cuda').manual_seed(1)
    M = torch.randn(n, n, device='cuda', generator=g)
    A = M @ M.T / n + 0.05 * torch.eye(n, device='cuda')
    ld = (n + 31) // 32 * 32                      # the padded leading dimension the library's own factor uses
    F = torch.zeros(n, ld, device='cuda')
    info = ctypes.c_int32(0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for block in blocks:
        for math in (1, 0):
            for _ in range(2):
                F[:, :n].copy_(A)
                ms, status = _event_ms(lambda: lib.pcbqs_gb300_cholesky_f32(n, F.data_ptr(), ld, block, math,
                                                                            ctypes.byref(info), stream))
                _lib.check(status, lib)
                print(f'potrf n={n} ld {ld} block {block} math {math}: {ms:.1f} ms, '
                      f'{n ** 3 / 3 / ms / 1e9:.1f} TFLOP/s', flush=True)
    for _ in range(2):
        ms, _ = _event_ms(lambda: torch.linalg.cholesky(A))
        print(f'potrf n={n} cuSOLVER (torch): {ms:.1f} ms', flush=True)


def dense(n, k=8):
    """A random symmetric n x n matrix (FP64 and its FP32 copy) against k complex columns."""
    from . import _lib
    n, k = int(n), int(k)
    lib = _lib.load()
    g = torch.Generator(device='cuda').manual_seed(1)
    M = torch.rand((n, n), dtype=torch.float64, device='cuda', generator=g)
    M = (M + M.T) / 2
    Mf = M.float()
    X = torch.randn((n, k), dtype=torch.complex128, device='cuda', generator=g)
    Y = torch.empty_like(X)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for name, fn in (('fp64', lambda: lib.pcbqs_gb300_dense_apply(n, k, M.data_ptr(), n, X.data_ptr(), Y.data_ptr(),
                                                                   stream)),
                     ('fp32', lambda: lib.pcbqs_gb300_dense_apply_single(n, k, Mf.data_ptr(), n, X.data_ptr(),
                                                                          Y.data_ptr(), stream))):
        for _ in range(3):
            ms, status = _event_ms(fn)
            _lib.check(status, lib)
            bytes_ = n * n * (8 if name == 'fp64' else 4)
            print(f'dense {name} n={n} k={k}: {ms:.3f} ms, {bytes_ / ms / 1e6:.0f} GB/s of matrix, '
                  f'{2 * n * n * 2 * k / ms / 1e9:.3f} TFLOP/s', flush=True)


def main(argv):
    if len(argv) < 2 or argv[0] not in ('fill', 'lu', 'dense', 'getrf', 'potrf'):
        print(__doc__)
        return 2
    if argv[0] == 'fill':
        fill(argv[1], argv[2] if len(argv) > 2 else None)
    elif argv[0] == 'potrf':
        potrf(argv[1], tuple(int(v) for v in argv[2:]) or (1024,))
    elif argv[0] == 'getrf':
        getrf(argv[1], tuple(int(v) for v in argv[2:]) or (1024,))
    elif argv[0] == 'dense':
        dense(argv[1], argv[2] if len(argv) > 2 else 8)
    else:
        lu(argv[1], tuple(int(v) for v in argv[2:]) or (8,))
    return 0


if __name__ == '__main__':
    sys.exit(main(sys.argv[1:]))
