"""pcbqs_gb300_complex_update: the tcgen05 GEMM behind the blocked LU's trailing update (c -= a b, complex64, BF16
part products with FP32 accumulation) against complex128 products on the same inputs, and against cuBLAS's own
FP32 complex GEMM (torch complex64 matmul) as the yardstick for the six-term form. Normwise errors are taken relative
to |a| |b| (the entrywise absolute product), the scale a product's rounding errors live on."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

# normwise error bounds relative to |a| |b| + |c|: six terms at FP32's level (and within 5x cuBLAS's FP32 GEMM on the
# same inputs: the tensor core's accumulation is restarted every 256 of the inner dimension and the chunks summed in
# FP32 registers); three terms about 2^-16 per product (the dropped part products).
TOL = {6: 2e-6, 3: 2e-4}


def _update(lib, a, b, c, terms, wait=1 << 32):
    """c -= a b through the C ABI; c a column-major view (the transpose of a row-major tensor)."""
    import torch
    rows, k = a.shape
    cols = b.shape[1]
    at, bt = a.T.contiguous(), b.T.contiguous()    # column-major a and b, held until the call has returned
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return lib.pcbqs_gb300_complex_update(rows, cols, k, at.data_ptr(), rows, bt.data_ptr(), k, c.data_ptr(),
                                          c.stride(1) if c.dim() == 2 else rows, terms, wait, stream)


def _rand(shape, g):
    import torch
    return torch.complex(torch.randn(*shape, device='cuda', generator=g), torch.randn(*shape, device='cuda', generator=g))


@pytest.mark.parametrize('terms', [6, 3])
@pytest.mark.parametrize('rows,cols,k', [(1, 1, 1), (130, 70, 33), (300, 200, 100), (1000, 700, 512),
                                         (2048, 2048, 2048), (4097, 300, 2048), (257, 1200, 96)])
def test_complex_update_matches_complex128(device_library, rows, cols, k, terms):
    import torch
    from pcbqs_gb300 import _lib
    g = torch.Generator(device='cuda').manual_seed(rows * 7 + cols * 3 + k + terms)
    a, b = _rand((rows, k), g), _rand((k, cols), g)
    c0 = _rand((rows, cols), g)
    # C column-major with a leading dimension larger than rows, inside a guard region that must stay untouched
    ld = rows + 5
    store = _rand((cols + 1, ld), g)
    guard = store.clone()
    view = store[:cols, :rows]                     # store row j = column j of C
    view.copy_(c0.T)
    at, bt = a.T.contiguous(), b.T.contiguous()    # column-major a and b (held until the call returns)
    _lib.check(device_library.pcbqs_gb300_complex_update(
        rows, cols, k, at.data_ptr(), rows, bt.data_ptr(), k, store.data_ptr(), ld,
        terms, 1 << 32, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), device_library)
    ours = store[:cols, :rows].T.to(torch.complex128)
    exact = c0.to(torch.complex128) - a.to(torch.complex128) @ b.to(torch.complex128)
    scale = torch.linalg.norm(a.abs().double() @ b.abs().double() + c0.abs().double()).item()
    err = torch.linalg.norm(ours - exact).item() / scale
    fp32 = torch.linalg.norm((c0 - a @ b).to(torch.complex128) - exact).item() / scale
    print(f'update {rows}x{cols}x{k} terms {terms}: error {err:.3e} of |a||b| + |c|, cuBLAS FP32 {fp32:.3e}')
    assert err < TOL[terms], err
    if terms == 6:
        assert err <= 5 * fp32 + 5e-8, (err, fp32)
    store[:cols, :rows] = guard[:cols, :rows]
    assert torch.equal(store, guard)               # nothing outside C written


@pytest.mark.parametrize('terms', [3, 6])
@pytest.mark.parametrize('rows,cols,k', [(200, 150, 64), (1030, 515, 300)])
def test_complex_update_exact_on_small_integers(device_library, rows, cols, k, terms):
    """Entries that are small integers are exact in BF16 and their products' sums exact in FP32, so the update must
    equal the exact product bit for bit: every tile, row, column and K slice lands where it belongs."""
    import torch
    from pcbqs_gb300 import _lib
    g = torch.Generator(device='cuda').manual_seed(rows + cols + k)
    ints = lambda *s: torch.randint(-8, 9, s, device='cuda', generator=g).float()
    a = torch.complex(ints(rows, k), ints(rows, k))
    b = torch.complex(ints(k, cols), ints(k, cols))
    c = torch.complex(ints(rows, cols), ints(rows, cols))
    at, bt, ct = a.T.contiguous(), b.T.contiguous(), c.T.contiguous()
    _lib.check(_update(device_library, a, b, ct.T, terms), device_library)
    exact = (c.to(torch.complex128) - a.to(torch.complex128) @ b.to(torch.complex128)).to(torch.complex64)
    assert torch.equal(ct.T, exact)


def test_complex_update_bounded_wait_returns_timeout(device_library):
    """A wait limit far too short for the first copy to land: every CTA gives up, waits for its own copies and
    products, frees its tensor memory and reports ERR_TIMEOUT; the next call with a normal limit is exact."""
    import torch
    from pcbqs_gb300 import _lib
    g = torch.Generator(device='cuda').manual_seed(5)
    a, b, c = _rand((512, 1024), g), _rand((1024, 384), g), _rand((512, 384), g)
    ct = c.T.contiguous()
    status = _update(device_library, a, b, ct.T, 6, wait=1)
    assert status == _lib.ERR_TIMEOUT, status
    torch.cuda.synchronize()
    ct = c.T.contiguous()
    assert _update(device_library, a, b, ct.T, 6) == 0
    exact = c.to(torch.complex128) - a.to(torch.complex128) @ b.to(torch.complex128)
    scale = torch.linalg.norm(a.abs().double() @ b.abs().double() + c.abs().double()).item()
    assert torch.linalg.norm(ct.T.to(torch.complex128) - exact).item() / scale < TOL[6]


# ---- pcbqs_gb300_dense_apply_tensor: Y = M X for a real M and complex128 X on the same GEMM ----

def _apply_tensor(lib, M, X, terms, wait=1 << 32):
    import torch
    rows, ld = M.shape[0], M.stride(0)
    Y = torch.full_like(X, float('nan'))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    status = lib.pcbqs_gb300_dense_apply_tensor(rows, X.shape[1], M.data_ptr(), ld, X.data_ptr(), Y.data_ptr(),
                                                terms, wait, stream)
    return status, Y


# relative to |M| |X|: three parts about 2^-16 per product, six FP32's (plus X's rounding to FP32)
APPLY_TOL = {3: 1e-4, 6: 1e-6}


@pytest.mark.parametrize('terms', [3, 6])
@pytest.mark.parametrize('rows,k', [(1, 1), (100, 16), (700, 33), (1000, 128), (4099, 130), (2500, 300)])
def test_dense_apply_tensor_matches_complex128(device_library, rows, k, terms):
    """The mixed solve's inner products over many right-hand sides: a symmetric FP32 M (leading dimension above
    its size) against complex128 X, to the parts' accuracy, and against the FP32 CUDA-core product."""
    import torch
    from pcbqs_gb300 import _lib
    g = torch.Generator(device='cuda').manual_seed(rows * 11 + k + terms)
    A = torch.randn(rows, rows, device='cuda', generator=g)
    store = torch.randn(rows, rows + 7, device='cuda', generator=g)
    store[:, :rows] = A + A.T
    M = store[:, :rows]
    X = torch.complex(torch.randn(rows, k, device='cuda', generator=g, dtype=torch.float64),
                      torch.randn(rows, k, device='cuda', generator=g, dtype=torch.float64))
    status, Y = _apply_tensor(device_library, store, X, terms)
    _lib.check(status, device_library)
    Md = M.double()
    exact = torch.complex(Md @ X.real, Md @ X.imag)
    scale = torch.linalg.norm(torch.complex(Md.abs() @ X.real.abs(), Md.abs() @ X.imag.abs())).item()
    err = torch.linalg.norm(Y - exact).item() / scale
    single = torch.empty_like(X)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(device_library.pcbqs_gb300_dense_apply_single(rows, k, store.data_ptr(), store.stride(0), X.data_ptr(),
                                                              single.data_ptr(), stream), device_library)
    fp32 = torch.linalg.norm(single - exact).item() / scale
    print(f'apply {rows} x {k} terms {terms}: error {err:.3e} of |M||X|, FP32 CUDA-core product {fp32:.3e}')
    assert err < APPLY_TOL[terms], err


@pytest.mark.parametrize('terms', [3, 6])
def test_dense_apply_tensor_exact_on_small_integers(device_library, terms):
    """Small integers are exact in BF16 and their sums exact in FP32: the product equals the exact one bit for bit,
    so every tile, row, column and K slice (3000 is not a multiple of 64 or 128) lands where it belongs."""
    import torch
    from pcbqs_gb300 import _lib
    g = torch.Generator(device='cuda').manual_seed(17 + terms)
    rows, k = 3000, 150
    A = torch.randint(-8, 9, (rows, rows), device='cuda', generator=g).float()
    M = (A + A.T).contiguous()
    ints = lambda: torch.randint(-8, 9, (rows, k), device='cuda', generator=g).double()
    X = torch.complex(ints(), ints())
    status, Y = _apply_tensor(device_library, M, X, terms)
    _lib.check(status, device_library)
    Md = M.double()
    assert torch.equal(Y, torch.complex(Md @ X.real, Md @ X.imag))


def test_dense_apply_tensor_bounded_wait_returns_timeout(device_library):
    import torch
    from pcbqs_gb300 import _lib
    g = torch.Generator(device='cuda').manual_seed(9)
    M = torch.randn(1024, 1024, device='cuda', generator=g)
    X = torch.complex(torch.randn(1024, 64, device='cuda', generator=g, dtype=torch.float64),
                      torch.randn(1024, 64, device='cuda', generator=g, dtype=torch.float64))
    status, _ = _apply_tensor(device_library, M, X, 3, wait=1)
    assert status == _lib.ERR_TIMEOUT, status
    torch.cuda.synchronize()
    status, Y = _apply_tensor(device_library, M, X, 3)
    assert status == 0
    Md = M.double()
    exact = torch.complex(Md @ X.real, Md @ X.imag)
    scale = torch.linalg.norm(torch.complex(Md.abs() @ X.real.abs(), Md.abs() @ X.imag.abs())).item()
    assert torch.linalg.norm(Y - exact).item() / scale < APPLY_TOL[3]


# ---- pcbqs_gb300_dense_apply_sliced: the FP64 product from integer slices on the same GEMM ----

def _apply_sliced(lib, M, X, slices, wait=1 << 32):
    import torch
    Y = torch.full_like(X, float('nan'))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    status = lib.pcbqs_gb300_dense_apply_sliced(M.shape[0], X.shape[1], M.data_ptr(), M.stride(0), X.data_ptr(),
                                                Y.data_ptr(), slices, wait, stream)
    return status, Y


def _wide_range(rows, g):
    """A symmetric FP64 matrix whose entries span many binades (decaying off the diagonal, as L and P do)."""
    import torch
    i = torch.arange(rows, device='cuda', dtype=torch.float64)
    decay = 1.0 / (1.0 + (i[:, None] - i[None, :]).abs())
    A = torch.randn(rows, rows, device='cuda', generator=g, dtype=torch.float64) * decay
    A = A + A.T
    A.diagonal().add_(4.0)
    return A * 1e-7


@pytest.mark.parametrize('slices', [5, 6, 7])
@pytest.mark.parametrize('rows,k', [(1, 1), (100, 4), (700, 33), (1000, 128), (3000, 130)])
def test_dense_apply_sliced_matches_fp64(device_library, rows, k, slices):
    """Errors within 2^(4 - 8 slices) of max_t |M[r,t]| sum_t |X[t,c]| per entry. Relative to |M| |X| that bound
    grows by about the ratio of a row's largest entry times sum |X| to sum |M| |X| (hundreds for this decaying
    matrix): seven slices are within FP64's own rounding, six within 1e-12, far below the 1e-8 residuals they
    check."""
    import torch
    from pcbqs_gb300 import _lib
    g = torch.Generator(device='cuda').manual_seed(rows * 13 + k + slices)
    store = torch.randn(rows, rows + 3, device='cuda', generator=g, dtype=torch.float64)
    store[:, :rows] = _wide_range(rows, g)
    M = store[:, :rows]
    X = torch.complex(torch.randn(rows, k, device='cuda', generator=g, dtype=torch.float64),
                      torch.randn(rows, k, device='cuda', generator=g, dtype=torch.float64)) * 3e4
    status, Y = _apply_sliced(device_library, store, X, slices)
    _lib.check(status, device_library)
    exact = torch.complex(M @ X.real, M @ X.imag)
    rowmax = M.abs().amax(1, keepdim=True)
    bound_re = rowmax * X.real.abs().sum(0, keepdim=True)
    bound_im = rowmax * X.imag.abs().sum(0, keepdim=True)
    err = max(((Y.real - exact.real).abs() / bound_re).max().item(),
              ((Y.imag - exact.imag).abs() / bound_im).max().item())
    scale = torch.linalg.norm(torch.complex(M.abs() @ X.real.abs(), M.abs() @ X.imag.abs())).item()
    normwise = torch.linalg.norm(Y - exact).item() / scale
    print(f'sliced {rows} x {k}, {slices} slices: {err:.3e} of the slice bound, {normwise:.3e} of |M||X|')
    assert err <= 2.0 ** (4 - 8 * slices), err
    assert normwise < {5: 1e-10, 6: 1e-12, 7: 1e-14}[slices], normwise


@pytest.mark.parametrize('slices', [3, 6])
def test_dense_apply_sliced_exact_on_integers(device_library, slices):
    """Integers of 14 bits are whole in two slices, so with three slices or more no slice pair they need is dropped:
    the product equals FP64's bit for bit, so every tile, row, column, slice pair and level carry lands where it
    belongs (3000 is not a multiple of 128 or 256)."""
    import torch
    from pcbqs_gb300 import _lib
    g = torch.Generator(device='cuda').manual_seed(29 + slices)
    rows, k = 3000, 150
    A = torch.randint(-8000, 8001, (rows, rows), device='cuda', generator=g).double()
    M = (A + A.T).contiguous()
    ints = lambda: torch.randint(-8000, 8001, (rows, k), device='cuda', generator=g).double()
    X = torch.complex(ints(), ints())
    status, Y = _apply_sliced(device_library, M, X, slices)
    _lib.check(status, device_library)
    assert torch.equal(Y, torch.complex(M @ X.real, M @ X.imag))


def test_dense_apply_sliced_non_finite_and_timeout(device_library):
    """A NaN in one column of X makes that column of Y NaN and leaves the others exact to the bound; a wait limit
    too short for the first copy returns status 6, and the next call is correct."""
    import torch
    from pcbqs_gb300 import _lib
    g = torch.Generator(device='cuda').manual_seed(31)
    rows, k = 1024, 64
    M = _wide_range(rows, g)
    X = torch.complex(torch.randn(rows, k, device='cuda', generator=g, dtype=torch.float64),
                      torch.randn(rows, k, device='cuda', generator=g, dtype=torch.float64))
    exact = torch.complex(M @ X.real, M @ X.imag)
    bad = X.clone()
    bad[7, 3] = complex(float('nan'), 1.0)
    status, Y = _apply_sliced(device_library, M, bad, 6)
    _lib.check(status, device_library)
    assert torch.isnan(Y[:, 3].real).all() and torch.isfinite(Y[:, 3].imag).all()
    keep = [c for c in range(k) if c != 3]
    scale = torch.linalg.norm(exact[:, keep]).item()
    assert torch.linalg.norm(Y[:, keep] - exact[:, keep]).item() / scale < 1e-11
    status, _ = _apply_sliced(device_library, M, X, 6, wait=1)
    assert status == _lib.ERR_TIMEOUT, status
    torch.cuda.synchronize()
    status, Y = _apply_sliced(device_library, M, X, 6)
    assert status == 0
    assert torch.linalg.norm(Y - exact).item() / torch.linalg.norm(exact).item() < 1e-11
