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
