"""pcbqs_gb300_pairs_no_alloc, the pair entry point that allocates no device memory, against
pcbqs_gb300_pairs_device on the same device inputs, through the C ABI. Collected last so that it also runs after
every other test in one process; it builds and loads everything it needs, so it also runs alone.

Tolerance: rel 2e-10, the pair-protocol tolerance of the other device tests (the two entry points run the same
kernels, so in practice the results are identical)."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

MAX_PAIRS = 1 << 20


def _pair_set(geo, rng, count):
    """Seeded pairs on the strip board: random pairs (mostly far), every self pair and index neighbours (near and
    outer-level pairs), with the reference's classification (near 3, outer level 1)."""
    nt = len(geo.tris)
    p = np.concatenate([rng.integers(0, nt, count), np.arange(nt), np.arange(nt - 1)]).astype(np.int32)
    q = np.concatenate([rng.integers(0, nt, count), np.arange(nt), np.arange(1, nt)]).astype(np.int32)
    d = geo.z[p] - geo.z[q]
    kind = O.kinds(geo, p, q, d, 3.0, 1)
    return p, q, d, kind


def _call(lib, name, handle, arrays, scalar, width):
    import torch
    from pcbqs_gb300 import _lib
    p, q, d, kind = (torch.as_tensor(a, device='cuda') for a in arrays)
    out = torch.full((len(p), width), float('nan'), dtype=torch.float64, device='cuda')
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(getattr(lib, name)(handle, p.data_ptr(), q.data_ptr(), d.data_ptr(), kind.data_ptr(), len(p),
                                  int(scalar), out.data_ptr(), stream), lib)
    return out.cpu().numpy()


@pytest.mark.parametrize('scalar', [False, True])
def test_no_alloc_pairs_match_pairs_device(device_library, scalar):
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.geometry import DeviceGeometry, prepare
    lib = device_library
    b = Board.load('strip')
    g = prepare(b.nodes, b.tris, b.z, 1)
    dg = DeviceGeometry(g, 0)
    try:
        rng = np.random.default_rng(11)
        width = 1 if scalar else 6
        # two calls in a row, the second smaller than the first: stale scratch from call 1 must not leak into 2
        for count in (300_000, 70_000):
            arrays = _pair_set(g, rng, count)
            assert (arrays[3] >= 0).any() and (arrays[3] == 1).any() and (arrays[3] == -1).any()
            expected = _call(lib, 'pcbqs_gb300_pairs_device', dg.handle, arrays, scalar, width)
            got = _call(lib, 'pcbqs_gb300_pairs_no_alloc', dg.handle, arrays, scalar, width)
            assert np.isfinite(got).all()
            assert got == pytest.approx(expected, rel=2e-10, abs=1e-26)
    finally:
        dg.close()


def test_no_alloc_rejects_more_pairs_than_its_scratch(device_library):
    from pcbqs_gb300 import _lib
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.geometry import DeviceGeometry, prepare
    lib = device_library
    b = Board.load('tiny')
    dg = DeviceGeometry(prepare(b.nodes, b.tris, b.z, 1), 0)
    try:
        status = lib.pcbqs_gb300_pairs_no_alloc(dg.handle, None, None, None, None, MAX_PAIRS + 1, 0, None, None)
        assert status == 1
        with pytest.raises(ValueError, match='exceed the fixed scratch'):
            _lib.check(status, lib)
    finally:
        dg.close()


def test_no_alloc_clears_flags_left_by_a_rejected_call(device_library):
    """A call whose pairs hold an out-of-range triangle index, then one with an out-of-range kind (both made on the
    host and caught by the kernels' own index checks), each return status 1 and leave the shared scratch's invalid
    flag set; the valid call after them must clear it, return 0 and match pcbqs_gb300_pairs_device."""
    import torch
    from pcbqs_gb300 import _lib
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.geometry import DeviceGeometry, prepare
    lib = device_library
    b = Board.load('strip')
    g = prepare(b.nodes, b.tris, b.z, 1)
    dg = DeviceGeometry(g, 0)
    try:
        rng = np.random.default_rng(5)
        p, q, d, kind = _pair_set(g, rng, 20_000)
        bad_index, bad_kind = p.copy(), kind.copy()
        bad_index[123] = len(g.tris)
        bad_kind[4567] = 7
        for arrays in ((bad_index, q, d, kind), (p, q, d, bad_kind)):
            pt, qt, dt, kt = (torch.as_tensor(a, device='cuda') for a in arrays)
            out = torch.zeros((len(pt), 6), dtype=torch.float64, device='cuda')
            stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
            status = lib.pcbqs_gb300_pairs_no_alloc(dg.handle, pt.data_ptr(), qt.data_ptr(), dt.data_ptr(),
                                                    kt.data_ptr(), len(pt), 0, out.data_ptr(), stream)
            assert status == 1
            with pytest.raises(ValueError, match='out of range'):
                _lib.check(status, lib)
        expected = _call(lib, 'pcbqs_gb300_pairs_device', dg.handle, (p, q, d, kind), False, 6)
        got = _call(lib, 'pcbqs_gb300_pairs_no_alloc', dg.handle, (p, q, d, kind), False, 6)
        assert got == pytest.approx(expected, rel=2e-10, abs=1e-26)
    finally:
        dg.close()
