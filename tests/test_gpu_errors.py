"""Failure paths on the device, in the manner of the reference's plugin contract tests (tests/test_static_backends.py:
96-113: a failing backend raises and nothing retries; a non-finite moment is rejected with FloatingPointError):

* fill_symmetric through the plugin object: its argument checks, and its device fill against the golden moments;
* a non-finite moment from a poisoned host input -- a valid mesh of two triangles 1e140 m across, whose areas'
  product overflows -- raises FloatingPointError from both evaluate and fill_symmetric;
* GMRES held to a few iterations reports non-convergence (status 5 from the C ABI, RuntimeError from the model);
* bounded device waits made to run out (pcbqs_gb300_set_wait_cycles far below any copy's or block's latency):
  the triangular sweeps' grid barriers return status 6, the fill returns status 6 or finishes, and in every case
  the next call with the normal limit on the same context is correct.
No failure here is made on the device: the GPU never faults, traps or hangs."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
NAMES = ('m0', 'mx', 'my', 'mrr')


@pytest.mark.parametrize('level', [0, 1])
@pytest.mark.parametrize('scalar', [False, True])
def test_backend_fill_symmetric_matches_reference(device_library, tiny8, level, scalar):
    from pcbqs_gb300.backend import Gb300Backend
    from pcbqs_gb300.geometry import prepare
    g = prepare(tiny8['nodes'], tiny8['tris'], tiny8['z'], level)
    backend = Gb300Backend(g, 1, 16384, 0)
    mats = [np.full((8, 8), np.nan) for _ in range(1 if scalar else 4)]
    analytic = backend.fill_symmetric(mats, 3.0, level, scalar)
    tag = f'l{level}_{"s" if scalar else "f"}'
    for name, m in zip(NAMES, mats):
        assert m == pytest.approx(tiny8[f'numpy_{tag}_{name}'], rel=2e-10, abs=1e-26)
    assert analytic == int(tiny8[f'numpy_{tag}_analytic'])
    assert backend.routing['device_fills'] == 1


def test_backend_fill_symmetric_rejects_bad_outputs(device_library, tiny8):
    from pcbqs_gb300.backend import Gb300Backend
    from pcbqs_gb300.geometry import prepare
    g = prepare(tiny8['nodes'], tiny8['tris'], tiny8['z'], 1)
    backend = Gb300Backend(g, 1, 16384, 0)
    good = lambda: [np.zeros((8, 8)) for _ in range(4)]
    with pytest.raises(ValueError, match='expects 4 output matrices'):
        backend.fill_symmetric(good()[:3], 3.0, 1, False)
    with pytest.raises(TypeError, match='C-contiguous float64'):
        backend.fill_symmetric([m.astype(np.float32) for m in good()], 3.0, 1, False)
    with pytest.raises(TypeError, match='C-contiguous float64'):
        backend.fill_symmetric([np.zeros((8, 16))[:, ::2] for _ in range(4)], 3.0, 1, False)
    frozen = good()
    frozen[2].setflags(write=False)
    with pytest.raises(TypeError):
        backend.fill_symmetric(frozen, 3.0, 1, False)
    with pytest.raises(ValueError, match='not prepared'):
        backend.fill_symmetric(good(), 3.0, 2, False)
    assert backend.routing['device_fills'] == 0


def _huge_pair():
    s = 1e140
    nodes = np.array([[0, 0], [1, 0], [0, 1], [1, 1]], float) * s
    return nodes, np.array([[0, 1, 2], [1, 3, 2]]), np.zeros(2)


def test_nonfinite_moment_raises(device_library):
    from pcbqs_gb300.backend import Gb300Backend
    from pcbqs_gb300.geometry import prepare
    from oracle import oracle as O
    nodes, tris, z = _huge_pair()
    with pytest.raises(FloatingPointError):              # the oracle rejects the same input
        O.fill(O.Geometry(nodes, tris, z, 1), 3.0, 1, False)
    g = prepare(nodes, tris, z, 1)
    backend = Gb300Backend(g, 1, 16384, 0)
    with pytest.raises(FloatingPointError):
        backend.fill_symmetric([np.zeros((2, 2)) for _ in range(4)], 3.0, 1, False)
    with pytest.raises(FloatingPointError):
        backend.evaluate(np.array([0], np.int32), np.array([1], np.int32), np.zeros(1), np.array([-1], np.int32),
                         False)


def test_gmres_nonconvergence_is_reported(device_library):
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    model = PeecModel(Board.load('tiny'), maxiter=3, restart=3)
    with pytest.raises(RuntimeError, match='GMRES did not reach'):
        model.solve([1e6], precondition='block_jacobi')
    ok = PeecModel(Board.load('tiny')).solve([1e6], precondition='block_jacobi')
    assert ok.residual.max() <= 5e-8


def test_bounded_waits_run_out_and_the_context_stays_usable(device_library):
    import torch
    from pcbqs_gb300 import _lib
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel, _csr_struct
    lib = device_library
    m = PeecModel(Board.load('tiny'))
    m.assemble(mixed=True)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    handle, _ = m._operator(np.array([2 * np.pi * 1e6]))
    try:
        desc = _csr_struct(m._krk_device())
        _lib.check(lib.pcbqs_gb300_peec_factor(handle, ctypes.byref(desc), 0, 2, stream), lib)
        g = torch.Generator(device='cuda').manual_seed(3)
        x = torch.complex(torch.randn(m.n, 4, device='cuda', generator=g, dtype=torch.float64),
                          torch.randn(m.n, 4, device='cuda', generator=g, dtype=torch.float64))
        ref = torch.empty_like(x)
        _lib.check(lib.pcbqs_gb300_peec_lu_solve(handle, 4, x.data_ptr(), ref.data_ptr(), 0, stream), lib)
        y = torch.empty_like(x)
        try:
            lib.pcbqs_gb300_set_wait_cycles(32)
            status = lib.pcbqs_gb300_peec_lu_solve(handle, 4, x.data_ptr(), y.data_ptr(), 0, stream)
        finally:
            lib.pcbqs_gb300_set_wait_cycles(0)
        assert status == _lib.ERR_TIMEOUT, status
        torch.cuda.synchronize()
        _lib.check(lib.pcbqs_gb300_peec_lu_solve(handle, 4, x.data_ptr(), y.data_ptr(), 0, stream), lib)
        assert torch.equal(y, ref)                        # the sweeps are deterministic
    finally:
        lib.pcbqs_gb300_peec_destroy(handle)
    # the fill: its bulk copies usually outlast a 1-cycle limit (status 6, copies drained before each block
    # exits); either way the next fill on the same context is the reference's
    from pcbqs_gb300.fill import DeviceFill
    f = DeviceFill(m.board.nodes, m.board.tris, m.board.z, 1, 3.0)
    good, analytic = f.moments()
    good = good.cpu()
    try:
        lib.pcbqs_gb300_set_wait_cycles(1)
        try:
            f.moments()
            short = 0
        except _lib.DeviceError as exc:
            short = exc.status
    finally:
        lib.pcbqs_gb300_set_wait_cycles(0)
    assert short in (0, _lib.ERR_TIMEOUT)
    again, analytic2 = f.moments()
    assert analytic2 == analytic and torch.equal(again.cpu(), good)
