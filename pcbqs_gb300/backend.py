"""The `gb300` fill backend: pcbqs's pair-integration plugin protocol on one GB300.

Registered through the `pcbqs.static_backends` entry-point group (pyproject.toml), so pcbqs loads it by name only
when selected: `fill_backend='gb300'`, `--fill-backend gb300` or `PCBQS_FILL_BACKEND=gb300`. It can also be
registered by hand with `pcbqs.static_backends.register_fill_backend('gb300', factory)`.

Protocol (src/pcbqs/static_backends.py:1-9, :246-336; the CuPy precedent src/pcbqs/static_cupy.py:64-197):
  factory(geometry, workers, chunk, device) -> backend with
    parallel_tiles        False: one device context serializes its calls
    min_batch_pairs       explicit pair-list callers batch at least this many pairs per call
    device_id, routing    reported in the engine's fill_info
    evaluate(p, q, d, kind, scalar_only) -> host float64 (n, 1|6): M0, Mro_x, Mro_y, Mrs_x, Mrs_y, Mrr
    fill_symmetric(matrices, near, outer_levels, scalar_only) -> analytic unordered-pair count
Failures raise; nothing is retried and nothing falls back to the CPU. A missing library or device raises
RuntimeError('GB300 fill unavailable: ...') at construction, as the CuPy backend does for a missing CuPy.
"""
import math
import ctypes
import threading

import numpy as np

from . import _lib
from .geometry import DeviceGeometry


class Gb300Backend:
    parallel_tiles = False
    min_batch_pairs = 1 << 20

    def __init__(self, geometry, workers=1, chunk=16384, device=None):
        self.device_id = 0 if device is None else int(device)
        try:
            self.device = DeviceGeometry(geometry, self.device_id)
        except (RuntimeError, OSError) as exc:
            raise RuntimeError(f'GB300 fill unavailable on device {device}: {exc}') from exc
        self.geometry = geometry     # the plugin contract: keep the (read-only) geometry arrays alive while used
        self.lib = self.device.lib
        self.chunk = chunk
        self.levels = set(geometry.levels)
        self._lock = threading.Lock()
        self.routing = dict(device_batches=0, device_pairs=0, device_fills=0)

    def evaluate(self, p, q, d, kind, scalar_only):
        p, q, kind = _lib.i32(p), _lib.i32(q), _lib.i32(kind)
        d = _lib.f64(np.broadcast_to(d, p.shape))
        n = len(p)
        out = np.empty((n, 1 if scalar_only else 6))
        if len(kind) and any(int(k) >= 0 and int(k) not in self.levels for k in np.unique(kind)):
            raise ValueError('pair kinds must select far (-1) or a prepared analytic level')
        with self._lock:
            self.routing['device_batches'] += 1
            self.routing['device_pairs'] += n
            if n:
                _lib.check(self.lib.pcbqs_gb300_pairs(self.device.handle, _lib.ptr(p, ctypes.c_int32),
                                                      _lib.ptr(q, ctypes.c_int32), _lib.ptr(d),
                                                      _lib.ptr(kind, ctypes.c_int32), n, int(bool(scalar_only)),
                                                      _lib.ptr(out)), self.lib)
        return out

    def fill_symmetric(self, matrices, near, outer_levels, scalar_only):
        n = self.device.nt
        width = 1 if scalar_only else 4
        if len(matrices) != width:
            raise ValueError(f'fill_symmetric expects {width} output matrices')
        for m in matrices:
            if not (isinstance(m, np.ndarray) and m.dtype == np.float64 and m.shape == (n, n)
                    and m.flags.c_contiguous and m.flags.writeable):
                raise TypeError('fill_symmetric outputs must be writable C-contiguous float64 n x n arrays')
        if outer_levels not in self.levels:
            raise ValueError('outer_levels was not prepared for this geometry')
        planes = (ctypes.c_void_p * 4)(*[m.ctypes.data for m in matrices], *([None] * (4 - width)))
        near = float(near)
        analytic = ctypes.c_uint64()
        with self._lock:
            self.routing['device_fills'] += 1
            _lib.check(self.lib.pcbqs_gb300_fill(self.device.handle, -1.0 if math.isinf(near) else near,
                                                 int(outer_levels), int(bool(scalar_only)), planes,
                                                 ctypes.byref(analytic)), self.lib)
        return int(analytic.value)

    def close(self):
        self.device.close()


def factory(geometry, workers, chunk, device):
    """Entry point of the `pcbqs.static_backends` group: factory(FillGeometry, workers, chunk, device)."""
    return Gb300Backend(geometry, workers, chunk, device)
