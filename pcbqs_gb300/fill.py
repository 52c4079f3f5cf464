"""Device-resident fill: moments, L and P stay in HBM as torch tensors; the kernels run through the C ABI.

    f = DeviceFill(nodes, tris, z, outer_levels=1, near=3.0)
    planes, analytic = f.moments()            # (4, nt, nt) float64: M0, Mx, My, Mrr
    L = f.inductance(planes)                  # (ne, ne): mu0/4pi diag(1/l) combine diag(1/l)   (static.py:103-128)
    P = f.potential(planes[0], node_of, er)   # (nn, nn): W^T M0 W / (4 pi eps0 er)            (mqs.py:532-552)

This is the path the solver uses: no host copy of any dense matrix. The pcbqs plugin (backend.py) is the drop-in
that returns host arrays.
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib
from .geometry import DeviceGeometry, prepare
from .rwg import RWG

MU0 = 4e-7 * np.pi
C0 = 299792458.0
EPS0 = 1.0 / (MU0 * C0 ** 2)


def _stream(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


class DeviceFill:
    def __init__(self, nodes, tris, z, outer_levels=1, near=3.0, device=0):
        if not torch.cuda.is_available():
            raise RuntimeError('GB300 fill unavailable: no CUDA device')
        self.device = torch.device('cuda', device)
        self.geometry = prepare(nodes, tris, z, outer_levels)
        self.dev = DeviceGeometry(self.geometry, device)
        self.lib = self.dev.lib
        self.near, self.outer_levels = near, outer_levels
        self.nt = len(self.geometry.tris)
        self._rwg = None
        self._edges = None

    @property
    def rwg(self):
        if self._rwg is None:
            self._rwg = RWG(self.geometry.nodes, self.geometry.tris)
        return self._rwg

    def moments(self, scalar_only=False, out=None, stream=None):
        """Reciprocal moment planes (1 or 4, nt, nt) float64 on the device, and the analytic pair count."""
        width = 1 if scalar_only else 4
        if out is None:
            out = torch.empty((width, self.nt, self.nt), dtype=torch.float64, device=self.device)
        planes = (ctypes.c_void_p * 4)(*[out[k].data_ptr() for k in range(width)], *([None] * (4 - width)))
        analytic = ctypes.c_uint64()
        near = float(self.near)
        _lib.check(self.lib.pcbqs_gb300_fill_device(self.dev.handle, -1.0 if math.isinf(near) else near,
                                                    int(self.outer_levels), int(scalar_only), planes,
                                                    out.stride(1), ctypes.byref(analytic), _stream(stream)),
                   self.lib)
        return out, int(analytic.value)

    def edge_arrays(self):
        if self._edges is None:
            tri, alpha, vertex = self.rwg.combine_arrays()
            scale = 1.0 / self.rwg.l
            t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a)).to(self.device, dt)
            self._edges = (t(tri, torch.int32), t(alpha, torch.float64), t(vertex, torch.float64),
                           t(scale, torch.float64))
        return self._edges

    def inductance(self, planes, factor=MU0 / (4 * np.pi), out=None, stream=None):
        """L = factor diag(1/l) combine(moments) diag(1/l) on the device, (ne, ne) float64."""
        tri, alpha, vertex, scale = self.edge_arrays()
        ne = self.rwg.Ne
        if out is None:
            out = torch.empty((ne, ne), dtype=torch.float64, device=self.device)
        m0, mx, my, rr = planes
        _lib.check(self.lib.pcbqs_gb300_edge_inductance_device(
            ne, tri.data_ptr(), alpha.data_ptr(), vertex.data_ptr(), scale.data_ptr(), float(factor), rr.data_ptr(),
            mx.data_ptr(), my.data_ptr(), m0.data_ptr(), planes.stride(1), out.data_ptr(), out.stride(0),
            _stream(stream)), self.lib)
        return out

    def potential(self, m0, node_of, er=1.0, out=None, stream=None):
        """P = W^T M0 W / (4 pi eps0 er) with W[t, node] = 1/A_node, (nn, nn) float64 on the device."""
        node_of = np.asarray(node_of)
        nn = int(node_of.max()) + 1
        members = np.argsort(node_of, kind='stable').astype(np.int32)
        start = np.zeros(nn + 1, np.int64)
        np.cumsum(np.bincount(node_of, minlength=nn), out=start[1:])
        area = np.bincount(node_of, weights=self.geometry.area, minlength=nn)
        dev = lambda a: torch.as_tensor(a).to(self.device)
        start_d, members_d, area_d = dev(start), dev(members), dev(area)
        if out is None:
            out = torch.empty((nn, nn), dtype=torch.float64, device=self.device)
        _lib.check(self.lib.pcbqs_gb300_potential_device(
            nn, start_d.data_ptr(), members_d.data_ptr(), area_d.data_ptr(), m0.data_ptr(), m0.stride(0),
            1.0 / (4 * np.pi * EPS0 * er), out.data_ptr(), out.stride(0), _stream(stream)), self.lib)
        return out

    # ---- mixed precision: FP32 far pairs in local coordinates, FP64 near pairs ----

    def moments_local(self, scalar_only=False, out=None, stream=None):
        """FP32 planes (1 or 4, nt, nt) of moments about each triangle's centroid, and the analytic pair count."""
        width = 1 if scalar_only else 4
        if out is None:
            out = torch.empty((width, self.nt, self.nt), dtype=torch.float32, device=self.device)
        planes = (ctypes.c_void_p * 4)(*[out[k].data_ptr() for k in range(width)], *([None] * (4 - width)))
        analytic = ctypes.c_uint64()
        near = float(self.near)
        _lib.check(self.lib.pcbqs_gb300_fill_local_device(self.dev.handle, -1.0 if math.isinf(near) else near,
                                                          int(self.outer_levels), int(scalar_only), planes,
                                                          out.stride(1), ctypes.byref(analytic), _stream(stream)),
                   self.lib)
        return out, int(analytic.value)

    def edge_arrays_local(self):
        if getattr(self, '_edges_local', None) is None:
            tri, alpha, vertex = self.rwg.combine_arrays()
            cent = self.geometry.cent
            off = cent[tri] - vertex                       # (2, ne, 2): centroid minus free vertex, in FP64
            t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a)).to(self.device, dt)
            self._edges_local = (t(tri, torch.int32), t(alpha, torch.float32), t(off, torch.float32),
                                 t(1.0 / self.rwg.l, torch.float32))
        return self._edges_local

    def inductance_local(self, planes, factor=MU0 / (4 * np.pi), out=None, out_single=None, stream=None):
        """(L FP64, L FP32) from the local FP32 moments, combined in FP32."""
        tri, alpha, off, scale = self.edge_arrays_local()
        ne = self.rwg.Ne
        if out is None:
            out = torch.empty((ne, ne), dtype=torch.float64, device=self.device)
        if out_single is None:
            out_single = torch.empty((ne, ne), dtype=torch.float32, device=self.device)
        m0, mx, my, rr = planes
        _lib.check(self.lib.pcbqs_gb300_edge_inductance_local_device(
            ne, tri.data_ptr(), alpha.data_ptr(), off.data_ptr(), scale.data_ptr(), float(factor), rr.data_ptr(),
            mx.data_ptr(), my.data_ptr(), m0.data_ptr(), planes.stride(1), out.data_ptr(), out.stride(0),
            out_single.data_ptr(), out_single.stride(0), _stream(stream)), self.lib)
        return out, out_single

    def potential_single(self, m0, node_of, er=1.0, out=None, out_single=None, stream=None):
        """(P FP64, P FP32) from FP32 M0, sums in FP64."""
        node_of = np.asarray(node_of)
        nn = int(node_of.max()) + 1
        members = np.argsort(node_of, kind='stable').astype(np.int32)
        start = np.zeros(nn + 1, np.int64)
        np.cumsum(np.bincount(node_of, minlength=nn), out=start[1:])
        area = np.bincount(node_of, weights=self.geometry.area, minlength=nn)
        dev = lambda a: torch.as_tensor(a).to(self.device)
        start_d, members_d, area_d = dev(start), dev(members), dev(area)
        if out is None:
            out = torch.empty((nn, nn), dtype=torch.float64, device=self.device)
        if out_single is None:
            out_single = torch.empty((nn, nn), dtype=torch.float32, device=self.device)
        _lib.check(self.lib.pcbqs_gb300_potential_single_device(
            nn, start_d.data_ptr(), members_d.data_ptr(), area_d.data_ptr(), m0.data_ptr(), m0.stride(0),
            1.0 / (4 * np.pi * EPS0 * er), out.data_ptr(), out_single.data_ptr(), out.stride(0), _stream(stream)),
            self.lib)
        return out, out_single

    def close(self):
        self.dev.close()
