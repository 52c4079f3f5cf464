"""Host preparation of a triangle mesh for the device fill, and its upload.

`prepare` restates pcbqs's FillGeometry.prepare (src/pcbqs/static_backends.py:104-130) with its observation rules
(_offplane_geometry, src/pcbqs/_numerics/sing.py:56-69; _split4, src/pcbqs/_numerics/currents.py:21-26; the
6-point and 3-point rules, src/pcbqs/_numerics/base.py:64-71; edge_frames, base.py:82-88). It is O(nt) NumPy work
done once per mesh, with the same NumPy expressions as the reference so that centroids and radii -- and with them
the near/far classification -- are bit-identical.

`DeviceGeometry` uploads either this or a reference FillGeometry (the plugin path) into a device context.
"""
from dataclasses import dataclass
import ctypes

import numpy as np

from . import _lib

# 6-point degree-4 rule and 3-point degree-2 rule (barycentric), as src/pcbqs/_numerics/base.py:64-71.
_A1, _A2 = 0.445948490915965, 0.091576213509771
BAR6 = np.array([[1 - 2 * _A1, _A1, _A1], [_A1, 1 - 2 * _A1, _A1], [_A1, _A1, 1 - 2 * _A1],
                 [1 - 2 * _A2, _A2, _A2], [_A2, 1 - 2 * _A2, _A2], [_A2, _A2, 1 - 2 * _A2]])
W6 = np.array([0.223381589678011] * 3 + [0.109951743655322] * 3)
BAR3 = np.array([[2 / 3, 1 / 6, 1 / 6], [1 / 6, 2 / 3, 1 / 6], [1 / 6, 1 / 6, 2 / 3]])
W3 = np.ones(3) / 3


def split4(V):
    """Each triangle (M, 3, 2) into its 4 midpoint triangles (4M, 3, 2), in the reference's order."""
    m01, m12, m20 = (V[:, 0] + V[:, 1]) / 2, (V[:, 1] + V[:, 2]) / 2, (V[:, 2] + V[:, 0]) / 2
    return np.concatenate([np.stack(t, 1) for t in ((V[:, 0], m01, m20), (m01, V[:, 1], m12),
                                                      (m20, m12, V[:, 2]), (m01, m12, m20))])


def edge_frames(V):
    """Edge vectors, lengths, unit tangents and outward normals of counter-clockwise triangles V (nt, 3, 2)."""
    e = np.roll(V, -1, axis=1) - V
    L = np.linalg.norm(e, axis=2)
    tau = e / L[..., None]
    return e, L, tau, np.stack([tau[..., 1], -tau[..., 0]], -1)


def level_geometry(nodes, tris, level):
    """(V, L, tau, un, area, P, W) of one observation refinement level: P (nt, 6*4^level, 2), W (6*4^level)."""
    V = nodes[tris]
    e, L, tau, un = edge_frames(V)
    area = 0.5 * np.abs(e[:, 0, 0] * (-e[:, 2, 1]) - e[:, 0, 1] * (-e[:, 2, 0]))
    bar, weights = BAR6, W6
    if level:
        ref = np.eye(3)[None]
        for _ in range(level):
            ref = split4(ref)
        bar = np.einsum('qk,tkc->tqc', BAR6, ref).reshape(-1, 3)
        weights = np.tile(W6, len(ref)) / len(ref)
    P = np.einsum('qk,tkc->tqc', bar, V)
    return V, L, tau, un, area, P, weights


@dataclass(frozen=True)
class MeshGeometry:
    """The fields of pcbqs's FillGeometry: centred nodes, int32 triangles, z, centroids, bounding radii, the
    three-point rule points and the per-level observation geometry."""
    nodes: np.ndarray
    tris: np.ndarray
    z: np.ndarray
    cent: np.ndarray
    radius: np.ndarray
    points: np.ndarray
    levels: dict

    @property
    def area(self):
        return self.levels[0][4]


def prepare(nodes, tris, z, outer_levels=1):
    """Validate and centre a mesh (ValueError as the reference raises it) and build its fill geometry."""
    nodes, tris, z = np.asarray(nodes, float), np.asarray(tris), np.asarray(z, float)
    if (nodes.ndim != 2 or nodes.shape[1] != 2 or not len(nodes) or
            tris.ndim != 2 or tris.shape[1] != 3 or not len(tris) or tris.dtype.kind not in 'iu' or
            z.shape != (len(tris),) or not np.isfinite(nodes).all() or not np.isfinite(z).all() or
            tris.min() < 0 or tris.max() >= len(nodes)):
        raise ValueError('fill requires finite planar nodes, integer triangles and one z per triangle')
    if outer_levels not in (0, 1, 2):
        raise ValueError('outer_levels must be 0, 1 or 2')
    nodes = np.ascontiguousarray(nodes - nodes.mean(0))
    tris = np.array(tris, dtype=np.int32, order='C', copy=True)
    z = np.array(z, order='C', copy=True)
    V = nodes[tris]
    edge = V[:, 1:] - V[:, :1]
    if (edge[:, 0, 0] * edge[:, 1, 1] - edge[:, 0, 1] * edge[:, 1, 0] <= 0).any():
        raise ValueError('fill triangles must be nondegenerate and counter-clockwise')
    cent = V.mean(1)
    radius = np.linalg.norm(V - cent[:, None], axis=2).max(1)
    points = np.einsum('qk,tkc->tqc', BAR3, V)
    levels = {}
    for level in {0, outer_levels}:
        g = level_geometry(nodes, tris, level)
        levels[level] = (*g[:-1], g[-1].copy())
    for array in (nodes, tris, z, cent, radius, points, *(a for g in levels.values() for a in g)):
        array.setflags(write=False)
    return MeshGeometry(nodes, tris, z, cent, radius, points, levels)


class DeviceGeometry:
    """A geometry resident on one GPU (a pcbqs_gb300 context). Accepts a MeshGeometry or pcbqs's FillGeometry."""

    def __init__(self, geometry, device=0):
        lib = _lib.load()
        self.lib, self.device = lib, int(device)
        self.nt = len(geometry.tris)
        V, L, tau, un, area, _, _ = geometry.levels[0]
        keep = dict(v=_lib.f64(V), len=_lib.f64(L), tau=_lib.f64(tau), un=_lib.f64(un), area=_lib.f64(area),
                    p3=_lib.f64(geometry.points), cent=_lib.f64(geometry.cent), radius=_lib.f64(geometry.radius),
                    z=_lib.f64(geometry.z))
        rules = []
        for level in range(3):
            g = geometry.levels.get(level, geometry.levels[0])
            rules.append((_lib.f64(g[5]), _lib.f64(g[6])))
        s = _lib.Geometry()
        s.nt = self.nt
        for name, array in keep.items():
            setattr(s, name, _lib.ptr(array))
        for k, (qp, qw) in enumerate(rules):
            s.qp[k], s.qw[k], s.nq[k] = _lib.ptr(qp), _lib.ptr(qw), len(qw)
        handle = ctypes.c_void_p()
        _lib.check(lib.pcbqs_gb300_create(ctypes.byref(s), self.device, ctypes.byref(handle)), lib)
        self.handle = handle
        self._keep = (keep, rules)   # host arrays stay alive with the context

    def close(self):
        if getattr(self, 'handle', None):
            self.lib.pcbqs_gb300_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 -- interpreter shutdown
            pass
