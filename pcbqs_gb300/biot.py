"""Biot-Savart near field of RWG sheet currents and filaments on the device.

    a, b = rwg_currents(rwg, I)                                # J = a r + b per triangle (A/m)
    H = h_sheets([(nodes, tris, a, b, z), ...], pts)           # (n, 3) complex, or (n, 3, k) for k excitations
    H += h_segments(p0, p1, I_seg, pts)                        # straight filaments (vias, parts)

Restates pcbqs.biot (src/pcbqs/biot.py:24-105) and _numerics.currents.rwg_currents (currents.py:5-18): the 6-point
rule per triangle, triangles near any observation point (centroid closer than near * 2 * size to a point, found with
a k-d tree as the reference does) split into 4 midpoint triangles `levels` times. The host builds the quadrature
points and current moments (O(sources x excitations)); the device (pcbqs_gb300_biot_sheets / _segments) does the
O(points x sources x excitations) sums, in FP64 (precision='f64', the parity path) or FP32 ('f32').
"""
import ctypes

import numpy as np
import torch
from scipy.spatial import cKDTree

from . import _lib
from .geometry import BAR6, W6, split4


def rwg_currents(rwg, I):
    """(a, b): J = a r + b on each triangle, a (nt,) or (nt, k), b (nt, 2) or (nt, 2, k), from RWG coefficients I
    (ne,) or (ne, k) (the RWG functions' amplitudes, total edge current / edge length)."""
    I = np.asarray(I)
    multi = I.ndim > 1
    I2 = I if multi else I[:, None]
    k = I2.shape[1]
    a = np.zeros((len(rwg.tris), k), complex)
    b = np.zeros((len(rwg.tris), 2, k), complex)
    for t, alpha, v in ((rwg.tp, rwg.l / (2 * rwg.area[rwg.tp]), rwg.vp),
                        (rwg.tm, -rwg.l / (2 * rwg.area[rwg.tm]), rwg.vm)):
        ia = I2 * alpha[:, None]
        np.add.at(a, t, ia)
        np.add.at(b, t, -ia[:, None, :] * v[:, :, None])
    return (a, b) if multi else (a[:, 0], b[:, :, 0])


def _sources(V, a, b, z):
    """Quadrature points (S, 4: x, y, z, 0) and current moments w J_x, w J_y (S, k) of triangles V (M, 3, 2)."""
    e1, e2 = V[:, 1] - V[:, 0], V[:, 2] - V[:, 0]
    area = 0.5 * np.abs(e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0])
    Q = np.einsum('qk,tkc->tqc', BAR6, V)                              # (M, 6, 2)
    w = (area[:, None] * W6[None]).reshape(-1)
    jx = (a[:, None, :] * Q[..., 0:1] + b[:, None, 0, :]).reshape(-1, a.shape[1]) * w[:, None]
    jy = (a[:, None, :] * Q[..., 1:2] + b[:, None, 1, :]).reshape(-1, a.shape[1]) * w[:, None]
    xyz = np.zeros((len(w), 4))
    xyz[:, 0], xyz[:, 1], xyz[:, 2] = Q[..., 0].reshape(-1), Q[..., 1].reshape(-1), np.repeat(z, 6)
    return xyz, jx, jy


def h_sheets(sheets, pts, near=1.5, levels=2, precision='f64', device=0):
    """H (n, 3) complex at pts (n, 3) m of the sheets [(nodes (N, 2) m, tris, a, b, z)], J = a r + b on each
    triangle; with a (M, k), b (M, 2, k): H (n, 3, k)."""
    pts = np.ascontiguousarray(pts, float)
    multi = None
    blocks = []
    for nodes, tris, a, b, z in sheets:
        a, b = np.asarray(a), np.asarray(b)
        multi = a.ndim > 1 if multi is None else multi
        a2 = a if a.ndim > 1 else a[:, None]
        b2 = b if b.ndim > 2 else b[:, :, None]
        V = nodes[tris]
        e1, e2 = V[:, 1] - V[:, 0], V[:, 2] - V[:, 0]
        size = np.sqrt(np.abs(e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]) / 2)
        cen = V.mean(1)
        tree = cKDTree(np.c_[pts[:, :2], pts[:, 2] - z])
        dist, _ = tree.query(np.c_[cen, np.zeros(len(cen))])
        far = dist > near * 2 * size
        blocks.append(_sources(V[far], a2[far], b2[far], np.full(far.sum(), z)))
        Vn, an, bn = V[~far], a2[~far], b2[~far]
        for _ in range(levels):
            if not len(Vn):
                break
            Vn = split4(Vn)
            an, bn = np.concatenate([an] * 4), np.concatenate([bn] * 4)
        if len(Vn):
            blocks.append(_sources(Vn, an, bn, np.full(len(Vn), z)))
    k = blocks[0][1].shape[1]
    xyz = np.ascontiguousarray(np.concatenate([s for s, _, _ in blocks]))
    jx = np.ascontiguousarray(np.concatenate([x for _, x, _ in blocks]).astype(complex))
    jy = np.ascontiguousarray(np.concatenate([y for _, _, y in blocks]).astype(complex))
    dev = torch.device('cuda', device)
    t = lambda arr: torch.as_tensor(arr, device=dev)
    pts_d, xyz_d, jx_d, jy_d = t(pts), t(xyz), t(jx), t(jy)
    H = torch.zeros((len(pts), 3, k), dtype=torch.complex128, device=dev)
    lib = _lib.load()
    _lib.check(lib.pcbqs_gb300_biot_sheets(len(pts), pts_d.data_ptr(), len(xyz), xyz_d.data_ptr(), jx_d.data_ptr(),
                                           jy_d.data_ptr(), k, int(precision == 'f32'), H.data_ptr(),
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), lib)
    out = H.cpu().numpy()
    return out if multi else out[:, :, 0]


def h_segments(p0, p1, I, pts, device=0):
    """H (n, 3) at pts of straight filaments p0 -> p1 ((m, 3) m) carrying I (m,) or (m, k) A: H (n, 3, k)."""
    p0, p1, pts = (np.ascontiguousarray(v, float).reshape(-1, 3) for v in (p0, p1, pts))
    I = np.asarray(I)
    multi = I.ndim > 1
    I2 = np.ascontiguousarray((I if multi else I[:, None]).astype(complex))
    k = I2.shape[1] if len(p0) else 1
    dev = torch.device('cuda', device)
    H = torch.zeros((len(pts), 3, k), dtype=torch.complex128, device=dev)
    if len(p0):
        t = lambda arr: torch.as_tensor(arr, device=dev)
        pts_d, a_d, b_d, i_d = t(pts), t(p0), t(p1), t(I2)
        lib = _lib.load()
        _lib.check(lib.pcbqs_gb300_biot_segments(len(pts), pts_d.data_ptr(), len(p0), a_d.data_ptr(),
                                                 b_d.data_ptr(), i_d.data_ptr(), k, H.data_ptr(),
                                                 ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), lib)
    out = H.cpu().numpy()
    return out if multi else out[:, :, 0]
