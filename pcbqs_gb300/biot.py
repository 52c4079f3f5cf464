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


def h_field(board, currents, pts, device=0):
    """H (n, 3) complex at pts (n, 3) m of a board's branch currents (nbranch,) or (nbranch, k) (edges' total
    currents, then the plated via segments', then the ports'): the sheets' RWG currents by Biot-Savart and the via
    segments as filaments along z; the ports are ideal sources without a radiating connector (the copper-port
    reduction zeroes their currents). MQS.h_field (src/pcbqs/mqs.py:891-913) for boards without lumped parts."""
    from .rwg import RWG
    I = np.asarray(currents)
    multi = I.ndim > 1
    I2 = I if multi else I[:, None]
    r = RWG(board.nodes, board.tris)             # the board's own coordinates (the fill's are centred)
    ne, nv = r.Ne, board.nv
    if I2.shape[0] < ne + nv:
        raise ValueError('currents must hold every edge and via segment')
    a, b = rwg_currents(r, I2[:ne] / r.l[:, None])
    sheets = [(board.nodes, board.tris[idx], a[idx], b[idx], float(board.z[idx[0]]))
              for idx in (np.flatnonzero(board.layer == lay) for lay in np.unique(board.layer))]
    H = h_sheets(sheets, pts, device=device)
    if nv:
        v = np.asarray(board.via_seg)
        H = H + h_segments(np.c_[v[:, 0], v[:, 1], v[:, 3]], np.c_[v[:, 0], v[:, 1], v[:, 4]], I2[ne:ne + nv], pts,
                           device)
    return H if multi else H[..., 0]


# ---- the FFT near field on a uniform grid (src/pcbqs/biot.py:108-181, h_grid) ------------------------------------

def current_grid(rwg, I, idx, gx, gy, per_cell=2.0, device=0):
    """Surface current density of the triangles `idx` on the uniform grid gx, gy (m): (jx, jy) (nx, ny, k) complex
    A/m on the device, for RWG amplitudes I (ne, k). Triangles larger than `per_cell` cells are split into four
    until they are not (at most 6 rounds), each integrated by the 6-point rule, each point's current moment spread
    onto its four grid points (cloud in cell, pcbqs_gb300_current_deposit). Restates current_deposit
    (src/pcbqs/_numerics/currents.py:28-61) for k excitations at once."""
    a, b = rwg_currents(rwg, I)
    V, aa, bb = rwg.nodes[rwg.tris[idx]][:, :, :2], a[idx], b[idx]
    dx, dy = gx[1] - gx[0], gy[1] - gy[0]
    area2 = lambda T: (T[:, 1, 0] - T[:, 0, 0]) * (T[:, 2, 1] - T[:, 0, 1]) - \
        (T[:, 1, 1] - T[:, 0, 1]) * (T[:, 2, 0] - T[:, 0, 0])
    for _ in range(6):
        big = np.sqrt(np.abs(area2(V)) / 2) > per_cell * min(dx, dy)
        if not big.any():
            break
        V = np.concatenate([V[~big], split4(V[big])])
        aa = np.concatenate([aa[~big], np.tile(aa[big], (4, 1))])
        bb = np.concatenate([bb[~big], np.tile(bb[big], (4, 1, 1))])
    area = 0.5 * np.abs(area2(V))
    Q = np.einsum('qk,tkc->tqc', BAR6, V)                                        # (M, 6, 2)
    w = (area[:, None] * W6[None])[..., None]                                     # (M, 6, 1)
    mx = ((aa[:, None, :] * Q[..., 0:1] + bb[:, None, 0, :]) * w).reshape(-1, aa.shape[1])
    my = ((aa[:, None, :] * Q[..., 1:2] + bb[:, None, 1, :]) * w).reshape(-1, aa.shape[1])
    dev = torch.device('cuda', device)
    t = lambda arr: torch.as_tensor(np.ascontiguousarray(arr), device=dev)
    qx, qy, mx_d, my_d = t(Q[..., 0].reshape(-1)), t(Q[..., 1].reshape(-1)), t(mx), t(my)
    k = aa.shape[1]
    jx = torch.zeros((len(gx), len(gy), k), dtype=torch.complex128, device=dev)
    jy = torch.zeros_like(jx)
    lib = _lib.load()
    _lib.check(lib.pcbqs_gb300_current_deposit(len(qx), qx.data_ptr(), qy.data_ptr(), mx_d.data_ptr(),
                                               my_d.data_ptr(), k, float(gx[0]), float(gy[0]), float(dx), float(dy),
                                               len(gx), len(gy), jx.data_ptr(), jy.data_ptr(),
                                               ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)), lib)
    return jx / (dx * dy), jy / (dx * dy)


def h_grid(rwg, layer_tris, z_of, I, x, y, heights, refine=1, filaments=None, device=0):
    """Open-boundary H (nx, ny, nh, 3) complex, or (nx, ny, nh, 3, k) for I (ne, k), on the uniform grids x, y (m) at
    absolute heights (m), from the RWG amplitudes I of the sheets `layer_tris` {layer: triangle indices} at z_of;
    `filaments` (p0, p1, currents) are added analytically. Each sheet's current is deposited on a source grid that
    covers all copper and the window (spacing / refine), and convolved with the magnetostatic kernel by zero-padded
    FFTs on the device (linear, not periodic, convolution). Restates h_grid (src/pcbqs/biot.py:108-181)."""
    from scipy.fft import next_fast_len
    x, y, heights = [np.asarray(v, float) for v in (x, y, np.atleast_1d(heights))]
    for axis in (x, y):
        if (axis.ndim != 1 or len(axis) < 2 or not np.isfinite(axis).all() or np.diff(axis).min() <= 0
                or not np.allclose(np.diff(axis), axis[1] - axis[0], rtol=1e-8, atol=1e-15)):
            raise ValueError('x and y must be increasing uniform grids (m)')
    if heights.ndim != 1 or not np.isfinite(heights).all():
        raise ValueError('heights must be finite absolute z coordinates (m)')
    if np.any(np.isclose(heights[:, None], np.unique(z_of)[None], rtol=0, atol=1e-15)):
        raise ValueError('FFT H must be evaluated away from copper planes')
    if not isinstance(refine, (int, np.integer)) or refine < 1:
        raise ValueError('refine must be a positive integer')
    I = np.asarray(I)
    multi = I.ndim > 1
    I2 = I if multi else I[:, None]
    nodes = rwg.nodes
    dx, dy = (x[1] - x[0]) / refine, (y[1] - y[0]) / refine
    grids, offsets = [], []
    for dim, axis, step in ((0, x, dx), (1, y, dy)):
        lo = min(0, int(np.floor((nodes[:, dim].min() - axis[0]) / step)) - 2)
        hi = max(refine * (len(axis) - 1), int(np.ceil((nodes[:, dim].max() - axis[0]) / step)) + 2)
        grids.append(axis[0] + np.arange(lo, hi + 1) * step)
        offsets.append(-lo)
    gx, gy = grids
    nx, ny = len(gx), len(gy)
    shape = (next_fast_len(3 * nx - 2), next_fast_len(3 * ny - 2))
    dev = torch.device('cuda', device)
    rx = torch.arange(1 - nx, nx, device=dev, dtype=torch.float64)[:, None] * dx
    ry = torch.arange(1 - ny, ny, device=dev, dtype=torch.float64)[None, :] * dy
    k = I2.shape[1]
    out = torch.zeros((len(x), len(y), len(heights), 3, k), dtype=torch.complex128, device=dev)
    cx = slice(nx - 1 + offsets[0], nx - 1 + offsets[0] + refine * len(x), refine)
    cy = slice(ny - 1 + offsets[1], ny - 1 + offsets[1] + refine * len(y), refine)
    fft2 = lambda v: torch.fft.fft2(v, s=shape, dim=(0, 1))
    for idx in layer_tris.values():
        idx = np.asarray(idx)
        jx, jy = current_grid(rwg, I2, idx, gx, gy, device=device)
        Jx, Jy = fft2(jx), fft2(jy)
        for h, height in enumerate(heights):
            dz = height - z_of[idx[0]]
            kernel = dx * dy / (4 * np.pi * (rx * rx + ry * ry + dz * dz) ** 1.5)
            kx, ky, kz = [fft2((v * kernel).to(torch.complex128))[..., None] for v in (rx + 0 * ry, ry + 0 * rx,
                                                                                       dz + 0 * rx * ry)]
            for c, spectrum in enumerate((Jy * kz, -Jx * kz, Jx * ky - Jy * kx)):
                out[:, :, h, c] += torch.fft.ifft2(spectrum, dim=(0, 1))[cx, cy]
    H = out.cpu().numpy()
    if filaments is not None and len(filaments[0]):
        p0, p1, currents = filaments
        X, Y, Z = np.meshgrid(x, y, heights, indexing='ij')
        pts = np.stack([X, Y, Z], axis=-1).reshape(-1, 3)
        cur = np.asarray(currents)
        H += h_segments(p0, p1, cur if cur.ndim > 1 else cur[:, None], pts, device).reshape(H.shape)
    return H if multi else H[..., 0]
