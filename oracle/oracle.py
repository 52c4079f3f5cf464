"""CPU oracle of the pcbqs static fill -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import this module, as the oracle (and as
the timed CPU restatement of the reference's compiled core). The product (pcbqs_gb300) never imports it.

Contents:
  * prepare()         FillGeometry.prepare restated (src/pcbqs/static_backends.py:104-130), written independently
                      of the product's copy so the oracle does not share the code it tests;
  * C restatement     liboracle.so built from oracle/pcbqs_oracle.c (make -C oracle): og_pair, og_kind,
                      og_pairs, og_fill, og_combine, og_potential (file:line citations in the C source);
  * rwg()             the RWG basis (src/pcbqs/_numerics/base.py:10-41);
  * node groups       terminal / via-fan merging into charge nodes and P = W^T M0 W (src/pcbqs/mqs.py:365-403,
                      :532-552).
Parity of this oracle is pinned against the reference's own outputs (tests/golden/, tests/test_oracle_golden.py).
"""
import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIBRARY = HERE / '_build' / 'liboracle.so'

MU0 = 4e-7 * np.pi
C0 = 299792458.0
EPS0 = 1.0 / (MU0 * C0 ** 2)

_a1, _a2 = 0.445948490915965, 0.091576213509771
_BAR6 = np.array([[1 - 2 * _a1, _a1, _a1], [_a1, 1 - 2 * _a1, _a1], [_a1, _a1, 1 - 2 * _a1],
                  [1 - 2 * _a2, _a2, _a2], [_a2, 1 - 2 * _a2, _a2], [_a2, _a2, 1 - 2 * _a2]])
_W6 = np.array([0.223381589678011] * 3 + [0.109951743655322] * 3)
_BAR3 = np.array([[2 / 3, 1 / 6, 1 / 6], [1 / 6, 2 / 3, 1 / 6], [1 / 6, 1 / 6, 2 / 3]])


def build():
    """Compile liboracle.so (gcc, OpenMP) when missing or stale; returns its path."""
    src = HERE / 'pcbqs_oracle.c'
    if not LIBRARY.exists() or LIBRARY.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(['make', '-s', '-C', str(HERE)], check=True)
    return LIBRARY


def build_reference():
    """Compile the reference's own core into oracle/_ref/ where its sources exist (this container only)."""
    from .reference import SOURCE
    core = SOURCE / 'pcbqs' / 'core' if SOURCE is not None else None
    if core is None or not core.exists():
        return None
    subprocess.run(['make', '-s', '-C', str(HERE), 'ref', f'REF_SRC={core}'], check=True)
    found = sorted((HERE / '_ref').glob('_core*.so'))
    return found[0] if found else None


class _Geo(ctypes.Structure):
    _fields_ = [('nt', ctypes.c_int),
                ('v', ctypes.c_void_p), ('len', ctypes.c_void_p), ('tau', ctypes.c_void_p),
                ('un', ctypes.c_void_p), ('area', ctypes.c_void_p), ('p3', ctypes.c_void_p),
                ('qp', ctypes.c_void_p * 3), ('qw', ctypes.c_void_p * 3), ('nq', ctypes.c_int * 3)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(str(build()))
        V = ctypes.c_void_p
        L.og_pairs.restype = ctypes.c_int
        L.og_pairs.argtypes = [ctypes.POINTER(_Geo), ctypes.c_long, V, V, V, V, ctypes.c_int, V, ctypes.c_int]
        L.og_fill.restype = ctypes.c_int
        L.og_fill.argtypes = [ctypes.POINTER(_Geo), V, V, V, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                              ctypes.c_int, ctypes.c_int, V, V, V, V, V]
        L.og_kind.restype = ctypes.c_int
        L.og_kind.argtypes = [V, V, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                              ctypes.c_int]
        L.og_combine.restype = None
        L.og_combine.argtypes = [ctypes.c_long, ctypes.c_long, V, V, V, V, ctypes.c_double, V, V, V, V, V,
                                 ctypes.c_int]
        L.og_potential.restype = None
        L.og_potential.argtypes = [ctypes.c_long, ctypes.c_long, V, V, V, V, ctypes.c_double, V, ctypes.c_int]
        _lib = L
    return _lib


def threads():
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


# ---- geometry (FillGeometry.prepare, _offplane_geometry, _split4, edge_frames) ----

def _split4(V):
    m01, m12, m20 = (V[:, 0] + V[:, 1]) / 2, (V[:, 1] + V[:, 2]) / 2, (V[:, 2] + V[:, 0]) / 2
    return np.concatenate([np.stack(t, 1) for t in ((V[:, 0], m01, m20), (m01, V[:, 1], m12),
                                                      (m20, m12, V[:, 2]), (m01, m12, m20))])


def _level(nodes, tris, level):
    V = nodes[tris]
    e = np.roll(V, -1, axis=1) - V
    L = np.linalg.norm(e, axis=2)
    tau = e / L[..., None]
    un = np.stack([tau[..., 1], -tau[..., 0]], -1)
    area = 0.5 * np.abs(e[:, 0, 0] * (-e[:, 2, 1]) - e[:, 0, 1] * (-e[:, 2, 0]))
    bar, w = _BAR6, _W6
    if level:
        ref = np.eye(3)[None]
        for _ in range(level):
            ref = _split4(ref)
        bar = np.einsum('qk,tkc->tqc', _BAR6, ref).reshape(-1, 3)
        w = np.tile(_W6, len(ref)) / len(ref)
    P = np.einsum('qk,tkc->tqc', bar, V)
    return V, L, tau, un, area, P, w.copy()


class Geometry:
    """Prepared mesh: centred nodes, int32 triangles, z, cent, radius, points (P3) and levels {k: (V, L, tau,
    un, area, P, W)} -- the reference FillGeometry's fields."""

    def __init__(self, nodes, tris, z, outer_levels=1):
        nodes, tris, z = np.asarray(nodes, float), np.asarray(tris), np.asarray(z, float)
        self.nodes = np.ascontiguousarray(nodes - nodes.mean(0))
        self.tris = np.array(tris, dtype=np.int32, order='C', copy=True)
        self.z = np.array(z, order='C', copy=True)
        V = self.nodes[self.tris]
        self.cent = V.mean(1)
        self.radius = np.linalg.norm(V - self.cent[:, None], axis=2).max(1)
        self.points = np.einsum('qk,tkc->tqc', _BAR3, V)
        self.levels = {level: _level(self.nodes, self.tris, level) for level in {0, outer_levels}}
        self.outer_levels = outer_levels
        self._struct = None

    @property
    def nt(self):
        return len(self.tris)

    @property
    def area(self):
        return self.levels[0][4]

    def struct(self):
        if self._struct is None:
            V, L, tau, un, area, _, _ = self.levels[0]
            keep = [np.ascontiguousarray(a, float) for a in (V, L, tau, un, area, self.points)]
            g = _Geo()
            g.nt = self.nt
            g.v, g.len, g.tau, g.un, g.area, g.p3 = [a.ctypes.data for a in keep]
            for k in range(3):
                lv = self.levels.get(k, self.levels[0])
                qp, qw = np.ascontiguousarray(lv[5], float), np.ascontiguousarray(lv[6], float)
                keep += [qp, qw]
                g.qp[k], g.qw[k], g.nq[k] = qp.ctypes.data, qw.ctypes.data, len(qw)
            self._struct = (g, keep)
        return self._struct[0]


def kinds(geo, p, q, d, near=3.0, outer=1):
    """FillEngine.kinds (src/pcbqs/static_backends.py:288-298) in NumPy."""
    distance = np.sqrt(((geo.cent[p] - geo.cent[q]) ** 2).sum(-1) + d * d)
    size = geo.radius[p] + geo.radius[q]
    refine = distance <= size
    if np.isinf(near):
        return np.where(refine, outer, 0).astype(np.int32)
    close = distance <= near * size
    kind = np.where(close, 0, -1).astype(np.int32)
    kind[close & refine] = outer
    return kind


def pairs(geo, p, q, d, kind, scalar_only=False, nthreads=None):
    p, q = np.ascontiguousarray(p, np.int32), np.ascontiguousarray(q, np.int32)
    d = np.ascontiguousarray(np.broadcast_to(np.asarray(d, float), p.shape))
    kind = np.ascontiguousarray(kind, np.int32)
    out = np.empty((len(p), 1 if scalar_only else 6))
    rc = lib().og_pairs(geo.struct(), len(p), p.ctypes.data, q.ctypes.data, d.ctypes.data, kind.ctypes.data,
                        int(scalar_only), out.ctypes.data, nthreads or threads())
    if rc:
        raise ValueError('oracle pairs: invalid index, kind or offset')
    return out


def fill(geo, near=3.0, outer=1, scalar_only=False, nthreads=None):
    """(M0, Mx, My, Mrr) (or (M0,)) and the analytic unordered-pair count (static_fill)."""
    n = geo.nt
    mats = [np.empty((n, n)) for _ in range(1 if scalar_only else 4)]
    ptrs = [m.ctypes.data for m in mats] + [None] * (4 - len(mats))
    analytic = ctypes.c_int64()
    all_near = int(np.isinf(near))
    rc = lib().og_fill(geo.struct(), geo.cent.ctypes.data, geo.radius.ctypes.data, geo.z.ctypes.data,
                       0.0 if all_near else float(near), all_near, int(outer), int(scalar_only),
                       nthreads or threads(), *ptrs, ctypes.byref(analytic))
    if rc:
        raise FloatingPointError('non-finite triangle-pair moments (oracle)')
    return mats, int(analytic.value)


# ---- RWG basis (src/pcbqs/_numerics/base.py:10-41) ----

class RWG:
    def __init__(self, nodes, tris):
        self.nodes, self.tris = nodes, np.asarray(tris)
        V = nodes[self.tris]
        e1, e2 = V[:, 1] - V[:, 0], V[:, 2] - V[:, 0]
        self.area = 0.5 * (e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0])
        self.cent = V.mean(1)
        d = {}
        for t, (a, b, c) in enumerate(self.tris):
            for i, (u, v) in enumerate(((a, b), (b, c), (c, a))):
                d.setdefault((min(u, v), max(u, v)), []).append((t, i))
        E = [(k, v) for k, v in d.items() if len(v) == 2]
        self.Ne = len(E)
        u, v = np.array([k for k, _ in E], int).reshape(-1, 2).T
        (t1, i1), (t2, i2) = np.array([s for _, s in E], int).reshape(-1, 2, 2).transpose(1, 2, 0)
        self.tp, self.tm = t1, t2
        self.vp, self.vm = nodes[self.tris[t1, (i1 + 2) % 3]], nodes[self.tris[t2, (i2 + 2) % 3]]
        pu, pv = nodes[u], nodes[v]
        self.l = np.linalg.norm(pv - pu, axis=1)
        self.mid = 0.5 * (pu + pv)
        tau = (pv - pu) / self.l[:, None]
        nrm = np.c_[tau[:, 1], -tau[:, 0]]
        nrm[((self.cent[t2] - self.cent[t1]) * nrm).sum(1) < 0] *= -1
        self.nrm = nrm

    def combine_arrays(self):
        """(tri (2,ne) int32, alpha (2,ne), vertex (2,ne,2)) as static.edge_inductance passes them."""
        tri = np.ascontiguousarray(np.stack([self.tp, self.tm]), np.int32)
        alpha = np.ascontiguousarray(np.stack([self.l / (2 * self.area[self.tp]), -self.l / (2 * self.area[self.tm])]))
        vertex = np.ascontiguousarray(np.stack([self.vp, self.vm]), float)
        return tri, alpha, vertex


def combine(rwg, mats, factor=MU0 / (4 * np.pi), scale=None, nthreads=None):
    """factor diag(scale) combine(moments) diag(scale), symmetric (static_combine)."""
    m0, mx, my, rr = [np.ascontiguousarray(m) for m in mats]
    tri, alpha, vertex = rwg.combine_arrays()
    scale = np.ascontiguousarray(1.0 / rwg.l if scale is None else scale, float)
    out = np.empty((rwg.Ne, rwg.Ne))
    lib().og_combine(rwg.Ne, len(m0), tri.ctypes.data, alpha.ctypes.data, vertex.ctypes.data, scale.ctypes.data,
                     float(factor), rr.ctypes.data, mx.ctypes.data, my.ctypes.data, m0.ctypes.data, out.ctypes.data,
                     nthreads or threads())
    return out


# ---- charge nodes and P (src/pcbqs/mqs.py:365-403, :532-552) ----

def node_groups(nt, merges):
    """node_of (nt) from groups of triangles merged into one node (terminals, via fans), numbered as the
    reference numbers them (np.unique of union-find roots)."""
    parent = np.arange(nt)

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a
    for ts in merges:
        ts = list(ts)
        if not ts:
            continue
        r0 = find(ts[0])
        for t in ts[1:]:
            parent[find(t)] = r0
    roots = np.array([find(t) for t in range(nt)])
    _, node_of = np.unique(roots, return_inverse=True)
    return node_of


def potential(m0, area, node_of, er=1.0, nthreads=None):
    """P = W^T M0 W / (4 pi eps0 er), W[t, node] = 1/A_node."""
    nt = len(node_of)
    nn = int(node_of.max()) + 1
    order = np.argsort(node_of, kind='stable').astype(np.int32)
    start = np.zeros(nn + 1, np.int64)
    np.cumsum(np.bincount(node_of, minlength=nn), out=start[1:])
    node_area = np.bincount(node_of, weights=area, minlength=nn)
    out = np.empty((nn, nn))
    m0 = np.ascontiguousarray(m0)
    lib().og_potential(nt, nn, start.ctypes.data, order.ctypes.data, node_area.ctypes.data, m0.ctypes.data,
                       1.0 / (4 * np.pi * EPS0 * er), out.ctypes.data, nthreads or threads())
    return out
