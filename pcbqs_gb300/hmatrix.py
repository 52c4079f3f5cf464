"""Compressed (H-matrix) partial inductance on the device: cluster tree and admissibility on the host, exact dense
near leaves and ACA far blocks built by device kernels, and the compressed product Y = L X on the device.

    H = DeviceHMatrix(fill, tol=1e-6, leaf=64, eta=1.0, rank=32)     # fill: a DeviceFill (its geometry and RWG)
    Y = H.matmat(X)                                                    # X (ne, k) complex torch tensor on the GPU

Restates pcbqs's HMatrix (src/pcbqs/hmatrix.py:59-221): the bisection tree on support-box centres (widest axis,
stable sort, halves), admissibility gap > eta * max(diameter) with 3-D boxes, level-by-level construction where a
block whose ACA is not accepted is subdivided (or made dense when both clusters are leaves), and diagonal blocks
symmetrized. The entries are those of compressed.edge_inductance (src/pcbqs/compressed.py:60-96) with the support
boxes of compressed._boxes (:54-57). ACA runs one CTA per block with a rank cap min(rank, 0.7 m n / (m + n)).
"""
import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .fill import EPS0, MU0


@dataclass
class Cluster:
    ids: np.ndarray
    lo: np.ndarray
    hi: np.ndarray
    children: tuple = ()


def cluster_tree(lo, hi, leaf):
    def tree(ids):
        node = Cluster(ids, lo[ids].min(0), hi[ids].max(0))
        if len(ids) > leaf:
            centers = (lo[ids] + hi[ids]) / 2
            axis = np.argmax(np.ptp(centers, axis=0))
            order = ids[np.argsort(centers[:, axis], kind='stable')]
            mid = len(ids) // 2
            node.children = (tree(order[:mid]), tree(order[mid:]))
        return node
    return tree(np.arange(len(lo)))


def _admissible(a, b, eta):
    gap = np.linalg.norm(np.maximum(0, np.maximum(a.lo - b.hi, b.lo - a.hi)))
    diameter = max(np.linalg.norm(a.hi - a.lo), np.linalg.norm(b.hi - b.lo))
    return a is not b and gap > eta * diameter


def _children(a, b):
    if a is b:
        x, y = a.children
        return [(x, x), (x, y), (y, y)]
    if a.children and (not b.children or len(a.ids) >= len(b.ids)):
        return [(child, b) for child in a.children]
    return [(a, child) for child in b.children]


def support_boxes(fill):
    """Per RWG edge, the box of its two support triangles in (x, y, z) (compressed._boxes and the support min/max)."""
    g = fill.geometry
    v = g.nodes[g.tris]
    lo_t, hi_t = np.c_[v.min(1), g.z], np.c_[v.max(1), g.z]
    r = fill.rwg
    support = np.stack((r.tp, r.tm), axis=1)
    return lo_t[support].min(1), hi_t[support].max(1)


class DeviceHMatrix:
    META = 8

    def __init__(self, fill, tol=1e-6, leaf=64, eta=1.0, rank=32, log=None, kernel='inductance', er=1.0):
        """kernel='inductance': L over RWG edges (mu0/4pi); kernel='potential': the triangle kernel
        M0 / (A_t A_u 4 pi eps0 er) of compressed.potential."""
        self.fill, self.tol, self.leaf, self.eta, self.rank = fill, tol, leaf, eta, rank
        dev = fill.device
        r = fill.rwg
        self.ne = r.Ne
        tri = np.ascontiguousarray(np.stack([r.tp, r.tm]), np.int32)
        alpha = np.ascontiguousarray(np.stack([1 / (2 * r.area[r.tp]), -1 / (2 * r.area[r.tm])]))
        vertex = np.ascontiguousarray(np.stack([r.vp, r.vm]), float)
        self._edges = [torch.as_tensor(a, device=dev) for a in (tri, alpha, vertex)]
        if kernel == 'inductance':
            self.kind, self.factor, self.n = 0, MU0 / (4 * np.pi), r.Ne
            lo, hi = support_boxes(fill)
        elif kernel == 'potential':
            self.kind, self.factor, self.n = 1, 1.0 / (4 * np.pi * EPS0 * er), fill.nt
            g = fill.geometry
            v = g.nodes[g.tris]
            lo, hi = np.c_[v.min(1), g.z], np.c_[v.max(1), g.z]
        else:
            raise ValueError("kernel must be 'inductance' or 'potential'")
        root = cluster_tree(lo, hi, leaf)
        lib = _lib.load()
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        near = float(fill.near)
        blocks, stores = [], []       # final (a_ids, b_ids, store index, offset, rank, cap, same)
        pending = [(root, root)]
        self.entries = 0
        while pending:
            admissible, dense, following = [], [], []
            for a, b in pending:
                if _admissible(a, b, eta):
                    cap = min(rank, int(0.7 * len(a.ids) * len(b.ids) / (len(a.ids) + len(b.ids))))
                    if cap >= 1:
                        admissible.append((a, b, cap))
                        continue
                if not a.children and not b.children:
                    dense.append((a, b))
                else:
                    following.extend(_children(a, b))
            failed_leaves = []
            if admissible:
                ranks, store, offsets = self._aca_round(admissible, lib, stream)
                for (a, b, cap), off, rk in zip(admissible, offsets, ranks):
                    if rk >= 0:
                        self.entries += cap * (len(a.ids) + len(b.ids))
                        blocks.append((a.ids, b.ids, len(stores), off, int(rk), cap, False))
                    elif not a.children and not b.children:
                        failed_leaves.append((a, b))        # not compressible: a dense leaf
                    else:
                        following.extend(_children(a, b))
                stores.append(store)
            if dense or failed_leaves:
                self._dense_round(dense + failed_leaves, blocks, stores, lib, stream)
            if log:
                log(f'hmatrix: {len(blocks):,} blocks so far')
            pending = following
        self._pack(blocks, stores)

    def _aca_round(self, admissible, lib, stream):
        """ACA of one level's admissible blocks on the device: (ranks (-1: not accepted), store, store offsets)."""
        dev = self.fill.device
        idx, meta, offset, ioff, offsets = [], [], 0, 0, []
        for a, b, cap in admissible:
            la, lb = len(a.ids), len(b.ids)
            meta.append([ioff, la, ioff + la, lb, offset, cap, 0, -1])
            offsets.append(offset)
            idx += [a.ids, b.ids]
            ioff += la + lb
            offset += la * cap + cap * lb + 32 * lb            # U, V and the check rows
        meta_d = torch.as_tensor(np.asarray(meta, np.int64), device=dev)
        idx_d = torch.as_tensor(np.concatenate(idx).astype(np.int64), device=dev)
        store = torch.empty(max(offset, 1), dtype=torch.float64, device=dev)
        ids = torch.as_tensor(np.arange(len(admissible), dtype=np.int64), device=dev)
        used_stride = max(len(a.ids) for a, _, _ in admissible)
        used = torch.empty(len(admissible) * used_stride, dtype=torch.uint8, device=dev)
        near = float(self.fill.near)
        _lib.check(lib.pcbqs_gb300_hmatrix_build(
            self.fill.dev.handle, -1.0 if np.isinf(near) else near, int(self.fill.outer_levels), self.kind,
            self._edges[0].data_ptr(), self._edges[1].data_ptr(), self._edges[2].data_ptr(), self.ne,
            self.factor, meta_d.data_ptr(), None, 0, ids.data_ptr(), len(admissible), idx_d.data_ptr(),
            self.tol, store.data_ptr(), used.data_ptr(), used_stride, stream), lib)
        return meta_d[:, 7].cpu().numpy(), store, offsets

    def _dense_round(self, pairs, blocks, stores, lib, stream):
        dev = self.fill.device
        idx, meta, offset, ioff = [], [], 0, 0
        for a, b in pairs:
            la, lb = len(a.ids), len(b.ids)
            meta.append([ioff, la, ioff + la, lb, offset, 0, int(a is b), -1])
            idx += [a.ids, b.ids]
            ioff += la + lb
            offset += la * lb
        meta_d = torch.as_tensor(np.asarray(meta, np.int64), device=dev)
        idx_d = torch.as_tensor(np.concatenate(idx).astype(np.int64), device=dev)
        store = torch.empty(max(offset, 1), dtype=torch.float64, device=dev)
        ids = torch.as_tensor(np.arange(len(pairs), dtype=np.int64), device=dev)
        near = float(self.fill.near)
        _lib.check(lib.pcbqs_gb300_hmatrix_build(
            self.fill.dev.handle, -1.0 if np.isinf(near) else near, int(self.fill.outer_levels), self.kind,
            self._edges[0].data_ptr(), self._edges[1].data_ptr(), self._edges[2].data_ptr(), self.ne,
            self.factor, meta_d.data_ptr(), ids.data_ptr(), len(pairs), None, 0, idx_d.data_ptr(),
            self.tol, store.data_ptr(), None, 0, stream), lib)
        for (a, b), m in zip(pairs, meta):
            self.entries += len(a.ids) * len(b.ids)
            blocks.append((a.ids, b.ids, len(stores), m[4], -1, 0, a is b))
        stores.append(store)

    def _pack(self, blocks, stores):
        """One store, the product's metadata, and the deterministic contribution slots (row order = block order)."""
        dev = self.fill.device
        base = np.cumsum([0] + [int(s.numel()) for s in stores])
        self.store = torch.cat(stores) if len(stores) > 1 else stores[0]
        meta, idx, ioff, targets, slot0, so = [], [], 0, [], [], 0
        for a, b, si, off, rk, cap, same in blocks:
            la, lb = len(a), len(b)
            meta.append([ioff, la, ioff + la, lb, base[si] + off, cap, int(same), rk])
            idx += [a, b]
            ioff += la + lb
            slot0.append([so, so + la])
            targets.append(a)
            so += la
            if not same:
                targets.append(b)
                so += lb
        targets = np.concatenate(targets)
        slots_of_row = np.argsort(targets, kind='stable').astype(np.int64)
        row_ptr = np.zeros(self.n + 1, np.int64)
        np.cumsum(np.bincount(targets, minlength=self.n), out=row_ptr[1:])
        t = lambda arr: torch.as_tensor(np.asarray(arr, np.int64), device=dev)
        self.meta, self.idx, self.slot0 = t(meta), t(np.concatenate(idx)), t(slot0)
        self.row_ptr, self.slots_of_row, self.nslots = t(row_ptr), t(slots_of_row), so
        self.nblocks = len(blocks)
        self.low_rank = sum(1 for blk in blocks if blk[4] >= 0)
        self.max_rank = max([blk[4] for blk in blocks] + [0])
        self.bytes = int(sum((len(a) * len(b)) if rk < 0 else rk * (len(a) + len(b))
                             for a, b, _, _, rk, _, _ in blocks) * 8)
        self.info = dict(blocks=self.nblocks, low_rank_blocks=self.low_rank, max_rank=self.max_rank,
                         bytes=self.bytes, dense_bytes=self.n * self.n * 8, evaluated_entries=self.entries,
                         tolerance=self.tol, leaf=self.leaf, eta=self.eta)

    _ARRAYS = ('store', 'meta', 'idx', 'slot0', 'row_ptr', 'slots_of_row')

    def __getstate__(self):
        """Pickle support, as HMatrix.__getstate__ (src/pcbqs/hmatrix.py:308-316): the blocks and the product's
        index arrays go to host memory; the fill (its device context, the exact-entry source) is not kept, so a
        loaded matrix applies its blocks but evaluates no new entries. The triangle areas stay for
        potential_operator."""
        state = {k: v for k, v in self.__dict__.items() if k not in ('fill', '_edges') + self._ARRAYS}
        for k in self._ARRAYS:
            state[k] = getattr(self, k).cpu().numpy()
        state['area'] = np.asarray(self.fill.geometry.area) if self.fill is not None else self.__dict__.get('area')
        return state

    def __setstate__(self, state):
        """Uploads the arrays to the current CUDA device (HMatrix.__setstate__ re-packs its blocks likewise)."""
        arrays = {k: state.pop(k) for k in self._ARRAYS}
        self.__dict__.update(state)
        self.fill, self._edges = None, None
        dev = torch.device('cuda', torch.cuda.current_device())
        for k, v in arrays.items():
            setattr(self, k, torch.as_tensor(v, device=dev))

    def potential_operator(self, node_of):
        """P x = W^T H W x for the charge nodes (compressed.PotentialOperator, src/pcbqs/compressed.py:194-204):
        W[t, node] = A_t / A_node. Returns a function of (nn, k) complex device tensors."""
        if self.kind != 1:
            raise ValueError('a potential operator needs the potential kernel')
        node_of = np.asarray(node_of)
        nn = int(node_of.max()) + 1
        area_t = self.fill.geometry.area if self.fill is not None else self.area
        device = self.store.device
        area_n = np.bincount(node_of, weights=area_t, minlength=nn)
        from scipy.sparse import coo_matrix
        W = coo_matrix((area_t / area_n[node_of], (np.arange(self.n), node_of)), shape=(self.n, nn))
        Wd = torch.sparse_coo_tensor(np.vstack([W.row, W.col]), W.data.astype(complex), W.shape,
                                     device=device).coalesce()
        Wt = Wd.t().coalesce()

        def apply(x):
            return torch.sparse.mm(Wt, self.matmat(torch.sparse.mm(Wd, x.reshape(nn, -1))))
        return apply

    def matmat(self, X):
        """Y = L X for X (ne, k) complex128 on the device (the product of HMatrix._matmat, deterministic)."""
        X = X.reshape(self.n, -1).to(torch.complex128).contiguous()
        k = X.shape[1]
        Y = torch.empty_like(X)
        slots = torch.empty((max(self.nslots, 1), k), dtype=torch.complex128, device=X.device)
        lib = _lib.load()
        _lib.check(lib.pcbqs_gb300_hmatrix_apply(self.n, self.nblocks, self.meta.data_ptr(), self.slot0.data_ptr(),
                                                 self.idx.data_ptr(), self.store.data_ptr(), self.row_ptr.data_ptr(),
                                                 self.slots_of_row.data_ptr(), self.max_rank, k, X.data_ptr(),
                                                 Y.data_ptr(), slots.data_ptr(),
                                                 ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), lib)
        return Y
