"""Compressed (H-matrix) partial inductance on the device: cluster tree and admissibility on the host, exact dense
near leaves and ACA far blocks built by device kernels, and the compressed product Y = L X on the device.

    H = DeviceHMatrix(fill, tol=1e-6, leaf=64, eta=1.0, rank=32)     # fill: a DeviceFill (its geometry and RWG)
    Y = H.matmat(X)                                                    # X (ne, k) complex torch tensor on the GPU

The counterpart of pcbqs's HMatrix (src/pcbqs/hmatrix.py:59-221), with a tree of its own: a flat-array binary tree
cut at the median of the support-box centres along their principal axis; the reference's admissibility (box gap >
eta * the larger diagonal, 3-D boxes); blocks decided a tree level at a time, both clusters refined together, a
block whose ACA is not accepted refined further (or made dense when both clusters are leaves), and only the upper
half of the symmetric block structure stored (each block applied both ways, diagonal blocks symmetrized). The entries are those of compressed.edge_inductance (src/pcbqs/compressed.py:60-96) with the support
boxes of compressed._boxes (:54-57). ACA runs one CTA per block with a rank cap min(rank, 0.7 m n / (m + n)).
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .fill import EPS0, MU0


class ClusterTree:
    """A binary cluster tree over n items with 3-D bounding boxes (lo, hi), held in flat arrays.

    Node k owns the items perm[start[k]:stop[k]]; kids[k] = (left, right) node indices, or (-1, -1) at a leaf.
    Nodes are made breadth first: a node with more than `leaf` items is cut through the median of its box
    centres projected on their principal axis (the dominant eigenvector of their covariance), so both halves hold
    half the items whatever the cloud's orientation, and every level of the tree is balanced."""

    def __init__(self, lo, hi, leaf):
        lo, hi = np.asarray(lo, float), np.asarray(hi, float)
        centre = 0.5 * (lo + hi)
        self.perm = np.arange(len(lo))
        start, stop, kids = [0], [len(lo)], [[-1, -1]]
        k = 0
        while k < len(start):
            a, b = start[k], stop[k]
            if b - a > leaf:
                seg = self.perm[a:b]
                c = centre[seg] - centre[seg].mean(0)
                _, vec = np.linalg.eigh(c.T @ c)
                proj = c @ vec[:, -1]
                half = (b - a) // 2
                self.perm[a:b] = seg[np.argpartition(proj, half)]
                kids[k] = [len(start), len(start) + 1]
                start += [a, a + half]
                stop += [a + half, b]
                kids += [[-1, -1], [-1, -1]]
            k += 1
        self.start, self.stop = np.asarray(start), np.asarray(stop)
        self.kids = np.asarray(kids)
        self.lo = np.array([lo[self.ids(k)].min(0) for k in range(len(start))])
        self.hi = np.array([hi[self.ids(k)].max(0) for k in range(len(start))])
        self.diam2 = ((self.hi - self.lo) ** 2).sum(1)

    def ids(self, k):
        return self.perm[self.start[k]:self.stop[k]]

    def size(self, k):
        return int(self.stop[k] - self.start[k])

    def leaf(self, k):
        return self.kids[k, 0] < 0

    def separated(self, i, j, eta):
        """Whether the block (i, j) is far enough to compress: the distance between the two boxes exceeds eta
        times the larger box diagonal (the admissibility of the reference's HMatrix, src/pcbqs/hmatrix.py:152-156,
        compared here in squares)."""
        if i == j:
            return False
        gap = np.maximum(0.0, np.maximum(self.lo[i] - self.hi[j], self.lo[j] - self.hi[i]))
        return float(gap @ gap) > eta * eta * max(self.diam2[i], self.diam2[j])

    def refine(self, i, j):
        """The sub-blocks that replace the block (i, j): both clusters cut where both have children (only the
        one that has, otherwise). A diagonal block keeps the upper pairs (p <= q) of its children, since a block
        below the diagonal is the transpose of one above it and the product applies each stored block both ways."""
        left = [i] if self.leaf(i) else list(self.kids[i])
        right = [j] if self.leaf(j) else list(self.kids[j])
        return [(int(p), int(q)) for p in left for q in right if i != j or p <= q]


def support_boxes(fill):
    """Per RWG edge, the box of its two support triangles in (x, y, z) (compressed._boxes and the support min/max)."""
    g = fill.geometry
    v = g.nodes[g.tris]
    lo_t, hi_t = np.c_[v.min(1), g.z], np.c_[v.max(1), g.z]
    r = fill.rwg
    support = np.stack((r.tp, r.tm), axis=1)
    return lo_t[support].min(1), hi_t[support].max(1)


def _pack_parts(store, jobs, map_all, plane, off2):
    """Write the BF16 parts of H-matrix entries into a tensor-core plane (pcbqs_gb300_pack_bf16_parts): each job
    (base, si, sj, ni, nj, row0, colbase, map_off) takes x = store[base + i si + j sj], i < ni, j < nj, and writes
    h = bf16(x) and m = bf16(x - h) to plane[row0 + i, c] and plane[row0 + i, off2 + c], c = colbase +
    map_all[map_off + j] (colbase + j when map_off < 0). Every read and write is checked on the host first."""
    if not jobs:
        return
    J = np.asarray(jobs, np.int64)
    base, si, sj, ni, nj, row0, colbase, moff = J.T
    assert (ni >= 0).all() and (nj >= 0).all()
    mapped = moff >= 0
    seg = nj - 1                                  # each job's largest column offset
    if mapped.any():
        # a list's maps are consecutive runs of map_all (never empty: a cluster has members); each run's maximum
        # by one reduceat over their span
        starts, counts = moff[mapped], nj[mapped]
        assert (counts > 0).all() and (np.diff(starts) == counts[:-1]).all()
        lo, hi = starts[0], starts[-1] + counts[-1]
        assert hi <= len(map_all) and map_all[lo:hi].min() >= 0
        seg[mapped] = np.maximum.reduceat(map_all[lo:hi], starts - lo)
    live = (ni > 0) & (nj > 0)                    # a rank-0 block's factors write nothing
    if not live.any():
        return
    J, base, si, sj, ni, nj, row0, colbase, seg = (a[live] for a in (J, base, si, sj, ni, nj, row0, colbase, seg))
    assert base.min() >= 0 and (base + (ni - 1) * si + (nj - 1) * sj).max() < store.numel()
    assert row0.min() >= 0 and (row0 + ni).max() <= plane.shape[0]
    assert colbase.min() >= 0 and (colbase + seg + off2).max() < plane.shape[1]
    assert plane.dtype == torch.bfloat16 and plane.is_contiguous() and store.dtype == torch.float64
    _pack_launch(store, np.ascontiguousarray(J), map_all, plane, off2)


def _pack_launch(store, J, map_all, plane, off2):
    """The launch of pcbqs_gb300_pack_bf16_parts for jobs checked by _pack_parts."""
    dev = plane.device
    jobs_d = torch.as_tensor(J, device=dev)
    map_d = torch.as_tensor(map_all, device=dev)
    lib = _lib.load()
    _lib.check(lib.pcbqs_gb300_pack_bf16_parts(store.data_ptr(), jobs_d.data_ptr(), len(J), map_d.data_ptr(),
                                               plane.data_ptr(), plane.shape[1], off2,
                                               ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)), lib)
    torch.cuda.current_stream(dev).synchronize()


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
        tree = ClusterTree(lo, hi, leaf)
        self.tree = tree
        lib = _lib.load()
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        blocks, stores = [], []       # final (a_ids, b_ids, store index, offset, rank, cap, same)
        self._nodes = []              # each block's (row cluster, column cluster) tree nodes
        level = [(0, 0)]              # the block (root, root), then each level's undecided blocks
        self.entries = 0
        while level:
            compress, exact, deeper = [], [], []
            for i, j in level:
                if tree.separated(i, j, eta):
                    m, n = tree.size(i), tree.size(j)
                    cap = min(rank, int(0.7 * m * n / (m + n)))
                    if cap >= 1:
                        compress.append((i, j, cap))
                        continue
                (exact if tree.leaf(i) and tree.leaf(j) else deeper).append((i, j))
            deeper = [sub for i, j in deeper for sub in tree.refine(i, j)]
            if compress:
                ranks, store, offsets = self._aca_round(compress, lib, stream)
                for (i, j, cap), off, rk in zip(compress, offsets, ranks):
                    if rk >= 0:
                        self.entries += cap * (tree.size(i) + tree.size(j))
                        blocks.append((tree.ids(i), tree.ids(j), len(stores), off, int(rk), cap, False))
                        self._nodes.append((i, j))
                    elif tree.leaf(i) and tree.leaf(j):
                        exact.append((i, j))                # ACA not accepted on two leaves: a dense block
                    else:
                        deeper.extend(tree.refine(i, j))
                stores.append(store)
            if exact:
                self._dense_round(exact, blocks, stores, lib, stream)
            if log:
                log(f'hmatrix: {len(blocks):,} blocks so far')
            level = deeper
        self._pack(blocks, stores)

    def _aca_round(self, admissible, lib, stream):
        """ACA of one level's admissible blocks (tree node pairs) on the device: (ranks (-1: not accepted), store,
        store offsets)."""
        dev, tree = self.fill.device, self.tree
        idx, meta, offset, ioff, offsets = [], [], 0, 0, []
        for i, j, cap in admissible:
            la, lb = tree.size(i), tree.size(j)
            meta.append([ioff, la, ioff + la, lb, offset, cap, 0, -1])
            offsets.append(offset)
            idx += [tree.ids(i), tree.ids(j)]
            ioff += la + lb
            offset += la * cap + cap * lb + 32 * lb            # U, V and the check rows
        meta_d = torch.as_tensor(np.asarray(meta, np.int64), device=dev)
        idx_d = torch.as_tensor(np.concatenate(idx).astype(np.int64), device=dev)
        store = torch.empty(max(offset, 1), dtype=torch.float64, device=dev)
        ids = torch.as_tensor(np.arange(len(admissible), dtype=np.int64), device=dev)
        used_stride = max(tree.size(i) for i, _, _ in admissible)
        used = torch.empty(len(admissible) * used_stride, dtype=torch.uint8, device=dev)
        near = float(self.fill.near)
        _lib.check(lib.pcbqs_gb300_hmatrix_build(
            self.fill.dev.handle, -1.0 if np.isinf(near) else near, int(self.fill.outer_levels), self.kind,
            self._edges[0].data_ptr(), self._edges[1].data_ptr(), self._edges[2].data_ptr(), self.ne,
            self.factor, meta_d.data_ptr(), None, 0, ids.data_ptr(), len(admissible), idx_d.data_ptr(),
            self.tol, store.data_ptr(), used.data_ptr(), used_stride, stream), lib)
        return meta_d[:, 7].cpu().numpy(), store, offsets

    def _dense_round(self, pairs, blocks, stores, lib, stream):
        """Exact dense blocks (tree node pairs) on the device, appended to `blocks`; a diagonal block is stored
        symmetrized."""
        dev, tree = self.fill.device, self.tree
        idx, meta, offset, ioff = [], [], 0, 0
        for i, j in pairs:
            la, lb = tree.size(i), tree.size(j)
            meta.append([ioff, la, ioff + la, lb, offset, 0, int(i == j), -1])
            idx += [tree.ids(i), tree.ids(j)]
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
        for (i, j), m in zip(pairs, meta):
            self.entries += tree.size(i) * tree.size(j)
            blocks.append((tree.ids(i), tree.ids(j), len(stores), m[4], -1, 0, i == j))
            self._nodes.append((i, j))
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

    def dense_entries(self, pairs, host=False):
        """Exact entries H[a][:, b] for each (a, b) pair of index arrays, evaluated on the device by the build's dense
        path (the fill's context is needed): a list of (len(a), len(b)) float64 device tensors (host=True: NumPy
        arrays, copied back at once)."""
        if self.fill is None:
            raise ValueError('a loaded H-matrix evaluates no new entries')
        dev = self.fill.device
        meta, idx, offset, ioff, shapes = [], [], 0, 0, []
        for a, b in pairs:
            la, lb = len(a), len(b)
            meta.append([ioff, la, ioff + la, lb, offset, 0, 0, -1])
            idx += [np.asarray(a, np.int64), np.asarray(b, np.int64)]
            shapes.append((offset, la, lb))
            ioff += la + lb
            offset += la * lb
        if not pairs:
            return []
        meta_d = torch.as_tensor(np.asarray(meta, np.int64), device=dev)
        idx_d = torch.as_tensor(np.concatenate(idx), device=dev)
        store = torch.empty(max(offset, 1), dtype=torch.float64, device=dev)
        ids = torch.arange(len(pairs), dtype=torch.int64, device=dev)
        near = float(self.fill.near)
        lib = _lib.load()
        _lib.check(lib.pcbqs_gb300_hmatrix_build(
            self.fill.dev.handle, -1.0 if np.isinf(near) else near, int(self.fill.outer_levels), self.kind,
            self._edges[0].data_ptr(), self._edges[1].data_ptr(), self._edges[2].data_ptr(), self.ne,
            self.factor, meta_d.data_ptr(), ids.data_ptr(), len(pairs), None, 0, idx_d.data_ptr(),
            self.tol, store.data_ptr(), None, 0, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), lib)
        if host:
            flat = store.cpu().numpy()
            return [flat[o:o + la * lb].reshape(la, lb) for o, la, lb in shapes]
        return [store[o:o + la * lb].view(la, lb) for o, la, lb in shapes]

    def desc(self):
        """The packed arrays as the C ABI's pcbqs_gb300_hmat (valid while this object lives)."""
        d = _lib.HmatDesc()
        d.n, d.nblocks, d.nslots = self.n, self.nblocks, self.nslots
        d.meta, d.slot0, d.idx = self.meta.data_ptr(), self.slot0.data_ptr(), self.idx.data_ptr()
        d.row_ptr, d.slots_of_row, d.store = self.row_ptr.data_ptr(), self.slots_of_row.data_ptr(), self.store.data_ptr()
        d.max_rank = self.max_rank
        return d

    def lowrank_plan(self, dense=False):
        """The low-rank blocks packed for the tensor cores (pcbqs_gb300_hmatrix_apply_lowrank): each block gives a
        group per direction, Y[I] += L (R X[J]) with (L, R) = (U, V) forward and (V^T, U^T) transposed, the factors
        split into BF16 parts h, m. X is read in a padded cluster order, each leaf's range rounded up to 64, so every
        cluster is a 64-aligned range the tensor copies can address. dense=True packs the dense leaves too (one
        group per block and direction, D or D^T at J's padded positions), so the whole product runs on the tensor
        cores. Returns (arrays kept alive, the C struct), or None when there is nothing to pack."""
        tree, dev = self.tree, self.store.device
        meta = self.meta.cpu().numpy()
        slot0 = self.slot0.cpu().numpy()
        low = np.flatnonzero(meta[:, 7] >= 0)
        if not len(low) and not dense:
            return None
        if self.max_rank > 64:
            raise ValueError('the tensor-core low-rank product takes ranks up to 64')
        leaves = sorted((k for k in range(len(tree.start)) if tree.leaf(k)), key=lambda k: tree.start[k])
        pos = np.empty(self.n, np.int32)
        pstart_of_start, pend_of_stop, off = {}, {}, 0
        for k in leaves:
            a, b = int(tree.start[k]), int(tree.stop[k])
            pos[tree.perm[a:b]] = off + np.arange(b - a)
            pstart_of_start[a] = off
            off += -(-(b - a) // 64) * 64
            pend_of_stop[b] = off
        n_pad = off
        span = lambda k: (pstart_of_start[int(tree.start[k])], pend_of_stop[int(tree.stop[k])])
        store = self.store
        # pack jobs (base, si, sj, ni, nj, row0, colbase, map_off): entry (i, j) = store[base + i si + j sj]. A block's
        # U (la x rk) holds U[r, c] = store[so + c la + r], its V (rk x lb) V[c, r] = store[so + la cap + c lb + r];
        # forward the group's left factor is U and its right V, transposed V^T and U^T.
        groups, ljobs, rjobs, maps = [], [], [], []
        a_row0, b_x0, map_n = 0, 0, 0
        for w in low:
            la, lb, so, cap, rk = (int(meta[w, 1]), int(meta[w, 3]), int(meta[w, 4]), int(meta[w, 5]),
                                   int(meta[w, 7]))
            i, j = self._nodes[w]
            for lbase, rows, rbase, ncols, cols_node, slot in ((so, la, so + la * cap, lb, j, slot0[w, 0]),
                                                               (so + la * cap, lb, so, la, i, slot0[w, 1])):
                p0, p1 = span(cols_node)
                cols_pos = pos[tree.ids(cols_node)] - p0
                groups.append((a_row0, rows, p0, b_x0, (p1 - p0) // 64, 256 * len(groups), rk, 0, int(slot)))
                ljobs.append((lbase, 1, rows, rows, rk, a_row0, 0, -1))
                rjobs.append((rbase, ncols, 1, rk, ncols, 0, b_x0, map_n))
                maps.append(cols_pos)
                map_n += len(cols_pos)
                a_row0 += rows
                b_x0 += p1 - p0
                if meta[w, 6]:                      # a diagonal block has no transposed half (none is low rank)
                    break
        lrows = a_row0 + 128
        rwidth = max(b_x0, 64)
        dgroups, djobs = [], []
        d_row0 = 0
        if dense:
            for w in np.flatnonzero(meta[:, 7] < 0):
                la, lb, so = int(meta[w, 1]), int(meta[w, 3]), int(meta[w, 4])
                i, j = self._nodes[w]
                # D (la x lb) row-major at so; forward D, transposed D^T
                for rows, ncols, si, sj, cols_node, slot in ((la, lb, lb, 1, j, slot0[w, 0]),
                                                             (lb, la, 1, lb, i, slot0[w, 1])):
                    p0, p1 = span(cols_node)
                    cols_pos = pos[tree.ids(cols_node)] - p0
                    dgroups.append((d_row0, rows, p0, 0, (p1 - p0) // 64, 0, 0, 0, int(slot)))
                    djobs.append((so, si, sj, rows, ncols, d_row0, 0, map_n))
                    maps.append(cols_pos)
                    map_n += len(cols_pos)
                    d_row0 += rows
                    if meta[w, 6]:                  # a diagonal block is stored whole: one direction
                        break
        dpitch = max([g[4] * 64 for g in dgroups] + [64])
        map_all = np.concatenate(maps).astype(np.int32) if maps else np.zeros(1, np.int32)
        lplane = torch.zeros((lrows, 128), dtype=torch.bfloat16, device=dev)
        rplane = torch.zeros((128, 2 * rwidth), dtype=torch.bfloat16, device=dev)
        _pack_parts(store, ljobs, map_all, lplane, 64)
        _pack_parts(store, rjobs, map_all, rplane, rwidth)
        gdt = np.dtype([('a_row0', '<i4'), ('rows', '<i4'), ('a_x0', '<i4'), ('b_x0', '<i4'), ('kb', '<i4'),
                        ('t_row0', '<i4'), ('rank', '<i4'), ('pad', '<i4'), ('slot0', '<i8')])
        assert gdt.itemsize == 40
        garr = np.array(groups, dtype=gdt)
        tiles = [(g, t) for g, grp in enumerate(groups) for t in range(-(-grp[1] // 128))]
        fp64_dense = np.flatnonzero(meta[:, 7] < 0) if not dense else np.zeros(0, np.int64)
        t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a, dt), device=dev)
        keep = dict(lplane=lplane, rplane=rplane, groups=t(garr.view(np.uint8), np.uint8),
                    tile_group=t([g for g, _ in tiles] or [0], np.int32), tile_m=t([m for _, m in tiles] or [0], np.int32),
                    pad_pos=t(pos, np.int32), meta_dense=t(meta[fp64_dense].reshape(-1, 8), np.int64),
                    slot0_dense=t(slot0[fp64_dense].reshape(-1, 2), np.int64))
        d = _lib.LowRankDesc()
        d.meta_dense, d.slot0_dense, d.ndense = (keep['meta_dense'].data_ptr(), keep['slot0_dense'].data_ptr(),
                                                 len(fp64_dense))
        if dgroups:
            dplane = torch.zeros((d_row0 + 128, 2 * dpitch), dtype=torch.bfloat16, device=dev)
            _pack_parts(store, djobs, map_all, dplane, dpitch)
            dtiles = [(g, tt) for g, grp in enumerate(dgroups) for tt in range(-(-grp[1] // 128))]
            keep.update(dplane=dplane, dgroups=t(np.array(dgroups, dtype=gdt).view(np.uint8), np.uint8),
                        dtile_group=t([g for g, _ in dtiles], np.int32), dtile_m=t([m for _, m in dtiles], np.int32))
            d.dplane, d.drows, d.dpitch = dplane.data_ptr(), d_row0 + 128, dpitch
            d.dgroups, d.ndgroups, d.ndtiles = keep['dgroups'].data_ptr(), len(dgroups), len(dtiles)
            d.dtile_group, d.dtile_m = keep['dtile_group'].data_ptr(), keep['dtile_m'].data_ptr()
        d.lplane, d.lrows = lplane.data_ptr(), lrows
        d.rplane, d.rwidth = rplane.data_ptr(), rwidth
        d.groups, d.ngroups, d.ntiles = keep['groups'].data_ptr(), len(groups), len(tiles)
        d.tile_group, d.tile_m, d.pad_pos = (keep['tile_group'].data_ptr(), keep['tile_m'].data_ptr(),
                                             keep['pad_pos'].data_ptr())
        d.n_pad = n_pad
        return keep, d

    def matmat_lowrank(self, X, dense=False):
        """Y = H X with the low-rank blocks on the tensor cores in BF16 (pcbqs_gb300_hmatrix_apply_lowrank); the
        dense blocks in FP64, or (dense=True) on the tensor cores too. X (n, k <= 128) complex128 on the device."""
        plans = self.__dict__.setdefault('_plans', {})
        if dense not in plans:
            plans[dense] = self.lowrank_plan(dense=dense)
        plan = plans[dense]
        X = X.reshape(self.n, -1).to(torch.complex128).contiguous()
        if plan is None:
            return self.matmat(X)
        Y = torch.empty_like(X)
        lib = _lib.load()
        d = self.desc()
        _lib.check(lib.pcbqs_gb300_hmatrix_apply_lowrank(ctypes.byref(d), ctypes.byref(plan[1]), X.shape[1],
                                                         X.data_ptr(), Y.data_ptr(),
                                                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
                   lib)
        return Y

    _ARRAYS = ('store', 'meta', 'idx', 'slot0', 'row_ptr', 'slots_of_row')

    def __getstate__(self):
        """Pickle support, as HMatrix.__getstate__ (src/pcbqs/hmatrix.py:308-316): the blocks and the product's
        index arrays go to host memory; the fill (its device context, the exact-entry source) is not kept, so a
        loaded matrix applies its blocks but evaluates no new entries. The triangle areas stay for
        potential_operator."""
        state = {k: v for k, v in self.__dict__.items() if k not in ('fill', '_edges', '_plans') + self._ARRAYS}
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
