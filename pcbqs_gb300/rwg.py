"""RWG basis on interior edges, restating src/pcbqs/_numerics/base.py:10-41 (same edge order and orientation).

Edge k joins T+ = tp[k] and T- = tm[k] (in the order the triangles first meet the edge), with free vertices
vp / vm, length l, and positive current direction nrm from T+ to T-; f = alpha (r - v) with alpha = +l/(2 A+)
on T+ and -l/(2 A-) on T-.
"""
import numpy as np


class RWG:
    def __init__(self, nodes, tris):
        self.nodes, self.tris = nodes, np.asarray(tris)
        V = nodes[self.tris]
        e1, e2 = V[:, 1] - V[:, 0], V[:, 2] - V[:, 0]
        self.area = 0.5 * (e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0])
        if not (self.area > 0).all():
            raise ValueError('triangles must be counter-clockwise')
        self.cent = V.mean(1)
        # Edges keyed by their sorted end nodes, in first-seen order (triangle-major, edge (a,b), (b,c), (c,a)), each
        # with its occurrences in that order: a stable sort by key groups the occurrences of one edge in sequence;
        # the interior edges are the keys met exactly twice, ordered by their first occurrence.
        tri = self.tris.astype(np.int64)
        ends = np.stack([tri, np.roll(tri, -1, axis=1)], axis=2).reshape(-1, 2)      # (3 nt, 2): edge i of t
        lo, hi = ends.min(1), ends.max(1)
        key = lo * (int(hi.max()) + 1) + hi
        order = np.argsort(key, kind='stable')
        sk = key[order]
        start = np.flatnonzero(np.r_[True, sk[1:] != sk[:-1]])
        count = np.diff(np.r_[start, len(sk)])
        keep = start[count == 2]
        first, second = order[keep], order[keep + 1]
        seq = np.argsort(first, kind='stable')
        first, second = first[seq], second[seq]
        self.Ne = len(first)
        u, v = lo[first], hi[first]
        t1, i1 = first // 3, first % 3
        t2, i2 = second // 3, second % 3
        self.tp, self.tm = t1, t2
        self.vp = nodes[self.tris[t1, (i1 + 2) % 3]]
        self.vm = nodes[self.tris[t2, (i2 + 2) % 3]]
        pu, pv = nodes[u], nodes[v]
        self.l = np.linalg.norm(pv - pu, axis=1)
        self.mid = 0.5 * (pu + pv)
        tau = (pv - pu) / self.l[:, None]
        nrm = np.c_[tau[:, 1], -tau[:, 0]]
        nrm[((self.cent[t2] - self.cent[t1]) * nrm).sum(1) < 0] *= -1
        self.nrm = nrm

    def combine_arrays(self):
        """(tri (2, ne) int32, alpha (2, ne), vertex (2, ne, 2)): the supports as static_combine takes them."""
        tri = np.ascontiguousarray(np.stack([self.tp, self.tm]), np.int32)
        alpha = np.ascontiguousarray(np.stack([self.l / (2 * self.area[self.tp]), -self.l / (2 * self.area[self.tm])]))
        vertex = np.ascontiguousarray(np.stack([self.vp, self.vm]), float)
        return tri, alpha, vertex
