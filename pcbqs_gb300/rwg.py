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
        # Edges keyed by their sorted end nodes, in first-seen order (a dict keeps insertion order).
        seen = {}
        for t, (a, b, c) in enumerate(self.tris.tolist()):
            for i, (u, v) in enumerate(((a, b), (b, c), (c, a))):
                seen.setdefault((u, v) if u < v else (v, u), []).append((t, i))
        interior = [(k, s) for k, s in seen.items() if len(s) == 2]
        self.Ne = len(interior)
        u, v = np.array([k for k, _ in interior], np.int64).reshape(-1, 2).T
        (t1, i1), (t2, i2) = np.array([s for _, s in interior], np.int64).reshape(-1, 2, 2).transpose(1, 2, 0)
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
