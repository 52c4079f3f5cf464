"""Boards: a meshed copper model (stacked sheets) with its terminals, via fans and ports.

The mesh comes from pcbqs's host mesher (here: seeded synthetic boards meshed by its constrained-Delaunay core and
stored as .npz, see tests/golden/make_meshes.py). This module restates the MQS model's graph bookkeeping that the
device path needs (src/pcbqs/mqs.py:365-403): one charge/circuit node per triangle, except that the triangles of
each terminal and of each via's fan are merged into one node, numbered as np.unique of the union-find roots.
"""
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parents[1] / 'tests' / 'golden'


def _csr_groups(ptr, items):
    return [np.asarray(items[ptr[i]:ptr[i + 1]], np.int64) for i in range(len(ptr) - 1)]


@dataclass
class Board:
    nodes: np.ndarray            # (N, 2) m
    tris: np.ndarray             # (nt, 3)
    z: np.ndarray                # (nt,) m
    layer: np.ndarray            # (nt,)
    terminals: dict              # name -> triangle indices
    fans: list                   # [triangle indices] merged into one node each
    ports: list                  # [(name, terminal a, terminal b)]: a current source from a to b
    thickness: float = 35e-6
    sigma: float = 5.8e7
    er: float = 1.0
    description: str = ''
    via_seg: np.ndarray = None   # (nv, 5): x, y, r, z0, z1 (m) of each plated via segment (MQS.vseg), or None
    via_fans: np.ndarray = None  # (nv, 2): the fans (merged nodes) the segment joins
    plating: float = 25e-6       # via barrel plating (m)
    _node_of: np.ndarray = field(default=None, repr=False)

    @classmethod
    def load(cls, name_or_path):
        path = Path(name_or_path)
        if not path.suffix:
            path = GOLDEN / f'{name_or_path}.npz'
        with np.load(path) as d:
            names = [str(n) for n in d['term_names']]
            terms = dict(zip(names, _csr_groups(d['term_ptr'], d['term_tris'])))
            fans = _csr_groups(d['fan_ptr'], d['fan_tris'])
            ports = [(str(p), names[a], names[b]) for p, a, b in zip(d['port_names'], d['port_a'], d['port_b'])]
            vias = (d['via_seg'].copy(), d['via_fans'].copy()) if 'via_seg' in d.files else (None, None)
            return cls(d['nodes'].copy(), d['tris'].copy(), d['z'].copy(), d['layer'].copy(), terms, fans, ports,
                       float(d['thickness']), float(d['sigma']), float(d['er']), str(d['description']), *vias)

    @property
    def nt(self):
        return len(self.tris)

    @property
    def node_of(self):
        """Triangle -> node: terminals and via fans merged (union-find, roots renumbered by np.unique)."""
        if self._node_of is None:
            nt = self.nt
            parent = np.arange(nt)

            def find(a):
                while parent[a] != a:
                    parent[a] = parent[parent[a]]
                    a = parent[a]
                return a
            for ts in list(self.terminals.values()) + list(self.fans):
                if len(ts):
                    r0 = find(int(ts[0]))
                    for t in ts[1:]:
                        parent[find(int(t))] = r0
            roots = np.array([find(t) for t in range(nt)])
            _, self._node_of = np.unique(roots, return_inverse=True)
        return self._node_of

    @property
    def n_nodes(self):
        return int(self.node_of.max()) + 1

    def term_node(self, name):
        return int(self.node_of[self.terminals[name][0]])

    @property
    def nv(self):
        return 0 if self.via_seg is None else len(self.via_seg)

    def via_ends(self):
        """(nv, 2) nodes each via segment joins (the branches after the RWG edges, MQS.br)."""
        if not self.nv:
            return np.zeros((0, 2), np.int64)
        first = np.array([int(f[0]) for f in self.fans], np.int64)
        return self.node_of[first[np.asarray(self.via_fans)]]

    def node_groups(self, area):
        """CSR of nodes -> member triangles (start (nn+1) int64, members (nt) int32) and node areas."""
        node_of = self.node_of
        nn = self.n_nodes
        members = np.argsort(node_of, kind='stable').astype(np.int32)
        start = np.zeros(nn + 1, np.int64)
        np.cumsum(np.bincount(node_of, minlength=nn), out=start[1:])
        node_area = np.bincount(node_of, weights=area, minlength=nn)
        return start, members, node_area
