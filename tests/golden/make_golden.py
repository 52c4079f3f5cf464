"""Golden vectors from the reference pcbqs itself (its NumPy path and its compiled core), for the oracle and the
device parity tests.

    PCBQS_REFERENCE_SRC=<checkout>/src python tests/golden/make_golden.py     (this container only: needs the reference checkout; builds oracle/_ref)

Writes tests/golden/golden_tiny8.npz and golden_<board>.npz for the boards of make_meshes.py:
  tiny8     the reference test suite's 8-triangle two-layer fixture (tests/test_static_backends.py:14-24):
            full moment matrices from static_moments(backend='numpy') and (backend='openmp') for outer levels
            0/1/2, full and scalar; the all-analytic path (near=inf); FillEngine.kinds for near 0/.5/3/inf;
            the explicit pair protocol on the reference test's pair list; L from static.edge_inductance.
  boards    geometry (centroids, radii), the analytic-pair count, per-plane checksums and sampled rows of the
            moments (static_fill), of L (static_combine via static.edge_inductance, factor mu0/4pi, scale 1/l),
            and of P (MQS._set_potential's W^T M0 W / (4 pi eps0 er) with the board's terminal and via-fan
            merges), with the RWG edge order (T+, T-).
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle.reference import load_reference  # noqa: E402

pcbqs = load_reference()
from pcbqs._numerics.base import MU0, EPS0, RWG, qform  # noqa: E402
from pcbqs.static import static_moments, edge_inductance  # noqa: E402
from pcbqs.static_backends import FillEngine  # noqa: E402
from scipy.sparse import coo_matrix  # noqa: E402

PAIR_P = np.array([0, 7, 1, 2, 3, 4, 0])
PAIR_Q = np.array([0, 2, 0, 5, 7, 2, 6])


def tiny8():
    nodes, tris, z = [], [], []
    for h in (0., .00013):
        for x in (0., .025):
            k = len(nodes)
            nodes.extend([[x, 0.], [x + .002, 0.], [x + .002, .001], [x, .001]])
            tris.extend([[k, k + 1, k + 2], [k, k + 2, k + 3]])
            z.extend([h, h])
    return np.array(nodes), np.array(tris), np.array(z)


def make_tiny8():
    mesh = tiny8()
    out = dict(nodes=mesh[0], tris=mesh[1], z=mesh[2], pair_p=PAIR_P, pair_q=PAIR_Q)
    for level in (0, 1, 2):
        for scalar in (False, True):
            tag = f'l{level}_{"s" if scalar else "f"}'
            for backend in ('numpy', 'openmp'):
                res, info = static_moments(*mesh, backend=backend, workers=2, outer_levels=level,
                                           scalar_only=scalar, return_info=True)
                for name, m in zip(('m0', 'mx', 'my', 'mrr'), res[1:]):
                    out[f'{backend}_{tag}_{name}'] = m
                out[f'{backend}_{tag}_analytic'] = info['analytic_pairs']
            e = FillEngine(*mesh, backend='numpy', outer_levels=level)
            d = e.geometry.z[PAIR_P] - e.geometry.z[PAIR_Q]
            out[f'pairs_{tag}'] = e.evaluate(PAIR_P, PAIR_Q, d, scalar_only=scalar)
            out[f'pairs_{tag}_kind'] = e.kinds(PAIR_P, PAIR_Q, d)
    res = static_moments(*mesh, backend='numpy', near=np.inf)
    for name, m in zip(('m0', 'mx', 'my', 'mrr'), res[1:]):
        out[f'allnear_{name}'] = m
    n = len(mesh[1])
    p, q = np.meshgrid(np.arange(n), np.arange(n), indexing='ij')
    p, q = p.ravel(), q.ravel()
    for near in (0., .5, 3., np.inf):
        for level in (0, 1, 2):
            e = FillEngine(*mesh, backend='numpy', near=near, outer_levels=level)
            out[f'kinds_{near}_{level}'] = e.kinds(p, q, e.geometry.z[p] - e.geometry.z[q])
    nodes, m0, mx, my, rr = static_moments(*mesh, backend='numpy')
    r = RWG(nodes, mesh[1])
    L, info = edge_inductance(r, rr, mx, my, m0, MU0 / (4 * np.pi), 1 / r.l, workers=2)
    out.update(L=L, L_backend=info['backend'], centred=nodes)
    np.savez_compressed(HERE / 'golden_tiny8.npz', **out)


def board_groups(b):
    """node_of from the board's terminal and via-fan merges (MQS's union-find numbering, mqs.py:365-403)."""
    nt = len(b['tris'])
    parent = np.arange(nt)

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a
    groups = [b['term_tris'][b['term_ptr'][i]:b['term_ptr'][i + 1]] for i in range(len(b['term_ptr']) - 1)]
    groups += [b['fan_tris'][b['fan_ptr'][i]:b['fan_ptr'][i + 1]] for i in range(len(b['fan_ptr']) - 1)]
    for ts in groups:
        if len(ts):
            r0 = find(ts[0])
            for t in ts[1:]:
                parent[find(t)] = r0
    _, node_of = np.unique([find(t) for t in range(nt)], return_inverse=True)
    return node_of


def checksums(m):
    return np.array([m.sum(), np.abs(m).sum(), np.sqrt((m * m).sum()), np.abs(m).max()])


def sample(m, rng, count=8192):
    i = rng.integers(0, m.shape[0], count)
    j = rng.integers(0, m.shape[1], count)
    return np.stack([i, j]), m[i, j]


def make_board(name, rows=8):
    b = dict(np.load(HERE / f'{name}.npz'))
    nodes, tris, z = b['nodes'], b['tris'], b['z']
    er = float(b['er'])
    res, info = static_moments(nodes, tris, z, near=3.0, outer_levels=1, backend='openmp', return_info=True)
    centred, m0, mx, my, rr = res
    nt = len(tris)
    pick = np.unique(np.r_[0, nt - 1, np.linspace(0, nt - 1, rows - 2).astype(int)])
    e = FillEngine(nodes, tris, z, backend='numpy')
    out = dict(analytic=info['analytic_pairs'], pairs=info['pairs'], rows=pick)
    if nt < 5000:         # the large board's geometry is checked through its checksums and samples only
        out.update(cent=e.geometry.cent, radius=e.geometry.radius, centred=centred)
    rng = np.random.default_rng(11)
    count = 8192 if nt < 5000 else 2048
    for key, m in zip(('m0', 'mx', 'my', 'mrr'), (m0, mx, my, rr)):
        out[f'{key}_rows'] = m[pick].copy()
        out[f'{key}_sum'] = checksums(m)
        out[f'{key}_at'], out[f'{key}_val'] = sample(m, rng, count)
    r = RWG(centred, tris)
    L, _ = edge_inductance(r, rr, mx, my, m0, MU0 / (4 * np.pi), 1 / r.l, workers=8)
    del rr, mx, my
    epick = np.unique(np.r_[0, r.Ne - 1, np.linspace(0, r.Ne - 1, rows - 2).astype(int)])
    out.update(L_rows=L[epick].copy(), L_sum=checksums(L), edge_rows=epick, tp=r.tp.astype(np.int32), tm=r.tm.astype(np.int32), ne=r.Ne,
               L_diag=np.diag(L).copy())
    out['L_at'], out['L_val'] = sample(L, rng, count)
    del L
    node_of = board_groups(b)
    nn = node_of.max() + 1
    area = np.bincount(node_of, weights=r.area, minlength=nn)
    W = coo_matrix((1 / area[node_of], (np.arange(nt), node_of)), shape=(nt, nn)).tocsr()
    P = qform(W, m0, W) / (4 * np.pi * EPS0 * er)
    P = np.asarray(P)
    npick = np.unique(np.r_[0, nn - 1, np.linspace(0, nn - 1, rows - 2).astype(int)])
    out.update(P_rows=P[npick].copy(), P_sum=checksums(P), node_rows=npick, node_of=node_of.astype(np.int32), P_diag=np.diag(P).copy())
    out['P_at'], out['P_val'] = sample(P, rng, count)
    np.savez_compressed(HERE / f'golden_{name}.npz', **out)
    print(name, 'triangles', nt, 'edges', r.Ne, 'nodes', nn, 'analytic', info['analytic_pairs'], 'of',
          info['pairs'], f'{info["seconds"]:.2f} s')


if __name__ == '__main__':
    make_tiny8()
    for name in sys.argv[1:] or ('tiny', 'strip', 'planes'):
        make_board(name, rows={'planes': 2, 'strip': 4}.get(name, 8))
