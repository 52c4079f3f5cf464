"""Golden layered-dielectric vectors from the reference itself (this container only: needs the reference checkout
and its compiled core in oracle/_ref).

    PCBQS_REFERENCE_SRC=<checkout>/src python tests/golden/make_layered_golden.py

Writes
  tests/golden/layered_spectral.npz  the reference's own spectral-network fixture for the image series
                                     (tests/fixtures/spectral-reference.npz, used by tests/test_electrostatic.py:13-20)
  tests/golden/layered_tiny.npz      the tiny two-layer board in a lossy FR-4 slab (0 .. 0.2 mm, er 4.3, tand 0.02,
                                     air outside): the image lists and spline arguments of every layer pair, sampled
                                     rows, the diagonal and checksums of M = potential_moments(model)
                                     (src/pcbqs/electrostatic.py:151-221, run through the compiled layered_pairs
                                     kernel) and of P = W^T M W / (4 pi eps0) as MQS._set_potential forms it.
"""
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle.reference import SOURCE, load_reference  # noqa: E402

REFERENCE = SOURCE.parent if SOURCE is not None else None      # the reference checkout
SLAB = dict(z0=0.0, z1=0.2e-3, er=4.3, tand=0.02)


def spectral():
    with np.load(REFERENCE / 'tests' / 'fixtures' / 'spectral-reference.npz') as d:
        np.savez_compressed(HERE / 'layered_spectral.npz', **{k: d[k] for k in d.files})


def board(name='tiny', rows=(0, 1, 77, 200, 311, 450), near=3.0, outer=1):
    load_reference()
    from pcbqs._numerics.base import EPS0
    from pcbqs.electrostatic import DielectricStack, potential_moments
    from pcbqs.static_backends import layered_spline_args
    from pcbqs_gb300.board import Board
    b = Board.load(name)
    eps = [1.0, SLAB['er'] * (1 - 1j * SLAB['tand']), 1.0]
    stack = DielectricStack(np.array([SLAB['z0'], SLAB['z1']]), eps, tol=1e-8)
    levels = np.unique(b.layer)
    layer_tris = {int(k): np.flatnonzero(b.layer == k) for k in levels}
    model = types.SimpleNamespace(nodes=b.nodes, tris=b.tris, z_of=b.z, near=near, outer_levels=outer,
                                  _fill_options=dict(backend='openmp', workers=8), layer_tris=layer_tris,
                                  _dielectric_stack=stack, fill_info={})
    M = potential_moments(model)
    e1, e2 = b.nodes[b.tris[:, 1]] - b.nodes[b.tris[:, 0]], b.nodes[b.tris[:, 2]] - b.nodes[b.tris[:, 0]]
    area = np.abs(e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]) / 2
    of = b.node_of
    nn = of.max() + 1
    W = np.zeros((len(b.tris), nn))
    W[np.arange(len(b.tris)), of] = 1 / np.bincount(of, weights=area, minlength=nn)[of]
    P = W.T @ M @ W / (4 * np.pi * EPS0)
    out = dict(rows=np.asarray(rows), M_rows=M[list(rows)], M_diag=np.diag(M).copy(),
               M_abs_sum=np.abs(M).sum(), M_sum=M.sum(), P_rows=P[list(rows)], P_diag=np.diag(P).copy(),
               P_abs_sum=np.abs(P).sum(), slab=np.array([SLAB['z0'], SLAB['z1'], SLAB['er'], SLAB['tand']]),
               near=near, outer=outer, image_terms=model.fill_info['capacitance']['image_terms'])
    # image series and spline arguments of every layer pair, in the order potential_moments visits them
    rho_max = np.linalg.norm(np.ptp(b.nodes - b.nodes.mean(0), axis=0))
    pairs = []
    for i, la in enumerate(levels):
        for lb in levels[i:]:
            o = stack.interface(b.z[layer_tris[int(la)][0]])
            s = stack.interface(b.z[layer_tris[int(lb)][0]])
            images = stack.images(s, o)
            pairs.append((o, s))
            d = np.array([x for x, _ in images])
            c = np.array([y for _, y in images])
            out[f'images_{o}_{s}_d'], out[f'images_{o}_{s}_c'] = d, c
            positive = [(x, y) for x, y in images if x > 0]
            smooth = None
            if len(positive) > 8:
                from scipy.interpolate import CubicSpline
                ngrid = max(257, int(np.ceil(32 * np.sqrt(rho_max / min(x for x, _ in positive)))))
                rho = rho_max * np.linspace(0, 1, ngrid) ** 2
                kernel = np.zeros(ngrid, complex)
                for x, y in positive:
                    kernel += y / np.hypot(rho, x)
                smooth = CubicSpline(rho, kernel)
            _, _, sx, sc = layered_spline_args(images, smooth)
            out[f'spline_{o}_{s}_x'], out[f'spline_{o}_{s}_c'] = sx, sc
    out['pairs'] = np.array(pairs)
    out['rho_max'] = rho_max
    np.savez_compressed(HERE / f'layered_{name}.npz', **out)
    print(name, 'image terms', out['image_terms'], 'pairs', pairs, '|M| sum', out['M_abs_sum'])


if __name__ == '__main__':
    spectral()
    board('tiny')
