"""Golden H-matrix products from the reference itself: pcbqs.hmatrix.HMatrix built natively with the compiled
RwgEntries provider, exactly as compressed.edge_inductance builds the compressed inductance
(src/pcbqs/compressed.py:60-96), applied to seeded random complex vectors.

    PCBQS_REFERENCE_SRC=<checkout>/src python tests/golden/make_hmatrix_golden.py      (this container only: needs the reference checkout)

Writes tests/golden/hmatrix_<board>.npz: X (ne, 3) complex, Y_h = H X (the reference's compressed product),
Y_dense = L X with the reference's dense L (static_moments + edge_inductance), and the build info.
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle.reference import load_reference  # noqa: E402

load_reference()
from pcbqs._numerics.base import MU0, RWG  # noqa: E402
from pcbqs.hmatrix import HMatrix  # noqa: E402
from pcbqs.static import static_moments, edge_inductance  # noqa: E402
from pcbqs.static_backends import FillEngine  # noqa: E402


def make(name, tol=1e-6, leaf=64, eta=1.0):
    from pcbqs_gb300.board import Board
    b = Board.load(name)
    engine = FillEngine(b.nodes, b.tris, b.z, 3.0, 1, backend='openmp')
    g = engine.geometry
    r = RWG(g.nodes, g.tris)
    v = g.nodes[g.tris]
    lo_t, hi_t = np.c_[v.min(1), g.z], np.c_[v.max(1), g.z]
    support = np.stack((r.tp, r.tm), axis=1)
    vertices = np.ascontiguousarray(np.stack((r.vp, r.vm), axis=1), float)
    alpha = np.ascontiguousarray(np.stack((1 / (2 * r.area[r.tp]), -1 / (2 * r.area[r.tm])), axis=1), float)
    core = engine.backend.core
    common = (engine.backend.data, g.z, g.cent, g.radius, 3.0, 1)
    provider = core.RwgEntries(*common, np.ascontiguousarray(support, np.int64), vertices, alpha, MU0 / (4 * np.pi))

    def entry(rows, cols):
        return core.rwg_inductance(*common, np.ascontiguousarray(support, np.int64), vertices, alpha,
                                   np.asarray(rows, np.int64), np.asarray(cols, np.int64), MU0 / (4 * np.pi), 8)
    H = HMatrix(entry, lo_t[support].min(1), hi_t[support].max(1), tol=tol, leaf=leaf, eta=eta, native=provider)
    rng = np.random.default_rng(3)
    X = rng.standard_normal((r.Ne, 3)) + 1j * rng.standard_normal((r.Ne, 3))
    Yh = H @ X
    nodes, m0, mx, my, rr = static_moments(b.nodes, b.tris, b.z, backend='openmp')
    L, _ = edge_inductance(RWG(nodes, b.tris), rr, mx, my, m0, MU0 / (4 * np.pi), 1 / r.l, workers=8)
    Yd = L @ X
    info = H.info
    np.savez_compressed(HERE / f'hmatrix_{name}.npz', X=X, Y_h=Yh, Y_dense=Yd, tol=tol, leaf=leaf, eta=eta,
                        blocks=info['blocks'], low_rank_blocks=info['low_rank_blocks'], bytes=info['bytes'])
    print(name, info, 'rel err H vs dense', np.abs(Yh - Yd).max() / np.abs(Yd).max())


if __name__ == '__main__':
    for name in sys.argv[1:] or ('strip',):
        make(name)
