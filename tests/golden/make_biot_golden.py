"""Golden Biot-Savart fields from the reference itself (pcbqs.biot.h_sheets / h_segments, pcbqs._numerics.currents
.rwg_currents) on the synthetic boards with seeded random RWG currents.

    PCBQS_REFERENCE_SRC=<checkout>/src python tests/golden/make_biot_golden.py      (this container only: needs the reference checkout)

Writes tests/golden/biot_<board>.npz: the RWG coefficients I (ne, k), observation points (grids at 0.5 and 2 mm
above the top sheet and points 50 um above the copper, inside the near-refinement zone), each sheet's field from
h_sheets with k excitations, and a set of seeded filaments with their h_segments field.
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle.reference import load_reference  # noqa: E402

load_reference()
from pcbqs._numerics.base import RWG  # noqa: E402
from pcbqs._numerics.currents import rwg_currents  # noqa: E402
from pcbqs.biot import h_sheets, h_segments  # noqa: E402


def make(name, k=3, seed=5):
    from pcbqs_gb300.board import Board
    b = Board.load(name)
    rng = np.random.default_rng(seed)
    r = RWG(b.nodes, b.tris)
    I = rng.standard_normal((r.Ne, k)) + 1j * rng.standard_normal((r.Ne, k))
    a, bb = rwg_currents(r, I)
    lo, hi = b.nodes.min(0), b.nodes.max(0)
    ztop = b.z.max()
    gx, gy = np.linspace(lo[0], hi[0], 7), np.linspace(lo[1], hi[1], 5)
    X, Y = np.meshgrid(gx, gy, indexing='ij')
    pts = [np.c_[X.ravel(), Y.ravel(), np.full(X.size, ztop + h)] for h in (0.5e-3, 2e-3)]
    cen = b.nodes[b.tris].mean(1)
    pick = rng.choice(len(cen), 12, replace=False)
    pts.append(np.c_[cen[pick], b.z[pick] + 50e-6])
    pts = np.vstack(pts)
    sheets = []
    for layer in np.unique(b.layer):
        idx = np.flatnonzero(b.layer == layer)
        sheets.append((b.nodes, b.tris[idx], a[idx], bb[idx], float(b.z[idx[0]])))
    H = h_sheets(sheets, pts)
    H1 = h_sheets(sheets, pts[:, :], near=1.5, levels=2)
    assert np.array_equal(H, H1)
    nseg = 5
    p0 = np.c_[rng.uniform(lo[0], hi[0], nseg), rng.uniform(lo[1], hi[1], nseg), np.zeros(nseg)]
    p1 = p0 + np.c_[rng.uniform(-1e-3, 1e-3, (nseg, 2)), np.full(nseg, 1e-3)]
    Iseg = rng.standard_normal((nseg, k)) + 1j * rng.standard_normal((nseg, k))
    Hs = h_segments(p0, p1, Iseg, pts)
    np.savez_compressed(HERE / f'biot_{name}.npz', I=I, pts=pts, H=H, p0=p0, p1=p1, Iseg=Iseg, Hseg=Hs)
    print(name, 'points', len(pts), 'max |H|', np.abs(H).max())


if __name__ == '__main__':
    for name in sys.argv[1:] or ('tiny', 'strip'):
        make(name)
