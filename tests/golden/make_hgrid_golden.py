"""Golden FFT near fields from the reference itself: pcbqs.biot.h_grid (src/pcbqs/biot.py:108-181) with its
current_deposit, for seeded random branch currents on the tiny two-layer board (this container only: needs the
reference checkout).

    PCBQS_REFERENCE_SRC=<checkout>/src python tests/golden/make_hgrid_golden.py

Writes tests/golden/hgrid_tiny.npz: the branch currents i (2, ne) (two excitations), the grids x, y, the heights, the
refinement and the field (nx, ny, nh, 3, 2).
"""
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle.reference import load_reference  # noqa: E402


def make(name='tiny', refine=2, seed=9):
    load_reference()
    from pcbqs._numerics.base import RWG
    from pcbqs.biot import h_grid
    from pcbqs_gb300.board import Board
    b = Board.load(name)
    r = RWG(b.nodes, b.tris)
    rng = np.random.default_rng(seed)
    i = rng.standard_normal((2, r.Ne)) + 1j * rng.standard_normal((2, r.Ne))
    layer_tris = {int(k): np.flatnonzero(b.layer == k) for k in np.unique(b.layer)}
    model = types.SimpleNamespace(nodes=b.nodes, z_of=b.z, layer_tris=layer_tris, rwg=r, ne=r.Ne, nv=0, vseg=[],
                                  parts=[])
    res = types.SimpleNamespace(i=i)
    lo, hi = b.nodes.min(0), b.nodes.max(0)
    x = np.linspace(lo[0] + 0.1e-3, hi[0] - 0.1e-3, 24)
    y = np.linspace(lo[1] + 0.1e-3, hi[1] - 0.1e-3, 18)
    heights = np.array([b.z.max() + 0.3e-3, b.z.max() + 1.0e-3, b.z.min() - 0.5e-3])
    H = h_grid(model, res, [0, 1], x, y, heights, refine=refine)
    np.savez_compressed(HERE / f'hgrid_{name}.npz', i=i, x=x, y=y, heights=heights, refine=refine, H=H)
    print(name, H.shape, np.abs(H).max())


if __name__ == '__main__':
    make()
