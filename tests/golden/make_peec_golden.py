"""Golden port impedances from the reference's own PEEC solve (pcbqs.peec.solve, dense LU) on the synthetic boards.

    PCBQS_REFERENCE_SRC=<checkout>/src python tests/golden/make_peec_golden.py [planes | viapair | board ...]

The reference's MQS model class needs shapely only for meshing and region handling, which these boards do not use
(their meshes are given). shapely is absent here, so a stand-in module that only provides its names is put in
sys.modules before pcbqs.mqs is imported; no stand-in function is ever called. The model object is then built
around the given mesh with the attributes MQS.__init__ would set (src/pcbqs/mqs.py:300-420): one node per triangle
with terminals and via fans merged, RWG edges as branches, then the board's plated via segments (the via pair; the
other boards' vias each join one sheet and have none), DC sheet resistance, homogeneous dielectric er, capacitance
on. Ports are 1 A current sources (MQS.source). The
reference's own methods then assemble and solve: MQS._assemble/_loops/_sheet_resistance/_set_potential,
static_moments/edge_inductance (compiled core) and peec.solve.

Writes tests/golden/peec_<board>.npz: freqs, port names, Z (nf, np, np) from the node potentials of each drive
(Z[f, i, j] = voltage of port i for 1 A in port j), and the reference's own diagonal Result.z.
"""
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))


def stub_shapely():
    """Names-only stand-ins so that pcbqs.mqs imports without shapely; calling any of them raises."""
    def unavailable(*args, **kwargs):
        raise RuntimeError('shapely is not available in this environment')

    class Unavailable:
        def __init__(self, *args, **kwargs):
            unavailable()
    root = types.ModuleType('shapely')
    for sub in ('geometry', 'ops', 'affinity', 'prepared', 'validation', 'strtree'):
        m = types.ModuleType(f'shapely.{sub}')
        m.__getattr__ = lambda name, _u=Unavailable: _u
        sys.modules[f'shapely.{sub}'] = m
        setattr(root, sub, m)
    root.__getattr__ = lambda name: Unavailable
    sys.modules['shapely'] = root


def reference_model(board, conductor_loss='dc'):
    from oracle.reference import load_reference
    stub_shapely()
    load_reference()
    from pcbqs.mqs import MQS
    from pcbqs._numerics.base import RWG
    q = object.__new__(MQS)
    q.matrix_backend, q.capacitance, q.dielectric, q.er = 'dense', True, 'homogeneous', board.er
    q.near, q.outer_levels = 3.0, 1
    q._fill_options = dict(backend='openmp', workers=None, chunk=16384, device=None)
    q.fill_info, q.log, q.solve_info = {}, (lambda *a, **k: None), []
    q.thick_kernel, q._thick_D, q.side_charge = False, None, False
    q.nodes, q.tris = board.nodes, board.tris
    q.z_of, q.t_of = board.z, np.full(board.nt, board.thickness)
    q.layer_of = board.layer
    q.sigma, q.conductor_loss, q.conductor_faces, q.thickness_sheets = board.sigma, conductor_loss, 2, 1
    q.layer_tris = {int(l): np.flatnonzero(board.layer == l) for l in np.unique(board.layer)}
    q.sheet_layer = {k: k for k in q.layer_tris}
    q.rwg = RWG(q.nodes, q.tris)
    q.node_of, q.charge_of = board.node_of, None
    q.n_nodes = board.n_nodes
    q.terms = {name: [] for name in board.terminals}
    q.term_tris = {name: np.asarray(ts) for name, ts in board.terminals.items()}
    q.term_node = {name: board.term_node(name) for name in board.terminals}
    r = q.rwg
    q.br = [(int(q.node_of[a]), int(q.node_of[b])) for a, b in zip(r.tp, r.tm)]
    q.n_rwg = r.Ne
    q.vseg, q.ne, q.nv = [], r.Ne, 0
    # plated via segments (a board that has them): branches after the RWG edges, from the lower sheet's fan node to
    # the upper one's (MQS.__init__, src/pcbqs/mqs.py:404-416)
    for (x, y, rr, z0, z1), (a, b) in zip(board.via_seg if board.nv else [], board.via_ends()):
        q.br.append((int(a), int(b)))
        q.vseg.append((float(x), float(y), float(rr), float(z0), float(z1)))
    q.nv = len(q.vseg)
    q.parts, q.plating = [], 25e-6
    q._mats = q._copper = q._potential = q._peec = q._mqs_iter = None
    q.ideal_terminals, q.factor_cache_bytes = True, 64 * 1024 ** 2
    for name, a, b in board.ports:
        q.source(name, a, b, part_h=0.0)
    return q


def port_matrix(q, board, freqs):
    names = [p for p, _, _ in board.ports]
    drives = [{n: (1.0 if n == m else 0.0) for n in names} for m in names]
    results = q.solve(freqs, drives)
    nf, npo = len(freqs), len(names)
    Z = np.zeros((nf, npo, npo), complex)
    diag = np.zeros((nf, npo), complex)
    for j, res in enumerate(results):
        for i, (n, a, b) in enumerate(board.ports):
            Z[:, i, j] = res.potential[:, board.term_node(b)] - res.potential[:, board.term_node(a)]
        diag[:, j] = res.z[names[j]]
    return names, Z, diag


def main(boards=('tiny', 'strip'), losses=('dc', 'slab')):
    """peec_<board>.npz: DC sheet resistance; peec_<board>_slab.npz: conductor_loss='slab' (finite-thickness sheet
    impedance, current from both faces, one sheet per layer), where R depends on frequency."""
    from pcbqs_gb300.board import Board
    freqs = np.array([1e5, 1e6, 1e7])
    for name in boards:
      for loss in losses:
        b = Board.load(name)
        q = reference_model(b, loss)
        names, Z, diag = port_matrix(q, b, freqs)
        assert np.allclose(np.diagonal(Z, axis1=1, axis2=2), diag, rtol=1e-9), 'port voltage convention'
        m = q._peec
        suffix = '' if loss == 'dc' else '_' + loss
        np.savez_compressed(HERE / f'peec_{name}{suffix}.npz', freqs=freqs, ports=np.array(names), Z=Z, z_diag=diag,
                            unknowns=m['K'].shape[1], loops=m['nl'], components=m['B'].shape[1],
                            conductor_loss=loss)
        print(name, 'unknowns', m['K'].shape[1], 'loops', m['nl'], 'components', m['B'].shape[1])
        print(np.round(Z[1], 6))


def stack(name='tiny', slab=(0.0, 0.2e-3, 4.3, 0.02)):
    """peec_<board>_stack.npz: dielectric='stack' (electrostatic images of a lossy FR-4 slab between the two copper
    layers, air outside; complex P), DC sheet resistance."""
    from pcbqs_gb300.board import Board
    b = Board.load(name)
    q = reference_model(b)
    from pcbqs.electrostatic import DielectricStack
    z0, z1, er, tand = slab
    q.dielectric = 'stack'
    q._dielectric_stack = DielectricStack(np.array([z0, z1]), [1.0, er * (1 - 1j * tand), 1.0], tol=1e-8)
    freqs = np.array([1e5, 1e6, 1e7])
    names, Z, diag = port_matrix(q, b, freqs)
    m = q._peec
    np.savez_compressed(HERE / f'peec_{name}_stack.npz', freqs=freqs, ports=np.array(names), Z=Z, z_diag=diag,
                        unknowns=m['K'].shape[1], loops=m['nl'], components=m['B'].shape[1], slab=np.array(slab))
    print(name, 'stack', np.round(Z[1], 6))


def planes(freqs=(1e6,), board='planes'):
    """peec_planes.npz: the plane pair (22,554 triangles, 32,990 unknowns, 8 ports), DC sheet resistance, at the
    benchmark's 1 MHz (peec_planes16.npz: its 16-port variant at a frequency of the batched sweep). The reference's MQS._solve_charge factors each frequency once for all 8 drives. The system
    is factored by the reference's double-precision path of lu_factor_rows (PCBQS_LU=double: LAPACK zgetrf in the
    system's own memory, src/pcbqs/kernels.py:265-284) rather than MixedLU, whose complex64 copy and kept double
    matrix do not fit beside the model's dense R, L and potential projections in a 62 GB host; MixedLU refines to
    1e-12 of that same double solve (kernels.py:157-172). The edge matrices (MQS._mats and the copper cache
    MQS._copper, src/pcbqs/mqs.py:639-661) are dropped once peec.prepare has projected them: with DC resistance the
    solve reads only the projections."""
    import os
    import time
    os.environ['PCBQS_LU'] = 'double'
    from pcbqs_gb300.board import Board
    b = Board.load(board)
    q = reference_model(b)
    from pcbqs.peec import prepare
    t = time.perf_counter()
    m = prepare(q)
    print(f'prepare {time.perf_counter() - t:.1f} s, unknowns {m["K"].shape[1]}', flush=True)
    q._mats = q._copper = None
    freqs = np.asarray(freqs, float)
    t = time.perf_counter()
    names, Z, diag = port_matrix(q, b, freqs)
    print(f'solve {time.perf_counter() - t:.1f} s', flush=True)
    assert np.allclose(np.diagonal(Z, axis1=1, axis2=2), diag, rtol=1e-9), 'port voltage convention'
    np.savez_compressed(HERE / f'peec_{board}.npz', freqs=freqs, ports=np.array(names), Z=Z, z_diag=diag,
                        unknowns=m['K'].shape[1], loops=m['nl'], components=m['B'].shape[1],
                        conductor_loss='dc', lu='double')
    print(board, np.round(Z[0], 6))


def graph(boards=('tiny', 'strip', 'viapair'), freqs=(1e5, 1e6, 1e7), maxiter=3000):
    """graph_<board>.npz: the reference's iterative PEEC solve (peec_iterative.solve, src/pcbqs/peec_iterative.py:
    229-346) on its compressed model with its graph preconditioner (solver_preconditioner='graph': the exact inverse of the loop block of
    a diagonal branch impedance through the node Laplacian's incomplete LU, then the charge-tree solve,
    peec_iterative.py:44-84), every port driven alone at each frequency: SciPy GMRES (restart 100, relative
    tolerance 1e-8) iterations and true residual per (frequency, drive), and the port impedance matrix. The
    comparator of the library's block-Jacobi and learned preconditioners."""
    from pcbqs_gb300.board import Board
    freqs = np.asarray(freqs, float)
    for name in boards:
        b = Board.load(name)
        q = reference_model(b)
        from pcbqs.peec_iterative import solve
        # the reference's compressed model, the one its iterative solve runs on (MQS(matrix_backend=
        # 'hierarchical'), src/pcbqs/mqs.py:220-221: H-matrix L and potential at their default compression)
        q.matrix_backend = 'hierarchical'
        q._compression_options = dict(tol=1e-6, leaf=64, eta=1.0)
        q.solver_tol, q.solver_maxiter, q.solver_restart, q.solver_preconditioner = 1e-8, maxiter, 100, 'graph'
        names = [p for p, _, _ in b.ports]
        its = np.zeros((len(freqs), len(names)), int)
        res = np.zeros((len(freqs), len(names)))
        Z = np.zeros((len(freqs), len(names), len(names)), complex)
        kinds = set()
        for j, drive in enumerate(names):
            r = solve(q, freqs, {n: (1.0 if n == drive else 0.0) for n in names})
            for fi, info in enumerate(q.solve_info):
                its[fi, j], res[fi, j] = info['iterations'], info['relative_residual']
                kinds.add(info['preconditioner'])
            for i, (n, a, c) in enumerate(b.ports):
                Z[:, i, j] = r.potential[:, b.term_node(c)] - r.potential[:, b.term_node(a)]
        np.savez_compressed(HERE / f'graph_{name}.npz', freqs=freqs, ports=np.array(names), iterations=its,
                            residual=res, Z=Z, preconditioner=np.array(sorted(kinds)))
        print(name, sorted(kinds), its.tolist(), float(res.max()))


if __name__ == '__main__':
    if sys.argv[1:] == ['viapair']:
        main(('viapair',), ('dc', 'slab'))
    elif sys.argv[1:] == ['planes']:
        planes()
    elif sys.argv[1:] == ['graph']:
        graph()
    elif sys.argv[1:] == ['planes16']:
        # a frequency of the batched sweep (np.geomspace(1e3, 1e8, 64)): its 39th, 1.04 MHz
        sweep = np.geomspace(1e3, 1e8, 64)
        planes((sweep[38],), board='planes16')
    else:
        main(tuple(sys.argv[1:]) or ('tiny', 'strip'))
        stack('tiny')
