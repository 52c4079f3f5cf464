"""Generate the seeded synthetic boards used by the tests and the benchmark, meshed with pcbqs's own mesher core.

    PCBQS_REFERENCE_SRC=<checkout>/src python tests/golden/make_meshes.py            (needs the reference checkout and oracle/_ref, this container)

Each board is written as tests/golden/<name>.npz with: nodes (N, 2) m, tris (nt, 3), z (nt) m, layer (nt),
terminal triangles (term_names, term_ptr, term_tris: CSR), via fans (fan_ptr, fan_tris: CSR, each merged into one
node), ports (port_a, port_b: terminal indices; a current source from a to b), and the board description.

The triangulation is the reference's constrained Delaunay core (`pcbqs._core.cdt_triangulate`, the kernel of its
mesher, src/pcbqs/core/cdt_mesh.hpp:18-64) run with a minimum-angle refinement; the points are outline, pad and via
outlines plus a seeded jittered hexagonal lattice, in the manner of src/pcbqs/_numerics/cdtmesh.py (hex seeding).
The boards themselves are synthetic stand-ins with the shapes and sizes of the benchmark configurations:
  strip  20 x 5 mm trace, h 0.31 mm, three terminals (both ends, middle), two ports         (~2,200 triangles)
  planes two 50 x 50 mm planes 0.2 mm apart, 40 vias (r 0.15 mm, seed-uniform), 8 ports   (~20,000 triangles)
  tiny   a 4 x 2 mm two-layer board for fast parity tests                                   (~300 triangles)
  viapair a 10 x 2 mm strip over its return strip 0.2 mm below, joined at the far end by two plated vias
          (via segments: via_seg (x, y, r, z0, z1) m and via_fans, the fan of each end), one port at the near
          end between the strips                                                              (~800 triangles)

    PCBQS_REFERENCE_SRC=<checkout>/src python tests/golden/make_meshes.py viapair    (that board alone; the others keep their meshes)
    PCBQS_REFERENCE_SRC=<checkout>/src python tests/golden/make_meshes.py planes16   (the plane pair with 16 ports, the batched
                                                   sweep's board)
    PCBQS_REFERENCE_SRC=<checkout>/src python tests/golden/make_meshes.py c5         (config C5's shape: four 100 x 80 mm pours with
                                                   voids, 200 plated vias, 16 ports, about 200,000 triangles)
    PCBQS_REFERENCE_SRC=<checkout>/src python tests/golden/make_meshes.py train      (train_0 .. train_5: seeded random small boards, alternately a
                                                   plane pair and a via-joined strip pair of random sizes, vias and
                                                   mesh sizes; the learned preconditioner's training systems)
"""
import sys
from pathlib import Path

import numpy as np
from scipy.spatial import cKDTree

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))


def reference_core():
    from oracle.reference import load_reference
    return load_reference()._core


def polygon(points):
    """Segments closing a point loop."""
    n = len(points)
    return [(i, (i + 1) % n) for i in range(n)]


def subdivide(a, b, h):
    n = max(1, int(np.ceil(np.linalg.norm(np.subtract(b, a)) / h)))
    t = np.arange(n) / n
    return np.asarray(a)[None] * (1 - t[:, None]) + np.asarray(b)[None] * t[:, None]


def rect_loop(x0, y0, x1, y1, h):
    corners = [(x0, y0), (x1, y0), (x1, y1), (x0, y1)]
    return np.vstack([subdivide(corners[i], corners[(i + 1) % 4], h) for i in range(4)])


def ngon(cx, cy, r, sides, phase=0.0):
    a = phase + 2 * np.pi * np.arange(sides) / sides
    return np.c_[cx + r * np.cos(a), cy + r * np.sin(a)]


def hex_lattice(x0, y0, x1, y1, h, rng, jitter=0.18):
    dy = h * np.sqrt(3) / 2
    pts = []
    for i, y in enumerate(np.arange(y0 + dy / 2, y1, dy)):
        xs = np.arange(x0 + h / 2 + (i % 2) * h / 2, x1, h)
        pts.append(np.c_[xs, np.full(len(xs), y)])
    pts = np.vstack(pts)
    return pts + rng.uniform(-jitter * h, jitter * h, pts.shape)


def mesh_sheet(core, outline, loops, holes, points, h, min_angle=20.0, lines=()):
    """Triangulate one sheet: outline loop, inner constraint loops (pads, via rings), holes (antipads; their
    triangles removed), extra fixed points (via centres), open constraint polylines whose end points lie on the
    outline (`lines`, interior points only), and lattice points kept clear of the constraints."""
    V, E = [], []

    def add_loop(loop):
        base = sum(len(v) for v in V)
        V.append(np.asarray(loop, float))
        E.extend((base + a, base + b) for a, b in polygon(loop))
    add_loop(outline)
    out = np.asarray(outline, float)
    for a, b in lines:
        ia = int(np.argmin(np.linalg.norm(out - a, axis=1)))
        ib = int(np.argmin(np.linalg.norm(out - b, axis=1)))
        inner = subdivide(a, b, h)[1:]
        base = sum(len(v) for v in V)
        V.append(inner)
        chain = [ia] + list(range(base, base + len(inner))) + [ib]
        E.extend(zip(chain[:-1], chain[1:]))
    for loop in loops:
        add_loop(loop)
    for loop in holes:
        add_loop(loop)
    fixed = np.vstack(V + ([np.asarray(points, float)] if len(points) else []))
    tree = cKDTree(fixed)
    lattice = hex_lattice(outline[:, 0].min(), outline[:, 1].min(), outline[:, 0].max(), outline[:, 1].max(), h,
                          RNG)
    x0, y0, x1, y1 = outline[:, 0].min(), outline[:, 1].min(), outline[:, 0].max(), outline[:, 1].max()
    inside = (lattice[:, 0] > x0 + 0.35 * h) & (lattice[:, 0] < x1 - 0.35 * h) & \
             (lattice[:, 1] > y0 + 0.35 * h) & (lattice[:, 1] < y1 - 0.35 * h)
    lattice = lattice[inside]
    lattice = lattice[tree.query(lattice)[0] > 0.5 * h]
    for loop in holes:
        c = loop.mean(0)
        r = np.linalg.norm(loop - c, axis=1).max()
        lattice = lattice[np.linalg.norm(lattice - c, axis=1) > r + 0.4 * h]
    allpts = np.vstack([fixed, lattice])
    vert, tri = core.cdt_triangulate(np.ascontiguousarray(allpts), np.ascontiguousarray(E, dtype=np.int32), 0.0,
                                     min_angle, 0)
    vert, tri = np.asarray(vert), np.asarray(tri)
    cen = vert[tri].mean(1)
    keep = np.ones(len(tri), bool)
    for loop in holes:
        c = loop.mean(0)
        r = np.linalg.norm(loop - c, axis=1).min()
        keep &= np.linalg.norm(cen - c, axis=1) > r * 0.999
    tri = tri[keep]
    used = np.unique(tri)
    remap = np.full(len(vert), -1)
    remap[used] = np.arange(len(used))
    vert, tri = vert[used], remap[tri]
    e1, e2 = vert[tri[:, 1]] - vert[tri[:, 0]], vert[tri[:, 2]] - vert[tri[:, 0]]
    assert (e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0] > 0).all(), 'triangles must be counter-clockwise'
    return vert, tri


def inside_box(cen, box):
    x0, y0, x1, y1 = box
    return np.flatnonzero((cen[:, 0] > x0) & (cen[:, 0] < x1) & (cen[:, 1] > y0) & (cen[:, 1] < y1))


def assemble(sheets, terminals, fans, ports, meta, vias=()):
    """Stack sheets (mm) into one mesh (m); terminals: name -> [(sheet, box mm)]; fans: [(sheet, centre mm)]."""
    nodes, tris, z, layer = [], [], [], []
    off = 0
    first = []
    for k, (vert, tri, zz) in enumerate(sheets):
        first.append(sum(len(t) for t in tris))
        nodes.append(vert * 1e-3)
        tris.append(tri + off)
        off += len(vert)
        z += [zz * 1e-3] * len(tri)
        layer += [k] * len(tri)
    nodes, tris = np.vstack(nodes), np.vstack(tris)
    cen_mm = nodes[tris].mean(1) * 1e3
    layer = np.array(layer)
    names, term = list(terminals), []
    for name in names:
        ids = np.concatenate([np.intersect1d(inside_box(cen_mm, box), np.flatnonzero(layer == s))
                              for s, box in terminals[name]])
        assert len(ids), f'terminal {name} has no triangles'
        term.append(np.sort(ids))
    fan = []
    for s, (cx, cy) in fans:
        sel = np.flatnonzero(layer == s)
        centre = np.argmin(np.linalg.norm(nodes * 1e3 - [cx, cy], axis=1) + np.where(
            np.isin(np.arange(len(nodes)), np.unique(tris[sel])), 0, 1e9))
        ids = sel[np.isin(tris[sel], centre).any(1)]
        assert len(ids) >= 3, 'via fan not found'
        fan.append(np.sort(ids))
    ptr = lambda groups: np.r_[0, np.cumsum([len(g) for g in groups])].astype(np.int64)
    cat = lambda groups: (np.concatenate(groups) if groups else np.zeros(0, int)).astype(np.int64)
    extra = {}
    if len(vias):     # (x, y, r mm, sheet a, sheet b, fan a, fan b): a plated barrel between two sheets' fans
        extra = dict(via_seg=np.array([(x * 1e-3, y * 1e-3, r * 1e-3, sheets[a][2] * 1e-3, sheets[b][2] * 1e-3)
                                       for x, y, r, a, b, _, _ in vias]),
                     via_fans=np.array([(fa, fb) for *_, fa, fb in vias], np.int64))
    return dict(**extra, nodes=nodes, tris=tris.astype(np.int64), z=np.array(z), layer=layer,
                term_names=np.array(names), term_ptr=ptr(term), term_tris=cat(term),
                fan_ptr=ptr(fan), fan_tris=cat(fan),
                port_a=np.array([names.index(a) for _, a, _ in ports]),
                port_b=np.array([names.index(b) for _, _, b in ports]),
                port_names=np.array([p for p, _, _ in ports]), **meta)


def strip(core):
    """20 x 5 mm trace, 35 um copper: terminals at both ends and in the middle, two ports."""
    h = 0.33
    cuts = [0.5, 9.75, 10.25, 19.5]
    # The outline carries a vertex at each terminal cut, and the cuts are constraint lines across the strip
    # (pads' outlines as mesh edges).
    xs = np.unique(np.r_[np.linspace(0, 20, int(np.ceil(20 / h)) + 1), cuts])
    ys = np.linspace(0, 5, int(np.ceil(5 / h)) + 1)
    outline = np.vstack([np.c_[xs[:-1], np.zeros(len(xs) - 1)], np.c_[np.full(len(ys) - 1, 20.0), ys[:-1]],
                         np.c_[xs[::-1][:-1], np.full(len(xs) - 1, 5.0)], np.c_[np.zeros(len(ys) - 1), ys[::-1][:-1]]])
    vert, tri = mesh_sheet(core, outline, [], [], [], h, lines=[((x, 0.0), (x, 5.0)) for x in cuts])
    terminals = {'left': [(0, (0, 0, cuts[0]))], 'mid': [(0, (cuts[1], 0, cuts[2]))],
                 'right': [(0, (cuts[3], 0, 20))]}
    terminals = {k: [(s, (b[0], 0.0, b[2], 5.0)) for s, b in v] for k, v in terminals.items()}
    ports = [('p1', 'left', 'mid'), ('p2', 'mid', 'right')]
    return assemble([(vert, tri, 0.0)], terminals, [], ports,
                    dict(thickness=0.035e-3, sigma=5.8e7, er=1.0, description='20 x 5 mm strip, h 0.31 mm'))


def planes(core, size=50.0, gap=0.2, n_vias=40, n_ports=8, h=0.75, seed=7, margin=2.0, spacing=2.0):
    """Two square planes `gap` mm apart (ground at z=0, power at z=gap); vias alternate power/ground, each a
    hexagonal ring (fan: one node) in its own plane and an antipad in the other; ports join a 0.6 mm pad on the
    power plane to one on the ground plane at the same place."""
    rng = np.random.default_rng(seed)
    sites = []
    for _ in range(100000):
        if len(sites) == n_vias + n_ports:
            break
        x, y = rng.uniform(margin, size - margin, 2)
        if all(np.hypot(x - a, y - b) > spacing for a, b in sites):
            sites.append((x, y))
    if len(sites) < n_vias + n_ports:
        raise ValueError('board too small for its vias and ports')
    vias, port_sites = sites[:n_vias], sites[n_vias:]
    r_via, r_anti, pad = 0.15, 0.35, 0.3
    sheets = []
    fans = []
    for s, zz in ((0, 0.0), (1, gap)):          # 0: ground, 1: power
        loops, holes, points = [], [], []
        for k, (x, y) in enumerate(vias):
            own = (k % 2 == 0) == (s == 1)      # even vias are power vias
            if own:
                loops.append(ngon(x, y, r_via, 6))
                points.append((x, y))
                fans.append((s, (x, y)))
            else:
                holes.append(ngon(x, y, r_anti, 8, np.pi / 8))
        for (x, y) in port_sites:
            loops.append(rect_loop(x - pad, y - pad, x + pad, y + pad, 0.3))
        vert, tri = mesh_sheet(core, rect_loop(0, 0, size, size, h), loops, holes, points, h)
        sheets.append((vert, tri, zz))
    terminals, ports = {}, []
    for i, (x, y) in enumerate(port_sites):
        box = (x - pad, y - pad, x + pad, y + pad)
        terminals[f'pwr{i}'] = [(1, box)]
        terminals[f'gnd{i}'] = [(0, box)]
        ports.append((f'port{i}', f'pwr{i}', f'gnd{i}'))
    return assemble(sheets, terminals, fans, ports,
                    dict(thickness=0.035e-3, sigma=5.8e7, er=4.3,
                         description=f'{size:g} x {size:g} mm plane pair, {gap} mm FR-4, {n_vias} vias, '
                                     f'{n_ports} ports, h {h} mm'))


def viapair(core, length=10.0, width=2.0, gap=0.2, h=0.3):
    """A strip (z = gap) over its return strip (z = 0), joined near the far end by two plated vias (r 0.15 mm,
    hexagonal rings, each a fan in both sheets); the port drives the near end from the top strip's pad to the bottom
    one's, so the current loop closes through the vias (magnetic and capacitive solves alike)."""
    r_via = 0.15
    sites = [(length - 1.0, 0.6), (length - 1.0, width - 0.6)]
    sheets, fans, vias = [], [], []
    for s, zz in ((0, 0.0), (1, gap)):
        loops = [ngon(x, y, r_via, 6) for x, y in sites]
        vert, tri = mesh_sheet(core, rect_loop(0, 0, length, width, h), loops, [], sites, h,
                               lines=[((0.6, 0.0), (0.6, width))])
        sheets.append((vert, tri, zz))
        for x, y in sites:
            fans.append((s, (x, y)))
    for k, (x, y) in enumerate(sites):
        vias.append((x, y, r_via, 0, 1, k, len(sites) + k))
    terminals = {'top': [(1, (0.0, 0.0, 0.6, width))], 'bottom': [(0, (0.0, 0.0, 0.6, width))]}
    return assemble(sheets, terminals, fans, [('loop', 'top', 'bottom')],
                    dict(thickness=0.035e-3, sigma=5.8e7, er=4.3,
                         description=f'{length:g} x {width:g} mm strip pair {gap} mm apart, 2 vias, h {h} mm'),
                    vias)


def c5(core, size=(100.0, 80.0), z=(0.0, 0.2, 1.4, 1.6), n_vias=200, n_ports=16, h=0.6, seed=11, voids=3):
    """Four copper pours of size[0] x size[1] mm at heights z mm, each with `voids` seeded circular cutouts (12-gons,
    r 2-5 mm); `n_vias` plated vias (r 0.15 mm) at seeded sites, each joining a pair of layers (1-2, 3-4, 2-3, 1-4 in
    turn: a hexagonal ring and its fan in both, an antipad in the layers between), and `n_ports` ports from a 0.6 mm
    pad on layer 2 to one on layer 1 at the same place. About 200,000 triangles at h = 0.6 mm."""
    rng = np.random.default_rng(seed)
    W, H = size
    r_via, r_anti, pad = 0.15, 0.35, 0.3
    holes_of = []
    for s in range(len(z)):
        holes_of.append([(float(rng.uniform(8, W - 8)), float(rng.uniform(8, H - 8)), float(rng.uniform(2, 5)))
                         for _ in range(voids)])
    clear = lambda x, y, m: all(np.hypot(x - a, y - b) > r + m for hs in holes_of for a, b, r in hs)
    sites = []
    for _ in range(200000):
        if len(sites) == n_vias + n_ports:
            break
        x, y = float(rng.uniform(2, W - 2)), float(rng.uniform(2, H - 2))
        if clear(x, y, 1.0) and all(np.hypot(x - a, y - b) > 1.6 for a, b in sites):
            sites.append((x, y))
    if len(sites) < n_vias + n_ports:
        raise ValueError('board too small for its vias and ports')
    vias, port_sites = sites[:n_vias], sites[n_vias:]
    joins = [(0, 1), (2, 3), (1, 2), (0, 3)]
    sheets, fans, barrels = [], [], []
    fan_index = {}
    for s, zz in enumerate(z):
        loops, holes, points = [], [], []
        for k, (x, y) in enumerate(vias):
            a, b = joins[k % len(joins)]
            if s in (a, b):
                loops.append(ngon(x, y, r_via, 6))
                points.append((x, y))
                fan_index[(k, s)] = len(fans)
                fans.append((s, (x, y)))
            elif a < s < b:
                holes.append(ngon(x, y, r_anti, 8, np.pi / 8))
        for x, y, r in holes_of[s]:
            holes.append(ngon(x, y, r, 12))
        if s in (0, 1):
            for (x, y) in port_sites:
                loops.append(rect_loop(x - pad, y - pad, x + pad, y + pad, 0.3))
        vert, tri = mesh_sheet(core, rect_loop(0, 0, W, H, h), loops, holes, points, h)
        sheets.append((vert, tri, zz))
        print(f'c5 layer {s}: {len(tri)} triangles', flush=True)
    for k, (x, y) in enumerate(vias):
        a, b = joins[k % len(joins)]
        barrels.append((x, y, r_via, a, b, fan_index[(k, a)], fan_index[(k, b)]))
    terminals, ports = {}, []
    for i, (x, y) in enumerate(port_sites):
        box = (x - pad, y - pad, x + pad, y + pad)
        terminals[f'pwr{i}'] = [(1, box)]
        terminals[f'gnd{i}'] = [(0, box)]
        ports.append((f'port{i}', f'pwr{i}', f'gnd{i}'))
    return assemble(sheets, terminals, fans, ports,
                    dict(thickness=0.035e-3, sigma=5.8e7, er=4.3,
                         description=f'{W:g} x {H:g} mm four-layer board, {voids} voids per pour, {n_vias} vias, '
                                     f'{n_ports} ports, h {h} mm'),
                    barrels)


def training_board(core, seed):
    """A seeded random small board: a plane pair (even seeds) or a via-joined strip pair (odd seeds)."""
    rng = np.random.default_rng(1000 + seed)
    if seed % 2 == 0:
        size = float(rng.uniform(3.5, 6.0))
        gap, n_vias, h = float(rng.uniform(0.15, 0.4)), int(rng.integers(2, 5)), float(rng.uniform(0.38, 0.5))
        for _ in range(20):              # a site draw that fits the vias and ports
            try:
                return planes(core, size=size, gap=gap, n_vias=n_vias, n_ports=2, h=h, seed=int(rng.integers(1 << 30)),
                              margin=0.8, spacing=1.1)
            except ValueError:
                continue
        raise ValueError('no site draw fits')
    return viapair(core, length=float(rng.uniform(6.0, 12.0)), width=float(rng.uniform(1.6, 2.8)),
                   gap=float(rng.uniform(0.15, 0.4)), h=float(rng.uniform(0.3, 0.42)))


RNG = np.random.default_rng(20261203)


def main():
    global RNG
    core = reference_core()
    RNG = np.random.default_rng(1)
    boards = {'strip': strip(core)}
    RNG = np.random.default_rng(2)
    boards['tiny'] = planes(core, size=4.0, gap=0.2, n_vias=2, n_ports=2, h=0.4, seed=3, margin=0.8, spacing=1.2)
    RNG = np.random.default_rng(3)
    boards['planes'] = planes(core)
    for name, data in boards.items():
        np.savez_compressed(HERE / f'{name}.npz', **data)
        print(name, len(data['tris']), 'triangles', len(data['nodes']), 'nodes')


if __name__ == '__main__':
    if sys.argv[1:] == ['viapair']:
        RNG = np.random.default_rng(4)
        data = viapair(reference_core())
        np.savez_compressed(HERE / 'viapair.npz', **data)
        print('viapair', len(data['tris']), 'triangles', len(data['nodes']), 'nodes', len(data['via_seg']), 'vias')
    elif sys.argv[1:] == ['planes16']:
        # the batched sweep's board: the plane pair with 16 ports (the same seed, so the first 40 sites are the same
        # vias and the first 8 ports the same pads)
        RNG = np.random.default_rng(3)
        data = planes(reference_core(), n_ports=16)
        np.savez_compressed(HERE / 'planes16.npz', **data)
        print('planes16', len(data['tris']), 'triangles', len(data['nodes']), 'nodes')
    elif sys.argv[1:] == ['c5']:
        # the large compressed board (config C5's shape: four layers, 100 x 80 mm, pours, 200 vias)
        RNG = np.random.default_rng(5)
        data = c5(reference_core())
        np.savez_compressed(HERE / 'c5.npz', **data)
        print('c5', len(data['tris']), 'triangles', len(data['nodes']), 'nodes', len(data['via_seg']), 'vias')
    elif sys.argv[1:] == ['train']:
        core = reference_core()
        for i in range(6):
            RNG = np.random.default_rng(100 + i)
            data = training_board(core, i)
            np.savez_compressed(HERE / f'train_{i}.npz', **data)
            print(f'train_{i}', len(data['tris']), 'triangles', data['description'])
    else:
        main()
