"""The host packing of the tensor-core low-rank product (DeviceHMatrix.lowrank_plan), checked on the CPU by
emulating the two GEMM phases exactly as the kernel addresses its planes (k_tc_update modes 4 and 5: the part
segments (h, m) x (h, m, h), the 64-wide K slices, the padded cluster order, the group and tile tables, the slot
rows), against the direct sum of U V^T x over the blocks in both directions. No GPU: a stand-in object carries a
real ClusterTree and random low-rank blocks in the packed layout of DeviceHMatrix._pack, and the planes' packing
kernel's launch (k_pack_parts, after the host's bounds checks) is replaced by its restatement here (the GPU tests
hold the kernel to it bit for bit)."""
import numpy as np
import torch

from pcbqs_gb300.hmatrix import ClusterTree, DeviceHMatrix

SEG_A, SEG_B = (0, 0, 1), (0, 1, 0)


class _Stand:
    pass


def _fake(seed=3, n=700, leaf=50):
    rng = np.random.default_rng(seed)
    pts = rng.uniform(0, 1, (n, 3)) * [1, 1, 0.01]
    tree = ClusterTree(pts, pts, leaf)
    nodes = range(len(tree.start))
    pairs = [(i, j) for i in nodes for j in nodes if i < j and tree.separated(i, j, 1.0)][:12]
    leaves = [k for k in nodes if tree.leaf(k)]
    near = [(leaves[0], leaves[0]), (leaves[1], leaves[2]), (leaves[3], leaves[3]), (leaves[2], leaves[5])]
    meta, slot0, store, so, ioff = [], [], [], 0, 0
    blocks, dense = [], []
    for i, j in near:                                 # dense leaves (a diagonal one stored whole)
        la, lb = tree.size(i), tree.size(j)
        D = rng.standard_normal((la, lb))
        if i == j:
            D = D + D.T
        store.append(D.ravel())
        meta.append([ioff, la, ioff + la, lb, so, 0, int(i == j), -1])
        dense.append((tree.ids(i), tree.ids(j), D, i == j))
        so += la * lb
        ioff += la + lb
    for i, j in pairs:
        la, lb = tree.size(i), tree.size(j)
        cap = 8
        rk = int(rng.integers(1, cap + 1))
        U = rng.standard_normal((la, cap))
        V = rng.standard_normal((cap, lb))
        store += [U.T.ravel(), V.ravel()]            # U column-major (la x cap), V row-major (cap x lb)
        meta.append([ioff, la, ioff + la, lb, so, cap, 0, rk])
        blocks.append((tree.ids(i), tree.ids(j), U[:, :rk], V[:rk]))
        so += la * cap + cap * lb
        ioff += la + lb
    s = 0
    for m in meta:
        slot0.append([s, s + m[1]])
        s += m[1] + (0 if m[6] else m[3])
    f = _Stand()
    f.tree, f.n, f.max_rank = tree, n, 8
    f.meta = torch.as_tensor(np.array(meta, np.int64))
    f.slot0 = torch.as_tensor(np.array(slot0, np.int64))
    f.store = torch.as_tensor(np.concatenate(store))
    f._nodes = near + pairs
    return f, blocks, dense, s


def _bf(x):
    return torch.as_tensor(x).float().to(torch.bfloat16).double().numpy()


def emulate_pack_parts(store, jobs, map_all, plane, off2):
    """k_pack_parts (csrc/hmatrix.cu) restated with torch's CPU roundings: each job writes h = bf16(fp32(x)) and
    m = bf16(fp32(x) - h) of its entries x = store[base + i si + j sj] to plane rows row0 + i, columns c and
    off2 + c, c = colbase + map_all[map_off + j] (colbase + j when map_off < 0)."""
    st = store.detach().cpu().numpy()
    out = torch.zeros(plane.shape, dtype=torch.bfloat16)
    for base, si, sj, ni, nj, row0, colbase, moff in np.asarray(jobs, np.int64).reshape(-1, 8):
        if ni == 0 or nj == 0:
            continue
        x = torch.as_tensor(st[base + np.arange(ni)[:, None] * si + np.arange(nj)[None, :] * sj]).float()
        h = x.to(torch.bfloat16)
        m = (x - h.float()).to(torch.bfloat16)
        cols = torch.as_tensor(colbase + (np.arange(nj) if moff < 0 else map_all[moff:moff + nj].astype(np.int64)))
        out[row0:row0 + ni][:, cols] = h
        out[row0:row0 + ni][:, off2 + cols] = m
    plane.copy_(out.to(plane.device))


GDT = np.dtype([('a_row0', '<i4'), ('rows', '<i4'), ('a_x0', '<i4'), ('b_x0', '<i4'), ('kb', '<i4'),
                ('t_row0', '<i4'), ('rank', '<i4'), ('pad', '<i4'), ('slot0', '<i8')])


def test_lowrank_plan_emulated_matches_direct_sum(monkeypatch):
    import pcbqs_gb300.hmatrix as hm
    monkeypatch.setattr(hm, '_pack_launch', emulate_pack_parts)
    f, blocks, dense, nslots = _fake()
    keep, d = DeviceHMatrix.lowrank_plan(f, dense=True)
    n, k = f.n, 5
    rng = np.random.default_rng(7)
    X = rng.standard_normal((n, k)) + 1j * rng.standard_normal((n, k))
    Xr = np.stack([X.real, X.imag], axis=2).reshape(n, 2 * k)          # real columns 2c, 2c + 1
    n_pad, rwidth = d.n_pad, d.rwidth
    pos = keep['pad_pos'].numpy()
    # X's transposed plane (256 x 2 n_pad): parts h, m at pad_pos
    xt = np.zeros((256, 2 * n_pad))
    h = _bf(Xr.astype(np.float32))
    m = _bf(Xr.astype(np.float32) - h)
    xt[:2 * k, pos] = h.T
    xt[:2 * k, n_pad + pos] = m.T
    rp = keep['rplane'].double().numpy()
    lp = keep['lplane'].double().numpy()
    groups = keep['groups'].numpy().view(GDT)
    tplane = np.zeros((len(groups) * 256, 128))
    for g in groups:                                  # phase one: one tile, rows = ranks, columns = real columns
        D = np.zeros((128, 256))
        for s in range(3):
            for kk in range(g['kb']):
                xa = SEG_A[s] * rwidth + g['b_x0'] + kk * 64
                xb = SEG_B[s] * n_pad + g['a_x0'] + kk * 64
                D += rp[:, xa:xa + 64] @ xt[:, xb:xb + 64].T
        T = np.where(np.arange(128)[:, None] < g['rank'], D, 0)[:64, :2 * k].astype(np.float32)
        th = _bf(T)
        tm = _bf(T - th)
        tplane[g['t_row0']:g['t_row0'] + 2 * k, :64] = th.T
        tplane[g['t_row0']:g['t_row0'] + 2 * k, 64:] = tm.T
    slots = np.zeros((nslots, 2 * k))
    for gi, mt in zip(keep['tile_group'].numpy(), keep['tile_m'].numpy()):
        g = groups[gi]
        r0 = g['a_row0'] + 128 * mt
        D = np.zeros((128, 256))
        for s in range(3):
            a = lp[r0:r0 + 128]
            a = np.vstack([a, np.zeros((128 - len(a), 128))])
            D += a[:, SEG_A[s] * 64:SEG_A[s] * 64 + 64] @ tplane[g['t_row0']:g['t_row0'] + 256,
                                                                  SEG_B[s] * 64:SEG_B[s] * 64 + 64].T
        rows = min(128, g['rows'] - 128 * mt)
        slots[g['slot0'] + 128 * mt:g['slot0'] + 128 * mt + rows] = D[:rows, :2 * k]
    # the dense leaves (MODE 6): D at J's padded positions against X's plane, into the slot rows
    dp = keep['dplane'].double().numpy()
    dpitch = d.dpitch
    dgroups = keep['dgroups'].numpy().view(GDT)
    for gi, mt in zip(keep['dtile_group'].numpy(), keep['dtile_m'].numpy()):
        g = dgroups[gi]
        r0 = g['a_row0'] + 128 * mt
        a = dp[r0:r0 + 128]
        a = np.vstack([a, np.zeros((128 - len(a), 2 * dpitch))])
        D = np.zeros((128, 256))
        for s in range(3):
            for kk in range(g['kb']):
                xa = SEG_A[s] * dpitch + kk * 64
                xb = SEG_B[s] * n_pad + g['a_x0'] + kk * 64
                D += a[:, xa:xa + 64] @ xt[:, xb:xb + 64].T
        rows = min(128, g['rows'] - 128 * mt)
        slots[g['slot0'] + 128 * mt:g['slot0'] + 128 * mt + rows] = D[:rows, :2 * k]
    # the slot rows of block w: forward rows a (slot0[w,0] ...), transposed rows b (slot0[w,1] ...)
    Y = np.zeros((n, 2 * k))
    exact = np.zeros((n, k), complex)
    s0 = f.slot0.numpy()
    for w, (a_ids, b_ids, D, same) in enumerate(dense):
        Y[a_ids] += slots[s0[w, 0]:s0[w, 0] + len(a_ids)]
        exact[a_ids] += D @ X[b_ids]
        if not same:
            Y[b_ids] += slots[s0[w, 1]:s0[w, 1] + len(b_ids)]
            exact[b_ids] += D.T @ X[a_ids]
    for w, (a_ids, b_ids, U, V) in enumerate(blocks, start=len(dense)):
        Y[a_ids] += slots[s0[w, 0]:s0[w, 0] + len(a_ids)]
        Y[b_ids] += slots[s0[w, 1]:s0[w, 1] + len(b_ids)]
        exact[a_ids] += U @ (V @ X[b_ids])
        exact[b_ids] += V.T @ (U.T @ X[a_ids])
    Yc = Y[:, 0::2] + 1j * Y[:, 1::2]
    err = np.linalg.norm(Yc - exact) / np.linalg.norm(exact)
    assert err < 2e-4, err
    assert d.ngroups == 2 * len(blocks) and n_pad % 64 == 0 and rwidth % 64 == 0
    assert d.ndgroups == sum(1 if same else 2 for *_, same in dense) and d.ndense == 0
    assert sorted(np.unique(pos)) == sorted(pos.tolist()) and pos.max() < n_pad
