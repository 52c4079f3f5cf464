"""Benchmark: fill + solve seconds per frequency of the plane-pair board on one GB300 (and the CPU reference arm).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--board planes] [--freq 1e6]
                    [--precondition lu32|block_jacobi]

Workload: the 50 x 50 mm plane pair (0.2 mm FR-4, er 4.3, 35 um copper, 40 vias of 0.3 mm diameter, 8 ports;
22,554 triangles, 33,368 RWG edges, 22,226 charge nodes, 32,990 loop/tree unknowns), seeded synthetic data meshed by
pcbqs's constrained-Delaunay core (tests/golden/planes.npz). One step = one frequency (1 MHz) of the whole hot path
with the mesh resident: the FP64 fill of the triangle-pair moments, the RWG combine into L (33k x 33k), the
aggregation into P (22k x 22k), the loop/tree system's preconditioner and the batched GMRES of all 8 port drives to a
1e-8 relative residual, and the port impedance matrix. Inputs (L alone is 8.9 GB) are far larger than the 129 MB
L2, so no flush is needed between steps.

`value` is seconds per frequency over the whole job (N GPUs solve N frequencies per step: replicas, weak
scaling); `e2e` is the same through the public API from host arrays (PeecModel(board).solve(f): geometry and
sparse topology uploaded, port matrix read back). The reference arm (--impl reference) times the CPU restatement
of the reference's path (the oracle: OpenMP C for the fill, combine and aggregation, run in full) on all host cores,
with the reference's dense solve (a complex64 LU, MixedLU) estimated from a timed bounded LU sample.

`roofline` is the step's dominant stage, the blocked complex64 LU of the 'lu32' preconditioner (about 55 % of the
step's kernel time), against the BF16x9 emulation's tensor ceiling; `fill_roofline` is the fill kernels' (FP32 far
pairs, FP64 near pairs) against the measured FP32/FP64 GEMM rates.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = 'fill+solve s/freq at 1e-8 residual: learned/mixed vs plain FP64 GPU; fill GB/s'
FAR_FLOP, NEAR_FLOP = 210, {0: 936, 1: 3744, 2: 14976}   # algorithmic flops per pair (full moments)
# transcendental evaluations per near pair (the analytic inner integrals: one log of positive terms and one
# arctangent per (observation point, edge) of the 3-point rule at level 0, 4x that per refinement level), which the
# algebraic flop count leaves out; and the FP64-pipe activity of k_fill_near measured by ncu on the plane pair's
# first 8,000 triangles (sm__pipe_fp64_cycles_active, the near kernel's bound)
NEAR_TRANSCENDENTALS = {0: 72, 1: 288, 2: 1152}
NEAR_FP64_PIPE_ACTIVE = 0.871


def parse():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=3)
    p.add_argument('--warmup', type=int, default=3)
    p.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    p.add_argument('--board', default='planes')
    p.add_argument('--freq', type=float, default=1e6)
    p.add_argument('--precondition', default='lu32', choices=['lu32', 'block_jacobi'])
    p.add_argument('--factor-math', default='tc6-blocked',
                   choices=['fp32', 'bf16x9', 'bf16x9-blocked', 'fp32-blocked', 'tc6-blocked', 'tc3-blocked'],
                   help='the lu32 factorization: cuSOLVER getrf or the blocked LU (-blocked) with cuBLAS trailing GEMMs '
                        'in FP32 or FP32 emulated on the tensor cores (bf16x9), or with this library\'s tcgen05 '
                        'update on six (tc6, FP32 accuracy) or three (tc3) BF16 part products')
    p.add_argument('--mode', default='mixed', choices=['mixed', 'fp64'],
                   help='mixed: FP32 far pairs in local coordinates and FP32 inner Krylov products under FP64 '
                        'refinement; fp64: the FP64 fill and FP64 GMRES')
    p.add_argument('--no-comparator', action='store_true', help='skip the one-step FP64 comparator')
    p.add_argument('--plain', action='store_true',
                   help='also time, once, the plain FP64 path: FP64 fill and block-Jacobi GMRES to the same residual')
    p.add_argument('--no-cpu-baseline', action='store_true')
    p.add_argument('--sweep', type=int, default=0,
                   help='also time a sweep of this many log-spaced frequencies (1 kHz to 100 MHz), all ports')
    p.add_argument('--anchors', type=int, default=6,
                   help='complex64 factors shared across the sweep (64 frequencies: 4 -> 15.4 s, 6 -> 14.0 s, 8 -> '
                        '14.9 s, 12 -> 21.0 s on one GB300)')
    p.add_argument('--sweep-board', default='planes16', help='the sweep\'s board (default: the 16-port plane pair)')
    p.add_argument('--inner-tol', type=float, default=1e-4,
                   help="the mixed solve's inner GMRES tolerance (relative to each outer step's residual)")
    p.add_argument('--product', default='tc3', choices=['tc3', 'tc6', 'fp32'],
                   help='the mixed solve\'s inner dense products over 16 or more columns')
    p.add_argument('--case', default=None,
                   help='time one kernel case small enough for a full ncu capture instead of the benchmark: '
                        'fill:BOARD[:TRIANGLES] | lu:BOARD[:K...] | dense:N[:K] | getrf:N[:BLOCK[:MATH...]] | '
                        'potrf:N[:BLOCK...] | update:ROWS:COLS:K (CUDA-event times after a warm-up call) | '
                        'c5 | c5solve[:FREQ[:MIXED[:PARTS]]] (the large compressed board)')
    return p.parse_args()


def rank_info():
    return int(os.environ.get('RANK', 0)), int(os.environ.get('WORLD_SIZE', 1)), int(os.environ.get('LOCAL_RANK', 0))


def replica_frequency(freq, rank):
    """Replicas: each rank solves its own frequency (1 % apart), the same work per rank (weak scaling)."""
    return freq * (1 + 0.01 * rank)


def job_seconds_per_frequency(ms_local, world, dist=None, device='cuda'):
    """(step ms, the maximum over ranks; whole-job seconds per frequency: world frequencies per step)."""
    ms = float(ms_local)
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([ms], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t)
    return ms, ms / 1e3 / world


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    QUERY = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
             'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
             'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.file = tempfile.NamedTemporaryFile('w+', suffix='.csv', delete=False)
        try:
            self.proc = subprocess.Popen(['nvidia-smi', f'--id={index}', f'--query-gpu={self.QUERY}',
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return dict(sm_mhz=None, sm_max_mhz=None, reasons=['nvidia-smi unavailable'])
        self.proc.terminate()
        self.proc.wait()
        self.file.flush()
        rows = [r.split(', ') for r in Path(self.file.name).read_text().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].replace('.', '').isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[i] for r in rows if len(r) >= 9 for i in range(4) if r[5 + i].strip() == 'Active'})
        return dict(sm_mhz=statistics.median(sm) if sm else None, sm_max_mhz=max(mx) if mx else None,
                    reasons=reasons, samples=len(rows))


def fill_roofline(model, fill_ms, mixed, peaks):
    """The fill kernel pair (far tiles + near lists): algorithmic flops per launch / their CUDA-event time.

    FP64 fill: every pair on the FP64 pipe, peak = the FP64 GEMM rate. Mixed fill: far pairs on the FP32 pipe and
    near pairs on the FP64 pipe, so the roofline time of one launch is far_flops / FP32 peak + near_flops / FP64
    peak, and `peak` is the flop rate that time implies (the pipes' rates weighted by this workload's flop mix)."""
    import ctypes
    from pcbqs_gb300 import _lib
    counts = (ctypes.c_uint64 * 2)()
    _lib.check(model.fill.lib.pcbqs_gb300_fill_counts(model.fill.dev.handle, counts))
    nt = model.fill.nt
    pairs = nt * (nt + 1) // 2
    near0, near1 = int(counts[0]), int(counts[1])
    far = pairs - near0 - near1
    far_flops = far * FAR_FLOP
    near_flops = near0 * NEAR_FLOP[0] + near1 * NEAR_FLOP[model.fill.outer_levels]
    flops = far_flops + near_flops
    achieved = flops / (fill_ms / 1e3) / 1e12
    if mixed:
        bound_s = far_flops / (peaks['fp32'] * 1e12) + near_flops / (peaks['fp64'] * 1e12)
        peak, bound = flops / bound_s / 1e12, 'fp32 (far) + fp64 (near)'
        source = (f"measured live: SGEMM {peaks['fp32']:.1f} and DGEMM {peaks['fp64']:.2f} TFLOP/s (cuBLAS 8192^3) on "
                  f"this GPU, weighted by the far/near flop split")
    else:
        peak, bound = peaks['fp64'], 'fp64'
        source = 'measured live: FP64 GEMM (cuBLAS DGEMM 8192^3) on this GPU'
    # DRAM bytes (read + written) of the far-tile kernel per launch, from an ncu capture of the same kernel on the
    # first 8,000 triangles of the plane pair (989.2 MB for its 32,004,000 unordered pairs: 30.9 B a pair against
    # the 32 B of the four FP32 planes written once), scaled by this launch's pair count; the FP64 fill has no
    # capture at a size above L2, so no figure
    traffic = round(pairs * 989.2e6 / 32004000) if mixed else None
    transcendentals = near0 * NEAR_TRANSCENDENTALS[0] + near1 * NEAR_TRANSCENDENTALS[model.fill.outer_levels]
    return dict(bound=bound, kernel='k_fill_tiles+k_fill_near', achieved=round(achieved, 4), peak=round(peak, 4),
                unit='TFLOP/s', frac=round(achieved / peak, 4), traffic=traffic, flops_per_launch=flops,
                far_pairs=far, near_pairs=[near0, near1], peak_source=source,
                traffic_source='ncu dram bytes of k_fill_tiles on 8,000 triangles, scaled by pairs' if mixed else None,
                near_transcendentals_per_launch=transcendentals,
                near_fp64_pipe_active=NEAR_FP64_PIPE_ACTIVE,
                near_fp64_pipe_source='profiles/k_fill_near_planes_8k.md (sm__pipe_fp64_cycles_active, ncu)')


def measured_peaks():
    """MEASURED_PEAKS.json beside this file (copy bandwidth and cuBLAS bf16 rates measured on this GPU model), or
    None."""
    path = Path(__file__).resolve().parent / 'MEASURED_PEAKS.json'
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return None


# DRAM bytes (read + written) per complex flop of the tcgen05 update, from an ncu capture of one six-term launch of
# C (8192 x 8192) -= A (8192 x 2048) B (2048 x 8192): 7.400 GB read + 0.529 GB written for 1.100e12 complex flops
TC_UPDATE_BYTES_PER_FLOP = (7.399611e9 + 0.529117e9) / (8.0 * 8192 * 8192 * 2048)


def factor_roofline(model, timings, factor_math):
    """The dominant stage's kernel. With the tcgen05 factor (tc3/tc6): this library's trailing update, its complex
    flops (8 rows cols k per launch) over its CUDA-event time summed on the factorization's stream, against the
    emulation's ceiling, the measured sustained BF16 tensor rate / terms (each complex-FP32 product is `terms` BF16
    part products; the updates run for most of a second inside the step, so the sustained figure); the whole LU
    (8 n^3 / 3 flops over its time) beside it. With cuBLAS's BF16x9 GEMMs: the LU against the bf16 rate / 9."""
    n = model.n
    lu_ms = statistics.median(t['factor_lu_ms'] for t in timings)
    lu_flops = 8 * n ** 3 / 3
    peaks = measured_peaks()
    if peaks and peaks.get('bf16_tflops_sustained'):
        bf16, source = float(peaks['bf16_tflops_sustained']), 'MEASURED_PEAKS.json bf16_tflops_sustained'
    else:
        bf16, source = 1700.0, 'fallback sustained bf16 1,700 TFLOP/s'
    if factor_math in ('tc6-blocked', 'tc3-blocked'):
        terms = 6 if factor_math == 'tc6-blocked' else 3
        t = timings[len(timings) // 2]
        ms, flops, launches = t['factor_update_ms'], t['factor_update_flops'], t['factor_update_launches']
        peak = bf16 / terms
        achieved = flops / (ms / 1e3) / 1e12
        per_launch = flops / max(launches, 1)
        return dict(bound='tensor', kernel=f'k_tc_update (this library: tcgen05 BF16x{terms} complex trailing update, '
                                           f'with its operand packing)',
                    achieved=round(achieved, 2), peak=round(peak, 2), unit='TFLOP/s', frac=round(achieved / peak, 4),
                    traffic=round(per_launch * TC_UPDATE_BYTES_PER_FLOP),
                    traffic_source='ncu dram bytes of one six-term launch (8192^2 x 2048), scaled by flops per launch',
                    flops_per_launch=per_launch, launches=launches, update_ms=round(ms, 2),
                    bf16_part_product_tflops=round(achieved * terms, 1),
                    peak_source=f'{source} / {terms} (of measured)',
                    lu=dict(ms=round(lu_ms, 2), tflops=round(lu_flops / (lu_ms / 1e3) / 1e12, 2),
                            update_share=round(ms / lu_ms, 3)))
    peak = bf16 / 9
    achieved = lu_flops / (lu_ms / 1e3) / 1e12
    return dict(bound='tensor', kernel='getrf_blocked (cuBLAS BF16x9 complex trailing GEMMs + cuSOLVER panels)',
                achieved=round(achieved, 2), peak=round(peak, 2), unit='TFLOP/s', frac=round(achieved / peak, 4),
                traffic=None, flops_per_launch=lu_flops, lu_ms=round(lu_ms, 2), peak_source=source + ' / 9 (of measured)')


def gemm_peak(dtype):
    """Best of three cuBLAS GEMMs of 8192^3 in `dtype` (FP32 without TF32), TFLOP/s."""
    import torch
    n = 8192
    allow = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    a = torch.randn(n, n, dtype=dtype, device='cuda')
    b = torch.randn(n, n, dtype=dtype, device='cuda')
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12)
    torch.backends.cuda.matmul.allow_tf32 = allow
    del a, b
    torch.cuda.empty_cache()
    return best


def cpu_front(board_name):
    """The oracle's fill of the moments, RWG combine into L and aggregation into P on every host core:
    (board, rwg, L, P, details)."""
    from oracle import oracle as O
    from pcbqs_gb300.board import Board
    b = Board.load(board_name)
    threads = O.threads()
    t0 = time.perf_counter()
    g = O.Geometry(b.nodes, b.tris, b.z, 1)
    mats, analytic = O.fill(g, 3.0, 1, False, threads)
    t1 = time.perf_counter()
    rwg = O.RWG(g.nodes, g.tris)
    L = O.combine(rwg, mats, nthreads=threads)
    t2 = time.perf_counter()
    P = O.potential(mats[0], g.area, b.node_of, b.er, threads)
    t3 = time.perf_counter()
    del mats
    return b, rwg, L, P, dict(cores=threads, fill_s=round(t1 - t0, 3), combine_s=round(t2 - t1, 3),
                              potential_s=round(t3 - t2, 3))


def cpu_reference(board_name, freq):
    """The CPU restatement of the reference's whole path (oracle), every host core, one frequency, in full: the fill
    of the moments, the RWG combine and the P aggregation (OpenMP C), then the reference's dense PEEC solve
    (oracle/peec_cpu.py: topology and projections, the scaled system, its complex64 LU with MixedLU's FP64
    refinement, every port drive). Returns (seconds, details, port impedance matrix, unknowns)."""
    from oracle import peec_cpu
    t0 = time.perf_counter()
    b, rwg, L, P, details = cpu_front(board_name)
    solver = peec_cpu.DenseSolve(b, rwg, L, P, details)
    del L
    Z = solver.solve(freq, details)
    seconds = time.perf_counter() - t0
    n = solver.n
    del solver
    return seconds, details, Z, n


def cpu_sample(board_name, n):
    """The bounded CPU baseline beside the GPU line: the oracle's fill, combine and aggregation in full, and the
    dense solve's complex64 LU from a timed 6144^2 LAPACK getrf scaled by (n / 6144)^3 (the factorization is most
    of the reference's solve; `--impl reference` runs it in full). Returns (seconds per frequency, details)."""
    from oracle import peec_cpu
    t0 = time.perf_counter()
    *_, details = cpu_front(board_name)
    front = time.perf_counter() - t0
    lu, sample_s = peec_cpu.lu_seconds(n, sample=6144, repeats=1)
    details.update(lu_estimate_s=round(lu, 2),
                   lu_sample='complex64 getrf 6144^2 in %.3f s, scaled by (n/6144)^3, n=%d' % (sample_s, n))
    return front + lu, details


def board_config(board_name, freq, unknowns=None, world=1):
    """The workload's configuration, the same keys on both arms."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.rwg import RWG
    from pcbqs_gb300.geometry import prepare
    b = Board.load(board_name)
    g = prepare(b.nodes, b.tris, b.z, 1)
    return dict(workload=f'{board_name}: fill+solve of all {len(b.ports)} ports at {freq:g} Hz', board=board_name,
                triangles=int(b.nt), edges=int(RWG(g.nodes, g.tris).Ne), nodes=int(b.n_nodes),
                unknowns=None if unknowns is None else int(unknowns), parallelism=f'replicas x{world}',
                l2='inputs larger than L2 (L 8.9 GB)' if board_name == 'planes' else 'inputs larger than L2')


def reference_arm(args):
    """The reference's CPU path on the host cores, run in full once (a step is minutes of CPU work: the complex64 LU
    of the 32,990-unknown system alone is about 10^14 flops), so `steps` reports the one step timed whatever
    --steps asked; no warm-up (nothing is cached between steps)."""
    rank, world, _ = rank_info()
    if rank != 0:
        return
    value, details, Z, n = cpu_reference(args.board, args.freq)
    golden = ROOT / 'tests' / 'golden' / f'peec_{args.board}.npz'
    if golden.exists():
        with np.load(golden) as ref:
            hit = np.flatnonzero(np.isclose(ref['freqs'], args.freq))
            if len(hit):
                Zr = ref['Z'][hit[0]]
                details['port_z_max_rel_err_vs_reference'] = float(np.abs(Z - Zr).max() / np.abs(Zr).max())
    line = dict(metric=METRIC, value=round(value, 4), unit='s/freq', n_gpus=args.gpus, steps=1,
                steps_requested=args.steps, warmup=0, ms_per_step=round(value * 1e3, 2), higher_is_better=False,
                scaling='weak', vs_baseline=None, dtype='f64 (complex64 LU refined in f64)',
                data='synthetic (seeded plane-pair board, CDT mesh)', impl='reference',
                config=board_config(args.board, args.freq, n, 1),
                cpu_baseline=dict(value=round(value, 4), unit='s/freq', cores=details['cores'], kind='port',
                                  sample=f'the whole path once, in full: oracle fill+combine+aggregation (OpenMP C) '
                                         f'and the restated dense PEEC solve ({details["lu"]} of all {n} unknowns, '
                                         f'MixedLU refinement, {len(Z)} drives); {details}'),
                e2e=dict(value=round(value, 4), unit='s/freq', h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line))


def _event_ms(fn):
    import torch
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    out = fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), out


def case_fill(board, triangles=None):
    """The mixed and the FP64 fill of the first `triangles` triangles of a board (k_fill_tiles, k_fill_near)."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.fill import DeviceFill
    b = Board.load(board)
    nt = len(b.tris) if triangles is None else int(triangles)
    tris = b.tris[:nt]
    used = np.unique(tris)
    remap = np.full(len(b.nodes), -1)
    remap[used] = np.arange(len(used))
    f = DeviceFill(b.nodes[used], remap[tris], b.z[:nt], 1, 3.0)
    for mode in ('mixed', 'fp64'):
        for _ in range(3):
            ms, (planes, analytic) = _event_ms(f.moments_local if mode == 'mixed' else f.moments)
            del planes
            print(f'fill {mode} {nt} triangles: {ms:.2f} ms, {analytic} analytic pairs', flush=True)


def case_lu(board, *ks):
    """A board's complex64 PEEC factor at 1 MHz (each factor math), then its triangular solves (k_tri_sweeps) for
    k right-hand sides."""
    import ctypes
    import torch
    from pcbqs_gb300 import _lib
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel, _csr_struct
    m = PeecModel(Board.load(board))
    m.assemble(mixed=True)
    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    handle, _ = m._operator(np.array([2 * np.pi * 1e6]))
    try:
        desc = _csr_struct(m._krk_device())
        for math in (1, 2, 3):
            ms, _ = _event_ms(lambda: _lib.check(lib.pcbqs_gb300_peec_factor(handle, ctypes.byref(desc), 0, math,
                                                                             stream), lib))
            print(f'factor n={m.n} math {math}: {ms:.1f} ms', flush=True)
        for k in (ks or (8,)):
            k = int(k)
            x = torch.randn(m.n, k, dtype=torch.complex128, device='cuda')
            y = torch.empty_like(x)
            for _ in range(3):
                ms, _ = _event_ms(lambda: _lib.check(lib.pcbqs_gb300_peec_lu_solve(handle, k, x.data_ptr(),
                                                                                   y.data_ptr(), 0, stream), lib))
                print(f'lu_solve k={k}: {ms:.2f} ms', flush=True)
    finally:
        lib.pcbqs_gb300_peec_destroy(handle)


def case_getrf(n, block=2048, *maths):
    """The blocked complex64 LU of a random n x n matrix with `block`-column panels, twice with each trailing update
    given (default all: cuBLAS BF16x9 = 1, this library's tcgen05 update with 3 and 6 BF16 part products = 2, 3)."""
    import ctypes
    import torch
    from pcbqs_gb300 import _lib
    n = int(n)
    lib = _lib.load()
    g = torch.Generator(device='cuda').manual_seed(1)
    A = torch.complex(torch.randn(n, n, device='cuda', generator=g), torch.randn(n, n, device='cuda', generator=g))
    F = torch.empty_like(A)
    piv = torch.zeros(n, dtype=torch.int32, device='cuda')
    singular = ctypes.c_int32(0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    flops = 8 / 3 * n ** 3
    for block in (int(block),):
        for math in tuple(int(m) for m in maths) or (1, 2, 3):
            for _ in range(2):
                F.copy_(A)
                ms, status = _event_ms(lambda: lib.pcbqs_gb300_lu_factor_c64(n, F.data_ptr(), piv.data_ptr(),
                                                                             int(block), math,
                                                                             ctypes.byref(singular), stream))
                _lib.check(status, lib)
                print(f'getrf n={n} block {block} math {math}: {ms:.1f} ms, {flops / ms / 1e9:.1f} TFLOP/s',
                      flush=True)


def case_update(rows, cols, k):
    """C -= A B (complex64, rows x k times k x cols) by this library's tcgen05 update with 3 and 6 BF16 part
    products, against cuBLAS's FP32 complex GEMM (torch complex64 matmul, TF32 off): TFLOP/s of 8 rows cols k."""
    import ctypes
    import torch
    from pcbqs_gb300 import _lib
    rows, cols, k = int(rows), int(cols), int(k)
    lib = _lib.load()
    g = torch.Generator(device='cuda').manual_seed(2)
    a = torch.complex(torch.randn(k, rows, device='cuda', generator=g), torch.randn(k, rows, device='cuda', generator=g))
    b = torch.complex(torch.randn(cols, k, device='cuda', generator=g), torch.randn(cols, k, device='cuda', generator=g))
    c = torch.zeros(cols, rows, dtype=torch.complex64, device='cuda')
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    flops = 8.0 * rows * cols * k
    for terms in (3, 6):
        for _ in range(3):
            ms, status = _event_ms(lambda: lib.pcbqs_gb300_complex_update(rows, cols, k, a.data_ptr(), rows,
                                                                          b.data_ptr(), k, c.data_ptr(), rows, terms,
                                                                          1 << 32, stream))
            _lib.check(status, lib)
            print(f'update {rows}x{cols}x{k} terms {terms}: {ms:.2f} ms, {flops / ms / 1e9:.1f} TFLOP/s', flush=True)
    allow = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    at, bt = a.T, b.T
    for _ in range(3):
        ms, _ = _event_ms(lambda: torch.matmul(at, bt))
        print(f'cuBLAS complex64 GEMM {rows}x{cols}x{k}: {ms:.2f} ms, {flops / ms / 1e9:.1f} TFLOP/s', flush=True)
    torch.backends.cuda.matmul.allow_tf32 = allow


def case_potrf(n, *blocks):
    """The blocked FP32 Cholesky of a random n x n positive definite matrix, against cuSOLVER's potrf."""
    import ctypes
    import torch
    from pcbqs_gb300 import _lib
    n = int(n)
    lib = _lib.load()
    g = torch.Generator(device='cuda').manual_seed(1)
    M = torch.randn(n, n, device='cuda', generator=g)
    A = M @ M.T / n + 0.05 * torch.eye(n, device='cuda')
    ld = (n + 31) // 32 * 32                      # the padded leading dimension the library's own factor uses
    F = torch.zeros(n, ld, device='cuda')
    info = ctypes.c_int32(0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for block in (blocks or (1024,)):
        for math in (1, 0):
            for _ in range(2):
                F[:, :n].copy_(A)
                ms, status = _event_ms(lambda: lib.pcbqs_gb300_cholesky_f32(n, F.data_ptr(), ld, int(block), math,
                                                                            ctypes.byref(info), stream))
                _lib.check(status, lib)
                print(f'potrf n={n} ld {ld} block {block} math {math}: {ms:.1f} ms, '
                      f'{n ** 3 / 3 / ms / 1e9:.1f} TFLOP/s', flush=True)


def case_dense(n, k=8, *forms):
    """A random symmetric n x n matrix (FP64 and its FP32 copy) against k complex columns: forms fp64 and fp32
    (k_dense_sym_apply, k_dense_apply_f32), tensor3 (the BF16x3 real-operand product, k_tc_update<1>) and sliced6
    (the FP64-accurate integer-slice product, k_tc_update<2>); the tensor forms pack M in each call. Default all."""
    import ctypes
    import torch
    from pcbqs_gb300 import _lib
    n, k = int(n), int(k)
    lib = _lib.load()
    g = torch.Generator(device='cuda').manual_seed(1)
    M = torch.rand((n, n), dtype=torch.float64, device='cuda', generator=g)
    M = (M + M.T) / 2
    Mf = M.float()
    X = torch.randn((n, k), dtype=torch.complex128, device='cuda', generator=g)
    Y = torch.empty_like(X)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    calls = dict(
        fp64=lambda: lib.pcbqs_gb300_dense_apply(n, k, M.data_ptr(), n, X.data_ptr(), Y.data_ptr(), stream),
        fp32=lambda: lib.pcbqs_gb300_dense_apply_single(n, k, Mf.data_ptr(), n, X.data_ptr(), Y.data_ptr(), stream),
        tensor3=lambda: lib.pcbqs_gb300_dense_apply_tensor(n, k, Mf.data_ptr(), n, X.data_ptr(), Y.data_ptr(), 3,
                                                           1 << 31, stream),
        sliced6=lambda: lib.pcbqs_gb300_dense_apply_sliced(n, k, M.data_ptr(), n, X.data_ptr(), Y.data_ptr(), 6,
                                                           1 << 31, stream))
    for name in (forms or tuple(calls)):
        fn = calls[name]
        for _ in range(3):
            ms, status = _event_ms(fn)
            _lib.check(status, lib)
            bytes_ = n * n * {'fp64': 8, 'fp32': 4, 'tensor3': 4, 'sliced6': 8}[name]
            print(f'dense {name} n={n} k={k}: {ms:.3f} ms, {bytes_ / ms / 1e6:.0f} GB/s of matrix, '
                  f'{2 * n * n * 2 * k / ms / 1e9:.3f} TFLOP/s', flush=True)


def case_lusolve(board, k=128, method=3, math=2):
    """A board's complex64 PEEC factor at 1 MHz (math 2: cuBLAS BF16x9 updates, so that no tcgen05 update precedes
    the solves), then two triangular solves of k columns by `method` (0 auto, 1 getrs, 2 streaming sweeps, 3 the
    blocked solve: k_cgemm_small, k_tc_update<3>, the factor's panels packed by the first)."""
    import ctypes
    import torch
    from pcbqs_gb300 import _lib
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel, _csr_struct
    k, method, math = int(k), int(method), int(math)
    m = PeecModel(Board.load(board))
    m.assemble(mixed=True)
    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    handle, _ = m._operator(np.array([2 * np.pi * 1e6]))
    try:
        desc = _csr_struct(m._krk_device())
        _lib.check(lib.pcbqs_gb300_peec_factor(handle, ctypes.byref(desc), 0, math, stream), lib)
        g = torch.Generator(device='cuda').manual_seed(1)
        x = torch.randn(m.n, k, dtype=torch.complex128, device='cuda', generator=g)
        y = torch.empty_like(x)
        for _ in range(2):
            ms, _ = _event_ms(lambda: _lib.check(lib.pcbqs_gb300_peec_lu_solve(handle, k, x.data_ptr(), y.data_ptr(),
                                                                               method, stream), lib))
            print(f'lu_solve n={m.n} k={k} method {method}: {ms:.2f} ms', flush=True)
    finally:
        lib.pcbqs_gb300_peec_destroy(handle)


def case_lowrank(board, k=128, leaf=256, tol=1e-6):
    """A board's inductance H-matrix (ACA to `tol`, leaves of `leaf`), then its product with k complex columns three
    times each: in FP64 (k_hm_apply_blocks), with the low-rank blocks in BF16 on the tensor cores (k_pack_xt,
    k_tc_update<4>, k_tc_update<5>; the dense leaves in FP64), and with every block on the tensor cores (the dense
    leaves by k_tc_update<6>)."""
    import torch
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.fill import DeviceFill
    from pcbqs_gb300.hmatrix import DeviceHMatrix
    k, leaf, tol = int(k), int(leaf), float(tol)
    b = Board.load(board)
    fill = DeviceFill(b.nodes, b.tris, b.z, 1, 3.0)
    t0 = time.perf_counter()
    H = DeviceHMatrix(fill, tol=tol, leaf=leaf, kernel='inductance')
    print(f'hmatrix {board}: n={H.n}, {H.nblocks} blocks ({H.low_rank} low rank, rank <= {H.max_rank}), '
          f'{H.bytes / 1e9:.2f} GB of {H.n * H.n * 8 / 1e9:.2f} GB dense, built in {time.perf_counter() - t0:.1f} s',
          flush=True)
    g = torch.Generator(device='cuda').manual_seed(1)
    X = torch.randn(H.n, k, dtype=torch.complex128, device='cuda', generator=g)
    H.matmat_lowrank(X)                              # packs the low-rank plans
    H.matmat_lowrank(X, dense=True)
    for name, fn in (('fp64', H.matmat), ('bf16 low-rank', H.matmat_lowrank),
                     ('bf16 all blocks', lambda v: H.matmat_lowrank(v, dense=True))):
        for _ in range(3):
            ms, Y = _event_ms(lambda: fn(X))
            print(f'hmatrix product {name} k={k}: {ms:.2f} ms', flush=True)


def case_c5(k=32, leaf=256, tol=1e-6):
    """The large compressed board (tests/golden/c5.npz, config C5's shape): the inductance H-matrix of its RWG edges
    and the potential H-matrix of its triangles (ACA to `tol`, leaves of `leaf`, rank up to 32), their products
    with k complex columns in FP64 and with the low-rank blocks in BF16 on the tensor cores, and the Biot-Savart
    field of random sheet currents on a 256 x 256 grid 1 mm above the board (h_grid). Prints one JSON line. No PEEC
    solve: block-Jacobi does not converge on pours, and the dense complex64 factor of its ~320,000 unknowns would
    take 820 GB."""
    import json as _json
    import torch
    from pcbqs_gb300.biot import h_grid
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.fill import DeviceFill
    from pcbqs_gb300.hmatrix import DeviceHMatrix
    k, leaf, tol = int(k), int(leaf), float(tol)
    b = Board.load('c5')
    out = dict(case='c5', triangles=int(len(b.tris)), vias=int(b.nv), ports=len(b.ports), k=k, leaf=leaf, tol=tol)
    t0 = time.perf_counter()
    fill = DeviceFill(b.nodes, b.tris, b.z, 1, 3.0)
    out['geometry_s'] = round(time.perf_counter() - t0, 2)
    g = torch.Generator(device='cuda').manual_seed(1)
    for name, kernel in (('L', 'inductance'), ('P', 'potential')):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        H = DeviceHMatrix(fill, tol=tol, leaf=leaf, kernel=kernel, er=b.er)
        torch.cuda.synchronize()
        rec = dict(n=H.n, build_s=round(time.perf_counter() - t0, 2), blocks=H.nblocks, low_rank=H.low_rank,
                   max_rank=H.max_rank, gbytes=round(H.bytes / 1e9, 3), dense_gbytes=round(H.n * H.n * 8 / 1e9, 1),
                   entries_per_s=round(H.entries / (time.perf_counter() - t0), 1))
        X = torch.randn(H.n, k, dtype=torch.complex128, device='cuda', generator=g)
        ref = H.matmat(X)
        H.matmat_lowrank(X)
        H.matmat_lowrank(X, dense=True)
        rec['fp64_ms'] = round(min(_event_ms(lambda: H.matmat(X))[0] for _ in range(3)), 2)
        rec['bf16_lowrank_ms'] = round(min(_event_ms(lambda: H.matmat_lowrank(X))[0] for _ in range(3)), 2)
        rec['bf16_all_ms'] = round(min(_event_ms(lambda: H.matmat_lowrank(X, dense=True))[0] for _ in range(3)), 2)
        rec['bf16_lowrank_vs_fp64'] = float((torch.linalg.norm(H.matmat_lowrank(X) - ref) /
                                             torch.linalg.norm(ref)).item())
        rec['bf16_all_vs_fp64'] = float((torch.linalg.norm(H.matmat_lowrank(X, dense=True) - ref) /
                                         torch.linalg.norm(ref)).item())
        out[name] = rec
        print(name, rec, flush=True)
        del H, X, ref
        torch.cuda.empty_cache()
    from pcbqs_gb300.rwg import RWG
    r = RWG(b.nodes, b.tris)                          # the board's own coordinates (the fill's are centred)
    rng = np.random.default_rng(2)
    I = rng.standard_normal(r.Ne) + 1j * rng.standard_normal(r.Ne)
    lt = {int(l): np.flatnonzero(b.layer == l) for l in np.unique(b.layer)}
    lo, hi = b.nodes.min(0), b.nodes.max(0)
    x, y = np.linspace(lo[0], hi[0], 256), np.linspace(lo[1], hi[1], 256)
    top = float(np.max(b.z)) + 1e-3
    h_grid(r, lt, b.z, I, x, y, [top])                # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    Hf = h_grid(r, lt, b.z, I, x, y, [top])
    torch.cuda.synchronize()
    out['h_grid'] = dict(points=256 * 256, seconds=round(time.perf_counter() - t0, 3), finite=bool(np.isfinite(Hf).all()))
    print(_json.dumps(out), flush=True)


def case_c5solve(freq=1e6, mixed=1, parts=0):
    """The PEEC solve of the large compressed board (tests/golden/c5.npz: 212,297 triangles, 16 ports): every port
    driven alone at one frequency through the compressed operator (H-matrices at tol 1e-6, leaves 256, rank <= 32),
    preconditioned by the graph preconditioner with its Laplacian split into domains (parts 0: by its size), the
    FP64 GMRES (mixed=0) or FP64 refinement around inner GMRES on BF16 products (mixed=1), to 1e-8. Prints one JSON
    line with the stage times, steps, residuals and the port matrix's diagonal."""
    import ctypes
    import json as _json
    import torch
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    freq, mixed, parts = float(freq), bool(int(mixed)), int(parts) or None
    b = Board.load('c5')
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    model = PeecModel(b, matrix='hierarchical')
    model.assemble()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    res = model.solve([freq], precondition='graph', mixed=mixed, graph_parts=parts)
    t2 = time.perf_counter()
    tm = model.timings
    Z = res.impedance[0]
    g = model.graph_structure()
    # per-application costs at the solve's column count: the FP64 operator, the graph preconditioner, and the BF16
    # H-matrix products of the inner solves (CUDA events, best of three after a warm-up)
    from pcbqs_gb300 import _lib
    lib = _lib.load()
    k = len(b.ports)
    nparts = model._graph_parts(parts)
    handle, _ = model._operator(np.array([2 * np.pi * freq]))
    gen = torch.Generator(device='cuda').manual_seed(3)
    rnd = lambda rows: torch.complex(torch.randn(rows, k, device='cuda', generator=gen, dtype=torch.float64),
                                     torch.randn(rows, k, device='cuda', generator=gen, dtype=torch.float64))
    per = {}
    try:
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        model._graph_precondition(handle, 0, freq, 2 if nparts else 1, stream, nparts)
        X = rnd(model.n)
        Y = torch.empty_like(X)
        sysidx = np.zeros(k, np.int32)
        calls = dict(graph_apply_ms=lambda: _lib.check(lib.pcbqs_gb300_peec_graph_apply(
                         handle, k, X.data_ptr(), Y.data_ptr(), stream), lib),
                     fp64_operator_ms=lambda: _lib.check(lib.pcbqs_gb300_peec_apply(
                         handle, k, _lib.ptr(sysidx, ctypes.c_int32), X.data_ptr(), Y.data_ptr(), stream), lib))
        Xe, Xt = rnd(model.HL.n), rnd(model.HP.n)
        calls['bf16_L_ms'] = lambda: model.HL.matmat_lowrank(Xe, dense=True)
        calls['bf16_P_ms'] = lambda: model.HP.matmat_lowrank(Xt, dense=True)
        for name, fn in calls.items():
            per[name] = round(min(_event_ms(fn)[0] for _ in range(3)), 2)
    finally:
        lib.pcbqs_gb300_peec_destroy(handle)
    out = dict(case='c5solve', triangles=int(len(b.tris)), unknowns=int(model.n), loops=int(model.nl),
               nodes=int(model.nn), ports=len(b.ports), freq=freq, mixed=mixed,
               graph_parts=int(model._graph_parts(parts)), laplacian_rows=int(g['nkeep']),
               tree_inverse_entries=int(len(g['tinv'][1])), assemble_s=round(t1 - t0, 2), solve_s=round(t2 - t1, 2),
               hmatrix_s=round(tm.get('hmatrix_s', 0.0), 2), host_topology_s=round(tm.get('host_topology_s', 0.0), 2),
               equilibrium_s=round(tm.get('equilibrium_s', 0.0), 2),
               precondition_ms=round(tm['precondition_ms'], 1), gmres_ms=round(tm['gmres_ms'], 1),
               graph_host_s=round(tm.get('graph_host_s', 0.0), 2), lowrank_plan_s=round(tm.get('lowrank_plan_s', 0.0), 2),
               rhs_s=round(tm.get('rhs_s', 0.0), 2), post_s=round(tm.get('post_s', 0.0), 2), per_application=per,
               gmres_steps_max=int(res.iterations.max()), outer_steps=tm.get('outer_steps'),
               residual_max=float(res.residual.max()),
               reciprocity=float(np.abs(Z - Z.T).max() / np.abs(Z).max()),
               z_diag=[[float(z.real), float(z.imag)] for z in np.diag(Z)],
               torch_peak_gbytes=round(torch.cuda.max_memory_allocated() / 1e9, 2))
    print(_json.dumps(out), flush=True)


CASES = dict(fill=case_fill, lu=case_lu, getrf=case_getrf, potrf=case_potrf, dense=case_dense, update=case_update,
             lusolve=case_lusolve, lowrank=case_lowrank, c5=case_c5, c5solve=case_c5solve)


def kernel_case(spec):
    name, *values = spec.split(':')
    if name not in CASES:
        raise SystemExit(f'unknown case {name!r}: one of {sorted(CASES)}')
    import torch
    torch.cuda.set_device(0)
    from pcbqs_gb300 import build
    build.build()
    CASES[name](*values)


BLOCKED_LU_MATH = {'fp32-blocked': 0, 'bf16x9-blocked': 1, 'tc3-blocked': 2, 'tc6-blocked': 3}


def autotune_lu_panel(lib, n, args, widths=(1024, 2048, 3072)):
    """The blocked LU's panel width for this order and math, from the tuning file (PCBQS_GB300_TUNE_FILE) when it
    holds one, else timed now (pcbqs_gb300_tune_lu_panel, outside the timed region); peec_factor then uses it."""
    import ctypes
    import torch
    from pcbqs_gb300 import _lib
    math = BLOCKED_LU_MATH.get(args.factor_math)
    if math is None:
        return None
    v = ctypes.c_int32()
    key = f'lu_panel n={n} math={math}'.encode()
    if lib.pcbqs_gb300_tune_lookup(key, ctypes.byref(v)) == 0:
        return dict(lu_panel=v.value, source='tuning file')
    w = np.array(widths, np.int32)
    t0 = time.perf_counter()
    _lib.check(lib.pcbqs_gb300_tune_lu_panel(n, math, _lib.ptr(w, ctypes.c_int32), len(w), ctypes.byref(v),
                                             ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), lib)
    return dict(lu_panel=v.value, candidates=list(widths), source='timed', tuning_s=round(time.perf_counter() - t0, 2))


def main():
    args = parse()
    if args.case:
        return kernel_case(args.case)
    if args.impl == 'reference':
        return reference_arm(args)
    import torch
    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl')
    from pcbqs_gb300 import _lib, build
    build.build()
    lib = _lib.load()
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import PeecModel
    board = Board.load(args.board)
    freq = replica_frequency(args.freq, rank)
    model = PeecModel(board, device=local, inner_tol=args.inner_tol)

    mixed = args.mode == 'mixed'

    def step(mode_mixed=mixed):
        model.assemble(mixed=mode_mixed)
        return model.solve([freq], precondition=args.precondition, mixed=mode_mixed, factor_math=args.factor_math)

    autotune = autotune_lu_panel(lib, model.n, args) if args.precondition == 'lu32' else None
    for _ in range(args.warmup):
        result = step()
    torch.cuda.synchronize()
    launches0 = lib.pcbqs_gb300_kernel_launches()
    clocks = Clocks(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    timings = []
    for _ in range(args.steps):
        result = step()
        timings.append(dict(model.timings))
    e1.record()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clock_info = clocks.stop()
    launches = lib.pcbqs_gb300_kernel_launches() - launches0
    ms, value = job_seconds_per_frequency(e0.elapsed_time(e1) / args.steps, world, dist)
    Z_headline = result.impedance[0]
    comparator = None
    fp64_timings = timings[-1]
    if mixed and not args.no_comparator:
        # the FP64 fill + FP64 GMRES on the same step, once (after one warm-up), for the error and speed-up
        step(False)
        torch.cuda.synchronize()
        c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c0.record()
        r64 = step(False)
        c1.record()
        torch.cuda.synchronize()
        Z64 = r64.impedance[0]
        fp64_timings = dict(model.timings)
        comparator = dict(mode='fp64 fill + fp64 GMRES (complex64-LU preconditioned)',
                          s_per_freq=round(c0.elapsed_time(c1) / 1e3, 4),
                          speedup_of_mixed=round(c0.elapsed_time(c1) / ms, 3),
                          port_z_max_rel_err_of_mixed=float(np.abs(Z_headline - Z64).max() / np.abs(Z64).max()),
                          gmres_iterations=r64.iterations.tolist(),
                          breakdown_ms={k: round(fp64_timings.get(k, 0), 2) for k in
                                        ('fill_ms', 'combine_ms', 'potential_ms', 'precondition_ms', 'gmres_ms')})
    # fill GB/s: bytes of L and P written once per step, over the fill + combine + aggregation time
    ne, nn = model.ne, model.nn
    fill_ms = statistics.median(t['fill_ms'] + t['combine_ms'] + t['potential_ms'] for t in timings)
    fill_gbs = 8 * (ne * ne + nn * nn) / (fill_ms / 1e3) / 1e9
    # end to end through the public API from host arrays: a new model from the board's host arrays each time (the
    # median of three, each timed by the host clock around a synchronized call)
    e2e_runs = []
    for _ in range(3):
        torch.cuda.synchronize()
        t_e2e = time.perf_counter()
        m2 = PeecModel(Board.load(args.board), device=local, inner_tol=args.inner_tol)
        m2.assemble(mixed=mixed)
        r2 = m2.solve([freq], precondition=args.precondition, mixed=mixed, factor_math=args.factor_math)
        torch.cuda.synchronize()
        e2e_runs.append(time.perf_counter() - t_e2e)
        h2d = m2.fill.dev.nt * (64 + 32 + 192) + sum(a.nbytes for a in m2.fill.geometry.levels[1][5:6])
        h2d += 16 * m2.n * len(m2.names)                 # right-hand sides
        d2h = 16 * m2.n * len(m2.names) + r2.impedance.nbytes
        del m2, r2
        torch.cuda.empty_cache()
    e2e_s = statistics.median(e2e_runs)
    if rank != 0:
        return
    import torch as _torch
    peaks = dict(fp64=gemm_peak(_torch.float64), fp32=gemm_peak(_torch.float32))
    head_fill_ms = statistics.median(t['fill_ms'] for t in timings)
    # the port impedances against the reference's own dense solve of this board (tests/golden/peec_<board>.npz)
    z_err_ref = None
    golden = ROOT / 'tests' / 'golden' / f'peec_{args.board}.npz'
    if golden.exists():
        with np.load(golden) as ref:
            hit = np.flatnonzero(np.isclose(ref['freqs'], freq))
            if len(hit):
                Zr = ref['Z'][hit[0]]
                z_err_ref = dict(headline=float(np.abs(Z_headline - Zr).max() / np.abs(Zr).max()))
                if comparator:
                    z_err_ref['fp64_comparator'] = float(np.abs(Z64 - Zr).max() / np.abs(Zr).max())
    # pair integrals per second: the fill's unordered triangle pairs (far and near, each kind counted) over its time
    nt = model.fill.nt
    fr = fill_roofline(model, head_fill_ms, mixed, peaks)
    pair_rate = dict(value=round(nt * (nt + 1) / 2 / (head_fill_ms / 1e3), 1), unit='pairs/s',
                     far=fr['far_pairs'], near_level0=fr['near_pairs'][0], near_level1=fr['near_pairs'][1],
                     fill_ms=round(head_fill_ms, 2))
    if comparator:
        comparator['fill_roofline'] = fill_roofline(model, fp64_timings['fill_ms'], False, peaks)
    line = dict(metric=METRIC, value=round(value, 4), unit='s/freq', n_gpus=world, steps=args.steps,
                warmup=args.warmup, ms_per_step=round(ms, 2), higher_is_better=False, scaling='weak',
                vs_baseline=None, dtype='f32+f64' if mixed else 'f64', data='synthetic (seeded plane-pair board, CDT mesh)',
                config=board_config(args.board, args.freq, model.n, world),
                solver=dict(precondition=args.precondition, factor_math=args.factor_math, mode=args.mode,
                            gmres_tol=model.tol, gmres_iterations=result.iterations.tolist(),
                            gmres_outer_steps=timings[-1].get('outer_steps')),
                port_z_max_rel_err_vs_reference=z_err_ref,
                fill_gbs=round(fill_gbs, 2),
                pair_integrals_per_s=pair_rate,
                fp64_comparator=comparator,
                breakdown_ms={k: round(statistics.median(t.get(k, 0) for t in timings), 2)
                              for k in ('fill_ms', 'combine_ms', 'potential_ms', 'precondition_ms', 'gmres_ms')},
                host_s={k: round(statistics.median(t.get(k, 0) for t in timings), 3)
                        for k in ('equilibrium_s', 'potential_solve_s', 'operator_setup_s', 'rhs_s', 'solve_s')},
                gpu_launches=int(launches),
                autotune=autotune,
                clocks=clock_info,
                roofline=(factor_roofline(model, timings, args.factor_math)
                          if args.precondition == 'lu32' else fill_roofline(model, head_fill_ms, mixed, peaks)),
                fill_roofline=fill_roofline(model, head_fill_ms, mixed, peaks),
                e2e=dict(value=round(e2e_s, 4), unit='s/freq', runs_s=[round(v, 4) for v in e2e_runs],
                         h2d_bytes_per_step=int(h2d),
                         d2h_bytes_per_step=int(d2h)))
    head_n = model.n
    if args.plain:
        # the plain FP64 GPU path of the same step (FP64 fill, FP64 operator, block-Jacobi GMRES), timed once
        model.assemble(mixed=False)
        torch.cuda.synchronize()
        p0 = time.perf_counter()
        try:
            rp = model.solve([freq], precondition='block_jacobi', mixed=False)
            plain = dict(s_per_freq=round(time.perf_counter() - p0, 3), gmres_iterations=rp.iterations.tolist(),
                         max_residual=float(rp.residual.max()))
            if z_err_ref is not None:
                plain['port_z_max_rel_err_vs_reference'] = float(np.abs(rp.impedance[0] - Zr).max() / np.abs(Zr).max())
        except RuntimeError as exc:
            plain = dict(s_per_freq=round(time.perf_counter() - p0, 3), error=str(exc)[:200])
        plain['speedup_of_headline'] = round(plain['s_per_freq'] / value, 2)
        line['plain_fp64_block_jacobi'] = plain
    if args.sweep:
        # the batched sweep (config C3): every (frequency, port) column of the sweep board, `anchors` shared factors,
        # one batched GMRES per run of frequencies, each restart cycle one CUDA graph launch
        fs = np.geomspace(1e3, 1e8, args.sweep)
        if args.sweep_board != args.board:
            del model
            torch.cuda.empty_cache()
            model = PeecModel(Board.load(args.sweep_board), device=local, inner_tol=args.inner_tol)
        model.assemble(mixed=mixed)
        sweep_tune = autotune_lu_panel(lib, model.n, args)
        torch.cuda.synchronize()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record()
        rs = model.solve(fs, precondition='lu32', mixed=mixed, factor_math=args.factor_math,
                         anchors=min(args.anchors, args.sweep), captured=True, product=args.product)
        s1.record()
        torch.cuda.synchronize()
        its = rs.iterations.reshape(len(fs), -1)
        sweep_err = None
        golden = ROOT / 'tests' / 'golden' / f'peec_{args.sweep_board}.npz'
        if golden.exists():
            with np.load(golden) as ref:
                errs = []
                for f, Zr in zip(ref['freqs'], ref['Z']):
                    fi = int(np.argmin(np.abs(fs - f)))
                    if abs(fs[fi] / f - 1) < 1e-9:
                        errs.append([float(f), float(np.abs(rs.impedance[fi] - Zr).max() / np.abs(Zr).max())])
                sweep_err = errs or None
        line['sweep'] = dict(board=args.sweep_board, unknowns=model.n, captured_cycles=True,
                             inner_product=args.product, outer_steps=rs.timings.get('outer_steps'),
                             autotune=sweep_tune,
                             port_z_max_rel_err_vs_reference=sweep_err,
                             frequencies=len(fs), range_hz=[1e3, 1e8], ports=len(model.names),
                             columns=int(its.size), anchors=rs.timings['factorizations'],
                             s_total=round(s0.elapsed_time(s1) / 1e3, 3),
                             s_per_freq=round(s0.elapsed_time(s1) / 1e3 / len(fs), 4),
                             precondition_ms=round(rs.timings['precondition_ms'], 1),
                             gmres_ms=round(rs.timings['gmres_ms'], 1),
                             iterations_per_frequency_max=its.max(axis=1).tolist(),
                             max_residual=float(rs.residual.max()))
    if not args.no_cpu_baseline:
        v, details = cpu_sample(args.board, head_n)
        line['cpu_baseline'] = dict(value=round(v, 3), unit='s/freq', cores=details['cores'], kind='port',
                                    sample=f'oracle fill+combine+aggregation in full; dense solve = complex64 LU '
                                           f'estimated from a bounded sample (--impl reference runs it in full); '
                                           f'{details}')
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
