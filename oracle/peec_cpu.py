"""CPU timing of the reference's dense PEEC solve for the benchmark's reference arm -- TEST INFRASTRUCTURE ONLY.

The reference solves a dense PEEC system per frequency by LU: peec.solve -> kernels.peec_system ->
lu_factor_rows, which is MixedLU (a complex64 LAPACK getrf refined to double accuracy) for systems of 4,000 unknowns
or more (src/pcbqs/peec.py:245-290, src/pcbqs/kernels.py:122-181). Its cost is the O(n^3) factorization; the
refinement and the system assembly are O(n^2). `lu_seconds` times LAPACK's complex64 getrf (SciPy, every BLAS
thread) on a bounded sample size and scales it by (n / sample)^3 to the system's size.
"""
import time

import numpy as np
import scipy.linalg as sl


def lu_seconds(n, sample=3072, repeats=2, seed=0):
    """Estimated seconds of a complex64 LU of an n x n matrix, from a timed `sample`-sized one."""
    rng = np.random.default_rng(seed)
    a = (rng.standard_normal((sample, sample)) + 1j * rng.standard_normal((sample, sample))).astype(np.complex64)
    a += sample * np.eye(sample, dtype=np.complex64)
    best = np.inf
    for _ in range(repeats):
        m = a.copy(order='F')
        t = time.perf_counter()
        sl.lu_factor(m, overwrite_a=True, check_finite=False)
        best = min(best, time.perf_counter() - t)
    return best * (n / sample) ** 3, best
