"""ctypes binding of the C ABI in include/pcbqs_gb300.h.

The library is built in-tree (pcbqs_gb300/build.py). There is no CPU fallback: if the library or a CUDA device is
missing, every entry point raises RuntimeError.
"""
import ctypes
import os
import threading
from pathlib import Path

import numpy as np

LIBRARY = Path(__file__).resolve().parent / 'libpcbqs_gb300.so'

STATUS = {0: 'ok', 1: 'invalid argument', 2: 'CUDA error', 3: 'non-finite result', 4: 'device allocation failed',
          5: 'no convergence', 6: 'bounded device wait gave up'}
OK, ERR_ARGUMENT, ERR_CUDA, ERR_NONFINITE, ERR_MEMORY, ERR_CONVERGENCE, ERR_TIMEOUT = range(7)

c_double_p = ctypes.POINTER(ctypes.c_double)
c_int32_p = ctypes.POINTER(ctypes.c_int32)
c_int64_p = ctypes.POINTER(ctypes.c_int64)
c_uint64_p = ctypes.POINTER(ctypes.c_uint64)
c_uint8_p = ctypes.POINTER(ctypes.c_uint8)
c_void_p = ctypes.c_void_p


class Geometry(ctypes.Structure):
    """pcbqs_gb300_geometry: host views of a prepared fill geometry."""
    _fields_ = [('nt', ctypes.c_int32),
                ('v', c_double_p), ('len', c_double_p), ('tau', c_double_p), ('un', c_double_p),
                ('area', c_double_p), ('p3', c_double_p), ('cent', c_double_p), ('radius', c_double_p),
                ('z', c_double_p),
                ('qp', c_double_p * 3), ('qw', c_double_p * 3), ('nq', ctypes.c_int32 * 3)]


class CsrDesc(ctypes.Structure):
    """pcbqs_gb300_csr: a device CSR matrix."""
    _fields_ = [('rows', ctypes.c_int64), ('cols', ctypes.c_int64), ('ptr', c_void_p), ('idx', c_void_p),
                ('val', c_void_p)]


class HmatDesc(ctypes.Structure):
    """pcbqs_gb300_hmat: a packed H-matrix's device arrays."""
    _fields_ = [('n', ctypes.c_int64), ('nblocks', ctypes.c_int64), ('nslots', ctypes.c_int64), ('meta', c_void_p),
                ('slot0', c_void_p), ('idx', c_void_p), ('row_ptr', c_void_p), ('slots_of_row', c_void_p),
                ('store', c_void_p), ('max_rank', ctypes.c_int32)]


class GraphDomainsDesc(ctypes.Structure):
    """pcbqs_gb300_graph_domains: the Laplacian's domain split (dom_ptr, bnd_ptr host arrays)."""
    _fields_ = [('parts', ctypes.c_int64), ('n_int', ctypes.c_int64), ('perm', c_void_p), ('pos', c_void_p),
                ('dom_ptr', c_void_p), ('bnd_ptr', c_void_p), ('bnd', c_void_p), ('bnd_nptr', c_void_p),
                ('bnd_local', c_void_p), ('bnd_branch', c_void_p)]


class GraphDesc(ctypes.Structure):
    """pcbqs_gb300_graph: the graph preconditioner's device arrays and one frequency's values."""
    _fields_ = [('nkeep', ctypes.c_int64), ('ncomp', ctypes.c_int64), ('nbranch', ctypes.c_int64), ('ac', CsrDesc),
                ('lap_ptr', c_void_p), ('lap_branch', c_void_p), ('lap_other', c_void_p), ('tinv', CsrDesc),
                ('tinvt', CsrDesc), ('branch', c_void_p), ('loop_ends', c_void_p), ('comp', c_void_p),
                ('member_ptr', c_void_p), ('members', c_void_p), ('zdiag', c_void_p), ('dinv', c_void_p),
                ('pinv', c_void_p), ('total', c_void_p), ('domains', ctypes.POINTER(GraphDomainsDesc))]


class LowRankDesc(ctypes.Structure):
    """pcbqs_gb300_lowrank: an H-matrix's low-rank blocks packed for the tensor cores."""
    _fields_ = [('meta_dense', c_void_p), ('slot0_dense', c_void_p), ('ndense', ctypes.c_int64), ('lplane', c_void_p),
                ('lrows', ctypes.c_int64), ('rplane', c_void_p), ('rwidth', ctypes.c_int64), ('groups', c_void_p),
                ('ngroups', ctypes.c_int32), ('ntiles', ctypes.c_int32), ('tile_group', c_void_p),
                ('tile_m', c_void_p), ('pad_pos', c_void_p), ('n_pad', ctypes.c_int64), ('dplane', c_void_p),
                ('drows', ctypes.c_int64), ('dpitch', ctypes.c_int64), ('dgroups', c_void_p),
                ('ndgroups', ctypes.c_int32), ('ndtiles', ctypes.c_int32), ('dtile_group', c_void_p),
                ('dtile_m', c_void_p)]


class PeecDesc(ctypes.Structure):
    """pcbqs_gb300_peec_desc: the loop/tree PEEC operator's device arrays and frequencies."""
    _fields_ = [('n', ctypes.c_int64), ('nb', ctypes.c_int64), ('ne', ctypes.c_int64), ('nn', ctypes.c_int64),
                ('K', CsrDesc), ('Kt', CsrDesc), ('T', CsrDesc), ('Tt', CsrDesc), ('R', CsrDesc),
                ('L', c_void_p), ('ldl', ctypes.c_int64), ('P', c_void_p), ('ldp', ctypes.c_int64),
                ('is_tree', c_void_p), ('pscale', ctypes.c_double), ('nsys', ctypes.c_int32),
                ('omega', c_double_p), ('zscale', c_double_p), ('rscale', c_double_p), ('Pim', c_void_p),
                ('nscaled', ctypes.c_int64)]


# name: (restype, argtypes)
PROTOTYPES = {
    'pcbqs_gb300_create': (ctypes.c_int, [ctypes.POINTER(Geometry), ctypes.c_int, ctypes.POINTER(c_void_p)]),
    'pcbqs_gb300_destroy': (None, [c_void_p]),
    'pcbqs_gb300_last_error': (ctypes.c_char_p, []),
    'pcbqs_gb300_triangles': (ctypes.c_int32, [c_void_p]),
    'pcbqs_gb300_kernel_launches': (ctypes.c_int64, []),
    'pcbqs_gb300_release_memory': (ctypes.c_int, [ctypes.c_int]),
    'pcbqs_gb300_fill_counts': (ctypes.c_int, [c_void_p, c_uint64_p]),
    'pcbqs_gb300_pairs': (ctypes.c_int, [c_void_p, c_int32_p, c_int32_p, c_double_p, c_int32_p, ctypes.c_int64,
                                         ctypes.c_int, c_double_p]),
    'pcbqs_gb300_pairs_device': (ctypes.c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, ctypes.c_int64,
                                                ctypes.c_int, c_void_p, c_void_p]),
    'pcbqs_gb300_pairs_no_alloc': (ctypes.c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                                  ctypes.c_int64, ctypes.c_int, c_void_p, c_void_p]),
    'pcbqs_gb300_fill': (ctypes.c_int, [c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                        ctypes.POINTER(c_void_p), c_uint64_p]),
    'pcbqs_gb300_fill_device': (ctypes.c_int, [c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                               ctypes.POINTER(c_void_p), ctypes.c_int64, c_uint64_p, c_void_p]),
    'pcbqs_gb300_edge_inductance_device': (ctypes.c_int, [ctypes.c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                                          ctypes.c_double, c_void_p, c_void_p, c_void_p, c_void_p,
                                                          ctypes.c_int64, c_void_p, ctypes.c_int64, c_void_p]),
    'pcbqs_gb300_edge_inductance': (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, c_int32_p, c_double_p,
                                                   c_double_p, c_double_p, ctypes.c_double, c_double_p, c_double_p,
                                                   c_double_p, c_double_p, c_double_p]),
    'pcbqs_gb300_potential_device': (ctypes.c_int, [ctypes.c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                                    ctypes.c_int64, ctypes.c_double, c_void_p, ctypes.c_int64,
                                                    c_void_p]),
    'pcbqs_gb300_fill_local_device': (ctypes.c_int, [c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                                     ctypes.POINTER(c_void_p), ctypes.c_int64, c_uint64_p, c_void_p]),
    'pcbqs_gb300_edge_inductance_local_device': (ctypes.c_int, [ctypes.c_int64, c_void_p, c_void_p, c_void_p,
                                                                c_void_p, ctypes.c_double, c_void_p, c_void_p,
                                                                c_void_p, c_void_p, ctypes.c_int64, c_void_p,
                                                                ctypes.c_int64, c_void_p, ctypes.c_int64, c_void_p]),
    'pcbqs_gb300_potential_single_device': (ctypes.c_int, [ctypes.c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                                           ctypes.c_int64, ctypes.c_double, c_void_p, c_void_p,
                                                           ctypes.c_int64, c_void_p]),
    'pcbqs_gb300_hmatrix_build': (ctypes.c_int, [c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int, c_void_p,
                                                 c_void_p,
                                                 c_void_p, ctypes.c_int64, ctypes.c_double, c_void_p, c_void_p,
                                                 ctypes.c_int64, c_void_p, ctypes.c_int64, c_void_p, ctypes.c_double,
                                                 c_void_p, c_void_p, ctypes.c_int64, c_void_p]),
    'pcbqs_gb300_hmatrix_apply': (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, c_void_p, c_void_p, c_void_p,
                                                 c_void_p, c_void_p, c_void_p, ctypes.c_int, ctypes.c_int, c_void_p,
                                                 c_void_p, c_void_p, c_void_p]),
    'pcbqs_gb300_loop_basis': (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, c_int32_p, c_int32_p, c_uint8_p,
                                              ctypes.c_int64, ctypes.c_int, c_uint8_p, ctypes.c_int64, c_int32_p,
                                              c_int32_p, c_double_p, c_int64_p, c_int32_p, c_int64_p]),
    'pcbqs_gb300_layered_device': (ctypes.c_int, [c_void_p, ctypes.c_double, ctypes.c_int, c_void_p, ctypes.c_int64,
                                                  c_void_p, ctypes.c_int64, ctypes.c_int, c_void_p, c_void_p,
                                                  ctypes.c_int, c_void_p, c_void_p, ctypes.c_int64, ctypes.c_double,
                                                  c_void_p, c_void_p, ctypes.c_int64, c_void_p]),
    'pcbqs_gb300_biot_sheets': (ctypes.c_int, [ctypes.c_int64, c_void_p, ctypes.c_int64, c_void_p, c_void_p,
                                               c_void_p, ctypes.c_int, ctypes.c_int, c_void_p, c_void_p]),
    'pcbqs_gb300_biot_segments': (ctypes.c_int, [ctypes.c_int64, c_void_p, ctypes.c_int64, c_void_p, c_void_p,
                                                 c_void_p, ctypes.c_int, c_void_p, c_void_p]),
    'pcbqs_gb300_current_deposit': (ctypes.c_int, [ctypes.c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                                   ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                                   ctypes.c_double, ctypes.c_int64, ctypes.c_int64, c_void_p,
                                                   c_void_p, c_void_p]),
    'pcbqs_gb300_peec_create': (ctypes.c_int, [ctypes.POINTER(PeecDesc), ctypes.POINTER(c_void_p)]),
    'pcbqs_gb300_peec_destroy': (None, [c_void_p]),
    'pcbqs_gb300_peec_apply': (ctypes.c_int, [c_void_p, ctypes.c_int, c_int32_p, c_void_p, c_void_p, c_void_p]),
    'pcbqs_gb300_peec_block_jacobi': (ctypes.c_int, [c_void_p, ctypes.c_int32, c_void_p, c_void_p]),
    'pcbqs_gb300_peec_graph': (ctypes.c_int, [c_void_p, ctypes.POINTER(GraphDesc), ctypes.c_int32, ctypes.c_int,
                                              c_void_p]),
    'pcbqs_gb300_pack_bf16_parts': (ctypes.c_int, [c_void_p, c_void_p, ctypes.c_int64, c_void_p, c_void_p,
                                                   ctypes.c_int64, ctypes.c_int64, c_void_p]),
    'pcbqs_gb300_peec_graph_apply': (ctypes.c_int, [c_void_p, ctypes.c_int, c_void_p, c_void_p, c_void_p]),
    'pcbqs_gb300_peec_factor': (ctypes.c_int, [c_void_p, ctypes.POINTER(CsrDesc), ctypes.c_int32, ctypes.c_int,
                                               c_void_p]),
    'pcbqs_gb300_peec_lu_solve': (ctypes.c_int, [c_void_p, ctypes.c_int, c_void_p, c_void_p, ctypes.c_int,
                                                 c_void_p]),
    'pcbqs_gb300_peec_factor_times': (ctypes.c_int, [c_void_p, ctypes.POINTER(ctypes.c_double),
                                                     ctypes.POINTER(ctypes.c_double)]),
    'pcbqs_gb300_peec_set_captured': (ctypes.c_int, [c_void_p, ctypes.c_int]),
    'pcbqs_gb300_peec_set_product': (ctypes.c_int, [c_void_p, ctypes.c_int]),
    'pcbqs_gb300_hmatrix_apply_lowrank': (ctypes.c_int, [c_void_p, c_void_p, ctypes.c_int, c_void_p, c_void_p,
                                                         c_void_p]),
    'pcbqs_gb300_peec_set_lowrank': (ctypes.c_int, [c_void_p, ctypes.c_int, c_void_p]),
    'pcbqs_gb300_peec_set_compressed': (ctypes.c_int, [c_void_p, c_void_p, c_void_p, ctypes.c_int64, c_void_p,
                                                       c_void_p, c_void_p]),
    'pcbqs_gb300_peec_block_jacobi_blocks': (ctypes.c_int, [c_void_p, ctypes.c_int32, c_void_p, c_void_p, c_void_p,
                                                            c_void_p]),
    'pcbqs_gb300_peec_potential_gmres': (ctypes.c_int, [c_void_p, ctypes.c_int, c_void_p, c_void_p, c_void_p,
                                                        ctypes.c_double, ctypes.c_int, ctypes.c_int, c_int32_p,
                                                        c_void_p, c_void_p]),
    'pcbqs_gb300_peec_set_fp64_product': (ctypes.c_int, [c_void_p, ctypes.c_int]),
    'pcbqs_gb300_tune_file': (ctypes.c_int, [ctypes.c_char_p]),
    'pcbqs_gb300_tune_lookup': (ctypes.c_int, [ctypes.c_char_p, c_int32_p]),
    'pcbqs_gb300_tune_count': (ctypes.c_int64, []),
    'pcbqs_gb300_tune_record': (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int32]),
    'pcbqs_gb300_tune_clear': (None, []),
    'pcbqs_gb300_tune_lu_panel': (ctypes.c_int, [ctypes.c_int64, ctypes.c_int, c_int32_p, ctypes.c_int, c_int32_p,
                                                 c_void_p]),
    'pcbqs_gb300_peec_factor_updates': (ctypes.c_int, [c_void_p, ctypes.POINTER(ctypes.c_double),
                                                       ctypes.POINTER(ctypes.c_double), c_int32_p]),
    'pcbqs_gb300_via_inductance': (ctypes.c_int, [ctypes.c_int64, c_void_p, ctypes.c_double, c_void_p,
                                                  ctypes.c_int64, c_void_p]),
    'pcbqs_gb300_learned_forward': (ctypes.c_int, [ctypes.c_int64, ctypes.c_int, ctypes.c_int, c_void_p, c_void_p,
                                                   c_void_p, c_void_p, c_void_p]),
    'pcbqs_gb300_learned_backward': (ctypes.c_int, [ctypes.c_int64, ctypes.c_int, ctypes.c_int, c_void_p, c_void_p,
                                                    c_void_p, c_void_p, c_void_p, c_void_p]),
    'pcbqs_gb300_learned_apply': (ctypes.c_int, [ctypes.c_int64, ctypes.c_int, ctypes.c_int64, c_void_p, c_void_p,
                                                 c_void_p, c_void_p, c_void_p, ctypes.c_int, c_void_p, c_void_p,
                                                 c_void_p, c_void_p]),
    'pcbqs_gb300_learned_edge_dots': (ctypes.c_int, [ctypes.c_int64, ctypes.c_int, ctypes.c_int64, c_void_p,
                                                     ctypes.c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    'pcbqs_gb300_learned_gmres': (ctypes.c_int, [ctypes.c_int64, c_void_p, ctypes.c_int64, ctypes.c_int, c_void_p,
                                                 c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                                 c_int32_p, c_double_p, c_void_p]),
    'pcbqs_gb300_lu_factor_c64': (ctypes.c_int, [ctypes.c_int64, c_void_p, c_void_p, ctypes.c_int, ctypes.c_int,
                                                 c_int32_p, c_void_p]),
    'pcbqs_gb300_set_wait_cycles': (ctypes.c_int, [ctypes.c_uint64]),
    'pcbqs_gb300_complex_update': (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.c_int, c_void_p,
                                                  ctypes.c_int64, c_void_p, ctypes.c_int64, c_void_p, ctypes.c_int64,
                                                  ctypes.c_int, ctypes.c_uint64, c_void_p]),
    'pcbqs_gb300_cholesky_f32': (ctypes.c_int, [ctypes.c_int64, c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                                c_int32_p, c_void_p]),
    'pcbqs_gb300_dense_apply': (ctypes.c_int, [ctypes.c_int64, ctypes.c_int, c_void_p, ctypes.c_int64, c_void_p,
                                               c_void_p, c_void_p]),
    'pcbqs_gb300_dense_apply_single': (ctypes.c_int, [ctypes.c_int64, ctypes.c_int, c_void_p, ctypes.c_int64,
                                                      c_void_p, c_void_p, c_void_p]),
    'pcbqs_gb300_dense_apply_tensor': (ctypes.c_int, [ctypes.c_int64, ctypes.c_int, c_void_p, ctypes.c_int64,
                                                      c_void_p, c_void_p, ctypes.c_int, ctypes.c_uint64, c_void_p]),
    'pcbqs_gb300_dense_apply_sliced': (ctypes.c_int, [ctypes.c_int64, ctypes.c_int, c_void_p, ctypes.c_int64,
                                                      c_void_p, c_void_p, ctypes.c_int, ctypes.c_uint64, c_void_p]),
    'pcbqs_gb300_to_single': (ctypes.c_int, [c_void_p, c_void_p, ctypes.c_int64, c_void_p]),
    'pcbqs_gb300_peec_single': (ctypes.c_int, [c_void_p, c_void_p, ctypes.c_int64, c_void_p, c_void_p,
                                               ctypes.c_int64]),
    'pcbqs_gb300_peec_solve_mixed': (ctypes.c_int, [c_void_p, ctypes.c_int, c_int32_p, c_void_p, c_void_p,
                                                    ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                                    ctypes.c_int, ctypes.c_int, c_int32_p, c_double_p, c_int32_p,
                                                    c_void_p]),
    'pcbqs_gb300_peec_gmres': (ctypes.c_int, [c_void_p, ctypes.c_int, c_int32_p, c_void_p, c_void_p, ctypes.c_double,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_int, c_int32_p, c_double_p,
                                              c_void_p]),
    'pcbqs_gb300_dense_gmres': (ctypes.c_int, [ctypes.c_int64, c_void_p, c_void_p, ctypes.c_int64, ctypes.c_int,
                                               c_void_p, c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_int, c_int32_p, c_double_p, c_void_p]),
}

_lock = threading.Lock()
_lib = None


class DeviceError(RuntimeError):
    """A status returned by the C ABI."""
    def __init__(self, status, message):
        self.status = status
        super().__init__(message)


def load():
    """The loaded library, with prototypes set. Raises RuntimeError when it was not built."""
    global _lib
    with _lock:
        if _lib is None:
            path = Path(os.environ.get('PCBQS_GB300_LIBRARY', LIBRARY))
            if not path.exists():
                raise RuntimeError(f'pcbqs_gb300 library not built ({path}): run python -m pcbqs_gb300.build')
            lib = ctypes.CDLL(str(path))
            for name, (restype, argtypes) in PROTOTYPES.items():
                fn = getattr(lib, name)
                fn.restype, fn.argtypes = restype, argtypes
            _lib = lib
        return _lib


def check(status, lib=None):
    """Raise the Python exception matching a C status (FloatingPointError for non-finite results)."""
    if status == 0:
        return
    lib = lib or load()
    message = (lib.pcbqs_gb300_last_error() or b'').decode(errors='replace') or STATUS.get(status, str(status))
    if status == 3:
        raise FloatingPointError(message)
    if status == 1:
        raise ValueError(message)
    raise DeviceError(status, message)


def ptr(array, ctype=ctypes.c_double):
    """ctypes pointer to a C-contiguous numpy array's data."""
    if not array.flags.c_contiguous:
        raise ValueError('array must be C-contiguous')
    return array.ctypes.data_as(ctypes.POINTER(ctype))


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)
