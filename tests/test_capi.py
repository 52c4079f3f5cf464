"""The C-ABI library builds for sm_103a, loads, and exports every entry point include/*.h declares (no GPU
calls here)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared():
    names = set()
    for header in (ROOT / 'include').glob('*.h'):
        text = re.sub(r'/\*.*?\*/', '', header.read_text(), flags=re.S)
        names |= set(re.findall(r'\b(pcbqs_gb300_\w+)\s*\(', text))
    return names


def test_header_declares_entry_points():
    names = declared()
    assert {'pcbqs_gb300_create', 'pcbqs_gb300_pairs', 'pcbqs_gb300_fill', 'pcbqs_gb300_fill_device',
            'pcbqs_gb300_edge_inductance_device', 'pcbqs_gb300_potential_device'} <= names


def test_library_exports_every_declared_symbol():
    from pcbqs_gb300 import build, _lib
    path = build.build()
    lib = ctypes.CDLL(str(path))
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding carries a prototype for every declared entry point
    assert declared() <= set(_lib.PROTOTYPES)


def test_library_reports_errors_without_a_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip('a device is present: covered by the GPU tests')
    from pcbqs_gb300 import _lib
    lib = _lib.load()
    g = _lib.Geometry()
    g.nt = 0
    handle = ctypes.c_void_p()
    status = lib.pcbqs_gb300_create(ctypes.byref(g), 0, ctypes.byref(handle))
    assert status == 1 and b'no triangles' in lib.pcbqs_gb300_last_error()
