"""The autotuner's memory (pcbqs_gb300_tune_*): choices kept per device and size, read from and written back to a
tuning file so that a later process takes them without timing. The CPU cases need no GPU (the device prefix is then
"unknown/0/"); the GPU case times the blocked LU's panel widths and finds the choice in the file."""
import ctypes
import shutil
from pathlib import Path

import numpy as np
import pytest

from pcbqs_gb300 import _lib

TUNE_DIR = Path(__file__).parent / '_tune'


@pytest.fixture
def tune_dir():
    shutil.rmtree(TUNE_DIR, ignore_errors=True)
    TUNE_DIR.mkdir()
    lib = _lib.load()
    yield TUNE_DIR
    lib.pcbqs_gb300_tune_file(None)
    lib.pcbqs_gb300_tune_clear()
    shutil.rmtree(TUNE_DIR, ignore_errors=True)


def test_tuning_file_round_trip(tune_dir):
    lib = _lib.load()
    lib.pcbqs_gb300_tune_clear()
    path = tune_dir / 'tune.txt'
    assert lib.pcbqs_gb300_tune_file(str(path).encode()) == 0
    assert lib.pcbqs_gb300_tune_record(b'dense_f32 rows=5', 3) == 0
    assert lib.pcbqs_gb300_tune_record(b'trisolve n=100 columns=32', 1) == 0
    v = ctypes.c_int32()
    assert lib.pcbqs_gb300_tune_lookup(b'dense_f32 rows=5', ctypes.byref(v)) == 0 and v.value == 3
    assert lib.pcbqs_gb300_tune_lookup(b'trisolve n=100 columns=32', ctypes.byref(v)) == 0 and v.value == 1
    assert lib.pcbqs_gb300_tune_lookup(b'dense_f32 rows=6', ctypes.byref(v)) == _lib.ERR_ARGUMENT
    assert lib.pcbqs_gb300_tune_count() == 2
    # the file is rewritten whole after each choice: tab-separated, the device's name and SM count before each key
    lines = path.read_text().splitlines()
    assert sorted(lines) == lines and len(lines) == 2
    assert lines[0].endswith('/dense_f32 rows=5\t3') and lines[1].endswith('/trisolve n=100 columns=32\t1')
    # a fresh memory (a later process) reads them back
    lib.pcbqs_gb300_tune_clear()
    assert lib.pcbqs_gb300_tune_count() == 0
    assert lib.pcbqs_gb300_tune_file(str(path).encode()) == 0
    assert lib.pcbqs_gb300_tune_lookup(b'dense_f32 rows=5', ctypes.byref(v)) == 0 and v.value == 3
    assert lib.pcbqs_gb300_tune_record(b'bad\tkey', 1) == _lib.ERR_ARGUMENT


def test_tuning_file_rejects_malformed_lines(tune_dir):
    lib = _lib.load()
    lib.pcbqs_gb300_tune_clear()
    path = tune_dir / 'good.txt'
    assert lib.pcbqs_gb300_tune_file(str(path).encode()) == 0
    assert lib.pcbqs_gb300_tune_record(b'y', 7) == 0
    good = path.read_text().strip()
    bad = tune_dir / 'bad.txt'
    bad.write_text('no value here\n' + good.replace('\t7', '\tnot-a-number') + '\n' + good + '\n')
    lib.pcbqs_gb300_tune_clear()
    assert lib.pcbqs_gb300_tune_file(str(bad).encode()) == _lib.ERR_ARGUMENT
    v = ctypes.c_int32()
    assert lib.pcbqs_gb300_tune_lookup(b'y', ctypes.byref(v)) == 0 and v.value == 7     # the good line is kept


@pytest.mark.gpu
def test_lu_panel_width_is_tuned_and_persisted(device_library, tune_dir):
    import torch
    lib = device_library
    lib.pcbqs_gb300_tune_clear()
    path = tune_dir / 'tune.txt'
    assert lib.pcbqs_gb300_tune_file(str(path).encode()) == 0
    widths = np.array([512, 1024], np.int32)
    best = ctypes.c_int32()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.pcbqs_gb300_tune_lu_panel(3000, 3, _lib.ptr(widths, ctypes.c_int32), 2, ctypes.byref(best),
                                             stream), lib)
    assert best.value in (512, 1024)
    text = path.read_text()
    assert f'lu_panel n=3000 math=3\t{best.value}' in text
    lib.pcbqs_gb300_tune_clear()
    assert lib.pcbqs_gb300_tune_file(str(path).encode()) == 0
    v = ctypes.c_int32()
    assert lib.pcbqs_gb300_tune_lookup(b'lu_panel n=3000 math=3', ctypes.byref(v)) == 0 and v.value == best.value
