"""Build the sm_103a shared library `libpcbqs_gb300.so` in-tree from `csrc/*.cu` with nvcc.

    python -m pcbqs_gb300.build [--force]

Each translation unit compiles in parallel to an object under `_build/`, then one `nvcc -shared` link. The
library is plain C ABI (include/pcbqs_gb300.h) with the CUDA runtime linked statically, so it loads with ctypes
and needs no PyTorch.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / 'csrc'
BUILD = HERE / '_build'
LIBRARY = HERE / 'libpcbqs_gb300.so'
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr']


def nvcc():
    path = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not Path(path).exists():
        raise RuntimeError('nvcc not found: the CUDA 13 toolkit is required to build pcbqs_gb300')
    return path


def sources():
    return sorted(CSRC.glob('*.cu'))


def _stale(target, deps):
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force=False, verbose=False, extra=()):
    """Compile (when sources changed) and return the library path."""
    headers = list(CSRC.glob('*.cuh')) + list((HERE.parent / 'include').glob('*.h'))
    BUILD.mkdir(exist_ok=True)
    compiler = nvcc()
    jobs = []
    for src in sources():
        obj = BUILD / (src.stem + '.o')
        if force or _stale(obj, [src, *headers]):
            jobs.append([compiler, *ARCH, *FLAGS, *extra, '-c', str(src), '-o', str(obj)])

    def run(cmd):
        result = subprocess.run(cmd, capture_output=True, text=True)
        if result.returncode:
            raise RuntimeError(f'nvcc failed: {" ".join(cmd)}\n{result.stdout}\n{result.stderr}')
        if verbose and (result.stdout or result.stderr):
            print(result.stdout, result.stderr, file=sys.stderr)
        return result

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as pool:
        list(pool.map(run, jobs))
    objects = [BUILD / (s.stem + '.o') for s in sources()]
    if force or jobs or _stale(LIBRARY, objects):
        tmp = LIBRARY.with_suffix('.so.tmp')
        run([compiler, *ARCH, '-shared', '-o', str(tmp), *map(str, objects), '-lcublas', '-lcusolver',
             '-Xlinker', f'-rpath={Path(compiler).resolve().parent.parent / "lib64"}'])
        os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))
