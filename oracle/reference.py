"""Import the reference pcbqs package from its read-only checkout, with its compiled core built into oracle/_ref/.

TEST INFRASTRUCTURE ONLY, and only in the container that holds the reference checkout: the golden-vector
generators (tests/golden/*.py) and the optional reference-arm tests use it. Nothing on the GPU path does.
"""
import glob
import importlib.machinery
import importlib.util
import os
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
_SOURCE = os.environ.get('PCBQS_REFERENCE_SRC')      # the reference checkout's src/ directory (required)
SOURCE = Path(_SOURCE) if _SOURCE else None


def available():
    return SOURCE is not None and (SOURCE / 'pcbqs' / '__init__.py').exists()


def load_reference(build=True):
    """The reference `pcbqs` package with `pcbqs._core` taken from oracle/_ref (built from its sources if
    needed). Raises ImportError when the checkout is absent."""
    if 'pcbqs' in sys.modules and hasattr(sys.modules['pcbqs'], '_core'):
        return sys.modules['pcbqs']
    if not available():
        raise ImportError(f'reference checkout not found (PCBQS_REFERENCE_SRC={SOURCE}): set it to the checkout\'s src '
                          'directory')
    found = sorted(glob.glob(str(HERE / '_ref' / '_core*.so')))
    if not found and build:
        from .oracle import build_reference
        build_reference()
        found = sorted(glob.glob(str(HERE / '_ref' / '_core*.so')))
    if str(SOURCE) not in sys.path:
        sys.path.insert(0, str(SOURCE))
    if found and 'pcbqs._core' not in sys.modules:
        loader = importlib.machinery.ExtensionFileLoader('pcbqs._core', found[0])
        spec = importlib.util.spec_from_loader('pcbqs._core', loader)
        module = importlib.util.module_from_spec(spec)
        loader.exec_module(module)
        sys.modules['pcbqs._core'] = module
    import pcbqs
    if 'pcbqs._core' in sys.modules:
        pcbqs._core = sys.modules['pcbqs._core']
    return pcbqs
