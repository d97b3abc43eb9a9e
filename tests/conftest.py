import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / 'tests' / 'golden'
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300, sm_103a) and the built libsosb')


def fixture_names():
    return [n for n in ('walk1', 'strato1', 'strato15', 'slow1', 'aer2', 'mie1', 'mie15') if (GOLDEN / f'{n}.npz').exists()]


@pytest.fixture(scope='session')
def host_transport_lib():
    """g++ build of the device transport (sos_math.cuh) for CPU checks."""
    import ctypes
    from sosfuse2_gb300 import _abi

    src = ROOT / 'tests' / 'native' / 'host_transport.cpp'
    out = ROOT / 'tests' / 'native' / '_build' / 'libhost_transport.so'
    deps = [src, ROOT / 'sosfuse2_gb300' / 'csrc' / 'sos_math.cuh', ROOT / 'sosfuse2_gb300' / 'csrc' / 'sos_pack.h',
            ROOT / 'include' / 'sosb.h']
    if not out.exists() or any(d.stat().st_mtime > out.stat().st_mtime for d in deps):
        out.parent.mkdir(parents=True, exist_ok=True)
        subprocess.run(['g++', '-O2', '-std=c++17', '-ffp-contract=off', '-fPIC', '-shared', str(src), '-o',
                        str(out)], check=True)
    lib = ctypes.CDLL(str(out))
    lib.host_transport.argtypes = [ctypes.POINTER(_abi.Dims), ctypes.POINTER(_abi.Constants),
                                   ctypes.POINTER(_abi.Bundle), ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]
    return lib


def rel_max(a, b):
    """max |a - b| / max |b|"""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))


def rel_l2_per_wave(a, b):
    """Source relative L2 per wavelength (the reference's numeric-gate measure)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    num = np.sqrt(np.sum((a - b) ** 2, axis=(0, 1)))
    den = np.maximum(np.sqrt(np.sum(b ** 2, axis=(0, 1))), 1e-300)
    return num / den


def ray_index(state, cells):
    off = state['cell_cell_off']
    return np.concatenate([np.arange(off[i], off[i + 1]) for i in cells])


def reference_history(meta):
    """The reference solve's per-evaluation (observer_relative, source_relative) arrays [evaluations, W]."""
    return np.asarray(meta['history_observer'], np.float64), np.asarray(meta['history_source'], np.float64)
