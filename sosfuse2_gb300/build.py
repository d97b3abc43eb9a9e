"""In-tree build of libsosb.so for sm_103a (one translation unit, nvcc)."""

import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / 'csrc'
OUT = PKG / '_lib' / 'libsosb.so'
SOURCES = [CSRC / 'sosb.cu', CSRC / 'tc_gemm.cu']
HEADERS = [CSRC / 'sos_math.cuh', CSRC / 'sos_pack.h', CSRC / 'tc_ptx.cuh', PKG.parent / 'include' / 'sosb.h']

NVCC_FLAGS = [
    '-gencode', 'arch=compute_103a,code=sm_103a',
    '-O3', '-lineinfo', '-std=c++17',
    '-ftz=true',           # the reference's device arithmetic: FP32 subnormals flushed
    '-Xcompiler', '-fPIC', '-shared', '--threads', '2',
]


def nvcc():
    exe = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not Path(exe).exists():
        raise RuntimeError('E_BUILD: nvcc not found')
    return exe


def stale():
    if not OUT.exists():
        return True
    t = OUT.stat().st_mtime
    return any(p.stat().st_mtime > t for p in SOURCES + HEADERS)


def build(force=False, verbose=False):
    """Compile libsosb.so if any source is newer than the library; returns its path."""
    if not force and not stale():
        return OUT
    OUT.parent.mkdir(parents=True, exist_ok=True)
    tmp = OUT.with_suffix('.so.tmp%d' % os.getpid())
    cmd = [nvcc(), *NVCC_FLAGS, '-o', str(tmp), *map(str, SOURCES)]
    if verbose:
        cmd.insert(1, '-Xptxas=-v')
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('E_BUILD: nvcc failed\n' + r.stdout + r.stderr)
    os.replace(tmp, OUT)
    if verbose:
        print(r.stdout + r.stderr)
    return OUT


if __name__ == '__main__':
    import sys

    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))
