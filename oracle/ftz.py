"""FP32 flush-to-zero mode of the host FPU, for the oracle only (test infrastructure).

The device build computes with -ftz=true: subnormal FP32 inputs and results are zero. The oracle reproduces that on
the CPU by setting the FPU control word around its FP32 arithmetic (x86-64 MXCSR FTZ|DAZ, AArch64 FPCR.FZ), the mode
the reference's NumPy mirror runs in (src/sosfuse2/backends/numpy_reference.py:19-78). An unsupported platform raises
instead of silently computing with subnormals.
"""

import contextlib
import ctypes
import ctypes.util
import platform

import numpy as np

_TINY = np.float32(np.finfo(np.float32).tiny)


class _X86Env(ctypes.Structure):
    _fields_ = [('x87', ctypes.c_uint8 * 28), ('mxcsr', ctypes.c_uint32)]


class _Arm64Env(ctypes.Structure):
    _fields_ = [('fpcr', ctypes.c_uint32), ('fpsr', ctypes.c_uint32)]


_STATE = None


def _platform():
    machine = platform.machine().lower()
    if platform.system() != 'Linux':
        raise RuntimeError(f'E_FTZ_UNSUPPORTED: {platform.system()} {machine}')
    if machine in ('x86_64', 'amd64'):
        env, field, bits = _X86Env, 'mxcsr', 0x8040  # FTZ (bit 15) | DAZ (bit 6)
    elif machine in ('aarch64', 'arm64'):
        env, field, bits = _Arm64Env, 'fpcr', 1 << 24  # FZ
    else:
        raise RuntimeError(f'E_FTZ_UNSUPPORTED: Linux {machine}')
    libm = ctypes.CDLL(ctypes.util.find_library('m') or ctypes.util.find_library('c'))
    return libm, env, field, bits


@contextlib.contextmanager
def flush_to_zero():
    """Run the block with FP32 subnormals flushed to zero; checks that the mode took effect."""
    global _STATE
    if _STATE is None:
        _STATE = _platform()
    libm, env, field, bits = _STATE
    saved, wanted = env(), env()
    if libm.fegetenv(ctypes.byref(saved)) != 0:
        raise RuntimeError('E_FTZ_FENV: fegetenv failed')
    ctypes.memmove(ctypes.byref(wanted), ctypes.byref(saved), ctypes.sizeof(env))
    setattr(wanted, field, getattr(wanted, field) | bits)
    if libm.fesetenv(ctypes.byref(wanted)) != 0:
        raise RuntimeError('E_FTZ_FENV: fesetenv failed')
    try:
        probe = np.full(64, _TINY, np.float32) * np.float32(0.5)
        if probe[0] != 0 or _TINY * np.float32(0.5) != 0:
            raise RuntimeError('E_FTZ_INACTIVE: subnormal results survived')
        yield
    finally:
        libm.fesetenv(ctypes.byref(saved))
