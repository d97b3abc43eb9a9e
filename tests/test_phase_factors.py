"""The factorisation behind the tensor-core ground sums (sosb_phase_factors, host only): the stratospheric phase
table over the wavelengths, lut[u][w] ~= sum_r U_r(u) V_r(w), at the smallest rank whose every row is within 2e-6 of
its largest magnitude. On the reference's golden states: strato15 (15 wavelengths) needs six factors, strato1 (one
wavelength) one; five do not reach the bound for strato15; the tabulated tropospheric Mie phase of mie15 needs more
than eight (that state keeps the CUDA-core ground sums)."""

import ctypes

import numpy as np
import pytest

from conftest import GOLDEN
from sosfuse2_gb300 import _abi

BINS = 4096  # the stratospheric table's bins (sosb_set_constants)


def strato_table(chi):
    """The table sosb_set_constants builds: the 33 Legendre moments summed in FP64 on u = -1 + 2 i / BINS, per sr,
    rounded to FP32."""
    u = -1.0 + 2.0 * np.arange(BINS + 1) / BINS
    p0, p1 = np.ones_like(u), u.copy()
    v = chi[0][None, :] + u[:, None] * chi[1][None, :]
    for l in range(2, 33):
        pn = ((2.0 * l - 1) * u * p1 - (l - 1.0) * p0) / l
        v = v + pn[:, None] * chi[l][None, :]
        p0, p1 = p1, pn
    return (v / (4.0 * np.pi)).astype(np.float32).astype(np.float64)


def factors(lut, rmax, tol=2e-6):
    lib = _abi.library()
    n, W = lut.shape
    lut = np.ascontiguousarray(lut)
    U = np.zeros(n * rmax)
    V = np.zeros(rmax * W)
    r = ctypes.c_int(-1)
    assert lib.sosb_phase_factors(lut.ctypes.data_as(_abi.P_f64), n, W, rmax, tol, U.ctypes.data_as(_abi.P_f64),
                                  V.ctypes.data_as(_abi.P_f64), ctypes.byref(r)) == 0
    k = r.value
    return k, U[:n * k].reshape(n, k), V[:k * W].reshape(k, W)


@pytest.mark.parametrize('name,rank', [('strato15', 6), ('strato1', 1)])
def test_stratospheric_table_factors(name, rank):
    lut = strato_table(np.load(GOLDEN / f'{name}.npz')['strato_chi'].astype(np.float64))
    k, U, V = factors(lut, 8)
    assert k == rank
    err = np.abs(lut - U @ V).max(axis=1) / np.abs(lut).max(axis=1)
    assert err.max() <= 2e-6
    if rank > 1:
        assert factors(lut, rank - 1)[0] == 0  # the rank is the smallest within the bound


def test_mie_table_needs_more_factors():
    lut = np.load(GOLDEN / 'mie15.npz')['tropo_lut'].astype(np.float64)
    assert factors(lut, 8)[0] == 0
