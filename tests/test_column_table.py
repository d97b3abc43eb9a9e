"""The native solar column table (sosb_column_table, host threads) against the NumPy restatement of the same
integrals (synth.column_rows): same cuts of every path and the same Gauss-Legendre sums in FP64, so the tables
agree to rounding (measured 2e-15 relative; bound 1e-12)."""

import numpy as np
import pytest


@pytest.mark.parametrize('top,strato', [(80.0, 0.0), (100.0, 0.01), (120.0, 0.02)])
def test_native_column_table_matches_numpy(top, strato):
    from sosfuse2_gb300 import synth

    atm = synth.Atmosphere(np.array([450.0, 650.0]), seed=4, top=top, strato_tau=strato, scale_height=1.5)
    shells = synth._shells(top)
    h = np.linspace(0, np.sqrt(top), 13) ** 2
    x = np.linspace(0, 1, 41)
    up, down = synth.native_column_table(atm, shells, h, x, threads=2)
    up0, down0 = synth.column_rows(atm, shells, h, x)
    for a, b in ((up, up0), (down, down0)):
        scale = np.abs(b).max(axis=(0, 1))
        assert np.all(np.abs(a - b) <= 1e-12 * np.maximum(scale, 1e-300))
    if not strato:
        assert np.all(up[..., 5] == 0) and np.all(down[..., 5] == 0)


def test_native_column_table_rejects_bad_sizes():
    import ctypes

    from sosfuse2_gb300 import _abi, build

    lib = _abi.library(build.build())
    one = np.zeros(1)
    p = _abi.ptr(one, _abi.P_f64)
    shape = _abi.ProfileShape(top=80.0, aerosol_height=1.2, ozone_peak=22.0, ozone_norm=1.0, no2_center=25.0)
    assert lib.sosb_column_table(0, p, 1, p, None, 0, p, p, 1, ctypes.byref(shape), p, p, 1) == 1
    assert lib.sosb_column_table(1, p, 1, p, p, 9, p, p, 1, ctypes.byref(shape), p, p, 1) == 1
