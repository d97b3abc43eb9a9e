"""Per-pixel relative error against an FP64 run (oracle.fp64): the reference's own float32 radiance table of the
walkthrough state (tests/golden/table_walk1.npz) and its observer boxes and application of the source
(tests/golden/walk1.npz) against the same computation in float64 on the same inputs. Measured: table max 3.1e-6, RMS
1.5e-6; the bounds below leave a factor of ten."""

import numpy as np
import pytest

from conftest import GOLDEN


@pytest.mark.skipif(not (GOLDEN / 'table_walk1.npz').exists(), reason='table fixture not generated')
def test_reference_table_against_float64():
    from oracle.fp64 import float64, relative_error
    from sosfuse2_gb300.table import _spectral
    from test_table_golden import table_state

    arrays, bundle, source, ref, hs, el, az = table_state()
    solar = np.asarray(arrays['solar'], np.float64)
    with float64() as so:
        pk = so.StatePack(arrays)
        zero = np.zeros(pk.shape, np.float64)
        one = so.transport(pk, bundle, zero, True, query=True)
        multiple = so.transport(pk, bundle, np.asarray(source, np.float64), False, query=True)
        assert one.dtype == np.float64
    exact = (_spectral(one, solar) + _spectral(multiple, solar)).reshape(ref.shape)
    mx, med, rms = relative_error(ref, exact)
    assert mx < 3e-5 and rms < 2e-5, (mx, med, rms)


def test_reference_boxes_against_float64():
    from oracle.fp64 import float64, relative_error

    with np.load(GOLDEN / 'walk1.npz') as z:
        arrays = {k: z[k] for k in z.files}
    with float64() as so:
        pk = so.StatePack(arrays)
        exact = so.boxes(pk, np.asarray(arrays['apply_zero'], np.float64))
    mx, med, rms = relative_error(arrays['boxes_g1'], exact)
    assert mx < 1e-4, (mx, med, rms)


def test_twilight_boxes_against_float64():
    """The FP32 arithmetic of the path (the oracle's, which the CUDA kernels restate operation for operation) against
    float64 on the same inputs, per observer elevation down to -18 deg, where the radiance is 8e-8 of the +6 deg value:
    a small state on 0-100 km at 450 nm with the stratospheric layer, NO2 and O4, its single-scatter source and the
    observer boxes of it. Measured max (RMS) relative error per row (+6, -6, -12, -18 deg): 2.5e-7 (2.0e-7), 3.0e-6
    (2.5e-6), 3.8e-6 (2.9e-6), 1.1e-5 (5.2e-6); the bound leaves a factor of ten at -18 deg."""
    from oracle import sos_oracle as so32
    from oracle.fp64 import float64, relative_error
    from sosfuse2_gb300 import synth

    wl = np.array([450.0])
    atm = synth.Atmosphere(wl, seed=6, top=100.0, strato_tau=0.02, no2_column=5e15, o4=True)
    h = np.r_[0.0, np.geomspace(0.5, 100.0, 6)]
    fam = synth.Family(h, [0.0, 60.0, 90.0, 96.0, 100.0, 105.0, 110.0, 180.0], 16, 1, 2, 4, atm, sun_scale=1,
                       monitor_elevations=[6.0, -6.0, -12.0, -18.0])
    arrays = fam.state(atm, 6)
    pk = so32.StatePack(dict(arrays))
    o = so32.Oracle(pk)
    b32 = o.boxes(o.apply(np.zeros(pk.shape, np.float32)))
    with float64() as so:
        pk64 = so.StatePack(dict(arrays))
        o64 = so.Oracle(pk64)
        b64 = o64.boxes(o64.apply(np.zeros(pk64.shape, np.float64)))
    rows = [relative_error(b32[r], b64[r])[0] for r in range(4)]
    assert b64[3].max() < 1e-5 * b64[0].max()  # -18 deg is deep twilight
    assert rows[0] < 1e-5 and max(rows[1:3]) < 5e-5 and rows[3] < 1e-4, rows
