"""Host side of the radiance table: the table axes of the reference (radiance_table.py:32-38) and the view rays of
`synth.Family.view_bundle` (one bundle cell per solar elevation, the observer frame and the (el, az) grid of
`Solver.query`, solve/engine_core.py:208-226)."""

import numpy as np
import pytest


def test_axes_reduced_and_full():
    from sosfuse2_gb300.table import axes

    wl, hs, el, az = axes(True)
    assert wl.tolist() == [550.0] and hs.tolist() == [-3.0, -6.0]
    assert np.allclose(el, [78.75, 56.25, 33.75, 11.25]) and np.allclose(az, 15.0 + 30.0 * np.arange(6))
    wl, hs, el, az = axes(False)
    assert len(wl) == 15 and len(hs) == 25 and hs[0] == 6.0 and hs[-1] == -18.0 and len(el) == 100 and len(az) == 180


def test_view_bundle_directions():
    from sosfuse2_gb300 import synth

    atm = synth.Atmosphere(np.array([550.0]), seed=3, top=80.0)
    h = np.r_[0.0, np.geomspace(0.5, 80.0, 4)]
    fam = synth.Family(h, [0.0, 60.0, 90.0, 96.0, 110.0, 180.0], 16, 1, 2, 4, atm, sun_scale=1)
    hs, el, az = [-3.0, -6.0], [80.0, 30.0, 5.0], [10.0, 100.0]
    b = fam.view_bundle(hs, el, az)
    assert b['cell_off'].tolist() == [0, 6, 12] and len(b['d']) == 12
    for j, hsj in enumerate(hs):
        p, up, ex = synth.frame(synth.R + synth.OBSERVER_KM, np.deg2rad(90 - hsj))
        ey = np.cross(up, ex)
        assert np.allclose(b['p'][j], p)
        for i, (e, z) in enumerate((e, z) for e in el for z in az):
            e, z = np.deg2rad(e), np.deg2rad(z)
            want = np.sin(e) * up + np.cos(e) * (np.cos(z) * ex + np.sin(z) * ey)
            assert np.allclose(b['d'][6 * j + i], want, atol=1e-12)


def test_make_table_validates_before_device_work():
    from sosfuse2_gb300.table import make_table

    with pytest.raises(ValueError, match='E_TABLE_GROUP'):
        make_table(None, None, [0.0], [0.0], [0.0], group=0, family=None)
    with pytest.raises(ValueError, match='E_TABLE_BATCH'):
        make_table(None, None, [0.0], [0.0], [0.0], batch=0, family=None)
