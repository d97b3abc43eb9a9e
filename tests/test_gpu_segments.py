"""The geometry CSR on the device (sosb_ray_segments_device, one thread per ray) against the host builder
(sosb_ray_segments, the reference's ray_geometry.pack restated and checked against its NumPy restatement in
tests/test_ray_segments.py), on every cell ray and observer ray of the config-0 family (27,224 + 560 rays, ground
columns from its solar column table): the same segments (validity and lower-end flags), the cuts to FP64 rounding
(CUT_RTOL: the host compiler and nvcc contract different products into fused multiply-adds, and the cuts are roots of
quadratics whose cancellation turns those last-bit differences into up to 3.3e-12 relative), the same ground-end
positions (interval + fraction: a ray whose ground point falls on a solar-zenith node within those last bits is
placed at the end of one interval by one builder and at the start of the next by the other, 1 ray in 27,224), the
same ground hits and columns. Then a whole bundle built under synth.device_geometry() equals the host-built one to
the same bounds."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CUT_RTOL = 1e-10


def _rays(fam, prefix):
    b = fam.cells if prefix == 'cell' else fam.query
    cell = np.repeat(np.arange(len(b['cell_off']) - 1), np.diff(b['cell_off']))
    return np.ascontiguousarray(b['p'][cell]), np.ascontiguousarray(b['d'])


def _same_end(j_dev, f_dev, j_host, f_host):
    """Ground-end positions interval + fraction within 1e-9; the intervals differ by at most one, at a node."""
    j_dev, j_host = np.asarray(j_dev), np.asarray(j_host)
    assert np.all(np.abs(j_dev - j_host) <= 1)
    pos_dev = j_dev + np.asarray(f_dev, np.float64)
    pos_host = j_host + np.asarray(f_host, np.float64)
    assert np.max(np.abs(pos_dev - pos_host)) <= 1e-9


def test_device_segments_equal_host():
    from sosfuse2_gb300 import synth

    fam = synth.config0_family()
    for prefix, ground in (('cell', True), ('query', False)):
        p, d = _rays(fam, prefix)
        host = synth._ray_block(p, d, fam.chi, fam.top, fam.table, ground)
        dev = synth.ray_block_device(p, d, fam.chi, fam.top, fam.table, ground)
        np.testing.assert_array_equal(dev['seg_off'], host['seg_off'])
        np.testing.assert_array_equal(dev['seg_lower'], host['seg_lower'])
        for k in ('seg_a', 'seg_b'):
            scale = np.maximum(np.abs(host[k]), 1.0)
            assert np.max(np.abs(dev[k] - host[k]) / scale) <= CUT_RTOL, k
        np.testing.assert_array_equal(dev['hits'], host['hits'])
        _same_end(dev['end_j'], dev['end_f'], host['end_j'], host['end_f'])
        for k in ('end_col', 'end_st'):
            assert np.max(np.abs(dev[k] - host[k]) / np.maximum(np.abs(host[k]), 1e-30)) <= 1e-6, k


def test_device_geometry_bundle_equals_host():
    from sosfuse2_gb300 import synth

    atm = synth.Atmosphere([550.0], seed=3, top=80.0)
    h = np.r_[0.0, np.geomspace(0.5, 80.0, 5)]
    host = synth.make_state(h, [0.0, 60.0, 90.0, 96.0, 110.0, 180.0], atm.wl, 16, 1, 2, 4, atm, seed=3, sun_scale=1)
    with synth.device_geometry():
        dev = synth.make_state(h, [0.0, 60.0, 90.0, 96.0, 110.0, 180.0], atm.wl, 16, 1, 2, 4, atm, seed=3,
                               sun_scale=1)
    for k in [k for k in host if k.startswith(('cell_', 'query_'))]:
        a, b = np.asarray(dev[k]), np.asarray(host[k])
        if k.endswith(('_end_j', '_end_f')):
            if k.endswith('_end_j'):
                pre = k[:-len('end_j')]
                _same_end(a, dev[pre + 'end_f'], b, host[pre + 'end_f'])
        elif a.dtype.kind == 'f':
            assert np.allclose(a, b, rtol=CUT_RTOL, atol=CUT_RTOL), k
        else:
            np.testing.assert_array_equal(a, b, err_msg=k)


def test_device_column_table_equals_host():
    """The solar column table on the device (sosb_column_table_device, one thread per (table, height, x)) against
    the host threads' table (sosb_column_table, itself checked against its NumPy restatement in
    tests/test_column_table.py) on 0-100 km with the shells and the stratospheric layer: every column within 1e-12 of
    the component's largest column. The two compilers contract the FP64 operations differently, which moves columns
    far below the largest by more than that relative to themselves: a ray from the top going up has a path of about
    1e-17 km whose length is rounding, and columns of 1e-26 and less differ in their twelfth digit."""
    from sosfuse2_gb300 import synth

    atm = synth.Atmosphere([550.0], seed=3, top=100.0, strato_tau=0.01, no2_column=5e15)
    shells = synth._shells(100.0)
    h = np.linspace(0, np.sqrt(100.0), 41) ** 2
    x = np.linspace(0, 1, 201)
    up, down = synth.native_column_table(atm, shells, h, x)
    up_d, down_d = synth.native_column_table(atm, shells, h, x, device='cuda:0')
    for a, b in ((up_d, up), (down_d, down)):
        top = np.abs(b).max(axis=(0, 1))  # per component
        assert np.all(np.abs(a - b).max(axis=(0, 1)) <= 1e-12 * top)
