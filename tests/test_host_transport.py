"""The device transport (sos_math.cuh) compiled for the host, against the reference's per-ray golden radiance.

This checks the CUDA path's arithmetic without a GPU: the same `transport_lane` source and the same packing
(sos_pack.h) run on the CPU under FP32 flush-to-zero. Tolerance: rtol 1e-3 on every radiance element above 1e-6 of
the maximum (the reference's numeric gate), and 1e-5 of the maximum overall.
"""

import ctypes

import numpy as np
import pytest

from conftest import GOLDEN, fixture_names, ray_index
from oracle.ftz import flush_to_zero
from sosfuse2_gb300.state import PackedState


def run(lib, ps, prefix, field, first, query, boundary=None):
    d, c, b = ps.dims(), ps.constants(), ps.abi_bundle(prefix)
    out = np.zeros((b.nray, ps.W, 4), np.float32)
    err = ctypes.create_string_buffer(256)
    f = np.ascontiguousarray(field, np.float32)
    bd = None if boundary is None else np.ascontiguousarray(boundary, np.float32)
    with flush_to_zero():
        rc = lib.host_transport(ctypes.byref(d), ctypes.byref(c), ctypes.byref(b), int(first), int(query),
                                f.ctypes.data, None if bd is None else bd.ctypes.data, out.ctypes.data, err, 256)
    assert rc == 0, err.value
    return out


def close(a, ref, rtol=1e-3, floor=1e-6):
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = np.max(np.abs(ref))
    big = np.abs(ref) > floor * scale
    assert np.max(np.abs(a - ref)) <= 1e-5 * scale
    assert np.all(np.abs(a[big] - ref[big]) <= rtol * np.abs(ref[big]))


@pytest.mark.parametrize('name', fixture_names())
def test_host_transport_matches_reference(host_transport_lib, name):
    ps = PackedState(GOLDEN / f'{name}.npz')
    idx = ray_index(ps, ps['pin_cells'])
    zero = np.zeros(ps.shape, np.float32)
    close(run(host_transport_lib, ps, 'cell', zero, True, False)[idx], ps['pin_first'])
    close(run(host_transport_lib, ps, 'cell', ps['apply_zero'], False, False, ps['pin_boundary'])[idx],
          ps['pin_warm'])
    close(run(host_transport_lib, ps, 'query', ps['apply_zero'], False, True), ps['pin_query'])


def _extended_state(air_end):
    """A small state on 0-120 km with a shell at 80 km, the components supported to 80 km and the air to `air_end`
    (numpy_reference.py:158-183: a top above 80 km; air_end 80 for a vacuum above, 120 for the upper-air profile)."""
    import json

    from sosfuse2_gb300 import synth

    atm = synth.Atmosphere([450.0, 650.0], seed=4, top=120.0, strato_tau=0.02, no2_column=5e15, o4=True)
    h = np.array([0.0, 2.0, 12.0, 40.0, 80.0, 100.0, 120.0])
    arrays = synth.make_state(h, [0.0, 60.0, 90.0, 96.0, 110.0, 180.0], atm.wl, 16, 1, 2, 4, atm, seed=4, sun_scale=1)
    meta = arrays['meta'] if isinstance(arrays['meta'], dict) else json.loads(str(arrays['meta']))
    meta = dict(meta, support=dict(lower_end=80.0, air_end=float(air_end)))
    return dict(arrays, meta=json.dumps(meta))


@pytest.mark.parametrize('air_end', [80.0, 120.0])
def test_extended_top_support_matches_oracle(host_transport_lib, air_end):
    """The extended top's support rules (profiles zero above their ends, the segment-end snap at 80 km, the warm
    density and aerosol source zero above their ends) in the device transport compiled for the host against the
    oracle's restatement of numpy_reference.py: first light, warm pass and observer pass. With a vacuum above 80 km
    the rules change the radiance: the rays of the cells at 100 and 120 km that stay above 80 km see no first light
    (their air is cut), which they do without the rules."""
    from oracle import sos_oracle as so

    arrays = _extended_state(air_end)
    ps = PackedState(dict(arrays))
    pk = so.StatePack(dict(arrays))
    zero = np.zeros(ps.shape, np.float32)
    rng = np.random.default_rng(4)  # a positive source: Rayleigh slots about 1e-3, SH slots smaller
    g1 = (rng.uniform(0.5, 1.5, ps.shape) * np.r_[np.full(10, 1e-3), np.full(ps.shape[1] - 10, 1e-4)][None, :, None])
    g1 = g1.astype(np.float32)
    for prefix, first, field in (('cell', True, zero), ('cell', False, g1), ('query', False, g1)):
        dev = run(host_transport_lib, ps, prefix, field, first, prefix == 'query')
        ref = so.transport(pk, pk.bundle(prefix), field, first, query=prefix == 'query')
        close(dev, ref)
    if air_end <= 80.0:
        import json

        plain = dict(arrays, meta=json.dumps({k: v for k, v in json.loads(arrays['meta']).items() if k != 'support'}))
        upper = ray_index(ps, range(5 * ps.nc, ps.ns))  # cells at 100 and 120 km
        first_plain = run(host_transport_lib, PackedState(plain), 'cell', zero, True, False)[upper]
        first = run(host_transport_lib, ps, 'cell', zero, True, False)[upper]
        dark = (np.abs(first).max(axis=(1, 2)) == 0) & (np.abs(first_plain).max(axis=(1, 2)) > 0)
        assert dark.sum() >= 10, dark.sum()
