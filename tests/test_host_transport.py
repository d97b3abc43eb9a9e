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
