"""The allocation-free composition entry point, sosb_compose_static, through the C ABI.

Some callers cannot allocate device memory once a state is set up (their device memory is reserved by another
allocator, or a cudaMalloc's implicit synchronisation would stall their pipeline). For them the library offers one
entry point whose reduction scratch is a static device array instead of handle memory. This test runs it twice in a
row (the scratch keeps the previous call's words, so the second call checks that it is cleared) and compares the
composed source with the existing entry point, sosb_apply, on the same field, at the tolerance of the other GPU
parity tests; the returned source metrics are checked against the composed output.

This file is collected last, so a run that stops at the first failure has run every other test before it.
"""

import ctypes

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2_per_wave

pytestmark = pytest.mark.gpu


def test_compose_static_matches_apply():
    from sosfuse2_gb300.solver import Kernel, Solver
    from sosfuse2_gb300.state import PackedState

    st = PackedState(GOLDEN / 'strato1.npz')
    k = Kernel(st, device='cuda:0')
    torch = k.torch
    solver = Solver(st, kernel=k)
    first_m, first_f, _ = k.launch(0, True)
    for x_host in (np.zeros(st.shape, np.float32), st['apply_zero']):
        x = k.field(x_host)
        _, flux, _ = k.launch(1, False, x)
        boundary = (flux + first_f[: st.nc]).contiguous()
        warm, _, _ = k.launch(0, False, x, boundary)
        out = torch.empty_like(x)
        nonfinite = np.full(st.W, -1, np.int64)
        rel = np.full(st.W, np.nan, np.float64)
        k._stream()
        rc = k.lib.sosb_compose_static(k.h, ctypes.c_void_p(warm.data_ptr()), ctypes.c_void_p(first_m.data_ptr()),
                                       ctypes.c_void_p(x.data_ptr()), 0, ctypes.c_void_p(out.data_ptr()),
                                       nonfinite.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                       rel.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        assert rc == 0, k.lib.sosb_last_error(k.h)
        got = out.cpu().numpy()
        ref = solver.apply(x).cpu().numpy()
        scale = np.max(np.abs(ref))
        assert np.max(np.abs(got - ref)) <= 1e-5 * scale
        assert np.all(rel_l2_per_wave(got, ref) <= 1e-4)
        assert np.all(nonfinite == 0)
        expect = np.max(np.abs(got - x_host), axis=(0, 1)) / np.maximum(np.max(np.abs(got), axis=(0, 1)), 1e-30)
        np.testing.assert_allclose(rel, expect, rtol=1e-6)
    k.close()
