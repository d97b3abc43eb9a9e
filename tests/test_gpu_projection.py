"""Projection forms on the tensor cores (tcgen05.mma against the per-bundle basis table) against the compensated FP32
CUDA-core projection and the oracle, on the small synthetic states of tests/test_gpu_synth.py (one wavelength, three
with L=32 and an 80-120 km grid, eight with L=24, 33 over two wavelength chunks). Bounds, relative L2 per
wavelength of apply(0) and of apply(oracle source): bf16x3 2e-5 (measured about 7e-6, inside the FP32 path's parity
bound of 1e-4 against the oracle), TF32 2e-3 (about 8e-4), BF16 6e-3 (about 3e-3). A converged bf16x3 solve reaches
the FP32 solve's fixed point within the solve tolerance."""

import numpy as np
import pytest

from conftest import rel_l2_per_wave
from test_gpu_synth import small_state

pytestmark = pytest.mark.gpu

CASES = {
    'w1_l16': dict(W=1, L=16, top=80.0, nh=6),
    'w3_l32_top120': dict(W=3, L=32, top=120.0, nh=7),
    'w8_l24': dict(W=8, L=24, top=80.0, nh=6),
    'w33_l16': dict(W=33, L=16, top=80.0, nh=5),
    'w6_l48': dict(W=6, L=48, top=120.0, nh=4),
}
BOUND = {1: 2e-5, 2: 2e-3, 3: 6e-3}  # bf16x3, TF32, BF16


def _applies(arrays, mode, start):
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

    s = Solver(PackedState(dict(arrays)), device='cuda:0')
    k = s.kernel
    k._check(k.lib.sosb_set_projection(k.h, mode))
    z = np.zeros(s.state.shape, np.float32)
    out = (s.apply(k.field(z)).cpu().numpy(), s.apply(k.field(start)).cpu().numpy())
    k.close()
    return out


@pytest.mark.parametrize('case', sorted(CASES))
def test_projection_forms(case):
    from oracle import sos_oracle as so

    arrays = small_state(**CASES[case])
    ref = so.Oracle(so.StatePack(dict(arrays)))
    g1_ref = ref.apply(np.zeros(ref.pk.shape, np.float32))
    base = _applies(arrays, 0, g1_ref)
    for mode, bound in BOUND.items():
        g1, g2 = _applies(arrays, mode, g1_ref)
        assert np.all(rel_l2_per_wave(g1, base[0]) <= bound), (case, mode)
        assert np.all(rel_l2_per_wave(g2, base[1]) <= bound), (case, mode)
    g1, _ = _applies(arrays, 1, g1_ref)
    assert np.all(rel_l2_per_wave(g1, g1_ref) <= 1e-4)


def test_bf16x3_solve_matches_fp32():
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

    arrays = small_state(**CASES['w8_l24'])
    out = {}
    for mode in (0, 1):
        s = Solver(PackedState(dict(arrays)), device='cuda:0')
        k = s.kernel
        k._check(k.lib.sosb_set_projection(k.h, mode))
        out[mode] = s.solve(64, 1e-3)
        k.close()
    x0, st0 = out[0]
    x1, st1 = out[1]
    assert abs(st1['evaluations'] - st0['evaluations']) <= 2
    assert np.all(rel_l2_per_wave(x1, x0) <= 1e-3)


def test_unknown_form_rejected():
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

    s = Solver(PackedState(dict(small_state(**CASES['w1_l16']))), device='cuda:0')
    k = s.kernel
    assert k.lib.sosb_set_projection(k.h, 7) != 0
    assert k.lib.sosb_last_error(k.h).decode().startswith('E_PROJECTION')
    k.close()
