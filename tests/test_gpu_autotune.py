"""Autotuned table launches (warps per ray timed once per launch shape) against the fixed rule: the two solves differ
only in the order of the per-ray sums, so their fields agree to rounding (relative L2 per wavelength 1e-5) and take
the same number of evaluations (within one)."""

import numpy as np
import pytest

from conftest import rel_l2_per_wave
from test_gpu_synth import small_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('case', [dict(W=1, L=16, top=80.0, nh=6), dict(W=3, L=32, top=120.0, nh=7)])
def test_autotune_matches_rule(case):
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

    arrays = small_state(**case)
    out = {}
    for tune in (True, False):
        s = Solver(PackedState(dict(arrays)), device='cuda:0')
        k = s.kernel
        k._check(k.lib.sosb_set_autotune(k.h, int(tune)))
        out[tune] = s.solve(64, 1e-3)
        k.close()
    (xa, sa), (xb, sb) = out[True], out[False]
    assert abs(sa['evaluations'] - sb['evaluations']) <= 1
    assert np.all(rel_l2_per_wave(xa, xb) <= 1e-5)
