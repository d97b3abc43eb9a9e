"""CUDA path against the oracle on small synthetic states that exercise the many-wavelength transport (W > 4), SH
orders other than 16 up to L = 48, two wavelength chunks (W > 32), and an 80-120 km extended grid. Same tolerances as
tests/test_gpu_parity.py (moments/sources relative L2 per wavelength <= 1e-4, observer radiance rtol 1e-3)."""

import numpy as np
import pytest

from conftest import rel_l2_per_wave

pytestmark = pytest.mark.gpu

CASES = {
    'w8_l24': dict(W=8, L=24, top=80.0, nh=6),
    'w33_l16': dict(W=33, L=16, top=80.0, nh=5),
    'w3_l32_top120': dict(W=3, L=32, top=120.0, nh=7),
    # the largest SH order of the batched configuration (L = 48, K = 1225), on the warp path and the wavelength path
    'w1_l48': dict(W=1, L=48, top=80.0, nh=5),
    'w6_l48_top120': dict(W=6, L=48, top=120.0, nh=4),
}


def small_state(W, L, top, nh, seed=7):
    from sosfuse2_gb300 import synth

    wl = np.linspace(420.0, 680.0, W)
    atm = synth.Atmosphere(wl, seed=seed, top=top, no2_column=5e15 if W > 4 else 0.0, o4=W > 4)
    h = np.r_[0.0, np.geomspace(0.5, top, nh - 1)]
    return synth.make_state(h, [0.0, 60.0, 90.0, 96.0, 110.0, 180.0], wl, L, 1, 2, 4, atm, seed=seed, sun_scale=1)


@pytest.mark.parametrize('case', sorted(CASES))
def test_apply_and_boxes_match_oracle(case):
    from oracle import sos_oracle as so
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

    arrays = small_state(**CASES[case])
    ref = so.Oracle(so.StatePack(dict(arrays)))
    solver = Solver(PackedState(dict(arrays)), device='cuda:0')
    k = solver.kernel
    zero = np.zeros(solver.state.shape, np.float32)
    g1_ref = ref.apply(zero)
    g1 = solver.apply(k.field(zero)).cpu().numpy()
    assert np.all(rel_l2_per_wave(g1, g1_ref) <= 1e-4)
    g2_ref = ref.apply(g1_ref)
    g2 = solver.apply(k.field(g1_ref)).cpu().numpy()
    assert np.all(rel_l2_per_wave(g2, g2_ref) <= 1e-4)
    b_ref = ref.boxes(g1_ref)
    b = solver.boxes(k.field(g1_ref))
    big = np.abs(b_ref) > 1e-6 * np.abs(b_ref).max()
    assert np.all(np.abs(b[big] - b_ref[big]) <= 1e-3 * np.abs(b_ref[big]))
    k.close()


@pytest.mark.parametrize('air_end', [80.0, 120.0])
def test_extended_top_matches_oracle(air_end):
    """An extended top (components supported to 80 km, the air to `air_end`) on the GPU against the oracle's
    restatement of the reference's support rules: apply(0), apply(g1) and the observer boxes."""
    from test_host_transport import _extended_state

    from oracle import sos_oracle as so
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

    arrays = _extended_state(air_end)
    ref = so.Oracle(so.StatePack(dict(arrays)))
    solver = Solver(PackedState(dict(arrays)), device='cuda:0')
    k = solver.kernel
    zero = np.zeros(solver.state.shape, np.float32)
    g1_ref = ref.apply(zero)
    g1 = solver.apply(k.field(zero)).cpu().numpy()
    assert np.all(rel_l2_per_wave(g1, g1_ref) <= 1e-4)
    g2_ref = ref.apply(g1_ref)
    g2 = solver.apply(k.field(g1_ref)).cpu().numpy()
    assert np.all(rel_l2_per_wave(g2, g2_ref) <= 1e-4)
    b_ref = ref.boxes(g1_ref)
    b = solver.boxes(k.field(g1_ref))
    big = np.abs(b_ref) > 1e-6 * np.abs(b_ref).max()
    assert np.all(np.abs(b[big] - b_ref[big]) <= 1e-3 * np.abs(b_ref[big]))
    k.close()
