"""First-light ground sums on the tensor cores (sosb_set_ground_mma: [items x directions] x [directions x W]
products, BF16 high and low parts, FP32 accumulation; the stratospheric pair phase through the leading factors of its
table over the wavelengths) against the CUDA-core kernel (ground_pairs_warp_kernel) on the same states: the first
light's moments and flux per wavelength within relative L2 1e-5 and every element within 1e-4 of the largest. On
synthetic many-wavelength states with a stratospheric layer and a bright ground (one factor: the synthetic
stratospheric phase does not depend on the wavelength), a state without that layer, and the reference's strato15
state (15 wavelengths, a phase table that needs six factors), whose first light is also held to the reference's own
moments."""

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2_per_wave

pytestmark = pytest.mark.gpu

CASES = {
    'w8_l24_strato': dict(W=8, L=24, strato=0.02),
    'w24_l16_strato': dict(W=24, L=16, strato=0.05),
    'w33_l16_strato': dict(W=33, L=16, strato=0.02),
    'w12_l16': dict(W=12, L=16, strato=0.0),
}


def _state(W, L, strato, seed=5):
    from sosfuse2_gb300 import synth

    wl = np.linspace(410.0, 690.0, W)
    atm = synth.Atmosphere(wl, seed=seed, top=80.0, strato_tau=strato, albedo=0.6, aod=0.2, no2_column=5e15, o4=True)
    h = np.r_[0.0, np.geomspace(0.5, 80.0, 6)]
    return synth.make_state(h, [0.0, 60.0, 90.0, 96.0, 110.0, 180.0], wl, L, 1, 2, 4, atm, seed=seed, sun_scale=1)


def _first_light(arrays, mma):
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

    solver = Solver(PackedState(arrays), device='cuda:0')
    k = solver.kernel
    k._check(k.lib.sosb_set_ground_mma(k.h, int(mma)))
    m, f, _ = k.launch(0, True)
    out = m.cpu().numpy(), f.cpu().numpy()
    k.close()
    return out


def _agree(a, b):
    assert np.all(rel_l2_per_wave(a, b) <= 1e-5), rel_l2_per_wave(a, b)
    assert np.abs(a - b).max() <= 1e-4 * np.abs(b).max()


@pytest.mark.parametrize('case', sorted(CASES))
def test_ground_mma_matches_cuda_cores(case):
    arrays = _state(**CASES[case])
    mm, mf = _first_light(dict(arrays), True)
    cm, cf = _first_light(dict(arrays), False)
    _agree(mm, cm)
    _agree(mf[:, None, :], cf[:, None, :])


def test_ground_mma_reference_strato15():
    from test_gpu_parity import close, close_field

    from sosfuse2_gb300.state import PackedState

    st = PackedState(GOLDEN / 'strato15.npz')
    mm, mf = _first_light(GOLDEN / 'strato15.npz', True)
    cm, cf = _first_light(GOLDEN / 'strato15.npz', False)
    _agree(mm, cm)
    close_field(mm, st['first_moments'])
    close(mf, st['first_flux'])
