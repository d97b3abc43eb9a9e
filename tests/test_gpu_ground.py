"""Ground preparation on the device (sosb_prepare_ground, the reference's engine_core.Solver.prepare_ground,
src/sosfuse2/solve/engine_core.py:103-147) against the host preparation of the same state (synth.Family.ground): a
handle whose ground arrays were prepared on the device gives the same first light, applications and observer boxes
as one given the host arrays. Both evaluate the ray values in FP64 and round once to FP32, so the bound is relative
1e-6 (the two exponentials may differ in the last bit of a double). Pinned to the reference: over the reference's own
ground rays of two golden states (tests/golden/ground_walk1.npz, ground_strato15.npz) the device preparation gives
the applications of the reference's prepared arrays, and the first light the reference's own first-light moments."""

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2_per_wave
from test_ground_host import reference_ground

pytestmark = pytest.mark.gpu

CASES = {
    'w1_l16': dict(W=1, L=16, strato=0.0),
    'w6_l16_strato': dict(W=6, L=16, strato=0.02),
}


def _family(W, L, strato, seed=11):
    from sosfuse2_gb300 import synth

    wl = np.linspace(420.0, 680.0, W)
    atm = synth.Atmosphere(wl, seed=seed, top=80.0, strato_tau=strato, albedo=0.4, aod=0.3)
    h = np.r_[0.0, np.geomspace(0.5, 80.0, 5)]
    fam = synth.Family(h, [0.0, 60.0, 90.0, 96.0, 110.0, 180.0], L, 1, 2, 4, atm, sun_scale=1)
    return fam, atm


@pytest.mark.parametrize('case', sorted(CASES))
def test_device_ground_matches_host(case):
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

    fam, atm = _family(**CASES[case])
    host = Solver(PackedState(fam.state(atm, 3)), device='cuda:0')
    dev = Solver(PackedState(fam.state(atm, 3, ground=False)), device='cuda:0')
    k = dev.kernel
    k.set_ground_rays(fam.ground_rays())
    k.prepare_ground(atm.albedo, atm.ext(), atm.strato_ext if atm.strato else None)
    zero = host.kernel.field()
    g_host, g_dev = host.apply(zero), dev.apply(dev.kernel.field())
    assert float(g_host.abs().max()) > 0
    assert np.all(rel_l2_per_wave(g_dev.cpu().numpy(), g_host.cpu().numpy()) <= 1e-6)
    g2_host, g2_dev = host.apply(g_host), dev.apply(g_host.clone())
    assert np.all(rel_l2_per_wave(g2_dev.cpu().numpy(), g2_host.cpu().numpy()) <= 1e-6)
    b_host, b_dev = host.boxes(g2_host), dev.boxes(g2_host.clone())
    assert np.max(np.abs(b_dev - b_host)) <= 1e-6 * np.abs(b_host).max()
    # a second state on the same handle: only the optics change
    from sosfuse2_gb300 import synth

    atm2 = synth.Atmosphere(atm.wl, seed=12, top=80.0, strato_tau=0.0 if not atm.strato else 0.03, albedo=0.1,
                            aod=0.05)
    host.kernel.update(PackedState(fam.state(atm2, 4)))
    k.update(PackedState(fam.state(atm2, 4, ground=False)))
    k.prepare_ground(atm2.albedo, atm2.ext(), atm2.strato_ext if atm2.strato else None)
    g_host, g_dev = host.apply(host.kernel.field()), dev.apply(dev.kernel.field())
    assert np.all(rel_l2_per_wave(g_dev.cpu().numpy(), g_host.cpu().numpy()) <= 1e-6)
    host.kernel.close()
    k.close()


def test_prepare_ground_needs_rays_and_strato_extinction():
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

    fam, atm = _family(W=2, L=16, strato=0.02)
    k = Solver(PackedState(fam.state(atm, 3, ground=False)), device='cuda:0').kernel
    with pytest.raises(RuntimeError, match='E_STATE'):
        k.prepare_ground(atm.albedo, atm.ext(), atm.strato_ext)
    k.set_ground_rays(fam.ground_rays())
    with pytest.raises(RuntimeError, match='E_CONSTANTS'):
        k.prepare_ground(atm.albedo, atm.ext(), None)
    k.close()


def test_table_of_device_ground_state_matches_host():
    """make_table on a handle whose ground arrays were prepared on the device carries them into its own handle: the
    first-order part (single scattering and the ground-reflected direct beam) equals the host-prepared state's."""
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState
    from sosfuse2_gb300.table import make_table

    fam, atm = _family(W=1, L=16, strato=0.0)
    host = Solver(PackedState(fam.state(atm, 3)), device='cuda:0')
    dev = Solver(PackedState(fam.state(atm, 3, ground=False)), device='cuda:0')
    dev.kernel.set_ground_rays(fam.ground_rays())
    dev.kernel.prepare_ground(atm.albedo, atm.ext(), None)
    field = host.apply(host.kernel.field())
    hs, el, az = [-3.0, -6.0], [60.0, 20.0, 5.0], [30.0, 150.0]
    a, _ = make_table(host, field, hs, el, az, log=lambda m: None, family=fam)
    b, _ = make_table(dev, field, hs, el, az, log=lambda m: None, family=fam)
    assert np.max(np.abs(a - b)) <= 1e-6 * np.abs(a).max()
    host.kernel.close()
    dev.kernel.close()


@pytest.mark.parametrize('name', ['walk1', 'strato15'])
def test_device_ground_matches_reference(name):
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState
    from test_gpu_parity import close_field

    rays, albedo, ext, strato_ext, _ = reference_ground(name)
    host = Solver(PackedState(GOLDEN / f'{name}.npz'), device='cuda:0')
    dev = Solver(PackedState(GOLDEN / f'{name}.npz'), device='cuda:0')
    dev.kernel.set_ground_rays(rays)
    dev.kernel.prepare_ground(albedo, ext, strato_ext)
    m, f, _ = dev.kernel.launch(0, True)
    close_field(m.cpu().numpy(), dev.state['first_moments'])
    g_host, g_dev = host.apply(host.kernel.field()), dev.apply(dev.kernel.field())
    assert np.all(rel_l2_per_wave(g_dev.cpu().numpy(), g_host.cpu().numpy()) <= 1e-6)
    host.kernel.close()
    dev.kernel.close()
