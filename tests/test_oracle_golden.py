"""The oracle against the reference's golden outputs (tests/golden/*.npz, made by tests/golden/make_fixtures.py).

Tolerances: the oracle restates the reference's FP32 arithmetic operation for operation, so the per-ray transport
and projection agree to a few FP32 ulps (ULPS = 2e-6 of the largest value: the steep boundary-layer profile of the
two-layer aerosol state spreads the regrouped sums' rounding furthest, 1.03e-6); the solve may take a different FP32 Gram rounding, so the converged field
is held to the reference's numeric gate (source relative L2 <= 1e-3 per wavelength, radiance rtol 1e-3).
"""

import numpy as np
import pytest

from conftest import GOLDEN, fixture_names, ray_index, reference_history, rel_l2_per_wave, rel_max
from oracle import sos_oracle as so

ULPS = 2e-6


@pytest.fixture(scope='module', params=fixture_names())
def pack(request):
    return so.StatePack(GOLDEN / f'{request.param}.npz')


def _cells(pk, cells):
    b = pk.bundle('cell')
    idx = ray_index(pk, cells)
    out = dict(b)
    off = b['cell_off']
    new_off = np.r_[0, np.cumsum([off[i + 1] - off[i] for i in cells])]
    segs = [np.arange(b['seg_off'][r], b['seg_off'][r + 1]) for r in idx]
    seg_idx = np.concatenate(segs)
    out.update(cell_off=new_off, p=b['p'][cells], target=b['target'][cells],
               seg_off=np.r_[0, np.cumsum([len(s) for s in segs])], seg_a=b['seg_a'][seg_idx],
               seg_b=b['seg_b'][seg_idx], seg_lower=b['seg_lower'][seg_idx],
               **{k: b[k][idx] for k in ('d', 'dloc', 'weight', 'end_j', 'end_f', 'end_col', 'end_st', 'hits')})
    return out


def test_transport_pins(pack):
    cells = list(pack['pin_cells'])
    b = _cells(pack, cells)
    zero = np.zeros((pack.ns, pack.source_size, pack.W), np.float32)
    assert rel_max(so.transport(pack, b, zero, True), pack['pin_first']) < ULPS
    warm = so.transport(pack, b, pack['apply_zero'], False, pack['pin_boundary'])
    assert rel_max(warm, pack['pin_warm']) < ULPS
    q = so.transport(pack, pack.bundle('query'), pack['apply_zero'], False, query=True)
    assert rel_max(q, pack['pin_query']) < ULPS


def test_projection_pin(pack):
    b = _cells(pack, [5])
    rad = so.transport(pack, b, pack['apply_zero'], False, pack['pin_boundary'])
    m, f = so.project(pack, b, rad)
    assert rel_max(m[0], pack['pin_project_moments']) < ULPS
    assert rel_max(f[0], pack['pin_project_flux']) < ULPS


def test_apply_and_boxes(pack):
    o = so.Oracle(pack)
    o.initialize()
    assert rel_max(o.first_moments, pack['first_moments']) < ULPS
    assert rel_max(o.first_flux, pack['first_flux']) < ULPS
    zero = np.zeros((pack.ns, pack.source_size, pack.W), np.float32)
    assert rel_max(o.apply(zero), pack['apply_zero']) < ULPS
    assert rel_max(o.apply(pack['apply_zero']), pack['apply_g1']) < ULPS
    assert rel_max(o.boxes(zero), pack['boxes_zero']) < ULPS
    assert rel_max(o.boxes(pack['apply_zero']), pack['boxes_g1']) < ULPS


@pytest.mark.parametrize('name', ['walk1', 'aer2', 'mie1'])
def test_solve_matches_reference(name):
    """The converged solve of the reference's states: the walkthrough state, its two-layer aerosol and its Mie phase
    variants."""
    if not (GOLDEN / f'{name}.npz').exists():
        pytest.skip(f'{name} fixture not generated')
    pk = so.StatePack(GOLDEN / f'{name}.npz')
    x, stats = so.Oracle(pk).solve()
    assert stats['converged'] == [True] * pk.W
    assert abs(stats['evaluations'] - pk.meta['evaluations']) <= 1
    assert np.all(rel_l2_per_wave(x, pk['solve_x']) <= 1e-3)
    assert rel_max(so.boxes(pk, x), pk['solve_boxes']) <= 1e-3


def test_solve_history_matches_reference():
    """The oracle's per-evaluation convergence measures follow the reference's history (walk1: 12 evaluations) within
    1 % (the last evaluations' changes are differences of nearly equal FP32 fields)."""
    pk = so.StatePack(GOLDEN / 'walk1.npz')
    _, stats = so.Oracle(pk).solve()
    ref_obs, ref_src = reference_history(pk.meta)
    obs = np.array([h['observer_relative'] for h in stats['history']])
    src = np.array([h['source_relative'] for h in stats['history']])
    assert obs.shape == ref_obs.shape
    assert np.all(np.abs(obs - ref_obs) <= 1e-2 * ref_obs + 1e-7), np.c_[obs, ref_obs]
    assert np.all(np.abs(src - ref_src) <= 1e-2 * ref_src + 1e-7), np.c_[src, ref_src]


@pytest.mark.skipif(not (GOLDEN / 'slow1.npz').exists(), reason='slow1 fixture not generated')
def test_nonconvergence_matches_reference():
    """The hazy forward-scattering state (AOD 0.3, g 0.78) does not converge in the reference's own solve (64
    evaluations, source change near 0.3 throughout); the oracle's iteration reproduces that history to the six digits
    the reference printed."""
    pk = so.StatePack(GOLDEN / 'slow1.npz')
    assert pk.meta['solve_error'].startswith('E_NOT_CONVERGED') and 'solve_x' not in pk
    ref_obs, ref_src = reference_history(pk.meta)
    hist = []
    with pytest.raises(RuntimeError, match='E_NOT_CONVERGED'):
        so.Oracle(pk).solve(log=lambda it, rr, ss, done: hist.append((rr, ss)))
    obs = np.array([h[0] for h in hist])
    src = np.array([h[1] for h in hist])
    assert obs.shape == ref_obs.shape == (64, 1)
    assert np.all(np.abs(obs - ref_obs) <= 2e-5 * ref_obs), np.c_[obs, ref_obs]
    assert np.all(np.abs(src - ref_src) <= 2e-5 * ref_src), np.c_[src, ref_src]


@pytest.mark.skipif(not (GOLDEN / 'mie15.npz').exists(), reason='mie15 fixture not generated')
def test_mie15_nonconvergence_matches_reference():
    """The Mie-phase state over 15 wavelengths does not converge in the reference's own solve (13 of 15 wavelengths
    within 1e-3 after 64 evaluations); over its first 12 evaluations (the CPU suite's time; the GPU parity test runs
    all 64) the oracle follows the history the reference printed (its maximum over the wavelengths, six digits)
    within 0.2 %: the largest gaps, 0.14 %, follow the Anderson steps where a wavelength's change jumps (evaluation
    11), from the FP32 regrouping of the sums."""
    pk = so.StatePack(GOLDEN / 'mie15.npz')
    assert pk.meta['solve_error'].startswith('E_NOT_CONVERGED') and 'solve_x' not in pk
    ref_obs, ref_src = reference_history(pk.meta)
    hist = []
    with pytest.raises(RuntimeError, match='E_NOT_CONVERGED'):
        so.Oracle(pk).solve(max_eval=12, log=lambda it, rr, ss, done: hist.append((max(rr), max(ss))))
    obs = np.array([[h[0]] for h in hist])
    src = np.array([[h[1]] for h in hist])
    assert ref_obs.shape == (64, 1) and obs.shape == (12, 1)
    ref_obs, ref_src = ref_obs[:12], ref_src[:12]
    assert np.all(np.abs(obs - ref_obs) <= 2e-3 * ref_obs), np.c_[obs, ref_obs]
    assert np.all(np.abs(src - ref_src) <= 2e-3 * ref_src), np.c_[src, ref_src]
