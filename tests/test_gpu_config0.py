"""CUDA path against the oracle on the states the benchmark reports, at their full size: the config-0 state (550 nm,
101 heights on 0-100 km x the 10-node solar-zenith grid = 1,010 cells, 27,224 rays, L=16, stratospheric layer) and
config-0 family states (seeded amounts from the batched configuration's ranges), one whose iteration converges and
one whose iteration does not (the reference's method itself stalls on such states: tests/golden/slow1.npz).

The oracle's per-cell work runs on every host core (oracle/parallel.py, bit-identical to one process). Tolerances are
those of tests/test_gpu_parity.py (the reference's numeric gate, src/sosfuse2/checks/gate.py:659-686): moments and
sources relative L2 <= 1e-4 per wavelength, radiance rtol 1e-3; the converged source relative L2 <= 1e-3 and its
observer radiance rtol 1e-3; the same evaluation count; the per-evaluation stopping measures within 2 % of the
oracle's."""

import numpy as np
import pytest

from conftest import rel_l2_per_wave, rel_max
from test_gpu_parity import close, close_field

pytestmark = pytest.mark.gpu

# held-out family seeds: 90001 (AOD 0.24, g 0.59) converges in 8 evaluations on the oracle; 90015 (AOD 0.43,
# g 0.78) keeps a source change near 0.37 for all 64
CONVERGING_SEED = 90001
STALLING_SEED = 90015


@pytest.fixture(scope='module')
def config0():
    from oracle.parallel import ParallelOracle
    from sosfuse2_gb300 import synth
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

    arrays = synth.config0()
    oracle = ParallelOracle(arrays)
    solver = Solver(PackedState(dict(arrays)), device='cuda:0')
    yield oracle, solver
    solver.kernel.close()
    oracle.close()


def test_config0_first_light(config0):
    oracle, solver = config0
    oracle.initialize()
    m, f, _ = solver.kernel.launch(0, True)
    close_field(m.cpu().numpy(), oracle.first_moments)
    close(f.cpu().numpy(), oracle.first_flux)


def test_config0_apply_and_boxes(config0):
    oracle, solver = config0
    k = solver.kernel
    zero = np.zeros(solver.state.shape, np.float32)
    g1_ref = oracle.apply(zero)
    close_field(solver.apply(k.field(zero)).cpu().numpy(), g1_ref)
    g2_ref = oracle.apply(g1_ref)
    close_field(solver.apply(k.field(g1_ref)).cpu().numpy(), g2_ref)
    close(solver.boxes(k.field(zero)), oracle.boxes(zero))
    close(solver.boxes(k.field(g1_ref)), oracle.boxes(g1_ref))


def _histories(stats_hist, oracle_hist):
    ours = np.array([[h['observer_relative'], h['source_relative']] for h in stats_hist])
    ref = np.array([[h['observer_relative'], h['source_relative']] for h in oracle_hist])
    return ours, ref


def _solve_pair(oracle, solver, max_eval, tol):
    """(x, stats, history) of the oracle and of the CUDA solve, with the E_NOT_CONVERGED message in place of x."""
    hist = []
    try:
        x_ref, st_ref = oracle.solve(max_eval, tol, log=lambda it, rr, ss, done: hist.append(
            dict(observer_relative=rr.tolist(), source_relative=ss.tolist())))
    except RuntimeError as exc:
        assert str(exc).startswith('E_NOT_CONVERGED'), exc
        x_ref, st_ref = str(exc), None
    try:
        x, st = solver.solve(max_eval, tol)
    except RuntimeError as exc:
        assert str(exc).startswith('E_NOT_CONVERGED'), exc
        x, st = str(exc), None
    return (x_ref, st_ref, hist), (x, st, solver.history())


def _assert_histories(h, h_ref):
    ours, ref = _histories(h, h_ref)
    assert ours.shape == ref.shape, (ours.shape, ref.shape)
    assert np.all(np.abs(ours - ref) <= 2e-2 * ref + 1e-6), np.c_[ours.reshape(len(ours), -1),
                                                                  ref.reshape(len(ref), -1)]
    return ref


def test_config0_solve(config0):
    oracle, solver = config0
    st = solver.state
    (x_ref, st_ref, h_ref), (x, stats, h) = _solve_pair(oracle, solver, int(st.meta['max_eval']),
                                                        float(st.meta['tolerance']))
    assert st_ref is not None and stats is not None, (x_ref, x)
    assert stats['evaluations'] == st_ref['evaluations']
    assert np.all(rel_l2_per_wave(x, x_ref) <= 1e-3)
    assert rel_max(solver.boxes(solver.kernel.field(x)), oracle.boxes(x_ref)) <= 1e-3
    _assert_histories(h, h_ref)


@pytest.mark.parametrize('seed', [CONVERGING_SEED, STALLING_SEED])
def test_family_solve(seed):
    """One held-out config-0 family state: the CUDA solve ends as the oracle's does (converged with the same
    evaluation count and field, or E_NOT_CONVERGED after the whole budget), and the stopping measures follow the
    oracle's evaluation by evaluation (all 64 for the state that stalls)."""
    from oracle.parallel import ParallelOracle
    from sosfuse2_gb300 import synth
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

    fam = synth.config0_family()
    arrays = synth.family_state(fam, seed)
    solver = Solver(PackedState(dict(arrays)), device='cuda:0')
    with ParallelOracle(arrays) as oracle:
        (x_ref, st_ref, h_ref), (x, stats, h) = _solve_pair(oracle, solver, 64, 1e-3)
        if st_ref is None:
            assert stats is None, 'the CUDA solve converged where the oracle does not'
        else:
            assert stats is not None, x
            assert stats['evaluations'] == st_ref['evaluations']
            assert np.all(rel_l2_per_wave(x, x_ref) <= 1e-3)
            assert rel_max(solver.boxes(solver.kernel.field(x)), oracle.boxes(x_ref)) <= 1e-3
    solver.kernel.close()
    ref = _assert_histories(h, h_ref)
    if seed == STALLING_SEED:
        assert st_ref is None and ref[-1].max() > 1e-2  # the stall is the oracle's (the method's), not the device's
    else:
        assert st_ref is not None
