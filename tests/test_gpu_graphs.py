"""Solve graphs and the one-thread batch driver: a solve whose evaluations after the first run inside one CUDA graph
(a WHILE node that the device's control kernel stops) gives the field, evaluation count and statistics of the same
solve launched kernel by kernel with the stop flag read after each evaluation (the same kernels on the same inputs,
so bit for bit), including a warm start that falls back and a solve that runs out of evaluations; the batch driver
with two solves in flight gives every state's single-solve result."""

import ctypes

import numpy as np
import pytest

from test_gpu_synth import small_state

pytestmark = pytest.mark.gpu

CASES = {
    'w1_l16': dict(W=1, L=16, top=80.0, nh=6),
    'w8_l24': dict(W=8, L=24, top=80.0, nh=6),
}


def _solve(arrays, graphs, max_eval=64):
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

    s = Solver(PackedState(dict(arrays)), device='cuda:0')
    k = s.kernel
    k.set_graphs(graphs)
    try:
        x, st = s.solve(max_eval, 1e-3)
        err = None
    except RuntimeError as exc:
        x, st, err = None, None, str(exc).split(':')[0]
    launches = int(s.last_stats.kernel_launches)
    k.close()
    return x, st, err, launches


@pytest.mark.parametrize('case', sorted(CASES))
def test_graph_solve_equals_direct(case):
    arrays = small_state(**CASES[case])
    _solve(arrays, True)  # the process's first solve of these shapes also times the launch shapes (autotuner)
    xg, sg, eg, lg = _solve(arrays, True)
    xd, sd, ed, ld = _solve(arrays, False)
    assert eg is None and ed is None
    assert sg['evaluations'] == sd['evaluations']
    assert np.array_equal(xg, xd)
    assert lg == ld + 1  # the solve graph counts its kernels, and its gate kernel is one more


def test_graph_budget_exhausted_equals_direct():
    arrays = small_state(**CASES['w1_l16'])
    g = _solve(arrays, True, max_eval=3)
    d = _solve(arrays, False, max_eval=3)
    assert g[2] == d[2] == 'E_NOT_CONVERGED'


def test_batch_driver_equals_single_solves():
    from sosfuse2_gb300.solver import BatchSolver, Solver
    from sosfuse2_gb300.state import PackedState

    states = [small_state(W=1, L=16, top=80.0, nh=6, seed=s) for s in (3, 4, 5)]
    singles = []
    for a in states:
        s = Solver(PackedState(dict(a)), device='cuda:0')
        singles.append(s.solve(64, 1e-3))
        s.kernel.close()
    b = BatchSolver([PackedState(dict(a)) for a in states], device='cuda:0')
    res = b.solve(64, 1e-3, threads=2)
    b.close()
    for (x, st), r in zip(singles, res):
        assert not isinstance(r, Exception)
        xb, sb = r
        assert sb['evaluations'] == st['evaluations']
        assert np.array_equal(xb, x)
