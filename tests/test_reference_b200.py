"""The `b200` backend inside the reference's own program (the reference imported from its source tree; skipped when it
is absent): after sosfuse2_gb300.b200.install(), the reference's create_configured(..., 'b200', ...) builds the
walkthrough state with a 'b200' kernel, and the reference's Solver(s, TransientGeometry(s, scope)).solve(64, tol)
hands the GPU solve exactly the packed inputs of the golden walkthrough fixture (tests/golden/walk1.npz, whose GPU
solve tests/test_gpu_parity.py checks against the reference's own solve) and returns what the GPU solve returns.
Here the GPU solve is replaced by a recorder (no GPU in this test); a NumPy-backend state is untouched."""

import os
import sys
import tempfile
from pathlib import Path

import numpy as np
import pytest

from conftest import GOLDEN

REFERENCE = Path(os.environ.get('SOSFUSE2_REFERENCE_SRC', '/root/reference/src'))
pytestmark = pytest.mark.skipif(not REFERENCE.exists() or not (GOLDEN / 'walk1.npz').exists(),
                                reason='reference source or golden fixture not present')
if REFERENCE.exists() and str(REFERENCE) not in sys.path:
    sys.path.insert(0, str(REFERENCE))


def _walkthrough(monkeypatch, root, backend):
    """The walkthrough state (clear_34, no stratospheric layer, 550 nm) by the reference's assembly."""
    from types import SimpleNamespace

    from sosfuse2.atmosphere.components import production_only
    from sosfuse2.jobs import run_state as rs
    from sosfuse2.jobs import walkthrough as wt
    from sosfuse2.solve import ray_geometry as gm

    for k, v in wt.example_environment(root).items():
        monkeypatch.setenv(k, v)
    for k in [k for k in os.environ if k.startswith('SOSFUSE2_') and k not in wt.example_environment(root)]:
        monkeypatch.delenv(k)
    cache = root / 'geometry_cache'
    monkeypatch.setenv('SOSFUSE2_COLUMN_CACHE_JOB', str(root))
    monkeypatch.setenv('SOSFUSE2_STATE_ID', 'walkthrough')
    monkeypatch.setenv('STRATO_ATTACH_CACHE', str(cache / 'attach_cache'))
    production_only()
    a = SimpleNamespace(reduced=True, settings_json=None, stratosphere=None)
    state = rs.effective_state(wt.example_state(), a)
    cfg = rs.resolve_settings(rs.settings_for(a), state)
    cfg['wavelengths_nm'] = [550.0]
    cfg['wavelengths'] = 1
    s, scope = rs.create_configured(root / 'tmp' / 'walk1' / 'prepare_0', cfg, np.asarray([550.0]), backend, state,
                                    128, geometry_cache=cache)
    return s, scope, gm.TransientGeometry(s, scope), cfg


def test_b200_solve_receives_the_golden_inputs(monkeypatch):
    from sosfuse2_gb300 import b200

    calls = []

    def record(arrays, max_eval, tolerance, device):
        calls.append((arrays, max_eval, tolerance))
        return np.zeros(1, np.float32), dict(evaluations=0, recorded=True)

    b200.install(solve_fn=record)
    try:
        root = Path(tempfile.mkdtemp(prefix='sosb_b200_'))
        s, scope, geometry, cfg = _walkthrough(monkeypatch, root, 'b200')
        assert s.kernel.backend == 'b200'
        from sosfuse2.solve.source_iteration import Solver

        x, stats = Solver(s, geometry).solve(64, cfg['anderson_tol'])
    finally:
        b200.uninstall()
    assert stats == dict(evaluations=0, recorded=True) and len(calls) == 1
    arrays, max_eval, tol = calls[0]
    assert max_eval == 64 and tol == cfg['anderson_tol']
    golden = np.load(GOLDEN / 'walk1.npz')
    # the inputs of the hot path: bundles of the cells and of the observer, the constants (the fixture stores the
    # solar column table only where first light reads it, so that table is compared there)
    keys = [k for k in golden.files if k.startswith(('cell_', 'query_'))] + [
        'u', 'wu', 'uq', 'wuq', 'h', 'chi', 'hr', 'ha', 'ext', 'asca', 'sun_h', 'gm', 'gd', 'gv', 'density_table', 'rf',
        'af', 'ext0', 'solar', 'box_ww']
    for k in keys:
        np.testing.assert_array_equal(np.asarray(arrays[k]), golden[k], err_msg=k)
    mask = golden['sun_mask']
    np.testing.assert_array_equal(np.asarray(arrays['sun_col'])[mask], golden['sun_col'][mask])


def test_other_backends_untouched():
    from sosfuse2.solve import source_iteration, source_solver

    from sosfuse2_gb300 import b200

    init, solve = source_solver.Kernel.__init__, source_iteration.Solver.solve
    b200.install(solve_fn=lambda *a: None)
    assert source_solver.Kernel.__init__ is not init and b200.installed()
    b200.uninstall()
    assert source_solver.Kernel.__init__ is init and source_iteration.Solver.solve is solve and not b200.installed()
