"""Learned warm start end to end on a small budget: the solver generates its own training solves (config-0 family,
tolerance 1e-4), the network trains on the tensor-core kernels, and on held-out states the warm-started solve (the
pair (0, g1) of the apply(0) that feeds the network kept in the Anderson history):
(a) converges under the unchanged test wherever the plain solve does;
(b) lands near the state's fixed point (the plain solve of the same state to tolerance 1e-6) as the plain solve to
    1e-4 does: max relative observer radiance within 1e-3 on at least 80 % of the states for each start and within
    2e-3 on all (stopping at 1e-4 bounds the last change, not the error: a slowly contracting state stops further
    from its fixed point, from either start);
(c) costs, counting the apply(0), no more than half an evaluation more than the plain start on average (the
    measured gain of the full training budget is reported by bench.py, forms.learned / forms.batched)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fixed_point_boxes(fam, seed):
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState
    from sosfuse2_gb300.synth import family_state

    s = Solver(PackedState(family_state(fam, seed)), device='cuda:0')
    try:
        x, _ = s.solve(256, 1e-6, device_out=True)
        return s.boxes(x)
    except RuntimeError:
        return None
    finally:
        s.kernel.close()


def test_learned_start_reaches_the_fixed_point():
    from sosfuse2_gb300 import learned, synth
    from sosfuse2_gb300.solver import Kernel, Solver
    from sosfuse2_gb300.state import PackedState
    from sosfuse2_gb300.synth import family_state

    fam = synth.config0_family()
    ws, report = learned.train_warm_start(fam, n_train=96, epochs=25, seed=10000, tolerance=1e-4, slow=40)
    assert report['loss_last'] < report['loss_first']
    plain_ev, learn_ev, errs = [], [], []
    for seed in range(90000, 90010):
        truth = _fixed_point_boxes(fam, seed)
        st = PackedState(family_state(fam, seed))
        k = Kernel(st, 'cuda:0')
        solver = Solver(st, kernel=k)
        try:
            xp, sp = solver.solve(64, 1e-4, device_out=True)
        except RuntimeError as exc:
            assert str(exc).startswith('E_NOT_CONVERGED')
            k.close()
            continue
        k.update(st)  # the learned path computes its own first light
        k._check(k.lib.sosb_set_warm_history(k.h, 1))
        g1 = solver.apply(k.field())
        x0 = ws.predict_start(st, g1)
        xl, sl = learned.solve_warm(solver, x0, g1, ws.fallback_ss, 64, 1e-4)
        bp, bl = solver.boxes(xp), solver.boxes(xl)
        k.close()
        plain_ev.append(sp['evaluations'])
        learn_ev.append(sl['evaluations'] + 1)  # the apply(0) that feeds the network
        if truth is not None:
            big = np.abs(truth) > 1e-6 * np.abs(truth).max()
            ep = np.max(np.abs(bp[big] - truth[big]) / np.abs(truth[big]))
            el = np.max(np.abs(bl[big] - truth[big]) / np.abs(truth[big]))
            errs.append((ep, el))
    e = np.array(errs)
    assert len(plain_ev) >= 5 and len(e) >= 5, (plain_ev, errs)
    assert np.all(e <= 2e-3) and np.all(np.mean(e <= 1e-3, axis=0) >= 0.8), errs
    assert np.mean(learn_ev) <= np.mean(plain_ev) + 0.5, (learn_ev, plain_ev)
