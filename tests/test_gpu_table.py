"""Radiance tables (make_table, src/sosfuse2/outputs/radiance_table.py:167-219) on the CUDA path against the oracle:
the same view rays transported by the oracle for the first-order and the multiple-scattering parts, reduced as
`Solver.query` reduces them. Tolerance: the reference's numeric gate, rtol 1e-3 on table entries above 1e-6 of the
largest. The reference's partition check (tests/test_a5_table.py: groups 4, 32, 64 agree) becomes: batches of one
solar elevation and of all of them give the same table within 1e-5."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = {
    'w1_l16': dict(W=1, L=16, top=80.0, nh=6),
    'w6_l16': dict(W=6, L=16, top=80.0, nh=5),
}


def _family(W, L, top, nh, seed=7):
    from sosfuse2_gb300 import synth

    wl = np.linspace(420.0, 680.0, W)
    atm = synth.Atmosphere(wl, seed=seed, top=top, no2_column=5e15 if W > 4 else 0.0, o4=W > 4)
    h = np.r_[0.0, np.geomspace(0.5, top, nh - 1)]
    fam = synth.Family(h, [0.0, 60.0, 90.0, 96.0, 110.0, 180.0], L, 1, 2, 4, atm, sun_scale=1)
    return fam, fam.state(atm, seed)


def _oracle_table(arrays, fam, field, hs, el, az):
    from oracle import sos_oracle as so

    pk = so.StatePack(dict(arrays))
    solar = np.asarray(arrays['solar'], np.float64)
    zero = np.zeros(pk.shape, np.float32)
    out = []
    for h in hs:
        b = fam.view_bundle([h], el, az)
        parts = []
        for first, f in ((True, zero), (False, field)):
            r = np.asarray(so.transport(pk, b, f, first, query=True), np.float64)
            parts.append(((r[..., 0] + r[..., 1]) + r[..., 2]) * solar[None, :])
        out.append((parts[0] + parts[1]).astype(np.float32).reshape(len(el), len(az), pk.W))
    return np.stack(out)


@pytest.mark.parametrize('case', sorted(CASES))
def test_table_matches_oracle(case):
    from oracle import sos_oracle as so
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState
    from sosfuse2_gb300.table import make_table

    fam, arrays = _family(**CASES[case])
    ref = so.Oracle(so.StatePack(dict(arrays)))
    field = ref.apply(ref.apply(np.zeros(ref.pk.shape, np.float32)))  # a multiple-scattering source
    hs = np.array([-3.0, -6.0])
    el = 90 - (np.arange(3) + 0.5) * 30.0
    az = (np.arange(4) + 0.5) * 45.0
    solver = Solver(PackedState(dict(arrays)), device='cuda:0')
    table, seconds = make_table(solver, field, hs, el, az, log=lambda m: None, family=fam)
    assert table.shape == (2, 3, 4, solver.state.W) and table.dtype == np.float32 and len(seconds) == 1
    want = _oracle_table(arrays, fam, field, hs, el, az)
    big = np.abs(want) > 1e-6 * np.abs(want).max()
    assert np.all(np.abs(table[big] - want[big]) <= 1e-3 * np.abs(want[big]))
    one_by_one, seconds = make_table(solver, field, hs, el, az, batch=1, log=lambda m: None, family=fam)
    assert len(seconds) == 2
    assert np.max(np.abs(one_by_one - table)) <= 1e-5 * np.abs(table).max()
    solver.kernel.close()


def test_table_rejects_bad_arguments():
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState
    from sosfuse2_gb300.table import make_table

    fam, arrays = _family(W=1, L=16, top=80.0, nh=5)
    solver = Solver(PackedState(dict(arrays)), device='cuda:0')
    good = np.zeros(solver.state.shape, np.float32)
    with pytest.raises(ValueError, match='E_TABLE_GROUP'):
        make_table(solver, good, [-3.0], [45.0], [90.0], group=0, family=fam)
    with pytest.raises(ValueError, match='E_TABLE_BATCH'):
        make_table(solver, good, [-3.0], [45.0], [90.0], batch=0, family=fam)
    with pytest.raises(ValueError, match='E_SOURCE_SHAPE'):
        make_table(solver, good[:, :5], [-3.0], [45.0], [90.0], family=fam)
    solver.kernel.close()


def test_table_matches_reference_golden():
    """make_table over the reference's own view rays of the walkthrough state (tests/golden/table_walk1.npz) against
    the reference's table (its make_table on the NumPy backend): the numeric gate, rtol 1e-3 on entries above 1e-6
    of the largest."""
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from test_table_golden import table_state

    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState
    from sosfuse2_gb300.table import make_table

    arrays, bundle, source, ref, hs, el, az = table_state()
    solver = Solver(PackedState(arrays), device='cuda:0')
    table, _ = make_table(solver, source, hs, el, az, batch=len(hs), log=lambda m: None,
                          views=lambda h, e, a: bundle)
    big = np.abs(ref) > 1e-6 * np.abs(ref).max()
    assert np.all(np.abs(table[big] - ref[big]) <= 1e-3 * np.abs(ref[big]))
    # per-pixel error against the FP64 run of the same rays (the reference's own table is within 3.1e-6 of it)
    from oracle.fp64 import float64, relative_error
    from sosfuse2_gb300.table import _spectral

    solar = np.asarray(arrays['solar'], np.float64)
    with float64() as so:
        pk = so.StatePack(arrays)
        one = so.transport(pk, bundle, np.zeros(pk.shape, np.float64), True, query=True)
        multiple = so.transport(pk, bundle, np.asarray(source, np.float64), False, query=True)
    exact = (_spectral(one, solar) + _spectral(multiple, solar)).reshape(ref.shape)
    assert relative_error(table, exact)[0] <= 1.1e-3
    solver.kernel.close()
