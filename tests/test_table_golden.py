"""The radiance table of the reference (outputs/radiance_table.make_table on its NumPy backend, tests/golden/
table_walk1.npz, made by tests/golden/make_table_fixture.py) against the oracle's transport of the same view rays
(the first-order and the multiple-scattering parts, reduced as `Solver.query` reduces them by
`sosfuse2_gb300.table._spectral`): this pins the table path's rays, reduction and solar factor to the reference's
own table. Tolerance: 1e-6 relative (the oracle's per-ray radiance matches the reference's to 2e-18)."""

import numpy as np
import pytest

from conftest import GOLDEN


def table_state():
    """walk1's packed state with the solar column table the view rays read, the view-ray bundle, the source and the
    reference's table."""
    t = np.load(GOLDEN / 'table_walk1.npz')
    with np.load(GOLDEN / 'walk1.npz') as z:
        arrays = {k: z[k] for k in z.files}
    arrays['sun_col'] = t['sun_col']
    if 'strato_sun_col' in t.files:
        arrays['strato_sun_col'] = t['strato_sun_col']
    bundle = {k[len('table_'):]: t[k] for k in t.files if k.startswith('table_') and k != 'table_ref'}
    return arrays, bundle, t['source'], t['table_ref'], t['hs'], t['el'], t['az']


@pytest.mark.skipif(not (GOLDEN / 'table_walk1.npz').exists(), reason='table fixture not generated')
def test_oracle_table_matches_reference():
    from oracle import sos_oracle as so
    from oracle.ftz import flush_to_zero
    from sosfuse2_gb300.table import _spectral

    arrays, bundle, source, ref, hs, el, az = table_state()
    pk = so.StatePack(arrays)
    solar = np.asarray(arrays['solar'], np.float64)
    zero = np.zeros(pk.shape, np.float32)
    with flush_to_zero():
        one = _spectral(so.transport(pk, bundle, zero, True, query=True), solar)
        multiple = _spectral(so.transport(pk, bundle, source, False, query=True), solar)
    got = (one + multiple).astype(np.float32).reshape(len(hs), len(el), len(az), pk.W)
    assert got.shape == ref.shape
    assert np.max(np.abs(got - ref)) <= 1e-6 * np.abs(ref).max()
