"""The native segment builder (sosb_ray_segments, host threads) against the NumPy restatement (synth.ray_block_numpy)
on the rays of a synthetic family's cell and observer bundles: the same cuts, segment choice, lower-end flags and
ground columns (FP64 arithmetic in the same order; ground columns to FP32), and the same end positions up to the last
bit of the arc cosine."""

import numpy as np
import pytest


@pytest.mark.parametrize('top,strato', [(80.0, 0.0), (100.0, 0.01)])
def test_native_segments_match_numpy(top, strato):
    from sosfuse2_gb300 import synth

    atm = synth.Atmosphere(np.array([550.0]), seed=2, top=top, strato_tau=strato)
    h = np.r_[0.0, np.geomspace(0.5, top, 5)]
    fam = synth.Family(h, [0.0, 60.0, 85.0, 90.0, 93.0, 96.0, 110.0, 180.0], 16, 2, 4, 4, atm, sun_scale=1)
    for b, ground in ((fam.cells, True), (fam.query, False)):
        ray_cell = np.repeat(np.arange(len(b['p'])), np.diff(b['cell_off']))
        p = b['p'][ray_cell]
        got = synth._ray_block(p, b['d'], fam.chi, fam.top, fam.table, ground)
        want = synth.ray_block_numpy(p, b['d'], fam.chi, fam.top, fam.table, ground)
        for k in ('seg_off', 'seg_lower', 'hits'):
            assert np.array_equal(got[k], want[k].astype(got[k].dtype)), k
        for k in ('seg_a', 'seg_b'):
            np.testing.assert_allclose(got[k], want[k], rtol=1e-14, atol=1e-12, err_msg=k)
        # the end's solar-zenith position j + f: the arc cosines may differ in the last bit, which at a grid node
        # moves the end between (j, 1) and (j + 1, 0), the same point
        np.testing.assert_allclose(got['end_j'] + got['end_f'], want['end_j'] + want['end_f'], rtol=0, atol=1e-12)
        assert np.mean(got['end_j'] == want['end_j']) > 0.99
        for k in ('end_col', 'end_st'):
            np.testing.assert_allclose(got[k], want[k], rtol=1e-6, atol=0, err_msg=k)
