"""The synthetic state generator: its restated ring quadrature against the reference's (when the reference source is
importable in this environment), its weights, and the packed state it writes."""

import math
import os
import sys
from pathlib import Path

import numpy as np
import pytest

from sosfuse2_gb300 import synth
from sosfuse2_gb300.state import PackedState

REFERENCE = Path(os.environ.get('SOSFUSE2_REFERENCE_SRC', '/root/reference/src'))


@pytest.mark.parametrize('h,chi,nmu,nphi,err', [(0.0, 60.0, 1, 2, 0.3), (40.0, 100.0, 3, 8, 1e-2),
                                                 (8.0, 95.0, 12, 16, 1e-3)])
def test_quadrature_weights_cover_the_sphere(h, chi, nmu, nphi, err):
    # the sinh-mapped Gauss-Legendre rule in mu is exact only in the limit; low orders are coarse
    loc, w = synth.ring_quadrature(synth.R + h, math.radians(chi), nmu, nphi, (0.0, 1.2, 8.0, 25.0, 40.0, 80.0))
    assert np.all(w > 0) and abs(w.sum() / (4 * math.pi) - 1) < err
    np.testing.assert_allclose(np.linalg.norm(loc, axis=1), 1.0, atol=1e-12)


@pytest.mark.skipif(not REFERENCE.exists(), reason='reference source not present')
@pytest.mark.parametrize('h,chi,nmu,nphi', [(0.0, 60.0, 1, 2), (8.0, 95.0, 2, 4), (40.0, 100.0, 12, 16)])
def test_quadrature_matches_reference(h, chi, nmu, nphi):
    sys.path.insert(0, str(REFERENCE))
    from sosfuse2.rays import incoming_rings

    ref_loc, ref_w = incoming_rings.incoming(synth.R + h, math.radians(chi), nmu, nphi, 4.0, True)
    loc, w = synth.ring_quadrature(synth.R + h, math.radians(chi), nmu, nphi, (0.0, 1.2, 8.0, 25.0, 40.0, 80.0))
    np.testing.assert_allclose(loc, ref_loc, rtol=0, atol=1e-12)
    np.testing.assert_allclose(w, ref_w, rtol=1e-12, atol=0)


def test_config0_state_shapes():
    st = PackedState(synth.config0())
    assert st.shape == (101 * 10, 10 + 2 * 153, 1)
    assert st.meta['rays'] == len(st['cell_d'])
    off = st['cell_seg_off']
    assert off[-1] == len(st['cell_seg_a']) and np.all(np.diff(off) >= 0)  # rays into the ground at h=0: none
    assert np.all(st['cell_seg_b'] - st['cell_seg_a'] > 1e-8)
    assert len(st['query_d']) == 5 * 7 * 16


def test_native_quadratures_match_numpy_restatement():
    """sosb_ring_quadrature (synth.quadratures) against the NumPy restatement ring_quadrature, cell by cell, with and
    without the shadow rings: the same directions and weights to rounding (measured 1.7e-15 and 2.8e-16)."""
    for rings in (True, False):
        specs = [(synth.R + hh, math.radians(c), 3, 8, (0.0, 1.2, 8.0, 25.0, 40.0, 80.0) if rings else (), rings)
                 for hh in (0.0, 0.7, 3.0, 12.0, 40.0, 79.0) for c in (0.0, 30.0, 60.0, 85.0, 88.0, 90.0, 93.0, 96.0,
                                                                     105.0, 140.0, 180.0)]
        for sp, (loc, w) in zip(specs, synth.quadratures(specs)):
            ref_loc, ref_w = synth.ring_quadrature(*sp[:5], rings=rings)
            assert loc.shape == ref_loc.shape, sp
            np.testing.assert_allclose(loc, ref_loc, rtol=0, atol=1e-12)
            # weights of 4 pi in total: a last-bit difference in a narrow interval's end is relatively large there
            np.testing.assert_allclose(w, ref_w, rtol=0, atol=1e-14)
