"""The combined SH plane of a reference state with the thin-layer skip (the C3/FW15 production flags:
sh_combine + sh_combine_skip, src/sosfuse2/solve/source_solver.py:1313-1314): the densities the adapter packs
(reference_adapter.thin_layer_cut) give, through the device's plane arithmetic (aerosol slots x ha, plus
stratospheric slots x density, each product and the sum rounded once in FP32), exactly the reference's own
sh_layout.combined_coefficients(..., skip_thin=True) of the same field. Skipped without the reference source."""

import os
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import GOLDEN

REFERENCE = Path(os.environ.get('SOSFUSE2_REFERENCE_SRC', '/root/reference/src'))
pytestmark = pytest.mark.skipif(not REFERENCE.exists(), reason='reference source not present')


def _device_plane(field, ha, sd, nc, K):
    """plane_kernel's arithmetic in NumPy FP32: [cells, K, W]."""
    hi = np.repeat(np.arange(len(ha)), nc)
    a = field[:, 10:10 + K] * ha[hi][:, None, None]
    b = field[:, 10 + K:] * sd[hi][:, None, None]
    return (a + b).astype(np.float32)


@pytest.mark.parametrize('name', ['strato1', 'strato15'])
def test_thin_layer_cut_gives_reference_combined_plane(name):
    if str(REFERENCE) not in sys.path:
        sys.path.insert(0, str(REFERENCE))
    from sosfuse2.backends.sh_layout import combined_coefficients

    from sosfuse2_gb300.reference_adapter import thin_layer_cut

    z = np.load(GOLDEN / f'{name}.npz')
    L = 16
    K = (L + 1) * (L + 2) // 2
    nc = len(z['chi'])
    rng = np.random.default_rng(7)
    field = rng.standard_normal((len(z['ha']) * nc, 10 + 2 * K, len(z['ext0']))).astype(np.float32)
    # thin layers on this grid: densities far below the air density at the upper heights
    arrays = dict(hr=z['hr'].copy(), ha=z['ha'].copy(), strato_density=z['strato_density'].copy())
    arrays['ha'][-1] = np.float32(1e-9) * arrays['hr'][-1]
    arrays['strato_density'][0] = np.float32(5e-8) * arrays['hr'][0]
    c = dict(ha=arrays['ha'], hr=arrays['hr'], strato_density=arrays['strato_density'], chi=z['chi'])
    want = combined_coefficients(field, c, L, skip_thin=True)
    cut = thin_layer_cut(dict(arrays), True)
    got = _device_plane(field, cut['ha'], cut['strato_density'], nc, K)
    assert np.array_equal(got, want)
    assert not np.array_equal(got, _device_plane(field, arrays['ha'], arrays['strato_density'], nc, K))
