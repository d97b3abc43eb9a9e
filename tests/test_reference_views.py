"""The adapter's view rays of a reference-assembled state (reference_adapter.view_rays) are the rays the reference's
own make_table transported for tests/golden/table_walk1.npz (runs where the reference source is importable)."""

import os
import shutil
import sys
import tempfile
from pathlib import Path

import numpy as np
import pytest

from conftest import GOLDEN

REFERENCE = Path(os.environ.get('SOSFUSE2_REFERENCE_SRC', '/root/reference/src'))


@pytest.mark.skipif(not REFERENCE.exists() or not (GOLDEN / 'table_walk1.npz').exists(),
                    reason='reference source or table fixture not present')
def test_view_rays_match_the_reference_table_rays():
    sys.path.insert(0, str(GOLDEN))
    import make_fixtures as mf

    saved = dict(os.environ)  # the reference's example environment replaces the process environment
    try:
        _check_views(mf)
    finally:
        os.environ.clear()
        os.environ.update(saved)


def _check_views(mf):
    root = Path(tempfile.mkdtemp(prefix='sosb_views_'))
    cache = mf._environment(root)
    from types import SimpleNamespace

    from sosfuse2.atmosphere.components import production_only
    from sosfuse2.jobs import run_state as rs
    from sosfuse2.jobs import walkthrough as wt

    from sosfuse2_gb300.reference_adapter import view_rays

    production_only()
    a = SimpleNamespace(reduced=True, settings_json=None, stratosphere=None)
    state = rs.effective_state(wt.example_state(), a)
    cfg = rs.resolve_settings(rs.settings_for(a), state)
    cfg['wavelengths_nm'], cfg['wavelengths'] = [550.0], 1
    s, _ = rs.create_configured(root / 'tmp' / 'views' / 'prepare_0', cfg, np.asarray([550.0]), 'numpy', state, 128,
                                geometry_cache=cache)
    try:
        t = np.load(GOLDEN / 'table_walk1.npz')
        got = view_rays(s, t['hs'], t['el'], t['az'])
        for k, v in got.items():
            assert np.array_equal(v, t['table_' + k]), k
    finally:
        shutil.rmtree(root, ignore_errors=True)
