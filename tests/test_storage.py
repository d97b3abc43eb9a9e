"""`sosfuse2_gb300.storage` writes the reference's source.npz, moment.npz and table.npz (jobs/run_storage.py:235-302):
the files written here from the inputs of tests/golden/make_storage_fixtures.py carry the same keys, dtypes, shapes
and values as the reference writer's files in tests/golden/storage/, and the readers return what was written."""

import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / 'golden'
sys.path.insert(0, str(GOLDEN))


def _same_npz(mine, ref):
    with np.load(mine) as a, np.load(ref) as b:
        assert sorted(a.files) == sorted(b.files)
        for k in b.files:
            assert a[k].dtype == b[k].dtype, k
            assert a[k].shape == b[k].shape, k
            assert np.array_equal(a[k], b[k]), k


@pytest.fixture(scope='module')
def written(tmp_path_factory):
    from make_storage_fixtures import inputs
    from sosfuse2_gb300 import storage

    a = inputs()
    d = tmp_path_factory.mktemp('storage')
    storage.write_source(d, a['fields'], a['h'], a['chi'], a['wl'], physical=a['physical'], optics=a['optics'],
                         contract=a['contract'])
    storage.write_moments(d, a['moments'], a['h'], a['chi'], a['wl'], a['order'])
    storage.write_table(d, a['table'], a['wl'], a['hs'], a['el'], a['az'])
    return d, a


@pytest.mark.parametrize('name', ['source.npz', 'moment.npz', 'table.npz'])
def test_files_match_reference_writer(written, name):
    d, _ = written
    _same_npz(d / name, GOLDEN / 'storage' / name)
    assert not list(d.glob('*.tmp'))


def test_readers_round_trip(written):
    from sosfuse2_gb300 import storage

    d, a = written
    src, h, chi, wl, meta = storage.read_source(d / 'source.npz')
    assert np.array_equal(src, np.concatenate(a['fields'], -1)) and np.array_equal(wl, a['wl'])
    assert meta['source_contract'] == a['contract'] and meta['optics_state'] == a['optics']
    rad, wl32, hs, el, az = storage.read_table(d / 'table.npz')
    assert np.array_equal(rad, a['table']) and hs.dtype == np.float32 and np.array_equal(az, a['az'].astype('f4'))


def test_contract_rejects_nan(tmp_path):
    from sosfuse2_gb300 import storage

    with pytest.raises(ValueError):
        storage.write_source(tmp_path, [np.zeros((1, 1, 1), np.float32)], [0.0], [0.0], [550.0], physical={},
                             optics={}, contract=dict(tolerance=float('nan')))
    assert not list(tmp_path.glob('*'))
