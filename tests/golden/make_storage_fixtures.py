"""Generate the files that pin `sosfuse2_gb300.storage` to the reference's writers.

Run in this container only (it imports the reference's `jobs/run_storage.py` from its source tree):

    python tests/golden/make_storage_fixtures.py

It writes source.npz, moment.npz and table.npz with the reference's `write_source`, `write_moments` and
`write_table` for the small seeded arrays of `inputs()` into tests/golden/storage/. The test writes the same inputs
with `sosfuse2_gb300.storage` and compares keys, dtypes, shapes and values.
"""

import os
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REFERENCE_SRC = Path(os.environ.get('SOSFUSE2_REFERENCE_SRC', '/root/reference/src'))


def inputs():
    rng = np.random.default_rng(20261203)
    h = np.array([0.0, 1.0, 2.5])
    chi = np.deg2rad([0.0, 90.0])
    wl = np.array([450.0, 550.0, 650.0])
    fields = [rng.random((6, 13, 2), dtype=np.float32), rng.random((6, 13, 1), dtype=np.float32)]
    moments = [rng.random((6, 7, 2), dtype=np.float32), rng.random((6, 7, 1), dtype=np.float32)]
    table = rng.random((2, 3, 4, 3), dtype=np.float32)
    hs, el, az = np.array([-3.0, -6.0]), np.array([80.0, 45.0, 10.0]), np.array([15.0, 60.0, 105.0, 150.0])
    physical = dict(model='sos', version=3, flags=['a', 'b'])
    optics = dict(aod=0.2, g=0.7, albedo=0.3)
    contract = dict(settings=dict(L=1, nq=4), tolerance=1e-3)
    return dict(fields=fields, moments=moments, table=table, h=h, chi=chi, wl=wl, hs=hs, el=el, az=az,
                physical=physical, optics=optics, contract=contract, order=1)


def main():
    sys.path.insert(0, str(REFERENCE_SRC))
    from sosfuse2.jobs import run_storage as rs

    a = inputs()
    out = HERE / 'storage'
    out.mkdir(exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        rs.write_source(tmp, a['fields'], a['h'], a['chi'], a['wl'], physical=a['physical'], optics=a['optics'],
                        contract=a['contract'])
        rs.write_moments(tmp, a['moments'], a['h'], a['chi'], a['wl'], a['order'])
        rs.write_table(tmp, a['table'], a['wl'], a['hs'], a['el'], a['az'])
        for name in ('source.npz', 'moment.npz', 'table.npz'):
            (out / name).write_bytes((tmp / name).read_bytes())
    print('wrote', sorted(p.name for p in out.iterdir()))


if __name__ == '__main__':
    main()
