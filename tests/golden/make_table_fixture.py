"""Generate the fixture that pins the radiance-table path (make_table) to the reference.

Run in this container only, after make_fixtures.py (it imports the reference from its source tree):

    python tests/golden/make_table_fixture.py

On the walkthrough state of walk1.npz (the same reference assembly), the script runs the reference's own
`outputs/radiance_table.make_table` on its NumPy backend over the reduced table axes (solar elevations -3 and -6
degrees, 4 x 6 views, 550 nm) for the source apply(apply(0)) of the reference's `Solver`, and stores

* `table_ref`: the reference's table [2, 4, 6, 1];
* the view rays the reference packed for that table (`radiance_table._capture`, i.e. `Solver.query`'s packs), in the
  packed-bundle layout under `table_*` keys (one bundle cell per 64-ray pack);
* `source`: the field the table was made from;
* `sun_col`/`sun_mask`: the solar column table where the first-light samples of the cells or of the view rays read
  it (zero elsewhere), replacing walk1.npz's narrower copy for the table's first-order part.
"""

import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))


def main():
    import make_fixtures as mf

    root = Path(tempfile.mkdtemp(prefix='sosb_table_fixture_'))
    cache = mf._environment(root)
    from types import SimpleNamespace

    from sosfuse2.atmosphere.components import production_only
    from sosfuse2.backends.sh_layout import source_size
    from sosfuse2.jobs import run_state as rs
    from sosfuse2.jobs import walkthrough as wt
    from sosfuse2.outputs import radiance_table as tf
    from sosfuse2.solve import ray_geometry as gm
    from sosfuse2.solve.source_solver import Solver

    production_only()
    a = SimpleNamespace(reduced=True, settings_json=None, stratosphere=None)
    state = rs.effective_state(wt.example_state(), a)
    cfg = rs.resolve_settings(rs.settings_for(a), state)
    wl = np.asarray([550.0])
    cfg['wavelengths_nm'] = wl.tolist()
    cfg['wavelengths'] = 1
    s, scope = rs.create_configured(root / 'tmp' / 'walk1' / 'prepare_0', cfg, wl, 'numpy', state, 128,
                                    geometry_cache=cache)
    geometry = gm.TransientGeometry(s, scope)
    groups = [geometry.cell(i) for i in range(s.geo.ns)]
    sys.path.insert(0, str(HERE.parents[1]))
    from sosfuse2_gb300.reference_adapter import _bundle

    c = s.kernel.setup(s, cfg['path_n'])
    strat = 'strato_ext' in c
    solver = Solver(s, geometry, fixed_boxes=False)
    zero = np.zeros((s.geo.ns, source_size(s), s.W), 'f4')
    source = np.asarray(solver.apply(solver.apply(zero)), 'f4')
    _, hs, el, az = tf.axes(True)
    t0 = time.time()
    table, _ = tf.make_table(s, source, hs, el, az, 32, 25, lambda m: None)
    seconds = time.time() - t0
    ee, aa = np.meshgrid(el, az, indexing='ij')
    raws = [r for h in hs for r in tf._capture(s, float(h), ee, aa, np.empty(0, 'f4'))]
    cq = s.kernel.setup(s, raws[0]['nq'])
    arrays = {'table_' + k: v for k, v in _bundle(raws, cq, strat).items()}
    mask = mf._touched_sun(c, groups, strat) | mf._touched_sun(cq, raws, strat)
    arrays.update(table_ref=np.asarray(table, 'f4'), source=source, hs=hs.astype('f8'), el=el.astype('f8'),
                  az=az.astype('f8'), sun_mask=mask,
                  sun_col=np.where(mask[..., None], c['sun_col'], np.float32(0)).astype('f4'),
                  packs=np.asarray([len(r['d']) for r in raws], 'i4'),
                  meta=np.asarray(f'{{"reference_seconds": {seconds:.2f}, "rays": {sum(len(r["d"]) for r in raws)}}}'))
    if strat:
        arrays['strato_sun_col'] = np.where(mask, c['strato_sun_col'], np.float32(0)).astype('f4')
    path = HERE / 'table_walk1.npz'
    np.savez_compressed(path, **arrays)
    print(f'{path.name}: {path.stat().st_size / 1e6:.2f} MB, table {table.shape}, reference {seconds:.1f} s')


if __name__ == '__main__':
    main()
