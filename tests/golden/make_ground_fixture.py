"""Generate the ground-illumination rays of the reference's own `Solver.prepare_ground` for golden states, with the
ground arrays that preparation produced, so that the device preparation (sosb_prepare_ground) is pinned to the
reference and not only to this project's host restatement.

Run in this container only (it imports the reference NumPy implementation from its source tree):

    python tests/golden/make_ground_fixture.py [walk1|strato15|all]

For each state (the walkthrough state at 550 nm; the stratospheric state over 15 wavelengths) the script assembles
the state by the reference's `create_configured` as make_fixtures.py does and records the exact per-ray inputs of the
reference's production ground preparation (the step engine_core.Solver.prepare_ground,
src/sosfuse2/solve/engine_core.py:103-147, defines): without a stratospheric layer, the cached candidate rays that
precompute/host_cache._ground_values receives (captured by wrapping that function during the assembly) with its solar
lookup at each ground point; with one, the per-cell geometry atmosphere/stratosphere.attach recomputes the ground
from (its in-process memo), whose optical depth adds (st + ssc) * strato_ext. Per ray it stores what
sosb_set_ground_rays takes: the cell, the local direction, the quadrature weight, the five slant columns (ground +
sun) and the stratospheric one, max(0, cos of the ground point's solar zenith) and the flag lit * (ground point on
the surface); with the state's albedo, its FP64 extinction (and the stratospheric one), and the gm, goff, gdir and
gval the reference produced.
"""

import copy
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import make_fixtures as mf  # noqa: E402

STATES = dict(walk1=mf.FIXTURES['walk1'], strato15=mf.FIXTURES['strato15'])


def _host_rays(s, z, aerosol):
    """Per-ray inputs of precompute/host_cache._ground_values (the production prepare_ground of a state without a
    stratospheric layer): its cached candidate rays, their slant columns with the aerosol column put back in place,
    and the solar lookup at each ground point, as that function evaluates them."""
    g, R = s.geo, s.ctx.b.R
    ray = np.flatnonzero(z['candidate'])
    cell = np.searchsorted(np.asarray(z['off']), ray, side='right') - 1
    col = np.empty((len(ray), 5))
    col[:, [0, 2, 3, 4]] = z['columns'][ray]
    col[:, 1] = aerosol
    q, r = z['q'][ray], z['r'][ray]
    sc, lit = g.sun.lookup(q, np.maximum(R, r))
    ch = np.arccos(np.clip(q[:, 2] / r, -1, 1))
    return dict(cell=cell.astype(np.int32), loc=np.asarray(z['loc'][ray], np.float64),
                weight=np.asarray(z['w'][ray], np.float64), cols=np.c_[sc + col, np.zeros(len(ray))],
                cos_sun=np.maximum(0.0, np.cos(ch)), ok=(np.asarray(lit, bool) & (r < R + 1e-5)).astype(np.uint8))


def _strato_rays(geom):
    """Per-ray inputs of atmosphere/stratosphere.attach's ground recomputation: per cell (loc, w, sc, lit, col, st,
    ssc, ec, re), the optical depth (sc + col) @ ext + (st + ssc) * strato_ext."""
    out = dict(cell=[], loc=[], weight=[], cols=[], cos_sun=[], ok=[])
    for c, (loc, w, sc, lit, col, st, ssc, ec, re) in enumerate(geom):
        out['cell'].append(np.full(len(loc), c, np.int32))
        out['loc'].append(np.asarray(loc, np.float64))
        out['weight'].append(np.asarray(w, np.float64))
        out['cols'].append(np.c_[sc + col, st + ssc])
        out['cos_sun'].append(np.maximum(0.0, np.cos(ec)))
        out['ok'].append((np.asarray(lit, bool) & (re < 6371.0 + 1e-5)).astype(np.uint8))
    return {k: np.concatenate(v) for k, v in out.items()}


def make(name, spec, out_dir=HERE):
    root = Path(tempfile.mkdtemp(prefix='sosb_ground_'))
    cache = mf._environment(root)
    from types import SimpleNamespace

    from sosfuse2.atmosphere.components import production_only
    from sosfuse2.jobs import run_state as rs
    from sosfuse2.jobs import walkthrough as wt

    production_only()
    a = SimpleNamespace(reduced=True, settings_json=None, stratosphere=None)
    st = wt.example_state()
    st['parameters'].update(spec.get('parameters', {}))
    if spec['strato']:
        st['stratosphere'] = dict(status='enabled', profile='gaussian', center_km=21.0, sigma_km=3.0, g=0.63, ssa=1.0)
    state = rs.effective_state(st, a)
    cfg = rs.resolve_settings(rs.settings_for(a), state)
    wl = np.asarray(spec['wavelengths'], float)
    cfg['wavelengths_nm'] = wl.tolist()
    cfg['wavelengths'] = len(wl)
    from sosfuse2.atmosphere import stratosphere
    from sosfuse2.precompute import host_cache

    seen = []
    original = host_cache._ground_values

    def record(s, scope, z, aerosol):
        seen.append((dict(z), np.asarray(aerosol)))
        return original(s, scope, z, aerosol)

    host_cache._ground_values = record
    stratosphere._GEOM_MEMO.clear()
    t0 = time.time()
    try:
        s, _ = rs.create_configured(root / 'tmp' / name / 'prepare_0', cfg, wl, 'numpy', state, 128,
                                    geometry_cache=cache)
    finally:
        host_cache._ground_values = original
    if spec['strato']:
        (_, geom), = stratosphere._GEOM_MEMO.values()
        rays = _strato_rays(geom)
        strato_ext = np.asarray(s.strato['ext'], np.float64)
    else:
        (z, aerosol), = seen
        rays = _host_rays(s, z, aerosol)
        strato_ext = np.zeros(0)
    arrays = {'ray_' + k: v for k, v in rays.items()}
    arrays.update(albedo=np.float64(s.fuse_state['parameters']['albedo']), ext=np.asarray(s.ext, np.float64),
                  strato_ext=strato_ext,
                  C=np.float64(s.ctx.C), gm=np.asarray(s.gm, np.float32), goff=np.asarray(s.goff, np.int64),
                  gdir=np.asarray(s.gdir, np.float32), gval=np.asarray(s.gval, np.float32))
    path = out_dir / f'ground_{name}.npz'
    np.savez_compressed(path, **arrays)
    print(f'ground_{name}: {len(rays["cell"])} rays, {len(s.gdir)} kept, {path.stat().st_size / 1e6:.2f} MB, '
          f'{time.time() - t0:.1f} s', flush=True)
    return path


if __name__ == '__main__':
    which = sys.argv[1] if len(sys.argv) > 1 else 'all'
    for key, spec in STATES.items():
        if which in ('all', key):
            make(key, copy.deepcopy(spec))
