"""Reference-facing side of the `b200` backend: runs the reference's own state assembly, then the GB300 solve.

The reference builds a state on the CPU (`create_configured`, src/sosfuse2/solve/build.py:14-118; the per-cell
rays of `TransientGeometry.cell`, src/sosfuse2/solve/ray_geometry.py:406-423; the constants of `Kernel.setup`,
src/sosfuse2/solve/source_solver.py:1243-1339). `pack_state` turns that assembled state into a packed state
(sosfuse2_gb300.state) and `solve` runs `Solver.solve` on the GPU with the reference's signature and return value
(src/sosfuse2/solve/source_iteration.py:309-663). Only the state assembly uses the reference; the iteration itself
never does.

Requires an importable `sosfuse2` package (the reference) for `pack_state`; the GPU solve does not.
"""

import json

import numpy as np


def _bundle(groups, c, strat):
    """One CSR bundle of per-cell ray packs (`ray_geometry.pack` dicts), segments compacted to b - a > 1e-8, the
    ground-end columns of `numpy_reference.boundary_end_columns` (what the transport's boundary term reads)."""
    from sosfuse2.backends import numpy_reference as nr

    cell_off = [0]
    p, target, d, dloc, weight = [], [], [], [], []
    seg_counts, seg_a, seg_b, seg_lower = [], [], [], []
    end_j, end_f, end_col, end_st, hits = [], [], [], [], []
    for g in groups:
        n = len(g['d'])
        cell_off.append(cell_off[-1] + n)
        if not np.all(g['p'] == g['p'][0]) or not np.all(g['target'] == g['target'][0]):
            raise ValueError('E_START: one start point and frame per cell expected')
        p.append(g['p'][0])
        target.append(g['target'][0])
        d.append(g['d'])
        dloc.append(g['dloc'])
        weight.append(g['weight'])
        e = np.asarray(g['edges'])
        valid = (e[:, 1:] - e[:, :-1]) > 1e-8
        seg_counts.append(valid.sum(1))
        seg_a.append(e[:, :-1][valid])
        seg_b.append(e[:, 1:][valid])
        seg_lower.append(np.asarray(g['lower'])[valid])
        end_j.append(g['end_index'])
        end_f.append(g['end_fraction'])
        hits.append(g['hits_ground'])
        if np.any(g['hits_ground']) and 'gm' in c:
            col, stcol = nr.boundary_end_columns(g, c, strat)
        else:
            col, stcol = g['end_columns'], None
        end_col.append(np.asarray(col, 'f4'))
        end_st.append(np.zeros(n, 'f4') if stcol is None else np.asarray(stcol, 'f4'))
    return dict(
        cell_off=np.asarray(cell_off, 'i8'), p=np.asarray(p, 'f8'), target=np.asarray(target, 'f8'),
        d=np.concatenate(d).astype('f8'), dloc=np.concatenate(dloc).astype('f8'),
        weight=np.concatenate(weight).astype('f8'),
        seg_off=np.r_[0, np.cumsum(np.concatenate(seg_counts))].astype('i8'),
        seg_a=np.concatenate(seg_a).astype('f8'), seg_b=np.concatenate(seg_b).astype('f8'),
        seg_lower=np.concatenate(seg_lower).astype('u1'), end_j=np.concatenate(end_j).astype('i4'),
        end_f=np.concatenate(end_f).astype('f8'), end_col=np.concatenate(end_col).astype('f4'),
        end_st=np.concatenate(end_st).astype('f4'), hits=np.concatenate(hits).astype('u1'))


def observer_rays(s):
    """The observer rays of engine_core.Solver.boxes, captured without transport (the reference's own recording
    trick of Solver.boxes_fixed, source_iteration.py:238-250)."""
    raws = []

    def record(raw, solver, _field, first=False):
        raws.append(raw)
        return np.zeros((len(raw['d']), solver.W, 2, 4), 'f8')

    s.kernel.transport = record
    try:
        s.boxes(np.empty(0, 'f4'), False)
    finally:
        del s.kernel.transport
    return raws


def thin_layer_cut(arrays, strat):
    """The thin-layer skip of the combined SH plane (sh_layout.combined_coefficients with skip_thin,
    src/sosfuse2/backends/sh_layout.py:135-152) applied to the packed densities: on grids of at most 128 heights the
    aerosol density ha and the stratospheric source density at or below 1e-7 of the air density hr become 0. Those
    densities enter only the plane, which the device forms as aerosol slots x ha + stratospheric slots x density."""
    hr = np.asarray(arrays['hr'], 'f4')
    if len(hr) > 128:
        return arrays
    cut = np.float32(1e-7) * hr
    for k in ('ha', 'strato_density') if strat else ('ha',):
        v = np.asarray(arrays[k], 'f4')
        arrays[k] = np.where(v > cut, v, np.float32(0)).astype('f4')
    return arrays


def pack_state(s, geometry, scope, tolerance=1e-3, max_eval=64):
    """Packed-state arrays of a reference-assembled state `s` (create_configured) with its TransientGeometry."""
    from sosfuse2.backends.sh_layout import source_size

    groups = [geometry.cell(i) for i in range(s.geo.ns)]
    nq = groups[0]['nq']
    c = s.kernel.setup(s, nq)
    strat = 'strato_ext' in c
    raws = observer_rays(s)
    cq = s.kernel.setup(s, raws[0]['nq'])
    L, K, W = s.kernel.L, s.kernel.K, s.W
    u4, w4 = np.polynomial.legendre.leggauss(4)
    opt = c['density_optics']
    meta = dict(
        L=L, K=K, W=W, nq=nq, nq_query=raws[0]['nq'], nh=len(s.geo.h), nc=len(s.geo.chi), ns=int(s.geo.ns),
        source_size=int(source_size(s)), strato=bool(strat), g=float(c['g']), mix=float(c['mix']),
        height=float(c['height']), albedo=float(c['albedo']), top_km=float(c['domain'].top_km),
        profile_step_km=float(c['domain'].step_km), density_mask=int(opt['mask']),
        air_surface=float(opt.get('air_surface', 1.0)), tolerance=float(tolerance), max_eval=int(max_eval),
        monitors=len(s.ctx.b.HS), n_dirs=len(s.ctx.b.DIRS), box_points=16, wavelengths_nm=list(map(float, s.wl)),
        C=float(scope.C))
    arrays = dict(
        u=np.asarray(c['u'], 'f8'), wu=np.asarray(c['wu'], 'f8'), uq=np.asarray(cq['u'], 'f8'),
        wuq=np.asarray(cq['wu'], 'f8'), h=c['h'], chi=c['chi'], hr=c['hr'], ha=c['ha'], ext=c['ext'], asca=c['asca'],
        sun_h=c['sun_h'], sun_col=c['sun_col'], gm=c['gm'], gd=c['gd'], gv=c['gv'],
        density_table=np.asarray(opt['table'], 'f4'), rf=np.asarray(s.rf, 'f4'), af=np.asarray(s.af[:K] if s.af is not None else np.zeros(K), 'f4'),
        ext0=np.asarray(s.ext[0], 'f4'), solar=np.asarray(s.solar, 'f8'), box_ww=(w4[:, None] * w4[None, :] / 4).ravel())
    if 'tropo_lut' in c:  # TROPO_MIE: the per-wavelength phase table and the SH eigenvalues chi_l / (2l + 1)
        from sosfuse2.atmosphere.tropo_mie import eigen_by_sh as tropo_eigen

        bins = int(c['tropo_bins'])
        arrays['tropo_lut'] = np.asarray(c['tropo_lut'], 'f4').reshape(bins + 1, W)
        arrays['tropo_eigen'] = np.asarray(tropo_eigen(s.tropo, L), 'f4')
        meta['tropo_bins'] = bins
    dom = c['domain']
    if dom.top_km > dom.lower_end:  # extended top: the components' support ends (numpy_reference.py:158-183)
        meta['support'] = dict(lower_end=float(dom.lower_end), air_end=float(dom.air_end))
    if 'aer2' in c:  # AEROSOL_2L: the two-layer profile's kernel vector
        arrays['aer2'] = np.asarray(c['aer2'], 'f4')
        meta['aerosol_profile'] = 'two_layer'
    if c.get('sh_combine') and c.get('sh_combine_skip'):
        # The device always forms the combined plane (aerosol slots x ha + stratospheric slots x their density); the
        # thin-layer skip of sh_layout.combined_coefficients (src/sosfuse2/backends/sh_layout.py:135-152) zeroes a
        # density at or below 1e-7 of the air density on grids of at most 128 heights, and those densities enter
        # only that plane.
        meta['sh_combine_skip'] = True
    if strat:
        from sosfuse2.atmosphere.stratosphere import eigen_by_sh

        prof = c['strato_profile']
        arrays.update(
            strato_ext=c['strato_ext'], strato_sca=c['strato_sca'], strato_chi=np.asarray(c['strato_chi'], 'f4'),
            strato_density=c['strato_density'], strato_sun_col=c['strato_sun_col'],
            strato_eigen=np.asarray(eigen_by_sh(s.strato, L), 'f4'), strato_sca_source=np.asarray(s.strato['sca'], 'f4'))
        meta.update(strato_center=float(prof['center']), strato_sigma=float(prof['sigma']),
                    strato_norm=float(prof['norm']))
    if meta.get('sh_combine_skip'):
        thin_layer_cut(arrays, strat)
    for k, v in _bundle(groups, c, strat).items():
        arrays['cell_' + k] = v
    for k, v in _bundle(raws, cq, strat).items():
        arrays['query_' + k] = v
    meta.update(rays=int(len(arrays['cell_d'])), segments=int(len(arrays['cell_seg_a'])),
                query_rays=int(len(arrays['query_d'])))
    arrays['meta'] = json.dumps(meta)
    return arrays


def solve_packed(arrays, max_eval=64, tolerance=1e-3, device=None):
    """Solver.solve of a packed state on the GPU: (field [cells, slots, W] f4 host array, stats with the reference's
    keys: seconds, evaluations, tolerance, converged, history); raises the reference's E_* errors."""
    from .solver import Solver
    from .state import PackedState

    solver = Solver(PackedState(arrays), device=device)
    try:
        return solver.solve(max_eval, tolerance)
    finally:
        solver.kernel.close()


def solve(s, geometry, scope, max_eval=64, tolerance=1e-3, device=None):
    """Solver.solve of a reference-assembled state on the GPU: (field [cells, slots, W] f4, stats)."""
    return solve_packed(pack_state(s, geometry, scope, tolerance, max_eval), max_eval, tolerance, device)


def view_rays(s, hs, el, az):
    """The view rays of a radiance table of a reference-assembled state as one packed bundle per call: the packs
    `Solver.query` builds for every solar elevation of `hs` over the (el, az) grid, captured without transport as
    outputs/radiance_table.py:43-54 does, one bundle cell per 64-ray pack."""
    from sosfuse2.outputs import radiance_table as tf

    ee, aa = np.meshgrid(np.asarray(el, float), np.asarray(az, float), indexing='ij')
    raws = [r for h in np.asarray(hs, float).ravel() for r in tf._capture(s, float(h), ee, aa, np.empty(0, 'f4'))]
    cq = s.kernel.setup(s, raws[0]['nq'])
    return _bundle(raws, cq, 'strato_ext' in cq)


def make_table(s, source, hs, el, az, group=32, batch=25, log=print, *, geometry, scope, device=None):
    """outputs/radiance_table.make_table (radiance_table.py:167-219) of a reference-assembled state on the GPU: the
    reference's own view rays (view_rays), both phase-2 transports on the device, `query`'s reduction; returns
    (table [len(hs), len(el), len(az), W] float32, seconds per batch) like the reference."""
    from .solver import Solver
    from .state import PackedState
    from .table import make_table as table

    solver = Solver(PackedState(pack_state(s, geometry, scope)), device=device)
    try:
        return table(solver, source, hs, el, az, group, batch, log, views=lambda h, e, a: view_rays(s, h, e, a))
    finally:
        solver.kernel.close()
