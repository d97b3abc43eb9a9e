"""Packed state: the per-state inputs of the source iteration in one flat container.

A packed state holds what the reference's `Kernel.setup` constants (src/sosfuse2/solve/source_solver.py:1243-1339),
its cell `Bundle` (src/sosfuse2/solve/ray_geometry.py:290-392) and the observer rays of `engine_core.Solver.boxes`
(src/sosfuse2/solve/engine_core.py:208-238) carry, as NumPy arrays:

    meta                      JSON: L, K, W, nq, nq_query, nh, nc, ns, source_size, strato, g, mix, height, albedo,
                              top_km, profile_step_km, density_mask, air_surface, tolerance, max_eval, n_dirs,
                              box_points, (strato_center, strato_sigma, strato_norm)
    u, wu / uq, wuq           Gauss-Legendre nodes and weights on [0, 1] (cell / observer transport)
    h, chi, hr, ha            grids and density shapes
    ext [5, W], asca [W]      extinction per unit profile and aerosol scattering
    density_table [rows, 3]   air, ozone, NO2 on the uniform profile grid
    sun_h, sun_col            solar slant-column table
    gm, gd, gv                first-light Rayleigh moments and ground directions/values per cell
    rf, af, ext0, solar, box_ww   composition and observer-box vectors
    strato_*                  stratospheric layer (when meta.strato)
    cell_* / query_*          ray bundles (cell_off, p, target, d, dloc, weight, seg_off, seg_a, seg_b, seg_lower,
                              end_j, end_f, end_col, end_st, hits)

Packs are written by tests/golden/make_fixtures.py from the reference's own assembly, or by sosfuse2_gb300.synth.
"""

import json

import numpy as np

from . import _abi

BUNDLE_KEYS = ('cell_off', 'p', 'target', 'd', 'dloc', 'weight', 'seg_off', 'seg_a', 'seg_b', 'seg_lower', 'end_j',
               'end_f', 'end_col', 'end_st', 'hits')
DTYPES = dict(cell_off='i8', p='f8', target='f8', d='f8', dloc='f8', weight='f8', seg_off='i8', seg_a='f8',
              seg_b='f8', seg_lower='u1', end_j='i4', end_f='f8', end_col='f4', end_st='f4', hits='u1')


class PackedState:
    def __init__(self, source):
        if isinstance(source, dict):
            arrays = dict(source)
        else:
            with np.load(source) as z:
                arrays = {k: z[k] for k in z.files}
        meta = arrays.pop('meta')
        self.meta = meta if isinstance(meta, dict) else json.loads(str(meta))
        self.arrays = arrays
        m = self.meta
        self.L, self.K, self.W = int(m['L']), int(m['K']), int(m['W'])
        self.nh, self.nc, self.ns = int(m['nh']), int(m['nc']), int(m['ns'])
        self.nq, self.nq_query = int(m['nq']), int(m['nq_query'])
        self.strato = bool(m['strato'])
        self.source_size = 10 + self.K * (2 if self.strato else 1)
        if int(m.get('source_size', self.source_size)) != self.source_size:
            raise ValueError('E_SHAPE: source size disagrees with L and the stratospheric flag')
        self._keep = []

    def __getitem__(self, k):
        return self.arrays[k]

    def __contains__(self, k):
        return k in self.arrays

    @property
    def shape(self):
        return (self.ns, self.source_size, self.W)

    def bundle(self, prefix):
        return {k: self.arrays[prefix + '_' + k] for k in BUNDLE_KEYS}

    # ------------------------------------------------------------------ ABI structs
    def _arr(self, a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        self._keep.append(a)
        return a

    def dims(self):
        m = self.meta
        rows = int(m.get('monitor_rows', m.get('monitors', 5)))
        n_q = len(self.arrays['query_d'])
        pts = int(m['box_points'])
        dirs = int(m['n_dirs'])
        if n_q != rows * dirs * pts:
            rows = n_q // (dirs * pts)
        d = _abi.Dims(
            L=self.L, W=self.W, nh=self.nh, nc=self.nc, nq=self.nq, nq_query=self.nq_query, strato=int(self.strato),
            density_rows=len(self.arrays['density_table']), density_mask=int(m['density_mask']),
            n_sun_h=len(self.arrays['sun_h']), n_sun_x=self.arrays['sun_col'].shape[1],
            monitors=int(m.get('monitors', 5)), n_monitor_rows=rows, n_dirs=dirs, box_points=pts,
            top_km=float(m['top_km']), profile_step_km=float(m['profile_step_km']), mix=float(m['mix']),
            g=float(m['g']), height=float(m['height']), albedo=float(m['albedo']),
            air_surface=float(m['air_surface']),
            strato_center=float(m.get('strato_center', 0.0)), strato_sigma=float(m.get('strato_sigma', 1.0)),
            strato_norm=float(m.get('strato_norm', 1.0)))
        sup = m.get('support')
        if sup:  # extended top: the components' support ends
            d.lower_end_km, d.air_end_km = float(sup['lower_end']), float(sup['air_end'])
        return d

    def ground_csr(self):
        """Ground directions per cell as CSR (rows of gd/gv whose values are all zero carry nothing)."""
        if 'goff' in self.arrays:
            return (np.asarray(self.arrays['goff'], 'i8'), np.asarray(self.arrays['gdir'], 'f4'),
                    np.asarray(self.arrays['gval'], 'f4'))
        gd, gv = self.arrays['gd'], self.arrays['gv']
        keep = np.any(gv != 0, axis=2)
        goff = np.r_[0, np.cumsum(keep.sum(1))].astype('i8')
        return goff, np.ascontiguousarray(gd[keep], 'f4'), np.ascontiguousarray(gv[keep], 'f4')

    def constants(self):
        a = self.arrays
        f4, f8 = np.float32, np.float64
        goff, gdir, gval = self.ground_csr()
        c = _abi.Constants()
        spec = dict(u=(a['u'], f8), wu=(a['wu'], f8), uq=(a['uq'], f8), wuq=(a['wuq'], f8), h=(a['h'], f4),
                    chi=(a['chi'], f4), hr=(a['hr'], f4), ha=(a['ha'], f4), ext=(a['ext'], f4), asca=(a['asca'], f4),
                    density_table=(a['density_table'], f4), sun_h=(a['sun_h'], f4), sun_col=(a['sun_col'], f4),
                    gm=(a['gm'], f4), goff=(goff, np.int64), gdir=(gdir, f4), gval=(gval, f4), rf=(a['rf'], f4),
                    af=(a['af'], f4), ext0=(a['ext0'], f4), solar=(a['solar'], f8), box_ww=(a['box_ww'], f8))
        if self.strato:
            spec.update(strato_ext=(a['strato_ext'], f4), strato_sca=(a['strato_sca'], f4),
                        strato_chi=(a['strato_chi'], f4), strato_density=(a['strato_density'], f4),
                        strato_sun_col=(a['strato_sun_col'], f4), strato_eigen=(a['strato_eigen'], f4),
                        strato_sca_source=(a['strato_sca_source'], f4))
        if 'aer2' in a:
            spec.update(aer2=(a['aer2'], f4))
        if 'tropo_lut' in a:
            spec.update(tropo_lut=(a['tropo_lut'], f4), tropo_eigen=(a['tropo_eigen'], f4))
            c.tropo_bins = len(a['tropo_lut']) - 1
        for name, (v, dt) in spec.items():
            arr = self._arr(v, dt)
            ct = dict((f[0], f[1]) for f in _abi.Constants._fields_)[name]
            setattr(c, name, arr.ctypes.data_as(ct))
        return c

    def abi_bundle(self, prefix):
        b = self.bundle(prefix)
        arrs = {k: self._arr(v, DTYPES[k]) for k, v in b.items()}
        out = _abi.Bundle(ncell=len(arrs['cell_off']) - 1, nray=len(arrs['d']), nseg=len(arrs['seg_a']))
        for name, ct in _abi.Bundle._fields_[3:]:
            setattr(out, name, arrs[name].ctypes.data_as(ct))
        return out
