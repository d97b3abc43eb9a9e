"""On-disk arrays of a solve in the reference's formats, so that `b200` results feed the reference's readers
(`tables_from_sources`, `check_anchor_rows`, the archive packer) unchanged.

Formats (src/sosfuse2/jobs/run_storage.py:235-302):

* `source.npz`: `source` [cells, slots, wavelengths] float32 (cell = ih * n_chi + ic, the solver's field layout,
  wavelength chunks joined along the last axis), `h` (km), `chi` (radians), `wavelength_nm`, and three JSON strings
  `physics`, `optics_state`, `source_contract` (sorted keys; the contract without NaN);
* `moment.npz`: `moment` [cells, 4 + K, wavelengths] float32, `h`, `chi`, `wavelength_nm`, `L` (int32) and the
  `layout` description;
* `table.npz`: `radiance` [solar elevation, view elevation, relative azimuth, wavelength] in W m^-2 sr^-1 nm^-1,
  the four axes as float32 (`wavelength_nm`, `solar_elevation_deg`, `view_elevation_deg`,
  `relative_azimuth_deg`) and `units`.

Each file is written to a temporary name and moved into place, so a reader never sees a partial file.
"""

import json
import os
from pathlib import Path

import numpy as np

UNITS = 'W m^-2 sr^-1 nm^-1'
MOMENT_LAYOUT = ('(cell=ih*n_chi+ic, slot, channel); slot [0:4] Rayleigh coherency, [4:4+K] scalar radiance SH '
                 'k=l(l+1)/2+m (m>=0, cos m phi), frame up=radial ex=sun-ward horizontal')


def _host(a):
    """A host array of a numpy array or a (CUDA) torch tensor."""
    if hasattr(a, 'detach'):
        a = a.detach().cpu().numpy()
    return np.asarray(a)


def _save(path, **arrays):
    path = Path(path)
    tmp = path.with_name(path.name + '.tmp')
    try:
        with tmp.open('wb') as f:
            np.savez(f, **arrays)
        os.replace(tmp, path)
    finally:
        tmp.unlink(missing_ok=True)
    return path


def write_source(prepare, fields, h, chi, wl, *, physical, optics, contract):
    """`prepare`/source.npz from the solver's converged fields (a list of wavelength chunks, each [cells, slots, W]
    on the host or the device)."""
    source = np.concatenate([_host(f).astype(np.float32, copy=False) for f in fields], axis=-1)
    return _save(Path(prepare) / 'source.npz', source=source, h=_host(h), chi=_host(chi), wavelength_nm=_host(wl),
                 physics=np.array(json.dumps(physical, sort_keys=True)),
                 optics_state=np.array(json.dumps(optics, sort_keys=True)),
                 source_contract=np.array(json.dumps(contract, sort_keys=True, allow_nan=False)))


def write_moments(prepare, moments, h, chi, wl, order):
    """`prepare`/moment.npz from moment chunks [cells, 4 + K, W]."""
    moment = np.concatenate([_host(m).astype(np.float32, copy=False) for m in moments], axis=-1)
    return _save(Path(prepare) / 'moment.npz', moment=moment, h=_host(h), chi=_host(chi), wavelength_nm=_host(wl),
                 L=np.int32(order), layout=np.array(MOMENT_LAYOUT))


def write_table(out, table, wl, hs, el, az):
    """`out`/table.npz from a radiance table [len(hs), len(el), len(az), W] (make_table's first result)."""
    return _save(Path(out) / 'table.npz', radiance=_host(table), wavelength_nm=_host(wl).astype('f4'),
                 solar_elevation_deg=_host(hs).astype('f4'), view_elevation_deg=_host(el).astype('f4'),
                 relative_azimuth_deg=_host(az).astype('f4'), units=np.array(UNITS))


def read_source(path):
    """(source [cells, slots, W] float32, h, chi, wavelength_nm, metadata dict) of a source.npz."""
    with np.load(path) as z:
        meta = {k: json.loads(str(z[k])) for k in ('physics', 'optics_state', 'source_contract')}
        return z['source'], z['h'], z['chi'], z['wavelength_nm'], meta


def read_table(path):
    """(radiance, wavelength_nm, solar_elevation_deg, view_elevation_deg, relative_azimuth_deg) of a table.npz."""
    with np.load(path) as z:
        if str(z['units']) != UNITS:
            raise ValueError(f'E_TABLE_UNITS: {z["units"]}')
        return (z['radiance'], z['wavelength_nm'], z['solar_elevation_deg'], z['view_elevation_deg'],
                z['relative_azimuth_deg'])
