"""Radiance tables from a converged source: the b200 counterpart of `make_table`
(src/sosfuse2/outputs/radiance_table.py:167-219).

The reference captures the rays of `Solver.query` for every solar elevation, launches them as one phase-2 bundle per
`first` flag, and replays `query`'s post-processing: per ray the first three Stokes-ordered components summed in
FP64, times the solar spectrum, the first-order (single scattering and the ground-reflected direct beam) and the
multiple-scattering parts added, cast to float32 (radiance_table.py:43-104,200-210; solve/engine_core.py:208-226).
Here the rays come from the state family's geometry builder (`synth.Family.view_bundle`, the same observer frame and
view grid as `query`), each batch of solar elevations is one observer bundle on a dedicated handle, and the two
phase-2 transports run on the GPU; the summation and the solar factor are the reference's host operations.
`group` only partitions CUDA blocks in the reference, so it is validated and has no effect on the values.
"""

import time

import numpy as np

from .solver import Kernel


def axes(reduced=False):
    """Wavelengths, solar elevations, view elevations and relative azimuths of a table (radiance_table.py:32-38)."""
    wl = np.array([550.0]) if reduced else 360 + (np.arange(15) + 0.5) * 470 / 15
    hs = np.array([-3.0, -6.0]) if reduced else np.arange(6.0, -19.0, -1.0)
    nr, nc = (4, 6) if reduced else (100, 180)
    el = 90 - (np.arange(nr) + 0.5) * 90 / nr
    az = (np.arange(nc) + 0.5) * 180 / nc
    return wl, hs, el, az


def _spectral(rad, solar):
    """query's reduction of per-ray radiance [rays, W, 4] (float32): components 0..2 summed in FP64, solar-scaled."""
    r = np.asarray(rad, np.float64)
    return ((r[..., 0] + r[..., 1]) + r[..., 2]) * solar[None, :]


def make_table(s, source, hs, el, az, group=32, batch=25, log=print, *, family=None, views=None):
    """(table [len(hs), len(el), len(az), W] float32, seconds per batch) for the converged `source` of Solver `s`.
    The view rays of a batch of solar elevations come from `views(hs_batch, el, az)` (a packed bundle, one cell per
    solar elevation or per 64-ray pack, rays in (elevation, view elevation, azimuth) order), by default from
    `family.view_bundle`, the synth.Family the state was built from."""
    if group < 1:
        raise ValueError('E_TABLE_GROUP: group must be positive')
    if batch < 1:
        raise ValueError('E_TABLE_BATCH: batch must be positive')
    if views is None:
        if family is None:
            raise ValueError('E_TABLE_GEOMETRY: make_table needs the state family or a view-ray builder')
        views = family.view_bundle
    st = s.state
    k0 = s.kernel
    torch = k0.torch
    if isinstance(source, torch.Tensor):
        if tuple(source.shape) != st.shape:
            raise ValueError(f'E_SOURCE_SHAPE: {tuple(source.shape)}')
        field = source.to(device=k0.device, dtype=torch.float32).contiguous()
    else:
        source = np.ascontiguousarray(source, np.float32)
        if source.shape != st.shape:
            raise ValueError(f'E_SOURCE_SHAPE: {source.shape}')
        field = k0.field(source)
    hs, el, az = (np.asarray(v, np.float64).ravel() for v in (hs, el, az))
    solar = np.asarray(st['solar'], np.float64)
    table = np.empty((len(hs), len(el), len(az), st.W), np.float32)
    views_n = len(el) * len(az)
    kernel = None
    seconds = []
    try:
        for b0 in range(0, len(hs), batch):
            t = time.monotonic()
            part = list(range(b0, min(b0 + batch, len(hs))))
            rays = views(hs[part], el, az)
            if len(rays['d']) != len(part) * views_n:
                raise ValueError(f'E_TABLE_GEOMETRY: {len(rays["d"])} view rays for {len(part)} x {views_n} entries')
            if kernel is None:
                kernel = Kernel(st, k0.device)
                if k0.ground_optics is not None:  # ground arrays prepared on the solver's handle: the same here
                    kernel.set_ground_rays(k0.ground_rays)
                    kernel.prepare_ground(*k0.ground_optics)
            kernel.set_observer(rays)
            one = _spectral(kernel.host(kernel.transport(None, True)), solar)
            multiple = _spectral(kernel.host(kernel.transport(field, False)), solar)
            spec = (one + multiple).astype(np.float32)
            if not np.isfinite(spec).all() or (spec < 0).any():
                raise RuntimeError('E_RADIANCE_INVALID: nonfinite/negative')
            table[part] = spec.reshape(len(part), len(el), len(az), st.W)
            seconds.append(time.monotonic() - t)
            log(f'TABLE_FAST sun={hs[part[0]]:+g}..{hs[part[-1]]:+g} rays={len(part) * views_n} '
                f'seconds={seconds[-1]:.2f}')
    finally:
        if kernel is not None:
            kernel.close()
    return table, seconds
