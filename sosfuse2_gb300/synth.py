"""Seeded synthetic states (packed states of sosfuse2_gb300.state) for the benchmark configurations.

The GPU machine has no reference installation, so the workloads are built here from a synthetic atmosphere on the
reference's geometry. The geometry restates the reference's ray construction:

* local frame of a cell point, src/sosfuse2/rays/shell_segments.py:37-40, and the target basis, solve/engine_core.py:8-20;
* ring-edge incoming-direction quadrature (sinh-mapped Gauss-Legendre in mu between the horizon, tangent, shadow
  and ring edges, trapezoid in azimuth), src/sosfuse2/rays/incoming_rings.py:11-126;
* segment ends: shell exit, opaque-ground hit, tangent point and shadow-cylinder crossings
  (rays/shell_segments.py:43-66), plus the extra shells at 10, 25, 40 (and 80) km (solve/ray_geometry.py:28-82);
* the observer boxes: 5 solar elevations x 7 directions x 4x4 Gauss-Legendre points at 0.1 km, 24 nodes per segment
  (solve/engine_core.py:208-238, solve/engine.py:435-446).

Slant columns (towards the sun from any point, and to the ground along any downward ray) depend only on the height
and the zenith cosine of a ray, because every profile here is a function of height alone; they are tabulated once per
state on a (height, x) grid like the reference's solar table (rays/shell_segments.py:109-112,230-325) and
interpolated bilinearly. The first-light ground term (solve/engine_core.py:103-147) is built from those tables.

The atmosphere: air exp(-h/8); ozone as a Chapman layer; tropospheric aerosol exp(-h/H) with Henyey-Greenstein
phase; optional stratospheric Gaussian layer with Henyey-Greenstein Legendre moments; optional NO2 Gaussian layer
and O4 proportional to the squared air density; Lambertian ground. Spectral shapes are seeded smooth curves.
"""

import ctypes
import json
import math

import numpy as np

R = 6371.0
OBSERVER_KM = 0.1
SUN_HEIGHT_INTERVALS = 80
MONITOR_ELEVATIONS = (2.0, -3.0, -6.0, -9.0, -12.0)
DIRS = ((2, 0), (10, 0), (30, 0), (10, 180), (30, 180), (10, 90), (89, 0))
DU = 2.687e16  # molecules cm^-2 per Dobson unit


def production_chi_deg():
    """The 75 solar-zenith nodes of the reference's full grid (rays/shell_segments.py:88-102)."""
    return np.unique(np.r_[np.arange(0, 81, 10), np.arange(80, 85, 1), np.arange(85, 110, 0.5),
                           np.arange(110, 120, 2), np.arange(120, 181, 10)]).astype(float)


REDUCED_CHI_DEG = np.array([0.0, 60.0, 85.0, 90.0, 93.0, 96.0, 105.0, 110.0, 140.0, 180.0])


def gauss01(n):
    x, w = np.polynomial.legendre.leggauss(n)
    return (x + 1) / 2, w / 2


def frame(r, chi):
    up = np.array([np.sin(chi), 0.0, np.cos(chi)])
    ex = np.array([-np.cos(chi), 0.0, np.sin(chi)])
    return r * up, up, ex


def target_basis(p):
    """Orthonormal local frame (east-like, north-like, up) of a point, as columns of a 3x3 matrix."""
    r = np.linalg.norm(p)
    up = p / r
    ex = np.array([0.0, 0.0, 1.0]) - up[2] * up
    n = np.linalg.norm(ex)
    ex = ex / n if n > 1e-12 else np.array([-(1.0 if up[2] >= 0 else -1.0), 0.0, 0.0])
    return np.stack([ex, np.cross(up, ex), up], -1)


# ------------------------------------------------------------------------------------------------ quadrature
def _ring_mus(r, chi, phi, heights, p, up, ex, ey):
    """Zenith cosines where the view plane at azimuth phi meets the shadow ring of each shell."""
    horizontal = np.cos(phi) * ex + np.sin(phi) * ey
    normal = np.cross(up, horizontal)
    amp = R * math.hypot(normal[0], normal[1])
    if amp < 1e-10:
        return []
    angle = math.atan2(normal[1], normal[0])
    out = []
    for h in heights:
        z = -math.sqrt(max(0.0, (R + h) ** 2 - R * R))
        target = -normal[2] * z / amp
        if abs(target) > 1:
            continue
        delta = math.acos(target)
        for az in (angle - delta, angle + delta):
            q = np.array([R * math.cos(az), R * math.sin(az), z])
            d = q - p
            length = math.sqrt(d @ d)
            if length < 1e-8:
                continue
            d /= length
            if d @ horizontal <= 1e-10:
                continue
            b = p @ d
            disc = b * b - r * r + R * R
            hit = -b - math.sqrt(max(0.0, disc))
            if disc >= 0 and b < 0 and hit >= -1e-7 and hit < length - 1e-5:
                continue
            out.append(float(d @ up))
    return out


def ring_quadrature(r, chi, nmu, nphi, heights, rings=True, a=4.0):
    """Incoming directions in the local frame (ex, ey, up) and solid-angle weights (sum 4 pi)."""
    mg = -math.sqrt(max(0.0, 1 - (R / r) ** 2))
    sa = math.sinh(a)
    u, wu = gauss01(nmu)
    sinchi, coschi = math.sin(chi), math.cos(chi)
    rp = r * sinchi
    p, up, ex = frame(r, chi)
    ey = np.cross(up, ex)
    mus, phis, ws = [], [], []
    for j, phi in enumerate(np.linspace(0, np.pi, nphi + 1)):
        edges = [-1.0, 1.0, mg, 0.0, mg - 0.05234, mg + 0.05234, mg - 0.0061, mg + 0.0061]
        if rp > R + 1e-8 and abs(sinchi) > 1e-8:
            kk = R / math.sqrt(rp * rp - R * R)
            for sign in (-1, 1):
                t = math.cos(phi) * coschi / sinchi + sign * math.sin(phi) / (kk * sinchi)
                mu = t / math.sqrt(1 + t * t)
                st = math.sqrt(1 - mu * mu)
                dx = mu * sinchi - st * math.cos(phi) * coschi
                dy = -st * math.sin(phi)
                dz = mu * coschi + st * math.cos(phi) * sinchi
                tmin = -rp * dx / max(dx * dx + dy * dy, 1e-25)
                if abs(dx) + abs(dy) < 1e-10 or (tmin > 0 and r * coschi + tmin * dz < 0):
                    edges.append(mu)
        if phi < np.pi / 6:
            mu = coschi / math.sqrt(coschi ** 2 + math.cos(phi) ** 2 * sinchi ** 2 + 1e-300)
            edges.extend([mu, mu - 0.012, mu + 0.012])
        if rings:
            edges += _ring_mus(r, chi, phi, heights, p, up, ex, ey)
        edges = np.unique(np.clip(edges, -1, 1))
        delta = edges - mg
        tt = np.sign(delta) * np.arcsinh(np.abs(delta) / np.where(delta < 0, 1 + mg, 1 - mg) * sa) / a
        keep = tt[1:] - tt[:-1] >= 1e-10
        left = tt[:-1][keep, None]
        right = tt[1:][keep, None]
        t = left + (right - left) * u
        den = np.where(t < 0, 1 + mg, 1 - mg)
        mus.append((mg + np.sign(t) * den * np.sinh(a * np.abs(t)) / sa).ravel())
        ws.append(((right - left) * wu * den * a * np.cosh(a * np.abs(t)) / sa * (2 * np.pi / nphi)
                   * (0.5 if j in (0, nphi) else 1.0)).ravel())
        phis.append(np.full(t.size, phi))
    mu = np.concatenate(mus)
    phi = np.concatenate(phis)
    st = np.sqrt(np.maximum(0, 1 - mu * mu))
    return np.column_stack([st * np.cos(phi), st * np.sin(phi), mu]), np.concatenate(ws)


_NATIVE = True
_DEVICE = None


class device_geometry:
    """Context in which the ray segments and ray-end quantities of the bundles (sosb_ray_segments) and the solar column
    tables (sosb_column_table) are built on the GPU `device` (sosb_ray_segments_device, one thread per ray;
    sosb_column_table_device, one thread per table entry) instead of on host threads; the quadratures and the CSR
    compaction stay on the host."""

    def __init__(self, device='cuda:0'):
        self.device = device

    def __enter__(self):
        global _DEVICE
        self.previous, _DEVICE = _DEVICE, self.device
        return self

    def __exit__(self, *exc):
        global _DEVICE
        _DEVICE = self.previous


class numpy_geometry:
    """Context in which the geometry builders (ring quadratures, solar column tables, ray segments) run their NumPy
    restatements instead of libsosb's host code, so that no native library is loaded (the CPU baseline's workload)."""

    def __enter__(self):
        global _NATIVE
        self.previous, _NATIVE = _NATIVE, False
        return self

    def __exit__(self, *exc):
        global _NATIVE
        _NATIVE = self.previous


def quadratures(specs):
    """The ring quadrature (loc, w) of every (r, chi, nmu, nphi, heights, rings) of `specs`, in order, by libsosb's
    sosb_ring_quadrature (host threads; the same rule as ring_quadrature). The specs of one call share nmu, nphi,
    heights and rings."""
    from . import _abi, build

    if not specs:
        return []
    if not _NATIVE:
        return [ring_quadrature(*sp) for sp in specs]
    nmu, nphi, heights, rings = specs[0][2:]
    if any(sp[2:] != (nmu, nphi, heights, rings) for sp in specs):
        raise ValueError('E_SYNTH: one quadrature rule per call')
    lib = _abi.library(build.build())
    r = np.ascontiguousarray([sp[0] for sp in specs], np.float64)
    chi = np.ascontiguousarray([sp[1] for sp in specs], np.float64)
    hh = np.ascontiguousarray(heights, np.float64)
    u, wu = (np.ascontiguousarray(v, np.float64) for v in gauss01(nmu))
    counts = np.zeros(len(specs), np.int64)
    args = (len(specs), _abi.ptr(r, _abi.P_f64), _abi.ptr(chi, _abi.P_f64), int(nmu), int(nphi),
            _abi.ptr(hh, _abi.P_f64) if len(hh) else None, len(hh), int(bool(rings)), 4.0, _abi.ptr(u, _abi.P_f64),
            _abi.ptr(wu, _abi.P_f64), _abi.ptr(counts, _abi.P_i64))
    if lib.sosb_ring_quadrature(*args, None, None, 0, 0):
        raise RuntimeError('E_SYNTH: sosb_ring_quadrature failed')
    total = int(counts.sum())
    loc = np.empty((total, 3))
    w = np.empty(total)
    if lib.sosb_ring_quadrature(*args, _abi.ptr(loc, _abi.P_f64), _abi.ptr(w, _abi.P_f64), total, 0):
        raise RuntimeError('E_SYNTH: sosb_ring_quadrature failed')
    off = np.r_[0, np.cumsum(counts)]
    return [(loc[off[i]:off[i + 1]], w[off[i]:off[i + 1]]) for i in range(len(specs))]


# ------------------------------------------------------------------------------------------------ segments
def ray_edges(p, d, top, shells):
    """Sorted path coordinates of every crossing: start, tangent, shadow-cylinder roots, extra shells, end."""
    b = np.sum(p * d, -1)
    pp = np.sum(p * p, -1)
    end = -b + np.sqrt(np.maximum(b * b - pp + (R + top) ** 2, 0))
    disc = b * b - pp + R * R
    hit = -b - np.sqrt(np.maximum(disc, 0))
    ground = (disc >= 0) & (b < 0) & (hit >= -1e-7)
    end = np.maximum(np.where(ground, np.maximum(hit, 0), end), 0)
    tangent = np.where((-b > 0) & (-b < end), -b, end)
    aa = d[:, 0] ** 2 + d[:, 1] ** 2
    bb = p[:, 0] * d[:, 0] + p[:, 1] * d[:, 1]
    cc = p[:, 0] ** 2 + p[:, 1] ** 2 - R * R
    ds = bb * bb - aa * cc
    cols = [np.zeros_like(end), tangent, end]
    for sign in (-1, 1):
        root = (-bb + sign * np.sqrt(np.maximum(ds, 0))) / np.maximum(aa, 1e-30)
        ok = (aa > 1e-20) & (ds >= 0) & (root > 0) & (root < end) & (p[:, 2] + root * d[:, 2] < 0)
        cols.append(np.where(ok, root, end))
    for height in shells:
        disc2 = b * b - pp + (R + height) ** 2
        for sign in (-1, 1):
            root = -b + sign * np.sqrt(np.maximum(disc2, 0))
            cols.append(np.where((disc2 > 0) & (root > 0) & (root < end), root, end))
    return np.sort(np.column_stack(cols), axis=-1), ground


def compact_segments(p, d, edges):
    """Valid segments (b - a > 1e-8) of each ray: CSR offsets, ends and the lower-end flag."""
    a, b = edges[:, :-1], edges[:, 1:]
    valid = (b - a) > 1e-8
    qa = p[:, None, :] + a[..., None] * d[:, None, :]
    qb = p[:, None, :] + b[..., None] * d[:, None, :]
    lower = np.sum(qa * qa, -1) <= np.sum(qb * qb, -1)
    counts = valid.sum(1)
    return (np.r_[0, np.cumsum(counts)].astype(np.int64), a[valid], b[valid], lower[valid].astype(np.uint8))


# ------------------------------------------------------------------------------------------------ atmosphere
class Atmosphere:
    """Synthetic seeded atmosphere on 0..top km for wavelengths `wl` (nm)."""

    def __init__(self, wl, seed=0, top=80.0, aod=0.1, ssa=0.95, g=0.7, scale_height=1.2, angstrom=1.3,
                 ozone_du=300.0, ozone_peak=22.0, ozone_sigma_cm2=3e-21, albedo=0.3,
                 strato_tau=0.01, strato_center=20.0, strato_sigma=3.0, strato_g=0.6,
                 no2_column=0.0, no2_center=25.0, o4=False):
        rng = np.random.default_rng(seed)
        self.aod = aod
        self.wl = np.asarray(wl, float)
        self.W = len(self.wl)
        self.top = float(top)
        self.g, self.ssa, self.H, self.albedo = g, ssa, scale_height, albedo
        w = self.wl
        # Rayleigh with the lambda^-4 law; ozone Chappuis-like smooth band scaled so 550 nm has ozone_sigma_cm2
        self.ray = 0.013558 * (550.0 / w) ** 4
        bump = lambda x, c, s: np.exp(-0.5 * ((x - c) / s) ** 2)  # noqa: E731
        jitter = 1 + 0.05 * rng.standard_normal(3)
        o3_shape = (bump(w, 600.0 * jitter[0] ** 0.02, 55.0) + 0.08) / (bump(550.0, 600.0 * jitter[0] ** 0.02, 55.0)
                                                                        + 0.08)
        self.o3_sigma = ozone_sigma_cm2 * o3_shape
        self.ozone_du = ozone_du
        self.ozone_peak = ozone_peak
        self.aer = aod / (scale_height * -math.expm1(-80.0 / scale_height)) * (550.0 / w) ** angstrom
        self.no2_column = no2_column
        self.no2_center = no2_center
        self.no2_sigma = (1.0 + 0.4 * rng.random()) * 1e-19 * (450.0 / w) ** 2.0 * (1 + 0.1 * np.sin(w / 7.0))
        self.o4 = bool(o4)
        self.o4_coeff = (1e-3 * (bump(w, 477.0, 4.0) + 0.6 * bump(w, 577.0, 5.0) + 0.9 * bump(w, 630.0, 4.0))
                         if o4 else np.zeros(self.W))
        self.strato = strato_tau > 0
        self.strato_tau, self.strato_center, self.strato_sigma, self.strato_g = (strato_tau, strato_center,
                                                                                 strato_sigma, strato_g)
        if self.strato:
            z = np.linspace(0, 80.0, 8001)
            self.strato_norm = float(np.trapezoid(np.exp(-0.5 * ((z - strato_center) / strato_sigma) ** 2), z))
            self.strato_ext = strato_tau * (550.0 / w) ** 0.8
        self.solar = 1.85 * (1 + 0.1 * np.sin(w / 13.0 + rng.random())) * np.exp(-((w - 480.0) / 400.0) ** 2)

    # ozone Chapman shape normalised to a 15 km column (the reference's triangle normalisation)
    def ozone_shape(self, h):
        if not hasattr(self, '_o3_norm'):
            zz = np.linspace(0, 120, 12001)
            z = (zz - self.ozone_peak) / 5.0
            self._o3_norm = 15.0 / np.trapezoid(np.exp(1 - z - np.exp(-z)), zz)
        z = (np.asarray(h, float) - self.ozone_peak) / 5.0
        return np.exp(1 - z - np.exp(-z)) * self._o3_norm

    def no2_shape(self, h):
        return np.exp(-0.5 * ((np.asarray(h, float) - self.no2_center) / 4.0) ** 2)

    def profiles(self, h):
        """[n, 5] air, aerosol, ozone, NO2, O4 shapes (the kernel's profile_at with the density table)."""
        h = np.clip(np.asarray(h, float), 0, self.top)
        air = np.exp(-h / 8.0)
        return np.stack([air, np.exp(-h / self.H), self.ozone_shape(h), self.no2_shape(h), air * air], -1)

    def strato_profile(self, h):
        if not self.strato:
            return np.zeros_like(np.asarray(h, float))
        return np.exp(-0.5 * ((np.asarray(h, float) - self.strato_center) / self.strato_sigma) ** 2) / self.strato_norm

    def ext(self):
        """[5, W] extinction per unit profile (km^-1)."""
        # beta [km^-1] = sigma [cm^2] * column [cm^-2] * shape / (column integral of the shape [km])
        o3 = self.o3_sigma * self.ozone_du * DU / 15.0
        no2_norm = 4.0 * math.sqrt(2 * math.pi)
        no2 = self.no2_sigma * self.no2_column / no2_norm
        return np.stack([self.ray, self.aer, o3, no2, self.o4_coeff])


# ------------------------------------------------------------------------------------------------ column tables
def _columns_along(r0, mu, atm, shells, n):
    """Columns (5 components + stratosphere) from radius r0 along zenith cosine mu to the top or the ground."""
    p = np.column_stack([np.zeros_like(mu), np.zeros_like(mu), np.full_like(mu, r0)])
    d = np.column_stack([np.sqrt(np.maximum(1 - mu * mu, 0)), np.zeros_like(mu), mu])
    edges, ground = ray_edges(p, d, atm.top, shells)
    u, wu = gauss01(n)
    out = np.zeros((len(mu), 6))
    for k in range(edges.shape[1] - 1):
        a, b = edges[:, k, None], edges[:, k + 1, None]
        t = a + (b - a) * u
        q = p[:, None, :] + t[..., None] * d[:, None, :]
        h = np.linalg.norm(q, axis=-1) - R
        w = (b - a) * wu
        prof = atm.profiles(h.ravel()).reshape(*h.shape, 5)
        out[:, :5] += np.einsum('rn,rnk->rk', w, prof)
        out[:, 5] += np.sum(w * atm.strato_profile(h), -1)
    return out, ground


def column_rows(atm, shells, h, x, n=32):
    """The (up, down) column tables [len(h), len(x), 6] by the NumPy restatement (_columns_along), row by row: the
    reference the native sosb_column_table is checked against."""
    up = np.empty((len(h), len(x), 6))
    down = np.empty_like(up)
    for i, hh in enumerate(h):
        r = R + hh
        mg = -math.sqrt(max(0.0, 1 - (R / r) ** 2))
        mu = mg + (1 - mg) * x ** 2
        mu[0] = mg + 1e-9
        up[i] = _columns_along(r, mu, atm, shells, n)[0]
        mud = mg - (1 + mg) * x ** 2
        mud[0] = mg - 1e-9
        down[i] = _columns_along(r, np.maximum(mud, -1.0), atm, shells, n)[0]
    return up, down


def native_column_table(atm, shells, h, x, n=32, threads=0, device=None):
    """The same tables by libsosb's sosb_column_table (host threads; built in-tree on first use), or by
    sosb_column_table_device on `device` (the same column function on the GPU, results back in host arrays)."""
    from . import _abi, build

    lib = _abi.library(build.build())
    atm.ozone_shape(0.0)  # sets the ozone normalisation
    shape = _abi.ProfileShape(top=atm.top, aerosol_height=atm.H, ozone_peak=atm.ozone_peak, ozone_norm=atm._o3_norm,
                              no2_center=atm.no2_center, strato=int(atm.strato),
                              strato_center=atm.strato_center, strato_sigma=atm.strato_sigma,
                              strato_norm=atm.strato_norm if atm.strato else 1.0)
    h = np.ascontiguousarray(h, np.float64)
    x = np.ascontiguousarray(x, np.float64)
    sh = np.ascontiguousarray(shells, np.float64)
    u, wu = (np.ascontiguousarray(v, np.float64) for v in gauss01(n))
    if device is not None:
        import torch

        dev = torch.device(device)
        t = lambda a: torch.as_tensor(a, device=dev)  # noqa: E731
        hd, xd, ud, wd = t(h), t(x), t(u), t(wu)
        upd = torch.empty((len(h), len(x), 6), dtype=torch.float64, device=dev)
        downd = torch.empty_like(upd)
        vp = lambda a: ctypes.c_void_p(a.data_ptr())  # noqa: E731
        stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        rc = lib.sosb_column_table_device(len(h), vp(hd), len(x), vp(xd), _abi.ptr(sh, _abi.P_f64), len(sh), vp(ud),
                                          vp(wd), n, ctypes.byref(shape), vp(upd), vp(downd), stream)
        if rc:
            raise RuntimeError(f'E_COLUMN_TABLE: sosb_column_table_device returned {rc}')
        return upd.cpu().numpy(), downd.cpu().numpy()
    up = np.empty((len(h), len(x), 6))
    down = np.empty_like(up)
    rc = lib.sosb_column_table(len(h), _abi.ptr(h, _abi.P_f64), len(x), _abi.ptr(x, _abi.P_f64),
                               _abi.ptr(sh, _abi.P_f64), len(sh), _abi.ptr(u, _abi.P_f64), _abi.ptr(wu, _abi.P_f64), n,
                               ctypes.byref(shape), _abi.ptr(up, _abi.P_f64), _abi.ptr(down, _abi.P_f64), int(threads))
    if rc:
        raise RuntimeError(f'E_COLUMN_TABLE: sosb_column_table returned {rc}')
    return up, down


class ColumnTable:
    """Slant columns on a (height, x) grid for upward (sun) and downward (ground) rays (sosb_column_table)."""

    def __init__(self, atm, shells, scale=2, n=32):
        self.top = atm.top
        self.h = np.linspace(0, math.sqrt(atm.top), SUN_HEIGHT_INTERVALS * scale + 1) ** 2
        self.x = np.linspace(0, 1, 400 * scale + 1)
        if _NATIVE and _DEVICE is not None:
            self.up, self.down = native_column_table(atm, shells, self.h, self.x, n, device=_DEVICE)
        else:
            build = native_column_table if _NATIVE else column_rows
            self.up, self.down = build(atm, shells, self.h, self.x, n)

    def lookup(self, h, mu):
        """Columns [n, 6] and whether the ray escapes (mu >= horizon cosine)."""
        h = np.clip(np.asarray(h, float), 0, self.top)
        mu = np.asarray(mu, float)
        r = R + h
        mg = -np.sqrt(np.maximum(0, 1 - (R / np.maximum(r, R)) ** 2))
        escape = mu >= mg
        x_up = np.sqrt(np.clip((mu - mg) / (1 - mg), 0, 1))
        x_dn = np.sqrt(np.clip((mg - mu) / (1 + mg), 0, 1))
        i = np.clip(np.searchsorted(self.h, h, side='right') - 1, 0, len(self.h) - 2)
        a = (h - self.h[i]) / (self.h[i + 1] - self.h[i])
        out = np.empty((len(h), 6))
        for sel, x, tab in ((escape, x_up, self.up), (~escape, x_dn, self.down)):
            f = x[sel] * (len(self.x) - 1)
            j = np.clip(f.astype(int), 0, len(self.x) - 2)
            bb = (f - j)[:, None]
            aa = a[sel][:, None]
            ii = i[sel]
            out[sel] = ((1 - aa) * (1 - bb) * tab[ii, j] + aa * (1 - bb) * tab[ii + 1, j] + (1 - aa) * bb * tab[ii, j + 1]
                        + aa * bb * tab[ii + 1, j + 1])
        return out, escape


# ------------------------------------------------------------------------------------------------ state
def _shells(top):
    return (10.0, 25.0, 40.0) + ((80.0,) if top > 80.0 else ())


def _ring_heights(top):
    return (0.0, 1.2, 8.0, 25.0, 40.0) + ((80.0, top) if top > 80.0 else (top,))


def _ray_block(p, d, chi_grid, top, table, with_ground_columns):
    """The segments and ray-end quantities of a block of rays by libsosb's sosb_ray_segments (host threads)."""
    from . import _abi, build

    lib = _abi.library(build.build())
    shells = np.ascontiguousarray(_shells(top), np.float64)
    p = np.ascontiguousarray(p, np.float64)
    d = np.ascontiguousarray(d, np.float64)
    chi = np.ascontiguousarray(chi_grid, np.float64)
    n, ncut = len(d), 5 + 2 * len(shells)
    edges = np.empty((n, ncut))
    valid = np.empty((n, ncut - 1), np.uint8)
    lower = np.empty((n, ncut - 1), np.uint8)
    end_j = np.empty(n, np.int32)
    end_f = np.empty(n)
    end_col = np.zeros((n, 5), np.float32)
    end_st = np.zeros(n, np.float32)
    hits = np.empty(n, np.uint8)
    grid = None
    if with_ground_columns:
        keep = [np.ascontiguousarray(table.h, np.float64), np.ascontiguousarray(table.up, np.float64),
                np.ascontiguousarray(table.down, np.float64)]
        grid = _abi.ColumnGrid(n_h=len(table.h), n_x=len(table.x), top=table.top, h=_abi.ptr(keep[0], _abi.P_f64),
                               up=_abi.ptr(keep[1], _abi.P_f64), down=_abi.ptr(keep[2], _abi.P_f64))
    rc = lib.sosb_ray_segments(n, _abi.ptr(p, _abi.P_f64), _abi.ptr(d, _abi.P_f64), float(top),
                               _abi.ptr(shells, _abi.P_f64), len(shells), len(chi), _abi.ptr(chi, _abi.P_f64),
                               None if grid is None else ctypes.byref(grid), _abi.ptr(edges, _abi.P_f64),
                               _abi.ptr(valid, _abi.P_u8), _abi.ptr(lower, _abi.P_u8), _abi.ptr(end_j, _abi.P_i32),
                               _abi.ptr(end_f, _abi.P_f64), _abi.ptr(end_col, _abi.P_f32), _abi.ptr(end_st, _abi.P_f32),
                               _abi.ptr(hits, _abi.P_u8), 0)
    if rc:
        raise RuntimeError(f'E_SEGMENTS: sosb_ray_segments returned {rc}')
    v = valid.astype(bool)
    return dict(seg_off=np.r_[0, np.cumsum(v.sum(1))].astype(np.int64), seg_a=edges[:, :-1][v], seg_b=edges[:, 1:][v],
                seg_lower=lower[v], end_j=end_j, end_f=end_f, end_col=end_col, end_st=end_st, hits=hits)


def ray_block_device(p, d, chi_grid, top, table, with_ground_columns, device='cuda:0'):
    """_ray_block with the segments built on the GPU (sosb_ray_segments_device); the results come back as the same
    host arrays."""
    import torch

    from . import _abi, build

    lib = _abi.library(build.build())
    dev = torch.device(device)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a, np.float64), device=dev)  # noqa: E731
    shells = t(_shells(top))
    pd, dd, chi = t(p), t(d), t(chi_grid)
    n, ncut = len(d), 5 + 2 * len(_shells(top))
    edges = torch.empty((n, ncut), dtype=torch.float64, device=dev)
    valid = torch.empty((n, ncut - 1), dtype=torch.uint8, device=dev)
    lower = torch.empty((n, ncut - 1), dtype=torch.uint8, device=dev)
    end_j = torch.empty(n, dtype=torch.int32, device=dev)
    end_f = torch.empty(n, dtype=torch.float64, device=dev)
    end_col = torch.zeros((n, 5), dtype=torch.float32, device=dev)
    end_st = torch.zeros(n, dtype=torch.float32, device=dev)
    hits = torch.empty(n, dtype=torch.uint8, device=dev)
    grid, keep = None, None
    if with_ground_columns:
        keep = [t(table.h), t(table.up), t(table.down)]
        grid = _abi.ColumnGrid(n_h=len(table.h), n_x=len(table.x), top=table.top,
                               h=ctypes.cast(keep[0].data_ptr(), _abi.P_f64),
                               up=ctypes.cast(keep[1].data_ptr(), _abi.P_f64),
                               down=ctypes.cast(keep[2].data_ptr(), _abi.P_f64))
    vp = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    rc = lib.sosb_ray_segments_device(n, vp(pd), vp(dd), float(top), vp(shells), len(shells), len(chi), vp(chi),
                                      None if grid is None else ctypes.byref(grid), vp(edges), vp(valid), vp(lower),
                                      vp(end_j), vp(end_f), vp(end_col), vp(end_st), vp(hits), stream)
    if rc:
        raise RuntimeError(f'E_SEGMENTS: sosb_ray_segments_device returned {rc}')
    v = valid.cpu().numpy().astype(bool)
    e = edges.cpu().numpy()
    return dict(seg_off=np.r_[0, np.cumsum(v.sum(1))].astype(np.int64), seg_a=e[:, :-1][v], seg_b=e[:, 1:][v],
                seg_lower=lower.cpu().numpy()[v], end_j=end_j.cpu().numpy(), end_f=end_f.cpu().numpy(),
                end_col=end_col.cpu().numpy(), end_st=end_st.cpu().numpy(), hits=hits.cpu().numpy())


def ray_block_numpy(p, d, chi_grid, top, table, with_ground_columns):
    """The NumPy restatement of _ray_block (ray_edges, compact_segments and the end quantities), the reference the
    native sosb_ray_segments is checked against."""
    shells = _shells(top)
    edges, ground = ray_edges(p, d, top, shells)
    seg_off, seg_a, seg_b, seg_lower = compact_segments(p, d, edges)
    end = edges[:, -1]
    qe = p + end[:, None] * d
    re = np.linalg.norm(qe, axis=-1)
    ch = np.arccos(np.clip(qe[:, 2] / re, -1, 1))
    j = np.clip(np.searchsorted(chi_grid, ch, side='right') - 1, 0, len(chi_grid) - 2)
    f = np.clip((ch - chi_grid[j]) / (chi_grid[j + 1] - chi_grid[j]), 0, 1)
    hits = re < R + 1e-5
    end_col = np.zeros((len(d), 5), np.float32)
    end_st = np.zeros(len(d), np.float32)
    if with_ground_columns and hits.any():
        r0 = np.linalg.norm(p[hits], axis=-1)
        mu = np.sum(p[hits] * d[hits], -1) / r0
        cols, _ = table.lookup(r0 - R, mu)
        end_col[hits] = cols[:, :5]
        end_st[hits] = cols[:, 5]
    return dict(seg_off=seg_off, seg_a=seg_a, seg_b=seg_b, seg_lower=seg_lower, end_j=j.astype(np.int32), end_f=f,
                end_col=end_col, end_st=end_st, hits=hits.astype(np.uint8))


def build_bundle(points, dirs_local, weights, chi_grid, top, table, atm, with_ground_columns=True, block=1 << 20):
    """points: (p, up, ex) per cell; dirs_local, weights: that cell's incoming directions in its local frame and
    their solid-angle weights. Rays are processed in blocks of about `block` to bound host memory."""
    cell_off = [0]
    P, T, D, DL, WT = [], [], [], [], []
    for (p, up, ex), loc, w in zip(points, dirs_local, weights):
        ey = np.cross(up, ex)
        d = loc[:, 0, None] * ex + loc[:, 1, None] * ey + loc[:, 2, None] * up
        B = target_basis(p)
        P.append(p)
        T.append(B)
        D.append(d)
        DL.append(d @ B)
        WT.append(w)
        cell_off.append(cell_off[-1] + len(d))
    cell_off = np.asarray(cell_off, np.int64)
    d = np.concatenate(D)
    P = np.asarray(P)
    ray_cell = np.repeat(np.arange(len(P)), np.diff(cell_off))
    parts = []
    for r0 in range(0, len(d), block):
        r1 = min(r0 + block, len(d))
        if _DEVICE is not None and _NATIVE:
            parts.append(ray_block_device(P[ray_cell[r0:r1]], d[r0:r1], chi_grid, top, table, with_ground_columns,
                                          _DEVICE))
        else:
            block_fn = _ray_block if _NATIVE else ray_block_numpy
            parts.append(block_fn(P[ray_cell[r0:r1]], d[r0:r1], chi_grid, top, table, with_ground_columns))
    seg_off = [np.zeros(1, np.int64)]
    base = 0
    for part in parts:
        seg_off.append(part['seg_off'][1:] + base)
        base += int(part['seg_off'][-1])
    out = dict(cell_off=cell_off, p=P, target=np.asarray(T), d=d, dloc=np.concatenate(DL), weight=np.concatenate(WT),
               seg_off=np.concatenate(seg_off))
    for k in ('seg_a', 'seg_b', 'seg_lower', 'end_j', 'end_f', 'end_col', 'end_st', 'hits'):
        out[k] = np.concatenate([part[k] for part in parts])
    return out


class Family:
    """Everything of a state that depends only on the grid and the profile shapes: the column tables, the cell and
    observer ray bundles, and the ground-illumination rays of every cell. States of one family differ only in the
    amounts (aerosol optical depth, single-scattering albedo, asymmetry, ozone column, albedo, stratospheric optical
    depth), so `state()` costs a fraction of a second."""

    def __init__(self, h, chi_deg, L, nmu, nphi, path_n, shape, query_n=24, sun_scale=2, tolerance=1e-3, max_eval=64,
                 name='synthetic', ground_nmu=3, ground_nphi=32, monitor_elevations=MONITOR_ELEVATIONS, cells=None,
                 table=None):
        self.h = np.asarray(h, float)
        self.chi = np.deg2rad(np.asarray(chi_deg, float))
        self.top = float(self.h[-1])
        if abs(self.top - shape.top) > 1e-9:
            raise ValueError('E_SYNTH: grid top and atmosphere top differ')
        self.L, self.path_n, self.query_n, self.name = L, path_n, query_n, name
        self.tolerance, self.max_eval = tolerance, max_eval
        self.shape = shape
        self.monitor_elevations = tuple(float(e) for e in monitor_elevations)
        shells = _shells(self.top)
        # the solar column table depends only on the profile shapes and the top: `table` reuses one built before
        self.table = table if table is not None else ColumnTable(shape, shells, scale=sun_scale)
        # the cells whose bundles are built (all by default; a subset for a timing sample), in cell order
        ncell = len(self.h) * len(self.chi)
        self.cell_ids = np.arange(ncell) if cells is None else np.unique(np.asarray(cells, int))
        points, dirs, weights = [], [], []
        specs = [(R + self.h[c // len(self.chi)], self.chi[c % len(self.chi)], nmu, nphi, _ring_heights(self.top), True)
                 for c in self.cell_ids]
        for sp, (loc, w) in zip(specs, quadratures(specs)):
            points.append(frame(sp[0], sp[1]))
            dirs.append(loc)
            weights.append(w)
        self.cells = build_bundle(points, dirs, weights, self.chi, self.top, self.table, shape)
        u4, w4 = np.polynomial.legendre.leggauss(4)
        self.box_ww = (w4[:, None] * w4[None, :] / 4).ravel()
        qpts, qdirs, qw = [], [], []
        for hs in self.monitor_elevations:
            el = np.array([e + de for e, z in DIRS for de in u4 for dz in u4])
            az = np.array([z + dz for e, z in DIRS for de in u4 for dz in u4])
            e, zz = np.deg2rad(el), np.deg2rad(az)
            loc = np.column_stack([np.cos(e) * np.cos(zz), np.cos(e) * np.sin(zz), np.sin(e)])
            qpts.append(frame(R + OBSERVER_KM, np.deg2rad(90 - hs)))
            qdirs.append(loc)
            qw.append(np.ones(len(loc)))
        self.query = build_bundle(qpts, qdirs, qw, self.chi, self.top, self.table, shape, with_ground_columns=False)
        self._ground_rays(ground_nmu, ground_nphi)

    def view_bundle(self, hs, el, az):
        """Rays of a radiance table (outputs/radiance_table.py:43-60 over solve/engine_core.py:208-226): for every
        solar elevation hs[j] the observer at OBSERVER_KM under solar zenith 90 - hs[j] (one bundle cell), looking
        along the (el, az) grid in meshgrid 'ij' order (elevation rows, azimuth columns), unit weights."""
        ee, aa = np.meshgrid(np.asarray(el, float), np.asarray(az, float), indexing='ij')
        e, z = np.deg2rad(ee.ravel()), np.deg2rad(aa.ravel())
        loc = np.column_stack([np.cos(e) * np.cos(z), np.cos(e) * np.sin(z), np.sin(e)])
        pts = [frame(R + OBSERVER_KM, np.deg2rad(90 - float(h))) for h in hs]
        return build_bundle(pts, [loc] * len(pts), [np.ones(len(loc))] * len(pts), self.chi, self.top, self.table,
                            self.shape, with_ground_columns=False)

    def _ground_rays(self, nmu, nphi):
        """Per cell: the directions of a ring quadrature without shadow rings, their weights, and for the downward
        ones the columns to the ground and from the ground point to the sun (solve/engine_core.py:103-147)."""
        table, h, chi = self.table, self.h, self.chi
        loc_all, w_all, col_all, sun_all, cos_all, ok_all, counts = [], [], [], [], [], [], []
        quads = quadratures([(R + h[cell // len(chi)], chi[cell % len(chi)], nmu, nphi, (), False)
                             for cell in self.cell_ids])
        for q_index, cell in enumerate(self.cell_ids):
            ih, ic = divmod(int(cell), len(chi))
            r = R + h[ih]
            loc, w = quads[q_index]
            p, up, ex = frame(r, chi[ic])
            ey = np.cross(up, ex)
            d = loc[:, 0, None] * ex + loc[:, 1, None] * ey + loc[:, 2, None] * up
            col, escape = table.lookup(np.full(len(d), h[ih]), loc[:, 2])
            b = d @ p
            disc = b * b - r * r + R * R
            t = -b - np.sqrt(np.maximum(disc, 0))
            q = p + t[:, None] * d
            cos_sun = q[:, 2] / np.linalg.norm(q, axis=-1)
            sun, lit = table.lookup(np.zeros(len(d)), cos_sun)
            loc_all.append(loc)
            w_all.append(w)
            col_all.append(col)
            sun_all.append(sun)
            cos_all.append(cos_sun)
            ok_all.append(lit & ~escape)
            counts.append(len(w))
        self.g_loc = np.concatenate(loc_all)
        self.g_w = np.concatenate(w_all)
        self.g_cols = np.concatenate(col_all) + np.concatenate(sun_all)
        self.g_cos = np.maximum(0, np.concatenate(cos_all))
        self.g_ok = np.concatenate(ok_all)
        self.g_cell = np.repeat(self.cell_ids, counts)
        lo = self.g_loc
        self.g_factor = np.stack([(1 - lo[:, 0] ** 2) / 2, (1 - lo[:, 1] ** 2) / 2, (1 - lo[:, 2] ** 2) / 2,
                                  -lo[:, 0] * lo[:, 2] / 2], -1)

    def ground_rays(self):
        """The ground-illumination rays of every cell for sosb_set_ground_rays: cell, local direction, weight, the
        six slant columns to the ground and on to the sun, the clipped solar cosine at the ground point and whether
        that point is lit (the geometry `ground` combines with a state's optics)."""
        return dict(cell=self.g_cell.astype(np.int32), loc=self.g_loc, weight=self.g_w, cols=self.g_cols,
                    cos_sun=self.g_cos, ok=self.g_ok.astype(np.uint8))

    def ground(self, atm, ext):
        """gm [ns, 4, W], goff, gdir, gval of one atmosphere (vectorised over all ground rays)."""
        od = self.g_cols[:, :5] @ ext
        if atm.strato:
            od += self.g_cols[:, 5, None] * atm.strato_ext[None, :]
        value = (atm.albedo / math.pi * self.g_cos[:, None] * np.exp(-od) * self.g_ok[:, None] * self.g_w[:, None])
        ns = len(self.h) * len(self.chi)
        gm = np.zeros((ns, 4, atm.W))
        for k in range(4):
            for w in range(atm.W):
                gm[:, k, w] = np.bincount(self.g_cell, weights=self.g_factor[:, k] * value[:, w], minlength=ns)
        gm *= (2 * (3 / (16 * math.pi)) * ext[0])[None, None, :]
        take = np.any(value > 0, axis=1)
        goff = np.r_[0, np.cumsum(np.bincount(self.g_cell[take], minlength=ns))].astype(np.int64)
        return (gm.astype(np.float32), goff, self.g_loc[take].astype(np.float32), value[take].astype(np.float32))

    def state(self, atm, seed=0, ground=True):
        """Packed-state arrays of atmosphere `atm` (same profile shapes as the family's). ground=False leaves the
        ground arrays empty for a handle that prepares them on the device (Kernel.prepare_ground)."""
        h, chi, L, W = self.h, self.chi, self.L, atm.W
        K = (L + 1) * (L + 2) // 2
        ext = atm.ext()
        if ground:
            gm, goff, gdir, gval = self.ground(atm, ext)
        else:
            ns = len(h) * len(chi)
            gm, goff = np.zeros((ns, 4, W), np.float32), np.zeros(ns + 1, np.int64)
            gdir, gval = np.zeros((0, 3), np.float32), np.zeros((0, W), np.float32)
        u, wu = gauss01(self.path_n)
        uq, wuq = gauss01(self.query_n)
        step = 0.5
        zt = np.arange(int(round(self.top / step)) + 1) * step
        prof = atm.profiles(zt)
        density_table = np.column_stack([prof[:, 0], prof[:, 2], prof[:, 3]]).astype(np.float32)
        levels = np.array([l for l in range(L + 1) for m in range(l + 1)])
        meta = dict(
            name=self.name, L=L, K=K, W=W, nq=self.path_n, nq_query=self.query_n, nh=len(h), nc=len(chi),
            ns=len(h) * len(chi), source_size=10 + K * (2 if atm.strato else 1), strato=atm.strato, g=atm.g,
            mix=(1 - 0.03) / (1 + 0.015), height=atm.H, albedo=atm.albedo, top_km=self.top, profile_step_km=step,
            density_mask=2, air_surface=1.0, tolerance=self.tolerance, max_eval=self.max_eval,
            monitors=len(self.monitor_elevations), n_dirs=len(DIRS), box_points=16, wavelengths_nm=atm.wl.tolist(),
            seed=seed, C=3 / (16 * math.pi), rays=int(len(self.cells['d'])), segments=int(len(self.cells['seg_a'])),
            query_rays=int(len(self.query['d'])),
            amounts=dict(aod=atm.aod, ssa=atm.ssa, g=atm.g, ozone_du=atm.ozone_du, albedo=atm.albedo,
                         strato_tau=atm.strato_tau))
        arrays = dict(
            u=u, wu=wu, uq=uq, wuq=wuq, h=h.astype(np.float32), chi=chi.astype(np.float32),
            hr=np.exp(-h / 8.0).astype(np.float32), ha=np.exp(-h / atm.H).astype(np.float32),
            ext=ext.astype(np.float32), asca=(ext[1] * atm.ssa).astype(np.float32),
            sun_h=self.table.h.astype(np.float32), sun_col=np.ascontiguousarray(self.table.up[:, :, :5], np.float32),
            gm=gm, goff=goff, gdir=gdir, gval=gval, density_table=density_table,
            rf=((levels[:6] == 0) + 0.1 * (levels[:6] == 2)).astype(np.float32),
            af=(atm.g ** levels).astype(np.float32), ext0=ext[0].astype(np.float32),
            solar=atm.solar.astype(np.float64), box_ww=self.box_ww)
        if atm.strato:
            lm = np.arange(33)
            chi_l = ((2 * lm + 1) * atm.strato_g ** lm)[:, None] * np.ones((1, W))
            cell_edges = np.r_[h[0], (h[:-1] + h[1:]) / 2, h[-1]]
            cdf = np.array([math.erf((z - atm.strato_center) / (math.sqrt(2) * atm.strato_sigma)) for z in cell_edges])
            avg = np.diff(cdf) * atm.strato_sigma * math.sqrt(math.pi / 2) / atm.strato_norm / np.diff(cell_edges)
            arrays.update(
                strato_ext=atm.strato_ext.astype(np.float32), strato_sca=atm.strato_ext.astype(np.float32),
                strato_chi=chi_l.astype(np.float32), strato_density=avg.astype(np.float32),
                strato_sun_col=np.ascontiguousarray(self.table.up[:, :, 5], np.float32),
                strato_eigen=(atm.strato_g ** levels[:, None] * np.ones((1, W))).astype(np.float32),
                strato_sca_source=atm.strato_ext.astype(np.float32))
            meta.update(strato_center=atm.strato_center, strato_sigma=atm.strato_sigma, strato_norm=atm.strato_norm)
        arrays['meta'] = json.dumps(meta)
        for k, v in self.cells.items():
            arrays['cell_' + k] = v
        for k, v in self.query.items():
            arrays['query_' + k] = v
        return arrays


def make_state(h, chi_deg, wl, L, nmu, nphi, path_n, atm, seed=0, query_n=24, sun_scale=2, tolerance=1e-3,
               max_eval=64, name='synthetic'):
    """A packed state (dict for sosfuse2_gb300.state.PackedState) of the synthetic atmosphere."""
    fam = Family(h, chi_deg, L, nmu, nphi, path_n, atm, query_n=query_n, sun_scale=sun_scale, tolerance=tolerance,
                 max_eval=max_eval, name=name)
    return fam.state(atm, seed)


# ------------------------------------------------------------------------------------------------ configurations
def config0(seed=0, **kw):
    """Plain SOS reduced grid: 550 nm, 101 heights on 0-100 km, the reduced 10-node solar-zenith grid, nmu 1, nphi 2,
    path_n 4, L=16, Chapman ozone 300 DU, tropospheric aerosol AOD 0.1 / ssa 0.95 / g 0.7 / H 1.2 km, stratospheric
    Gaussian 20 km (sigma 3 km, AOD 0.01, g 0.6), NO2/O4 off, albedo 0.3."""
    atm = Atmosphere([550.0], seed=seed, top=100.0)
    return make_state(np.arange(101.0), REDUCED_CHI_DEG, atm.wl, 16, 1, 2, 4, atm, seed=seed, name='config0', **kw)


def config0_family(**kw):
    """The state family of config 0's grid (amounts vary, profile shapes fixed)."""
    atm = Atmosphere([550.0], seed=0, top=100.0)
    return Family(np.arange(101.0), REDUCED_CHI_DEG, 16, 1, 2, 4, atm, name='config0-family', **kw)


def random_amounts(seed):
    """Amounts drawn from the batched configuration's ranges: AOD U(0.02, 0.5), g U(0.5, 0.8), ozone U(250, 400) DU,
    albedo U(0.05, 0.8)."""
    rng = np.random.default_rng(seed)
    return dict(aod=float(rng.uniform(0.02, 0.5)), g=float(rng.uniform(0.5, 0.8)),
                ozone_du=float(rng.uniform(250, 400)), albedo=float(rng.uniform(0.05, 0.8)))


def family_atmosphere(family, seed):
    """The atmosphere of `family` with amounts random_amounts(seed)."""
    a = random_amounts(seed)
    return Atmosphere(family.shape.wl, seed=seed, top=family.top, scale_height=family.shape.H,
                      no2_column=family.shape.no2_column, o4=family.shape.o4, **a)


def family_state(family, seed, ground=True):
    """A state of `family` with amounts random_amounts(seed) (ground=False: see Family.state)."""
    return family.state(family_atmosphere(family, seed), seed, ground=ground)


def config1(seed=0, nh=241, W=30, nmu=12, nphi=16, path_n=12, L=32, chi_deg=None, **kw):
    """Plain SOS full table: 30 wavelengths 400-700 nm, 241 heights on 0-120 km, the 75 production solar-zenith
    nodes, nmu 12, nphi 16, path_n 12, L=32; config-0 atmosphere plus an NO2 Gaussian layer at 25 km (5e15 cm^-2)
    and O4. Smaller grids of the same construction are available through the keyword arguments."""
    wl = np.linspace(400.0, 700.0, W)
    atm = Atmosphere(wl, seed=seed, top=120.0, no2_column=5e15, o4=True)
    chi = production_chi_deg() if chi_deg is None else np.asarray(chi_deg, float)
    return make_state(np.linspace(0.0, 120.0, nh), chi, wl, L, nmu, nphi, path_n, atm, seed=seed, name='config1',
                      **kw)


# the batched configuration: 64 seeded states (seeds 1000 + i) of uneven sizes
CONFIG3_STATES = 64
CONFIG3_TOP = 120.0


def config3_spec(i):
    """Sizes and amounts of batched state i (seed 1000 + i): height levels U{121..481} on 0-120 km, wavelengths
    U{8..64} linear on 400-700 nm, L in {16, 24, 32, 48}, observer solar elevations +6 to -18 deg in 1 or 2 deg steps
    (the stop rows), and the amounts of random_amounts (AOD U(0.02, 0.5), g U(0.5, 0.8), ozone U(250, 400) DU, albedo
    U(0.05, 0.8)). The rest follows the reduced configuration (10-node solar-zenith grid, nmu 1, nphi 2, path_n 4)
    and the full-table atmosphere (NO2 layer at 25 km, O4)."""
    seed = 1000 + int(i)
    rng = np.random.default_rng(seed)
    amounts = dict(aod=float(rng.uniform(0.02, 0.5)), g=float(rng.uniform(0.5, 0.8)),
                   ozone_du=float(rng.uniform(250, 400)), albedo=float(rng.uniform(0.05, 0.8)))  # random_amounts(seed)
    nh = int(rng.integers(121, 482))
    W = int(rng.integers(8, 65))
    L = int(rng.choice([16, 24, 32, 48]))
    step = int(rng.choice([1, 2]))
    return dict(index=int(i), seed=seed, nh=nh, W=W, L=L, solar_step=step, **amounts)


def config3_family(i, cells=None, table=None):
    """The geometry of batched state i (its grid, bundles, observer rows and ground rays); `cells`: only those
    cells' bundles and ground rays (a timing sample); `table`: a column table of config3_table() to reuse."""
    sp = config3_spec(i)
    wl = np.linspace(400.0, 700.0, sp['W'])
    shape = Atmosphere(wl, seed=sp['seed'], top=CONFIG3_TOP, no2_column=5e15, o4=True)
    elevations = np.arange(6.0, -18.0 - 1e-9, -float(sp['solar_step']))
    return Family(np.linspace(0.0, CONFIG3_TOP, sp['nh']), REDUCED_CHI_DEG, sp['L'], 1, 2, 4, shape,
                  name=f'config3-{i}', monitor_elevations=elevations, cells=cells, table=table)


def config3_table():
    """The solar column table shared by every batched state (same profile shapes and top)."""
    shape = Atmosphere([550.0], seed=1000, top=CONFIG3_TOP, no2_column=5e15, o4=True)
    return ColumnTable(shape, _shells(CONFIG3_TOP))


def config3(i, family=None, ground=True):
    """Packed-state arrays of batched state i (seed 1000 + i; see config3_spec)."""
    sp = config3_spec(i)
    fam = family or config3_family(i)
    a = {k: sp[k] for k in ('aod', 'g', 'ozone_du', 'albedo')}
    atm = Atmosphere(fam.shape.wl, seed=sp['seed'], top=CONFIG3_TOP, no2_column=5e15, o4=True, **a)
    arrays = fam.state(atm, sp['seed'], ground=ground)
    meta = json.loads(arrays['meta'])
    meta.update(config3=sp)
    arrays['meta'] = json.dumps(meta)
    return arrays


def config3_training_family(L, table=None):
    """The geometry the learned start of the batched configuration trains on for SH order L: the smallest grid of
    the batched ranges (121 heights on 0-120 km, 8 wavelengths 400-700 nm, observer rows every 2 deg), the batched
    states' atmosphere shapes; its states draw their amounts like the batched states (family_state, seeds 10000+)."""
    shape = Atmosphere(np.linspace(400.0, 700.0, 8), seed=10000, top=CONFIG3_TOP, no2_column=5e15, o4=True)
    return Family(np.linspace(0.0, CONFIG3_TOP, 121), REDUCED_CHI_DEG, int(L), 1, 2, 4, shape,
                  name=f'config3-train-L{L}', monitor_elevations=np.arange(6.0, -18.0 - 1e-9, -2.0), table=table)
