"""CPU oracle of the successive-orders-of-scattering source iteration (TEST INFRASTRUCTURE ONLY).

Only the tests, `__graft_entry__.smoke()` and the `cpu_baseline` / `--impl reference` legs of `bench.py` may import
this module, and only as the checker or the timed CPU baseline. The product path never calls it.

It restates, in NumPy FP32 with flush-to-zero, the reference's NumPy mirror of its CUDA transport:

* double-single (two-float) coordinates, src/sosfuse2/backends/arithmetic.py:15-66;
* SH basis recurrence and cos(m phi) table, arithmetic.py:69-119; the 32-lane shuffle-tree sum, arithmetic.py:122-130;
* per-sample geometry, numpy_reference.py:294-387; Simpson optical-depth prefix, numpy_reference.py:236-291;
* the transport of one evaluation (first light, warm, ground boundary), numpy_reference.py:467-643;
* the FP64-sum projection, numpy_reference.py:689-711;
* `Solver.apply` composition, src/sosfuse2/solve/source_iteration.py:161-216;
* the observer boxes, src/sosfuse2/solve/engine_core.py:208-238 and source_iteration.py:218-222;
* `Solver.solve` with per-wavelength Anderson depth 4, source_iteration.py:25-33,309-663 (the default
  device-history path that keeps the rings as lists, source_iteration.py:618-635).

Inputs are the packed states written by tests/golden/make_fixtures.py (or by sosfuse2_gb300.synth): every ray of
every cell in one CSR bundle, segments compacted to the valid ones (b - a > 1e-8, the only ones the reference's
transport integrates). Rays are processed all at once, vectorised over rays, one segment slot at a time; the per-ray
arithmetic is the reference's, operation for operation, so the oracle agrees with the reference to FP32 rounding of
the transcendental functions.

Pins: tests/test_oracle_golden.py against the reference's outputs of tests/golden/{walk1,strato1,strato15}.npz
(per-ray radiance, moments, apply, boxes, the converged field) and tests/test_table_golden.py against the reference's
radiance table of the walkthrough state (tests/golden/table_walk1.npz). oracle/fp64.py evaluates the same operations
in float64 for the per-pixel error report.

Optional state features follow the reference where a golden state carries them: the two-layer tropospheric aerosol
profile (tests/golden/aer2.npz) and the tabulated tropospheric Mie phase with its per-wavelength eigenvalues
(tests/golden/mie1.npz, mie15.npz); the component support of an extended top above 80 km (meta 'support': the ends
of the lower components and of the air, numpy_reference.py:158-183,221-222,254-256,606-609), restated from the
reference's code, which builds such a top only on its full grid, so no golden state pins it.
"""

import json
import math

import numpy as np

from .ftz import flush_to_zero

F = np.float32
EARTH_R = F(6371)
TRACE_MIN = F(np.finfo(np.float32).tiny)
PAIRS = ((0, 0), (1, 1), (2, 2), (0, 2))


# ---------------------------------------------------------------- double-single arithmetic (arithmetic.py:15-66)

def ds(x):
    """Split an FP64 value into (hi, lo) FP32 words."""
    x = np.asarray(x, np.float64)
    hi = x.astype(F)
    return hi, (x - hi.astype(np.float64)).astype(F)


def ds_add(a, b):
    s = a[0] + b[0]
    v = s - a[0]
    e = ((a[0] - (s - v)) + (b[0] - v)) + (a[1] + b[1])
    h = s + e
    return h, e - (h - s)


def ds_neg(a):
    return -a[0], -a[1]


def ds_sub(a, b):
    return ds_add(a, ds_neg(b))


def ds_mul(a, b):
    p = a[0] * b[0]
    # fmaf(a.hi, b.hi, -p) with its single rounding, through an exact FP64 product
    e = (a[0].astype(np.float64) * b[0].astype(np.float64) - p.astype(np.float64)).astype(F)
    e = (e + a[0] * b[1]) + a[1] * b[0]
    h = p + e
    return h, e - (h - p)


def _hi(x):
    return x, np.zeros_like(x)


def ds_sqrt(a):
    h = np.sqrt(np.maximum(a[0], F(0)))
    e = ds_sub(a, ds_mul(_hi(h), _hi(h)))
    lo = (e[0] + e[1]) / np.maximum(F(2) * h, F(1e-30))
    return ds_add(_hi(h), _hi(lo))


def ds_div(a, b):
    h = a[0] / b[0]
    e = ds_sub(a, ds_mul(_hi(h), b))
    lo = (e[0] + e[1]) / b[0]
    return ds_add(_hi(h), _hi(lo))


def ds_value(a):
    return a[0] + a[1]


# ---------------------------------------------------------------- SH basis and azimuth table (arithmetic.py:69-130)

def sh_count(L):
    return (L + 1) * (L + 2) // 2


def sh_constants(L):
    K = sh_count(L)
    a = np.zeros(K)
    b = np.zeros(K)
    diag = np.zeros(L + 1)
    for m in range(1, L + 1):
        diag[m] = -math.sqrt((2.0 * m + 1) / (2 * m))
    for l in range(1, L + 1):
        for m in range(l):
            k = l * (l + 1) // 2 + m
            a[k] = math.sqrt((4.0 * l * l - 1) / (l * l - m * m))
            if l > m + 1:
                b[k] = math.sqrt((2.0 * l + 1) * ((l - 1.0) ** 2 - m * m) / ((2.0 * l - 3) * (l * l - m * m)))
    return a, b, diag


def sh_basis(mu, L):
    """Orthonormal real SH at azimuth 0 for k = l(l+1)/2 + m: FP64 recurrence, rounded to FP32."""
    mu = np.clip(np.asarray(mu, np.float64), -1, 1)
    sin_t = np.sqrt(np.maximum(0.0, 1 - mu * mu))
    a, b, dg = sh_constants(L)
    out = np.empty((len(mu), sh_count(L)), F)
    pmm = np.full_like(mu, 1 / math.sqrt(4 * math.pi))
    for m in range(L + 1):
        if m:
            pmm = (pmm * dg[m]) * sin_t
        scale = math.sqrt(2.0) if m else 1.0
        p0 = pmm
        out[:, m * (m + 1) // 2 + m] = scale * p0
        if m < L:
            p1 = (math.sqrt(2.0 * m + 3) * mu) * p0
            out[:, (m + 1) * (m + 2) // 2 + m] = scale * p1
            for l in range(m + 2, L + 1):
                k = l * (l + 1) // 2 + m
                p2 = (a[k] * mu) * p1 - b[k] * p0
                out[:, k] = scale * p2
                p0, p1 = p1, p2
    return out


def cos_multiples(cp, n=33):
    """cos(m phi), m = 0..n-1 (the reference's table has n = 33, L <= 32), by the Chebyshev recurrence in FP32."""
    cp = np.clip(cp, F(-1), F(1)).astype(F)
    out = np.empty((len(cp), n), F)
    out[:, 0] = F(1)
    out[:, 1] = cp
    for m in range(2, n):
        out[:, m] = (F(2) * cp) * out[:, m - 1] - out[:, m - 2]
    return out


def lane_tree_sum(x):
    """Sum over m = 0..32 as a 32-lane shuffle-down tree with m = 32 folded into lane 0 first (orders above 32, which
    the reference does not take, are folded into lanes m - 32 the same way)."""
    x = x.copy()
    x[:, : x.shape[1] - 32] = x[:, : x.shape[1] - 32] + x[:, 32:]
    x = x[:, :32]
    for stride in (16, 8, 4, 2, 1):
        old = x.copy()
        x[:, : 32 - stride] = old[:, : 32 - stride] + old[:, stride:]
    return x[:, 0]


def kahan_add(total, comp, value):
    y = value - comp
    t = total + y
    return t, (t - total) - y


def sh_levels(L):
    return np.array([l for l in range(L + 1) for m in range(l + 1)])


# ---------------------------------------------------------------- packed state

class StatePack:
    """A packed state: meta, transport constants, the cell bundle and the observer (query) bundle."""

    def __init__(self, source):
        z = np.load(source) if not isinstance(source, dict) else source
        self.arrays = {k: z[k] for k in z.keys()} if not isinstance(source, dict) else dict(source)
        meta = self.arrays['meta']
        self.meta = json.loads(str(meta)) if not isinstance(meta, dict) else meta
        for k in ('L', 'K', 'W', 'nq', 'nq_query', 'nh', 'nc', 'ns', 'source_size'):
            setattr(self, k, int(self.meta[k]))
        self.strato = bool(self.meta['strato'])
        self.shape = (self.ns, self.source_size, self.W)
        if 'gd' not in self.arrays:
            # ground directions given as CSR (goff, gdir, gval): pad per cell; zero values add nothing
            goff = self.arrays['goff']
            ng = int(np.diff(goff).max(initial=0))
            gd = np.zeros((self.ns, max(ng, 1), 3), F)
            gv = np.zeros((self.ns, max(ng, 1), self.W), F)
            for c in range(self.ns):
                a, b = goff[c], goff[c + 1]
                gd[c, : b - a] = self.arrays['gdir'][a:b]
                gv[c, : b - a] = self.arrays['gval'][a:b]
            self.arrays['gd'], self.arrays['gv'] = gd, gv

    def __getitem__(self, key):
        return self.arrays[key]

    def __contains__(self, key):
        return key in self.arrays

    def subset(self, cells):
        """Cell bundle restricted to the listed cells (rays and segments of those cells, in order)."""
        b = self.bundle('cell')
        off = b['cell_off']
        rays = np.concatenate([np.arange(off[i], off[i + 1]) for i in cells])
        segs = [np.arange(b['seg_off'][r], b['seg_off'][r + 1]) for r in rays]
        seg_idx = np.concatenate(segs) if segs else np.zeros(0, int)
        out = dict(cell_off=np.r_[0, np.cumsum([off[i + 1] - off[i] for i in cells])], p=b['p'][cells],
                   target=b['target'][cells], seg_off=np.r_[0, np.cumsum([len(x) for x in segs])],
                   seg_a=b['seg_a'][seg_idx], seg_b=b['seg_b'][seg_idx], seg_lower=b['seg_lower'][seg_idx])
        for k in ('d', 'dloc', 'weight', 'end_j', 'end_f', 'end_col', 'end_st', 'hits'):
            out[k] = b[k][rays]
        return out

    def bundle(self, prefix, cells=None):
        """Bundle dict ('cell' or 'query'); `cells` selects the first n cells (the ground pass uses nc)."""
        b = {k[len(prefix) + 1:]: v for k, v in self.arrays.items() if k.startswith(prefix + '_')}
        if cells is not None and cells < len(b['cell_off']) - 1:
            nr = int(b['cell_off'][cells])
            ne = int(b['seg_off'][nr])
            b = dict(b, cell_off=b['cell_off'][: cells + 1], p=b['p'][:cells], target=b['target'][:cells],
                     seg_off=b['seg_off'][: nr + 1], seg_a=b['seg_a'][:ne], seg_b=b['seg_b'][:ne],
                     seg_lower=b['seg_lower'][:ne],
                     **{k: b[k][:nr] for k in ('d', 'dloc', 'weight', 'end_j', 'end_f', 'end_col', 'end_st', 'hits')})
        return b


# ---------------------------------------------------------------- optics primitives (numpy_reference.py:187-458)

def profile_at(h, pk):
    """Air, tropospheric aerosol, O3, NO2, O4 number-density shapes at FP32 heights (numpy_reference.py:187-223).
    Density table columns: air, ozone, NO2 on the uniform profile grid; mask bit 0/1 selects tabulated air/ozone; a
    state with the two-layer tropospheric aerosol (array 'aer2') takes that shape for the aerosol
    (atmosphere/tropo_profile.py:295-304)."""
    h = np.asarray(h, F)
    tab = pk['density_table']
    inv = 1.0 / pk.meta['profile_step_km']
    last = len(tab) - 2
    hc = np.clip(h, F(0), F(pk.meta['top_km']))
    x = hc * F(inv)
    i = np.minimum(x.astype(np.int32), last)
    f = x - i.astype(F)
    t = tab[i] + f[:, None] * (tab[i + 1] - tab[i])
    prof = np.stack([np.exp(-h / F(8)), np.exp(-h / F(pk.meta['height'])),
                     np.maximum(F(0), F(1) - abs(h - F(25)) / F(15)), t[:, 2], np.zeros_like(h)], -1)
    mask = pk.meta['density_mask']
    if mask & 1:
        prof[:, 0] = t[:, 0]
    if mask & 2:
        prof[:, 2] = t[:, 1]
    if 'aer2' in pk:
        prof[:, 1] = aerosol_two_layer(h, pk['aer2'])
    q = prof[:, 0] / F(pk.meta['air_surface'])
    prof[:, 4] = q * q
    sup = support(pk)
    if sup is not None:  # zero strictly above each component's support end (numpy_reference.py:168-172,221-222)
        prof[:, 0] = np.where(h > sup[1], F(0), prof[:, 0])
        prof[:, 1:] = np.where(h[:, None] > sup[0], F(0), prof[:, 1:])
    return prof


def support(pk):
    """(lower end, air end) of an extended top (FP32 km), or None: the components other than air end at the lower
    end, the air at the air end (numpy_reference.py:158-166, foundation/top.py:26-32)."""
    s = pk.meta.get('support')
    return None if not s else (F(s['lower_end']), F(s['air_end']))


def support_height(h, inside_h, sup):
    """A segment end's height within one FP32 ulp of a support end moves to the side the segment lies on
    (numpy_reference.py:175-183)."""
    for edge in sup:
        above = np.nextafter(edge, F(np.inf))
        near = (h >= np.nextafter(edge, F(-np.inf))) & (h <= above)
        h = np.where(near, np.where(inside_h > edge, above, edge), h)
    return h


def aerosol_two_layer(h, k):
    """FP32 two-layer aerosol shape: smoothstep blend of the boundary-layer and free-troposphere exponentials
    (atmosphere/tropo_profile.py:295-304, kernel.cu aerosol_two_layer)."""
    h = np.asarray(h, F)
    k = np.asarray(k, F)
    x = np.clip((h - k[0]) * k[1], F(0), F(1))
    s = x * x * (F(3) - F(2) * x)
    return ((k[2] * np.exp(-h * k[3])) * (F(1) - s) + (k[4] * np.exp(-(np.maximum(h, k[0]) - k[6]) * k[5])) * s).astype(F)


def tropo_phase(u, pk):
    """Tabulated tropospheric phase per sr, linear in u on tropo_bins + 1 nodes, FP32: u[...] -> [..., W]
    (numpy_reference.py:409-420)."""
    lut = pk['tropo_lut']
    bins = len(lut) - 1
    x = (np.clip(np.asarray(u, F), F(-1), F(1)) + F(1)) * F(bins / 2)
    i = np.minimum(x.astype(np.int32), bins - 1)
    f = (x - i.astype(F))[..., None]
    a = lut[i]
    return a + f * (lut[i + 1] - a)


def strato_profile(h, pk):
    t = (h - F(pk.meta['strato_center'])) / F(pk.meta['strato_sigma'])
    out = np.exp(F(-0.5) * (t * t)) / F(pk.meta['strato_norm'])
    sup = support(pk)
    return out if sup is None else np.where(h > sup[0], F(0), out)


def extinction(prof, pk, st_prof=None):
    out = np.zeros((len(prof), pk.W), F)
    for k in range(5):
        out += prof[:, k, None] * pk['ext'][k]
    if pk.strato:
        out += st_prof[:, None] * pk['strato_ext']
    return out


def hg_phase(u, g):
    den = np.maximum(F(1e-20), (F(1) + g * g) - (F(2) * g) * u)
    return (F(1) - g * g) / (F(4 * math.pi) * (den * np.sqrt(den)))


def legendre_phase(u, chi):
    """Scalar phase from 33 Legendre moments chi[l, w], per steradian, FP32 recurrence."""
    u = np.asarray(u, F)
    p0 = np.ones_like(u)
    p1 = u.copy()
    val = p0[..., None] * chi[0]
    val += p1[..., None] * chi[1]
    for l in range(2, 33):
        pn = ((F(2 * l - 1) * u) * p1 - F(l - 1) * p0) / F(l)
        val += pn[..., None] * chi[l]
        p0, p1 = p1, pn
    return val / F(4 * math.pi)


def ftz_value(a):
    h, l = (np.where(np.abs(x) < TRACE_MIN, F(0), x) for x in a)
    v = h + l
    return np.where(np.abs(v) < TRACE_MIN, F(0), v)


def sun_columns(q, pk):
    """Slant columns towards the sun at the sample (numpy_reference.py:431-458): bilinear in (height, x)."""
    top = F(pk.meta['top_km'])
    hh = np.clip(q['h'], F(0), top)
    height = ds_sub(q['r'], (EARTH_R, F(0)))
    height = tuple(np.where(ftz_value(height) > F(0), x, F(0)) for x in height)
    rad = ds_add((EARTH_R, F(0)), height)
    mg = ds_neg(ds_sqrt(ds_div(ds_mul(height, ds_add((F(2) * EARTH_R, F(0)), height)), ds_mul(rad, rad))))
    delta = ds_sub(ds_div(q['qz'], q['r']), mg)
    zero = ftz_value(delta) == F(0)
    delta = tuple(np.where(zero, F(0), x) for x in delta)
    lit = ds_value(delta) >= F(0)
    delta = tuple(np.where(lit, x, F(0)) for x in delta)
    x = np.clip(ds_value(ds_sqrt(ds_div(delta, ds_sub((F(1), F(0)), mg)))), F(0), F(1))
    sun_h = pk['sun_h']
    col_t = pk['sun_col']
    i = np.clip(np.searchsorted(sun_h, hh, side='right') - 1, 0, len(sun_h) - 2)
    a = (hh - sun_h[i]) / (sun_h[i + 1] - sun_h[i])
    f = x * F(col_t.shape[1] - 1)
    j = np.clip(f.astype(np.int32), 0, col_t.shape[1] - 2)
    b = f - j.astype(F)
    col = ((F(1) - a) * (F(1) - b))[:, None] * col_t[i, j]
    col += (a * (F(1) - b))[:, None] * col_t[i + 1, j]
    col += ((F(1) - a) * b)[:, None] * col_t[i, j + 1]
    col += (a * b)[:, None] * col_t[i + 1, j + 1]
    st = np.zeros(len(col), F)
    if pk.strato:
        s = pk['strato_sun_col']
        st = ((F(1) - a) * (F(1) - b)) * s[i, j]
        st += (a * (F(1) - b)) * s[i + 1, j]
        st += ((F(1) - a) * b) * s[i, j + 1]
        st += (a * b) * s[i + 1, j + 1]
    return col, lit, st


# ---------------------------------------------------------------- per-sample geometry (numpy_reference.py:294-387)

def sample(rays, seg, u, wu, pk):
    """Quadrature node `u` of segment `seg` (dict of a, b, lower per active ray) in double-single FP32."""
    a = ds(seg['a'])
    b = ds(seg['b'])
    length = ds_sub(b, a)
    uu = ds(u)
    ww = ds(wu)
    lower = seg['lower']
    v1 = ds_sub((F(1), F(0)), uu)
    v = (np.where(lower, uu[0], v1[0]), np.where(lower, uu[1], v1[1]))
    tl = ds_add(a, ds_mul(length, ds_mul(uu, uu)))
    tr = ds_sub(b, ds_mul(length, ds_mul(v, v)))
    tt = tuple(np.where(lower, x, y) for x, y in zip(tl, tr))
    dsl = ds_value(ds_mul(ds_mul(length, v), ww)) * F(2)
    q, q2, r = path_point(rays['pp'], rays['dd'], tt)
    h = np.clip(ds_value(ds_sub(r, (EARTH_R, F(0)))), F(0), F(pk.meta['top_km']))
    xy = ds_sqrt(ds_add((q2[0][:, 0], q2[1][:, 0]), (q2[0][:, 1], q2[1][:, 1])))
    rho = ds_value(xy)
    far = rho > F(1e-12)
    den = (np.maximum(xy[0], F(1e-30)), xy[1])
    cx = np.where(far, ds_value(ds_div((q[0][:, 0], q[1][:, 0]), den)), F(1))
    sx = np.where(far, ds_value(ds_div((q[0][:, 1], q[1][:, 1]), den)), F(0))
    angle = np.arctan2(rho, ds_value((q[0][:, 2], q[1][:, 2])))
    hg_, chi = pk['h'], pk['chi']
    ir = np.clip(np.searchsorted(hg_, h, side='right') - 1, 0, len(hg_) - 2)
    j = np.clip(np.searchsorted(chi, angle, side='right') - 1, 0, len(chi) - 2)
    ah = np.clip((h - hg_[ir]) / (hg_[ir + 1] - hg_[ir]), F(0), F(1))
    ac = np.clip((angle - chi[j]) / (chi[j + 1] - chi[j]), F(0), F(1))
    ang = chi[j] + ac * (chi[j + 1] - chi[j])
    sn, cc = np.sin(ang), np.cos(ang)
    Q = np.stack([-cc * cx, sx, sn * cx, -cc * sx, -cx, sn * sx, sn, np.zeros_like(sn), cc], -1).reshape(-1, 3, 3)
    B = rays['B']
    dloc = rays['dloc']
    d = rays['d32']
    A = np.zeros((len(h), 3, 3), F)
    dot = np.zeros((len(h), 3), F)
    for k in range(3):
        A += B[:, k, :, None] * Q[:, k, None, :]
        dot += d[:, k, None] * Q[:, k]
    Km = A - dloc[:, :, None] * dot[:, None, :]
    T = np.stack([np.stack([Km[:, i, 0] * Km[:, k, 0], Km[:, i, 1] * Km[:, k, 1], Km[:, i, 2] * Km[:, k, 2],
                            Km[:, i, 0] * Km[:, k, 2] + Km[:, i, 2] * Km[:, k, 0]], -1) for i, k in PAIRS], 1)
    st = rays['st']
    cp = np.where(st > F(1e-12), (d[:, 0] * cx + d[:, 1] * sx) / np.maximum(st, F(1e-30)), F(1))
    nc = len(chi)
    cells = np.stack([ir * nc + j, ir * nc + j + 1, (ir + 1) * nc + j, (ir + 1) * nc + j + 1], -1)
    sw = np.stack([(F(1) - ah) * (F(1) - ac), (F(1) - ah) * ac, ah * (F(1) - ac), ah * ac], -1)
    prof = profile_at(h, pk)
    return dict(h=h, ds=dsl, cells=cells, sw=sw, ir=ir, T=T, cm=cos_multiples(cp, max(33, pk.L + 1)), prof=prof,
                st_prof=strato_profile(h, pk) if pk.strato else None, Q=Q, r=r, qz=(q[0][:, 2], q[1][:, 2]), t=tt)


def path_point(pp, dd, t):
    q = ds_add(pp, ds_mul((t[0][:, None], t[1][:, None]), dd))
    q2 = ds_mul(q, q)
    r = ds_sqrt(ds_add(ds_add((q2[0][:, 0], q2[1][:, 0]), (q2[0][:, 1], q2[1][:, 1])), (q2[0][:, 2], q2[1][:, 2])))
    return q, q2, r


def beta_at(rays, t, pk, inside=None):
    """Extinction [n, W] at DS path coordinate t; at a segment end (inside = the segment's midpoint) its height
    snaps to the segment's side of a support end (numpy_reference.py:250-257)."""
    r = path_point(rays['pp'], rays['dd'], t)[2]
    h = np.clip(ds_value(ds_sub(r, (EARTH_R, F(0)))), F(0), F(pk.meta['top_km']))
    sup = support(pk)
    if inside is not None and sup is not None:
        ri = path_point(rays['pp'], rays['dd'], inside)[2]
        ih = np.clip(ds_value(ds_sub(ri, (EARTH_R, F(0)))), F(0), F(pk.meta['top_km']))
        h = support_height(h, ih, sup)
    return extinction(profile_at(h, pk), pk, strato_profile(h, pk) if pk.strato else None)


# ---------------------------------------------------------------- transport (numpy_reference.py:467-643)

def _ray_table(pk, b, rows):
    """Per-ray constants for the selected rays."""
    ray_cell = np.searchsorted(b['cell_off'], np.arange(len(b['d'])), side='right') - 1
    cell = ray_cell[rows]
    d = b['d'][rows]
    p = b['p'][cell]
    Bm = b['target'][cell].astype(F)
    dloc = b['dloc'][rows].astype(F)
    d32 = d.astype(F)
    pu = np.stack([F(1) - dloc[:, 0] * dloc[:, 0], F(1) - dloc[:, 1] * dloc[:, 1], F(1) - dloc[:, 2] * dloc[:, 2],
                   -dloc[:, 0] * dloc[:, 2]], -1)
    u = Bm[:, 2]
    dot = (dloc[:, 0] * u[:, 0] + dloc[:, 1] * u[:, 1]) + dloc[:, 2] * u[:, 2]
    e = u - dloc * dot[:, None]
    direct = np.stack([(pu[:, k] - e[:, i] * e[:, j]) / F(2) for k, (i, j) in enumerate(PAIRS)], -1)
    st = np.sqrt(np.maximum(0.0, 1 - d[:, 2] ** 2)).astype(F)
    return dict(pp=ds(p), dd=ds(d), B=Bm, dloc=dloc, d32=d32, pu=pu, direct=direct, st=st,
                Y=sh_basis(d[:, 2], pk.L))


def _sub(rt, idx):
    out = {}
    for k, v in rt.items():
        out[k] = tuple(x[idx] for x in v) if isinstance(v, tuple) else v[idx]
    return out


def transport(pk, b, field, first=False, boundary=None, query=False):
    """Per-ray radiance [rays, W, 4] (xx, yy, zz, xz coherency components) of bundle `b`."""
    with flush_to_zero():
        return _transport(pk, b, field, first, boundary, query)


def _transport(pk, b, field, first, boundary, query):
    n, W, L, K = len(b['d']), pk.W, pk.L, pk.K
    u, wu = (pk['uq'], pk['wuq']) if query else (pk['u'], pk['wu'])
    rows = np.arange(n)
    rt = _ray_table(pk, b, rows)
    g = F(pk.meta['g'])
    mix = F(pk.meta['mix'])
    phase = tropo_phase(rt['d32'][:, 2], pk) if 'tropo_lut' in pk else hg_phase(rt['d32'][:, 2], g)
    if pk.strato:
        sphase = legendre_phase(rt['d32'][:, 2], pk['strato_chi'])
    total = np.zeros((n, W, 4), F)
    corr = np.zeros_like(total)
    tau = np.zeros((n, W), F)
    tauc = np.zeros_like(tau)
    nseg = np.diff(b['seg_off'])
    field = np.asarray(field, F)
    hr, ha = pk['hr'], pk['ha']
    for slot in range(int(nseg.max(initial=0))):
        act = np.flatnonzero(nseg > slot)
        si = b['seg_off'][act] + slot
        seg = dict(a=b['seg_a'][si], b=b['seg_b'][si], lower=b['seg_lower'][si].astype(bool))
        r = _sub(rt, act)
        # Simpson prefix over the panels [a, t_0], [t_0, t_1], ..., [t_{nq-1}, b] (numpy_reference.py:236-291)
        t0 = ds(seg['a'])
        inside = ds((seg['a'] + seg['b']) / 2)
        beta0 = beta_at(r, t0, pk, inside)
        acc = np.zeros((len(act), W), F)
        for step in range(len(u)):
            q = sample(r, seg, u[step], wu[step], pk)
            beta1 = extinction(q['prof'], pk, q['st_prof'])
            tm = ds_add(t0, q['t'])
            tm = (tm[0] * F(0.5), tm[1] * F(0.5))
            wpan = ds_value(ds_sub(q['t'], t0)) / F(6)
            acc = acc + wpan[:, None] * ((beta0 + beta1) + F(4) * beta_at(r, tm, pk))
            t0, beta0 = q['t'], beta1
            mid = (tau[act] - tauc[act]) + acc
            att = q['ds'][:, None] * np.exp(-mid)
            val = _sample_value(pk, r, q, field, first, phase[act], sphase[act] if pk.strato else None, g, mix,
                                hr, ha)
            t, c = kahan_add(total[act], corr[act], val * att[:, :, None])
            total[act], corr[act] = t, c
        tend = ds(seg['b'])
        tm = ds_add(t0, tend)
        tm = (tm[0] * F(0.5), tm[1] * F(0.5))
        wpan = ds_value(ds_sub(tend, t0)) / F(6)
        beta_end = beta_at(r, tend, pk, inside)
        acc = acc + wpan[:, None] * ((beta0 + beta_end) + F(4) * beta_at(r, tm, pk))
        t, c = kahan_add(tau[act], tauc[act], acc)
        tau[act], tauc[act] = t, c
    if boundary is not None:
        bnd = np.asarray(boundary).astype(F)
        ef = b['end_f'].astype(F)
        E = (F(1) - ef)[:, None] * bnd[b['end_j']]
        E += ef[:, None] * bnd[b['end_j'] + 1]
        optical = np.zeros((n, W), F)
        for k in range(5):
            optical += b['end_col'][:, k, None] * pk['ext'][k]
        if pk.strato:
            optical += b['end_st'][:, None] * pk['strato_ext']
        E *= np.exp(-optical) * b['hits'][:, None].astype(F)
        for k in range(4):
            total[:, :, k] += (E * rt['pu'][:, k, None]) / F(2)
    return total


def _sample_value(pk, r, q, field, first, phase, sphase, g, mix, hr, ha):
    n, W, L, K = len(q['h']), pk.W, pk.L, pk.K
    pu = r['pu']
    val = np.zeros((n, W, 4), F)
    logs = np.zeros((n, W), F)
    wg = np.zeros_like(logs)
    am = np.zeros_like(logs)
    strat = pk.strato
    if first:
        sc, lit, st_sc = sun_columns(q, pk)
        optical = np.zeros((n, W), F)
        for k in range(5):
            optical += sc[:, k, None] * pk['ext'][k]
        if strat:
            optical += st_sc[:, None] * pk['strato_ext']
        sun = np.exp(-optical) * lit[:, None]
        ground = np.zeros((n, W), F)
        sground = np.zeros((n, W), F)
        d = r['d32']
        Q = q['Q']
        mu = np.zeros(n, F)
        exd = np.zeros(n, F)
        eyd = np.zeros(n, F)
        for k in range(3):
            mu += d[:, k] * Q[:, k, 2]
            exd += d[:, k] * Q[:, k, 0]
            eyd += d[:, k] * Q[:, k, 1]
        gd, gv = pk['gd'], pk['gv']
        for corner in range(4):
            cells = q['cells'][:, corner]
            gdc = gd[cells]
            m0 = mu[:, None] * gdc[:, :, 2] + exd[:, None] * gdc[:, :, 0]
            m1 = abs(eyd)[:, None] * gdc[:, :, 1]
            if 'tropo_lut' in pk:  # per wavelength from the table
                ph = (tropo_phase(np.clip(m0 + m1, F(-1), F(1)), pk)
                      + tropo_phase(np.clip(m0 - m1, F(-1), F(1)), pk)) / F(2)
                wph = q['sw'][:, corner, None, None] * ph
            else:
                ph = (hg_phase(np.clip(m0 + m1, F(-1), F(1)), g) + hg_phase(np.clip(m0 - m1, F(-1), F(1)), g)) / F(2)
                wph = q['sw'][:, corner, None] * ph
            if strat:
                sph = (legendre_phase(np.clip(m0 + m1, F(-1), F(1)), pk['strato_chi'])
                       + legendre_phase(np.clip(m0 - m1, F(-1), F(1)), pk['strato_chi'])) / F(2)
                swph = q['sw'][:, corner, None, None] * sph
            # sum over the cell's ground directions (the reference adds them one by one, in the same order)
            gvc = gv[cells]
            ground += np.einsum('ngw,ngw->nw' if wph.ndim == 3 else 'ng,ngw->nw', wph, gvc, dtype=F)
            if strat:
                sground += np.einsum('ngw,ngw->nw', swph, gvc, dtype=F)
        beam = (q['prof'][:, 1, None] * pk['asca']) * (sun * (phase if phase.ndim == 2 else phase[:, None]) + ground)
        if strat:
            sbeam = (q['st_prof'][:, None] * pk['strato_sca']) * (sun * sphase + sground)
        ray = (sun * q['prof'][:, 0, None]) * pk['ext'][0]
        for k in range(4):
            val[:, :, k] = ray * (mix * F(3 / (8 * math.pi)) * r['direct'][:, k, None]
                                  + (F(1) - mix) * F(1 / (8 * math.pi)) * pu[:, k, None]) + beam * pu[:, k, None] / F(2)
            if strat:
                val[:, :, k] += (sbeam * pu[:, k, None]) / F(2)
    Y = r['Y']
    for corner in range(4):
        cell = q['cells'][:, corner]
        irc = q['ir'] + corner // 2
        if first:
            rm = pk['gm'][cell].transpose(0, 2, 1)
            aero = np.zeros((n, W), F)
            density = q['prof'][:, 0]
        else:
            cache = np.zeros((n, max(33, L + 1), W), F)
            scache = np.zeros((n, max(33, L + 1), W), F) if strat else None
            for l in range(L + 1):
                for m in range(l + 1):
                    k = l * (l + 1) // 2 + m
                    cache[:, m] += Y[:, k, None] * field[cell, 10 + k]
                    if strat:
                        scache[:, m] += Y[:, k, None] * field[cell, 10 + K + k]
            aero = lane_tree_sum(q['cm'][:, :, None] * cache) * ha[irc, None]
            if strat:
                saero = lane_tree_sum(q['cm'][:, :, None] * scache) * pk['strato_density'][irc, None]
            rm = field[cell, :4].transpose(0, 2, 1)
            density = hr[irc]
            sup = support(pk)
            if sup is not None:  # numpy_reference.py:606-609
                density = np.where(q['h'] > sup[1], F(0), density)
                aero = np.where(q['h'][:, None] > sup[0], F(0), aero)
                if strat:
                    saero = np.where(q['h'][:, None] > sup[0], F(0), saero)
        trace = (rm[:, :, 0] + rm[:, :, 1]) + rm[:, :, 2]
        tensor = np.zeros((n, W, 4), F)
        for k in range(4):
            rot = np.zeros((n, W), F)
            for uu in range(4):
                rot += q['T'][:, k, uu, None] * rm[:, :, uu]
            tensor[:, :, k] = density[:, None] * (mix * rot + ((F(1) - mix) / F(3) * trace) * pu[:, k, None])
            tensor[:, :, k] += (aero * pu[:, k, None]) / F(2)
            if strat and not first:
                tensor[:, :, k] += (saero * pu[:, k, None]) / F(2)
            val[:, :, k] += q['sw'][:, corner, None] * tensor[:, :, k]
        if not first:
            tr = (tensor[:, :, 0] + tensor[:, :, 1]) + tensor[:, :, 2]
            good = tr >= TRACE_MIN
            t = np.where(good, tr, F(1))
            w = np.where(good, q['sw'][:, corner, None], F(0))
            logs += w * np.log(t)
            wg += w
            am += w * t
    if not first:
        ok = (wg > F(0)) & (am >= TRACE_MIN)
        mean = np.where(ok, am, F(1)) / np.where(ok, wg, F(1))
        val = val * np.exp(np.where(ok, logs - wg * np.log(mean), F(0)))[:, :, None]
    return val


# ---------------------------------------------------------------- projection (numpy_reference.py:689-711)

def project(pk, b, rad, ground_only=False):
    """Per-cell moments [cells, 4+K, W] (FP64 sums of FP32 products) and ground flux [cells, W]."""
    with flush_to_zero():
        return _project(pk, b, rad, ground_only)


def _project(pk, b, rad, ground_only):
    d = b['d']
    L, K, W = pk.L, pk.K, pk.W
    Y = sh_basis(d[:, 2], L)
    st = np.sqrt(np.maximum(0.0, 1 - d[:, 2] ** 2))
    cp = np.where(st > 1e-12, d[:, 0] / np.maximum(st, 1e-30), 1.0).astype(F)
    cm = cos_multiples(cp, max(33, L + 1))
    weight = b['weight'].astype(F)
    trace = (rad[:, :, 0] + rad[:, :, 1]) + rad[:, :, 2]
    weighted = trace * weight[:, None]
    ncell = len(b['cell_off']) - 1
    ray_cell = np.searchsorted(b['cell_off'], np.arange(len(d)), side='right') - 1
    out = np.zeros((ncell, 4 + K, W))
    if not ground_only:
        for k in range(4):
            np.add.at(out[:, k], ray_cell, (rad[:, :, k] * weight[:, None]).astype(np.float64))
        m_of_k = np.array([m for l in range(L + 1) for m in range(l + 1)])
        basis = Y * cm[:, m_of_k]
        prod = (weighted[:, None, :] * basis[:, :, None]).astype(np.float64)
        np.add.at(out[:, 4:], ray_cell, prod)
    g = (trace * (weight * np.maximum(F(0), b['dloc'][:, 2].astype(F)))[:, None]).astype(np.float64)
    flux = np.zeros((ncell, W))
    np.add.at(flux, ray_cell, g)
    return out, flux * pk.meta['albedo'] / math.pi


# ---------------------------------------------------------------- evaluation, apply, boxes, solve

def evaluate(pk, field, first=False, phase=0, boundary=None):
    """TransientGeometry.evaluate (src/sosfuse2/solve/ray_geometry.py:425-451) over the whole bundle."""
    if phase == 1:
        b = pk.bundle('cell', pk.nc)
        rad = transport(pk, b, field, first)
        return project(pk, b, rad, ground_only=True)
    b = pk.bundle('cell')
    rad = transport(pk, b, field, first, boundary)
    return project(pk, b, rad)


class Oracle:
    """Solver.initialize/apply/boxes/solve over one packed state."""

    def __init__(self, pk):
        self.pk = pk if isinstance(pk, StatePack) else StatePack(pk)
        self.first_moments = None
        self.first_flux = None

    def initialize(self):
        if self.first_moments is None:
            pk = self.pk
            zero = np.zeros((pk.ns, pk.source_size, pk.W), F)
            self.first_moments, self.first_flux = evaluate(pk, zero, first=True, phase=0)

    def apply(self, field):
        self.initialize()
        pk = self.pk
        _, flux = evaluate(pk, field, phase=1)
        boundary = flux + self.first_flux[: pk.nc]
        moment, _ = evaluate(pk, field, phase=0, boundary=boundary)
        moment = moment + self.first_moments
        return compose(pk, moment)

    def boxes(self, field):
        return boxes(self.pk, field)

    def solve(self, max_eval=None, tolerance=None, initial=None, log=None):
        pk = self.pk
        return anderson_solve(self.apply, self.boxes, (pk.ns, pk.source_size, pk.W),
                              pk.meta['max_eval'] if max_eval is None else max_eval,
                              pk.meta['tolerance'] if tolerance is None else tolerance, initial,
                              monitors=int(pk.meta.get('monitors', 5)), log=log)


def compose(pk, moment):
    """Next source from the incident moments (source_iteration.py:176-212)."""
    K = pk.K
    ext0 = pk['ext0'].astype(F)
    out = np.empty((pk.ns, pk.source_size, pk.W), F)
    out[:, :4] = (moment[:, :4] * (F(3 / (8 * math.pi)) * ext0)[None, None, :]).astype(F)
    out[:, 4:10] = (moment[:, 4:10] * pk['rf'][None, :, None] * ext0[None, None, :]).astype(F)
    eigen = pk['tropo_eigen'][None, :, :] if 'tropo_lut' in pk else pk['af'][None, :, None]
    out[:, 10:10 + K] = (moment[:, 4:] * eigen * pk['asca'][None, None, :]).astype(F)
    if pk.strato:
        out[:, 10 + K:] = (moment[:, 4:] * pk['strato_eigen'][None, :, :]
                           * pk['strato_sca_source'][None, None, :]).astype(F)
    out[np.abs(out) < TRACE_MIN] = 0
    return out


def boxes(pk, field):
    """Observer values [monitors, 7, W]: GL-weighted trace radiance of the box rays times the solar spectrum."""
    b = pk.bundle('query')
    rad = transport(pk, b, field, first=False, query=True)
    I = rad[..., :3].astype(np.float64).sum(-1) * pk['solar'][None, :]
    pts = int(pk.meta['box_points'])
    I = I.reshape(-1, pk.meta['n_dirs'], pts, pk.W)
    return np.einsum('hdnw,n->hdw', I, pk['box_ww'])


def anderson_weights(products):
    """Regularised Gram solve, weights normalised to sum 1, rejected unless finite and max|w| < 8
    (source_iteration.py:25-33)."""
    gram = np.array(products, dtype=np.float64, copy=True)
    gram[np.diag_indices_from(gram)] += max(float(np.trace(gram)) * 1e-10, 1e-30)
    w = np.linalg.solve(gram, np.ones(len(gram)))
    w /= w.sum()
    if np.isfinite(w).all() and np.max(np.abs(w)) < 8:
        return w.astype(np.float32)
    return None


def anderson_solve(apply, boxes_fn, shape, max_eval, tolerance, initial=None, monitors=5, log=None):
    """Solver.solve (source_iteration.py:309-663) with the list-ring Anderson path (618-635)."""
    W = shape[2]
    x = np.zeros(shape, F) if initial is None else np.asarray(initial, F).copy()
    gs = [[] for _ in range(W)]
    fs = [[] for _ in range(W)]
    done = np.zeros(W, bool)
    history = []
    it = 0
    for it in range(1, max_eval + 1):
        old = boxes_fn(x)
        g = apply(x)
        bad = int(np.count_nonzero(~np.isfinite(g)))
        if bad:
            raise RuntimeError(f'E_NONFINITE_SOURCE: {bad} values after evaluation {it}')
        if done.any():
            g = np.where(done[None, None, :], x, g)
        new = boxes_fn(g)
        so, sn = old[:monitors], new[:monitors]
        rr = np.max(abs(sn - so) / np.maximum(abs(sn), 1e-30), axis=(0, 1))
        ss = np.max(abs(g - x), axis=(0, 1)) / np.maximum(np.max(abs(g), axis=(0, 1)), F(1e-30))
        if it >= 2:
            done |= np.maximum(rr, ss) <= tolerance
        history.append(dict(evaluation=it, observer_relative=rr.tolist(), source_relative=ss.tolist(),
                            converged=done.tolist()))
        if log:
            log(it, rr, ss, done)
        if done.all():
            x = g
            break
        for w in range(W):
            if done[w]:
                gs[w], fs[w] = [], []
        nxt = g.copy()
        for w in range(W):
            if done[w]:
                continue
            gw = g[:, :, w]
            norm = np.linalg.norm(gw, axis=1)
            scale = np.maximum(norm, norm.max() * 1e-8)
            feature = ((gw - x[:, :, w]) / scale[:, None]).astype(F).ravel()
            obs = np.asarray(((sn[:, :, w] - so[:, :, w]) / np.maximum(abs(sn[:, :, w]), 1e-20)).ravel()
                             * math.sqrt(len(feature) / (sn.shape[0] * sn.shape[1])), F)
            gs[w].append(gw.copy())
            fs[w].append(np.concatenate([feature, obs]))
            if len(fs[w]) > 4:
                gs[w].pop(0)
                fs[w].pop(0)
            if len(fs[w]) > 1:
                f = np.stack(fs[w], 1)
                try:
                    ah = anderson_weights(f.T @ f)
                except np.linalg.LinAlgError:
                    ah = None
                if ah is not None:
                    nxt[:, :, w] = sum(c * q for c, q in zip(ah, gs[w]))
        x = nxt
    if not done.all():
        raise RuntimeError(f'E_NOT_CONVERGED: {done.sum()}/{W} within {tolerance}')
    return x, dict(evaluations=it, tolerance=tolerance, converged=done.tolist(), history=history)
