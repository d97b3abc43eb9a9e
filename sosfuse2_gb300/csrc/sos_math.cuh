// Device math of the SOS transport, compiled both for sm_103a (by nvcc) and for the host (by g++, for CPU tests).
//
// One call of `transport_lane` integrates one incoming ray of one destination cell for one wavelength: the ray's
// segments (shell crossings) are walked node by node with the reference's double-single (two-float) geometry
// (src/sosfuse2/backends/numpy_reference.py:294-387, arithmetic.py:15-66), the optical depth to each node is the
// Simpson prefix of the extinction (numpy_reference.py:236-291), and each node adds the scattered source of its
// four bracketing (height, solar-zenith) cells, rotated into the ray's frame, attenuated and Kahan-summed
// (numpy_reference.py:467-643). The aerosol source of a corner cell is the SH plane of that cell contracted with
// the ray's SH basis row (numpy_reference.py:588-600) and kept per corner while the corner cell does not change.
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define SOS_HD __host__ __device__ __forceinline__
#else
#define SOS_HD inline
struct float4 {
    float x, y, z, w;
};
struct float2 {
    float x, y;
};
#endif

// Error-free transformations need every add and multiply rounded on its own: no contraction into FMA.
#if defined(__CUDA_ARCH__)
#define SOS_ADD(a, b) __fadd_rn((a), (b))
#define SOS_SUB(a, b) __fsub_rn((a), (b))
#define SOS_MUL(a, b) __fmul_rn((a), (b))
#define SOS_DIV(a, b) __fdiv_rn((a), (b))
#define SOS_SQRT(a) __fsqrt_rn(a)
#define SOS_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#else
// the host build uses -ffp-contract=off
#define SOS_ADD(a, b) ((a) + (b))
#define SOS_SUB(a, b) ((a) - (b))
#define SOS_MUL(a, b) ((a) * (b))
#define SOS_DIV(a, b) ((a) / (b))
#define SOS_SQRT(a) sqrtf(a)
#define SOS_FMA(a, b, c) fmaf((a), (b), (c))
#endif

namespace sos {

constexpr float EARTH_R = 6371.0f;
constexpr float TRACE_MIN = 1.17549435e-38f;  // FLT_MIN
constexpr float PI_F = 3.14159265358979f;
constexpr float C_3_8PI = 0.119366207318921505f;   // 3 / (8 pi), rounded once
constexpr float C_1_8PI = 0.0397887357729738339f;  // 1 / (8 pi), rounded once
constexpr float C_4PI = 12.5663706143591725f;      // 4 pi, rounded once
constexpr int MAX_L = 48;

// ------------------------------------------------------------------ double-single arithmetic
struct DS {
    float h, l;
};

SOS_HD DS ds_make(float h) { return DS{h, 0.0f}; }

SOS_HD DS ds_add(DS a, DS b) {
    float s = SOS_ADD(a.h, b.h);
    float v = SOS_SUB(s, a.h);
    float e = SOS_ADD(SOS_ADD(SOS_SUB(a.h, SOS_SUB(s, v)), SOS_SUB(b.h, v)), SOS_ADD(a.l, b.l));
    float h = SOS_ADD(s, e);
    return DS{h, SOS_SUB(e, SOS_SUB(h, s))};
}

SOS_HD DS ds_neg(DS a) { return DS{-a.h, -a.l}; }
SOS_HD DS ds_sub(DS a, DS b) { return ds_add(a, ds_neg(b)); }

SOS_HD DS ds_mul(DS a, DS b) {
    float p = SOS_MUL(a.h, b.h);
    float e = SOS_FMA(a.h, b.h, -p);  // exact low part of a.h * b.h, one rounding
    e = SOS_ADD(SOS_ADD(e, SOS_MUL(a.h, b.l)), SOS_MUL(a.l, b.h));
    float h = SOS_ADD(p, e);
    return DS{h, SOS_SUB(e, SOS_SUB(h, p))};
}

SOS_HD DS ds_sqrt(DS a) {
    float h = SOS_SQRT(fmaxf(a.h, 0.0f));
    DS e = ds_sub(a, ds_mul(ds_make(h), ds_make(h)));
    float lo = SOS_DIV(SOS_ADD(e.h, e.l), fmaxf(SOS_MUL(2.0f, h), 1e-30f));
    return ds_add(ds_make(h), ds_make(lo));
}

SOS_HD DS ds_div(DS a, DS b) {
    float h = SOS_DIV(a.h, b.h);
    DS e = ds_sub(a, ds_mul(ds_make(h), b));
    float lo = SOS_DIV(SOS_ADD(e.h, e.l), b.h);
    return ds_add(ds_make(h), ds_make(lo));
}

SOS_HD float ds_val(DS a) { return SOS_ADD(a.h, a.l); }

SOS_HD float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

// Index i in [0, n-2] with grid[i] <= x < grid[i+1] (searchsorted right, minus one, clipped).
SOS_HD int bracket(const float* grid, int n, float x) {
    int lo = 0, hi = n;  // count of grid values <= x by binary search
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (grid[mid] <= x) lo = mid + 1; else hi = mid;
    }
    int i = lo - 1;
    return i < 0 ? 0 : (i > n - 2 ? n - 2 : i);
}

// ------------------------------------------------------------------ inputs
// Per-state optics and grids (device pointers, or host pointers in the host build).
struct Optics {
    int L, K, W, nh, nc, ns, src;   // src = source slots per cell (10 + K or 10 + 2K)
    int strato;
    float top_km, mix, g, height, air_surface, inv_step;
    int density_last, density_mask;
    float strato_center, strato_sigma, strato_norm;
    const float* h;        // [nh]
    const float* chi;      // [nc]
    const float* hr;       // [nh] air density shape at the cell heights
    const float* ext;      // [5][W] extinction per unit profile: air, aerosol, O3, NO2, O4
    const float* asca;     // [W]  aerosol scattering
    const float* table;    // [rows][3] air, ozone, NO2 on the uniform profile grid
    int n_sun_h, n_sun_x;
    const float* sun_h;    // [n_sun_h]
    const float* sun_col;  // [n_sun_h][n_sun_x][5]
    const float* strato_sun_col;  // [n_sun_h][n_sun_x]
    const float* gm;       // [ns][4][W] first-light direct-ground Rayleigh moments
    const int* goff;       // [ns+1] ground directions per cell
    const float* gdir;     // [*][3]
    const float* gval;     // [*][W]
    const float* strato_ext;  // [W]
    const float* strato_sca;  // [W]
    const float* strato_chi;  // [33][W] Legendre moments of the stratospheric phase function
    const float* sh_a;     // [K] recurrence coefficients (FP32)
    const float* sh_b;     // [K]
    const float* sh_d;     // [L+1] diagonal factors
    const float* strato_lut;  // [STRATO_LUT_BINS + 1][W] stratospheric phase per sr on a uniform grid of u in [-1, 1]
    const uint8_t* gsame;  // [ns] 1 when cell c + 1 (same height, next solar zenith) has c's ground directions, or null
    const float2* strato_lut2;  // [STRATO_LUT_BINS][W] (value, next value - value) of strato_lut, or null
    const float4* gdir4;        // [*] gdir padded to 16 bytes, or null
    int aer2_on;                // two-layer tropospheric aerosol profile instead of exp(-h / height)
    float aer2[7];              // its vector [bl_top - w/2, 1/w, a_bl, k_bl, a_ft, k_ft, bl_top]
    int support;                // extended top: components vanish above their support ends
    float lower_end, air_end;   // support ends of the components other than air and of the air (km)
    int tropo_bins;             // tabulated tropospheric phase (TROPO_MIE) on tropo_bins + 1 nodes, or 0 for HG
    const float* tropo_lut;     // [tropo_bins + 1][W] tropospheric phase per sr on a uniform grid of u in [-1, 1]
    const float2* tropo_lut2;   // [tropo_bins][W] (value, next value - value) of tropo_lut, or null
};

constexpr int STRATO_LUT_BINS = 4096;

// One bundle of rays: cells (destination points) with their incoming rays and compacted segments.
struct Rays {
    int ncell, nray;
    const int* cell_off;   // [ncell+1]
    const int* ray_cell;   // [nray]
    const float* p;        // [ncell][6] start point, double-single (hi xyz, lo xyz)
    const float* frame;    // [ncell][9] target frame B[k][i]
    const float4* dir;     // [nray] (dx, dy, dz, sin theta) FP32
    const float4* dir_lo;  // [nray] (dx_lo, dy_lo, dz_lo, weight)
    const float4* dloc;    // [nray] (local direction xyz, end fraction)
    const int* seg_off;    // [nray+1]
    const float4* seg;     // [nseg] (a_hi, a_lo, b_hi, b_lo) path coordinates of the segment ends
    const uint8_t* lower;  // [nseg] segment runs upward (its lower end is at a)
    const int* end_j;      // [nray] solar-zenith interval of the ray's ground end
    const float* end_col;  // [nray][6] component columns (5) and stratospheric column to the ground end
    const uint8_t* hits;   // [nray]
    const float* pcp;      // [nray] cos of the ray's global azimuth, d_x / sin(theta) (projection)
};

// ------------------------------------------------------------------ optics primitives
struct Profile {
    float v[5];
};

// Two-layer tropospheric aerosol shape (kernel.cu aerosol_two_layer, FP32 mirror atmosphere/tropo_profile.py:295-304):
// a smoothstep over [P0, P0 + 1/P1] from the boundary layer P2 exp(-h P3) to the free troposphere
// P4 exp(-(max(h, P0) - P6) P5), each product and sum rounded on its own.
SOS_HD float aerosol_two_layer(float h, const float* P) {
    const float x = clampf(SOS_MUL(SOS_ADD(h, -P[0]), P[1]), 0.0f, 1.0f);
    const float s = SOS_MUL(SOS_MUL(x, x), SOS_ADD(3.0f, -SOS_MUL(2.0f, x)));
    const float bl = SOS_MUL(SOS_MUL(P[2], expf(-SOS_MUL(h, P[3]))), SOS_ADD(1.0f, -s));
    const float ft = SOS_MUL(SOS_MUL(P[4], expf(-SOS_MUL(SOS_ADD(fmaxf(h, P[0]), -P[6]), P[5]))), s);
    return SOS_ADD(bl, ft);
}

SOS_HD Profile profile_at(const Optics& o, float h) {
    float hc = clampf(h, 0.0f, o.top_km);
    float x = hc * o.inv_step;
    int i = (int)x;
    if (i > o.density_last) i = o.density_last;
    float f = x - (float)i;
    const float* t0 = o.table + 3 * i;
    const float* t1 = t0 + 3;
    float tab0 = t0[0] + f * (t1[0] - t0[0]);
    float tab1 = t0[1] + f * (t1[1] - t0[1]);
    float tab2 = t0[2] + f * (t1[2] - t0[2]);
    Profile p;
    p.v[0] = (o.density_mask & 1) ? tab0 : expf(-h / 8.0f);
    p.v[1] = o.aer2_on ? aerosol_two_layer(h, o.aer2) : expf(-h / o.height);
    p.v[2] = (o.density_mask & 2) ? tab1 : fmaxf(0.0f, 1.0f - fabsf(h - 25.0f) / 15.0f);
    p.v[3] = tab2;
    float q = p.v[0] / o.air_surface;
    p.v[4] = q * q;
    if (o.support) {  // zero strictly above each component's support end (numpy_reference.py:168-172,221-222)
        if (h > o.air_end) p.v[0] = 0.0f;
        if (h > o.lower_end)
            for (int k = 1; k < 5; ++k) p.v[k] = 0.0f;
    }
    return p;
}

// A segment end's height within one FP32 ulp of a support end moves to the side the segment lies on (inside_h: the
// height of the segment's midpoint; numpy_reference.py:175-183).
SOS_HD float support_height(const Optics& o, float h, float inside_h) {
    if (!o.support) return h;
    const float edges[2] = {o.lower_end, o.air_end};
    for (int i = 0; i < 2; ++i) {
        const float edge = edges[i];
        const float above = nextafterf(edge, INFINITY);
        if (h >= nextafterf(edge, -INFINITY) && h <= above) h = inside_h > edge ? above : edge;
    }
    return h;
}

SOS_HD float strato_profile(const Optics& o, float h) {
    if (o.support && h > o.lower_end) return 0.0f;
    float t = (h - o.strato_center) / o.strato_sigma;
    return expf(-0.5f * (t * t)) / o.strato_norm;
}

SOS_HD float extinction(const Optics& o, const Profile& p, float st, int w) {
    float b = 0.0f;
    for (int k = 0; k < 5; ++k) b += p.v[k] * o.ext[k * o.W + w];
    if (o.strato) b += st * o.strato_ext[w];
    return b;
}

SOS_HD float hg_phase(float u, float g) {
    float den = fmaxf(1e-20f, (1.0f + g * g) - (2.0f * g) * u);
    return (1.0f - g * g) / (C_4PI * (den * sqrtf(den)));
}

SOS_HD float legendre_phase(const Optics& o, float u, int w) {
    float p0 = 1.0f, p1 = u;
    float val = p0 * o.strato_chi[w] + p1 * o.strato_chi[o.W + w];
    for (int l = 2; l < 33; ++l) {
        float pn = (((float)(2 * l - 1) * u) * p1 - (float)(l - 1) * p0) / (float)l;
        val += pn * o.strato_chi[l * o.W + w];
        p0 = p1;
        p1 = pn;
    }
    return val / C_4PI;
}

SOS_HD float ftz_value(DS a) {
    float h = fabsf(a.h) < TRACE_MIN ? 0.0f : a.h;
    float l = fabsf(a.l) < TRACE_MIN ? 0.0f : a.l;
    float v = h + l;
    return fabsf(v) < TRACE_MIN ? 0.0f : v;
}

// ------------------------------------------------------------------ one quadrature node
struct Node {
    DS t;             // path coordinate
    DS r;             // distance from the Earth's centre
    DS qz;            // z of the node
    float h, ds;      // height (clipped), quadrature weight along the path
    float sw[4];      // bilinear weights of the four corner cells
    int cell[4];      // corner cells (ir, j), (ir, j+1), (ir+1, j), (ir+1, j+1)
    int ir;           // height interval
    float T[4][4];    // Rayleigh coherency rotation
    float cp;         // cos of the azimuth between the ray and the node's meridian
    float mu, exd, eyd;  // ray direction in the node's local frame (first light)
    Profile prof;
    float st_prof;
    float fr[4];      // cos, sin of the interpolated cell angle; cos, sin of the node's longitude (frame inputs)
    float ah, ac;     // bilinear fractions in height and solar zenith
    int j;            // solar-zenith interval
    int above;        // extended top: bit 0 above the lower components' support end, bit 1 above the air's
};

struct RayConst {
    DS p[3], d[3];
    float B[3][3];    // frame rows B[k][i]
    float d32[3], dloc[3], pu[4], direct[4], st, weight, end_f;
};

SOS_HD DS ds_half(DS a) { return DS{a.h * 0.5f, a.l * 0.5f}; }  // exact

SOS_HD void path_point(const RayConst& rc, DS t, DS q[3], DS q2[3], DS& r) {
    for (int k = 0; k < 3; ++k) {
        q[k] = ds_add(rc.p[k], ds_mul(t, rc.d[k]));
        q2[k] = ds_mul(q[k], q[k]);
    }
    r = ds_sqrt(ds_add(ds_add(q2[0], q2[1]), q2[2]));
}

SOS_HD float path_height(const Optics& o, DS r) { return clampf(ds_val(ds_sub(r, ds_make(EARTH_R))), 0.0f, o.top_km); }

SOS_HD float beta_at(const Optics& o, const RayConst& rc, DS t, int w) {
    DS q[3], q2[3], r;
    path_point(rc, t, q, q2, r);
    float h = path_height(o, r);
    Profile p = profile_at(o, h);
    return extinction(o, p, o.strato ? strato_profile(o, h) : 0.0f, w);
}

// Height h of an end of segment [a, b] with the support snap of an extended top (the segment's midpoint decides the
// side; numpy_reference.py:250-257).
SOS_HD float segment_end_height(const Optics& o, const RayConst& rc, float h, DS a, DS b) {
    if (!o.support) return h;
    DS q[3], q2[3], r;
    path_point(rc, ds_half(ds_add(a, b)), q, q2, r);
    return support_height(o, h, path_height(o, r));
}

// beta_at at an end t of segment [a, b].
SOS_HD float beta_end(const Optics& o, const RayConst& rc, DS t, DS a, DS b, int w) {
    DS q[3], q2[3], r;
    path_point(rc, t, q, q2, r);
    const float h = segment_end_height(o, rc, path_height(o, r), a, b);
    Profile p = profile_at(o, h);
    return extinction(o, p, o.strato ? strato_profile(o, h) : 0.0f, w);
}

// Rotation of the Rayleigh coherency tensor into the ray frame, the ray direction in the node's local frame and the
// azimuth cosine, from the cos/sin of the node's interpolated cell angle (cc, sn) and of its longitude (cx, sx)
// (numpy_reference.py:515-545).
SOS_HD void node_frame(const RayConst& rc, float cc, float sn, float cx, float sx, Node& n) {
    n.fr[0] = cc;
    n.fr[1] = sn;
    n.fr[2] = cx;
    n.fr[3] = sx;
    // Q rows: local (east, north, up) of the node in global coordinates, columns indexed [k][j]
    float Q[3][3] = {{-cc * cx, sx, sn * cx}, {-cc * sx, -cx, sn * sx}, {sn, 0.0f, cc}};
    float A[3][3], dot[3];
    for (int i = 0; i < 3; ++i)
        for (int jj = 0; jj < 3; ++jj) {
            float s = 0.0f;
            for (int k = 0; k < 3; ++k) s += rc.B[k][i] * Q[k][jj];
            A[i][jj] = s;
        }
    for (int jj = 0; jj < 3; ++jj) {
        float s = 0.0f;
        for (int k = 0; k < 3; ++k) s += rc.d32[k] * Q[k][jj];
        dot[jj] = s;
    }
    float Km[3][3];
    for (int i = 0; i < 3; ++i)
        for (int jj = 0; jj < 3; ++jj) Km[i][jj] = A[i][jj] - rc.dloc[i] * dot[jj];
    const int PI_[4] = {0, 1, 2, 0}, PK_[4] = {0, 1, 2, 2};
    for (int pr = 0; pr < 4; ++pr) {
        int i = PI_[pr], k = PK_[pr];
        n.T[pr][0] = Km[i][0] * Km[k][0];
        n.T[pr][1] = Km[i][1] * Km[k][1];
        n.T[pr][2] = Km[i][2] * Km[k][2];
        n.T[pr][3] = Km[i][0] * Km[k][2] + Km[i][2] * Km[k][0];
    }
    n.mu = dot[2];
    n.exd = dot[0];
    n.eyd = dot[1];
    n.cp = rc.st > 1e-12f ? (rc.d32[0] * cx + rc.d32[1] * sx) / fmaxf(rc.st, 1e-30f) : 1.0f;
}

// Corner cells (ir, j), (ir, j+1), (ir+1, j), (ir+1, j+1) and their bilinear weights.
SOS_HD void node_corners(const Optics& o, int ir, int j, float ah, float ac, Node& n) {
    n.ah = ah;
    n.ac = ac;
    n.j = j;
    n.ir = ir;
    n.cell[0] = ir * o.nc + j;
    n.cell[1] = ir * o.nc + j + 1;
    n.cell[2] = (ir + 1) * o.nc + j;
    n.cell[3] = (ir + 1) * o.nc + j + 1;
    n.sw[0] = (1.0f - ah) * (1.0f - ac);
    n.sw[1] = (1.0f - ah) * ac;
    n.sw[2] = ah * (1.0f - ac);
    n.sw[3] = ah * ac;
}

SOS_HD void sample_node(const Optics& o, const RayConst& rc, DS a, DS b, bool lower, DS u, DS wu, Node& n) {
    DS length = ds_sub(b, a);
    DS v = lower ? u : ds_sub(ds_make(1.0f), u);
    DS tt = lower ? ds_add(a, ds_mul(length, ds_mul(u, u))) : ds_sub(b, ds_mul(length, ds_mul(v, v)));
    n.t = tt;
    n.ds = ds_val(ds_mul(ds_mul(length, v), wu)) * 2.0f;
    DS q[3], q2[3], r;
    path_point(rc, tt, q, q2, r);
    n.r = r;
    n.qz = q[2];
    float h = path_height(o, r);
    n.h = h;
    n.above = o.support ? (h > o.lower_end ? 1 : 0) | (h > o.air_end ? 2 : 0) : 0;
    DS xy = ds_sqrt(ds_add(q2[0], q2[1]));
    float rho = ds_val(xy);
    float cx = 1.0f, sx = 0.0f;
    if (rho > 1e-12f) {
        DS den = DS{fmaxf(xy.h, 1e-30f), xy.l};
        cx = ds_val(ds_div(q[0], den));
        sx = ds_val(ds_div(q[1], den));
    }
    float angle = atan2f(rho, ds_val(q[2]));
    int ir = bracket(o.h, o.nh, h);
    int j = bracket(o.chi, o.nc, angle);
    float ah = clampf((h - o.h[ir]) / (o.h[ir + 1] - o.h[ir]), 0.0f, 1.0f);
    float ac = clampf((angle - o.chi[j]) / (o.chi[j + 1] - o.chi[j]), 0.0f, 1.0f);
    float ang = o.chi[j] + ac * (o.chi[j + 1] - o.chi[j]);
    node_frame(rc, cosf(ang), sinf(ang), cx, sx, n);
    node_corners(o, ir, j, ah, ac, n);
    n.prof = profile_at(o, h);
    n.st_prof = o.strato ? strato_profile(o, h) : 0.0f;
}

// Slant columns towards the sun at the node: bilinear in (height, x), x from the node's solar elevation relative to
// the geometric horizon (numpy_reference.py:431-458).
SOS_HD void sun_columns(const Optics& o, const Node& n, float col[5], float& st, float& lit) {
    float hh = clampf(n.h, 0.0f, o.top_km);
    DS height = ds_sub(n.r, ds_make(EARTH_R));
    if (!(ftz_value(height) > 0.0f)) height = DS{0.0f, 0.0f};
    DS rad = ds_add(ds_make(EARTH_R), height);
    DS mg = ds_neg(ds_sqrt(ds_div(ds_mul(height, ds_add(ds_make(2.0f * EARTH_R), height)), ds_mul(rad, rad))));
    DS delta = ds_sub(ds_div(n.qz, n.r), mg);
    if (ftz_value(delta) == 0.0f) delta = DS{0.0f, 0.0f};
    bool is_lit = ds_val(delta) >= 0.0f;
    if (!is_lit) delta = DS{0.0f, 0.0f};
    float x = clampf(ds_val(ds_sqrt(ds_div(delta, ds_sub(ds_make(1.0f), mg)))), 0.0f, 1.0f);
    int i = bracket(o.sun_h, o.n_sun_h, hh);
    float a = (hh - o.sun_h[i]) / (o.sun_h[i + 1] - o.sun_h[i]);
    float f = x * (float)(o.n_sun_x - 1);
    int j = (int)f;
    j = j < 0 ? 0 : (j > o.n_sun_x - 2 ? o.n_sun_x - 2 : j);
    float bb = f - (float)j;
    const float* c00 = o.sun_col + ((size_t)i * o.n_sun_x + j) * 5;
    const float* c10 = c00 + (size_t)o.n_sun_x * 5;
    const float* c01 = c00 + 5;
    const float* c11 = c10 + 5;
    float w00 = (1.0f - a) * (1.0f - bb), w10 = a * (1.0f - bb), w01 = (1.0f - a) * bb, w11 = a * bb;
    for (int k = 0; k < 5; ++k) {
        float v = w00 * c00[k];
        v += w10 * c10[k];
        v += w01 * c01[k];
        v += w11 * c11[k];
        col[k] = v;
    }
    st = 0.0f;
    if (o.strato) {
        const float* s00 = o.strato_sun_col + (size_t)i * o.n_sun_x + j;
        st = w00 * s00[0];
        st += w10 * s00[o.n_sun_x];
        st += w01 * s00[1];
        st += w11 * s00[o.n_sun_x + 1];
    }
    lit = is_lit ? 1.0f : 0.0f;
}

SOS_HD void ray_constants(const Rays& b, int ray, RayConst& rc) {
    int cell = b.ray_cell[ray];
    const float* p = b.p + 6 * cell;
    float4 d = b.dir[ray], dl = b.dir_lo[ray], lo = b.dloc[ray];
    rc.p[0] = DS{p[0], p[3]};
    rc.p[1] = DS{p[1], p[4]};
    rc.p[2] = DS{p[2], p[5]};
    rc.d[0] = DS{d.x, dl.x};
    rc.d[1] = DS{d.y, dl.y};
    rc.d[2] = DS{d.z, dl.z};
    rc.d32[0] = d.x;
    rc.d32[1] = d.y;
    rc.d32[2] = d.z;
    rc.st = d.w;
    rc.weight = dl.w;
    const float* f = b.frame + 9 * cell;
    for (int k = 0; k < 3; ++k)
        for (int i = 0; i < 3; ++i) rc.B[k][i] = f[3 * k + i];
    rc.dloc[0] = lo.x;
    rc.dloc[1] = lo.y;
    rc.dloc[2] = lo.z;
    rc.end_f = lo.w;
    rc.pu[0] = 1.0f - lo.x * lo.x;
    rc.pu[1] = 1.0f - lo.y * lo.y;
    rc.pu[2] = 1.0f - lo.z * lo.z;
    rc.pu[3] = -lo.x * lo.z;
    const float* u = rc.B[2];
    float dot = (lo.x * u[0] + lo.y * u[1]) + lo.z * u[2];
    float e[3] = {u[0] - lo.x * dot, u[1] - lo.y * dot, u[2] - lo.z * dot};
    const int PI_[4] = {0, 1, 2, 0}, PK_[4] = {0, 1, 2, 2};
    for (int k = 0; k < 4; ++k) rc.direct[k] = (rc.pu[k] - e[PI_[k]] * e[PK_[k]]) / 2.0f;
}

// Aerosol SH contraction for one corner cell: cache[m] = sum_l Y_lm(mu) plane[cell][k(l,m)] for m = 0..L, with the
// normalised associated-Legendre recurrence evaluated on the fly (FP32) from the ray's mu = d_z.
SOS_HD void sh_contract(const Optics& o, float mu, float st, const float* plane_cell, int wstride, float* cache,
                        int cstride) {
    const int L = o.L;
    float pmm = 0.28209479177387814f;  // 1 / sqrt(4 pi)
    for (int m = 0; m <= L; ++m) {
        if (m) pmm = (pmm * o.sh_d[m]) * st;
        const float scale = m ? 1.41421356237309515f : 1.0f;
        float p0 = pmm;
        int k = m * (m + 1) / 2 + m;
        float acc = (scale * p0) * plane_cell[(size_t)k * wstride];
        if (m < L) {
            float p1 = (sqrtf(2.0f * m + 3.0f) * mu) * p0;
            k = (m + 1) * (m + 2) / 2 + m;
            acc += (scale * p1) * plane_cell[(size_t)k * wstride];
            for (int l = m + 2; l <= L; ++l) {
                k = l * (l + 1) / 2 + m;
                float p2 = (o.sh_a[k] * mu) * p1 - o.sh_b[k] * p0;
                acc += (scale * p2) * plane_cell[(size_t)k * wstride];
                p0 = p1;
                p1 = p2;
            }
        }
        cache[m * cstride] = acc;
    }
}

// Sum over m of cos(m phi) * cache[m], cos(m phi) by the Chebyshev recurrence of cp.
SOS_HD float azimuth_sum(int L, float cp, const float* cache, int cstride) {
    cp = clampf(cp, -1.0f, 1.0f);
    float c0 = 1.0f, c1 = cp;
    float s = cache[0];
    if (L >= 1) s += c1 * cache[cstride];
    for (int m = 2; m <= L; ++m) {
        float c2 = (2.0f * cp) * c1 - c0;
        s += c2 * cache[m * cstride];
        c0 = c1;
        c1 = c2;
    }
    return s;
}

SOS_HD void kahan(float& total, float& comp, float value) {
    float y = value - comp;
    float t = total + y;
    comp = (t - total) - y;
    total = t;
}

// Everything one lane needs that is shared by all rays of a launch.
struct LaneInputs {
    const float* field;     // [ns][src][W] current source
    const float* plane;     // aerosol (+ stratospheric) SH plane, already scaled by the cell density: [ns][K][W]
                            // (kp = 0), or [ns][W][kp] rows padded to kp = K rounded up to 4 (few wavelengths)
    const float* boundary;  // [nc][W] ground flux at the surface nodes, or null
    const float* u_hi;      // quadrature nodes on [0, 1] and weights, double-single
    const float* u_lo;
    const float* wu_hi;
    const float* wu_lo;
    int nq;
    int first;
    int kp;
    int table_only;         // write the node table only (no radiance): the corner path computes the values after it
};

// Henyey-Greenstein phase (per sr) of the pair of scattering cosines (up, dn), averaged:
// ((1 - g^2) / 4 pi) (den_up^-3/2 + den_dn^-3/2) / 2 with den = 1 + g^2 - 2 g u, by reciprocal square roots.
struct HgPair {
    float a, b, c;  // 1 + g^2, 2 g, (1 - g^2) / (8 pi)
};

SOS_HD HgPair hg_pair_constants(float g) { return HgPair{1.0f + g * g, 2.0f * g, (1.0f - g * g) / (2.0f * C_4PI)}; }

SOS_HD float rsqrt_fast(float x) {
#if defined(__CUDA_ARCH__)
    return rsqrtf(x);
#else
    return 1.0f / sqrtf(x);
#endif
}

SOS_HD float hg_pair(const HgPair& k, float up, float dn) {
    const float r1 = rsqrt_fast(fmaxf(1e-20f, k.a - k.b * up));
    const float r2 = rsqrt_fast(fmaxf(1e-20f, k.a - k.b * dn));
    return k.c * ((r1 * r1) * r1 + (r2 * r2) * r2);
}

// Stratospheric phase by linear interpolation in its table (built from the same 33 Legendre moments in FP64), the
// form the reference's CUDA path evaluates it in (kernel.cu strato_lut_build); used in the first-light ground sums.
// Position of u in the table: bin i and fraction f.
SOS_HD void strato_lut_pos(float u, int& i, float& f) {
    const float x = (clampf(u, -1.0f, 1.0f) + 1.0f) * (0.5f * STRATO_LUT_BINS);
    i = (int)x;
    i = i > STRATO_LUT_BINS - 1 ? STRATO_LUT_BINS - 1 : i;
    f = x - (float)i;
}

SOS_HD float strato_lut_at(const Optics& o, int i, float f, int w) {
    if (o.strato_lut2) {
        const float2 p = o.strato_lut2[(size_t)i * o.W + w];
        return p.x + f * p.y;
    }
    const float a = o.strato_lut[(size_t)i * o.W + w], b = o.strato_lut[(size_t)(i + 1) * o.W + w];
    return a + f * (b - a);
}

// Tabulated tropospheric phase (TROPO_MIE), linear in u between the table's nodes (numpy_reference.tropo_phase,
// numpy_reference.py:409-420; kernel.cu tropo_phase): position of u, value at a position, value at u.
SOS_HD void tropo_lut_pos(const Optics& o, float u, int& i, float& f) {
    const float x = (clampf(u, -1.0f, 1.0f) + 1.0f) * (0.5f * (float)o.tropo_bins);
    i = (int)x;
    i = i > o.tropo_bins - 1 ? o.tropo_bins - 1 : i;
    f = x - (float)i;
}

SOS_HD float tropo_lut_at(const Optics& o, int i, float f, int w) {
    if (o.tropo_lut2) {
        const float2 p = o.tropo_lut2[(size_t)i * o.W + w];
        return p.x + f * p.y;
    }
    const float a = o.tropo_lut[(size_t)i * o.W + w], b = o.tropo_lut[(size_t)(i + 1) * o.W + w];
    return a + f * (b - a);
}

SOS_HD float tropo_phase_at(const Optics& o, float u, int w) {
    int i;
    float f;
    tropo_lut_pos(o, u, i, f);
    return tropo_lut_at(o, i, f, w);
}

// strato_lut_pos for u already in [-1, 1].
SOS_HD void strato_lut_pos_clamped(float u, int& i, float& f) {
    const float x = (u + 1.0f) * (0.5f * STRATO_LUT_BINS);
    i = (int)x;
    i = i > STRATO_LUT_BINS - 1 ? STRATO_LUT_BINS - 1 : i;
    f = x - (float)i;
}

// Light from the lit ground scattered at the node, wavelengths w0 .. w0 + nw - 1 (nw <= NW): for every ground
// direction of every corner cell, the aerosol (Henyey-Greenstein) and stratospheric (table) phase of the pair of
// cosines (m0 + m1, m0 - m1) weighted by the corner weight and the direction's ground value
// (numpy_reference.py:548-566). Corner pairs (ir, j), (ir, j+1) whose cells share their ground directions evaluate
// the phases once for both cells.
template <int NW>
SOS_HD void ground_sums(const Optics& o, const Node& n, int w0, int nw, float ground[NW], float sground[NW]) {
    const int W = o.W;
    const HgPair hk = hg_pair_constants(o.g);
    const float aeyd = fabsf(n.eyd);
    for (int w = 0; w < NW; ++w) ground[w] = sground[w] = 0.0f;
    for (int pr = 0; pr < 2; ++pr) {
        const int ca = n.cell[2 * pr], cb = n.cell[2 * pr + 1];
        const float wa = n.sw[2 * pr], wb = n.sw[2 * pr + 1];
        const bool merged = o.gsame != nullptr && o.gsame[ca] != 0;
        for (int side = 0; side < (merged ? 1 : 2); ++side) {
            const int cell = side ? cb : ca;
            const float wc = side ? wb : wa;
            const int g0 = o.goff[cell], g1 = o.goff[cell + 1];
            const int shift = merged ? o.goff[cb] - g0 : 0;
            for (int gi = g0; gi < g1; ++gi) {
                const float* gd = o.gdir + 3 * gi;
                const float m0 = n.mu * gd[2] + n.exd * gd[0];
                const float m1 = aeyd * gd[1];
                const float up = clampf(m0 + m1, -1.0f, 1.0f), dn = clampf(m0 - m1, -1.0f, 1.0f);
                const float ph = o.tropo_bins ? 0.0f : hg_pair(hk, up, dn);
                int iu = 0, id = 0, tu = 0, td = 0;
                float fu = 0.0f, fd = 0.0f, gu = 0.0f, gd_ = 0.0f;
                if (o.strato) {
                    strato_lut_pos(up, iu, fu);
                    strato_lut_pos(dn, id, fd);
                }
                if (o.tropo_bins) {
                    tropo_lut_pos(o, up, tu, gu);
                    tropo_lut_pos(o, dn, td, gd_);
                }
                for (int k = 0; k < NW; ++k) {
                    if (k >= nw) break;
                    const int w = w0 + k;
                    float gv = wc * o.gval[(size_t)gi * W + w];
                    if (merged) gv += wb * o.gval[(size_t)(gi + shift) * W + w];
                    const float phw =
                        o.tropo_bins ? (tropo_lut_at(o, tu, gu, w) + tropo_lut_at(o, td, gd_, w)) * 0.5f : ph;
                    ground[k] += phw * gv;
                    if (o.strato) {
                        const float sph = (strato_lut_at(o, iu, fu, w) + strato_lut_at(o, id, fd, w)) * 0.5f;
                        sground[k] += sph * gv;
                    }
                }
            }
        }
    }
}

// First-light value of one node for wavelength w: single scattering of the attenuated sun (Rayleigh tensor,
// aerosol and stratospheric phase), light from the lit ground through the cell ground directions (ground, sground:
// ground_sums for w), and the direct ground Rayleigh moments of the four corners (numpy_reference.py:515-568,573-622
// with first=True).
SOS_HD void first_light_value(const Optics& o, const RayConst& rc, const Node& n, int w, float phase, float sphase,
                              float ground, float sground, float val[4]) {
    const int W = o.W;
    const float mix = o.mix;
    float col[5], stc, lit;
    sun_columns(o, n, col, stc, lit);
    float optical = 0.0f;
    for (int k = 0; k < 5; ++k) optical += col[k] * o.ext[k * W + w];
    if (o.strato) optical += stc * o.strato_ext[w];
    const float sun = expf(-optical) * lit;
    const float ph = o.tropo_bins ? tropo_phase_at(o, rc.d32[2], w) : phase;  // TROPO_MIE: the table, per wavelength
    const float beam = (n.prof.v[1] * o.asca[w]) * (sun * ph + ground);
    const float ray_ = (sun * n.prof.v[0]) * o.ext[w];
    const float sbeam = o.strato ? (n.st_prof * o.strato_sca[w]) * (sun * sphase + sground) : 0.0f;
    for (int k = 0; k < 4; ++k) {
        val[k] = ray_ * (mix * C_3_8PI * rc.direct[k] + (1.0f - mix) * C_1_8PI * rc.pu[k]) + beam * rc.pu[k] / 2.0f;
        if (o.strato) val[k] += (sbeam * rc.pu[k]) / 2.0f;
    }
    for (int c = 0; c < 4; ++c) {
        const float* gm = o.gm + (size_t)n.cell[c] * 4 * W + w;
        const float rm[4] = {gm[0], gm[W], gm[2 * W], gm[3 * W]};
        const float trace = (rm[0] + rm[1]) + rm[2];
        const float dens = n.prof.v[0];
        for (int k = 0; k < 4; ++k) {
            float rot = 0.0f;
            for (int u = 0; u < 4; ++u) rot += n.T[k][u] * rm[u];
            val[k] += n.sw[c] * (dens * (mix * rot + ((1.0f - mix) / 3.0f * trace) * rc.pu[k]));
        }
    }
}

SOS_HD void first_light_value(const Optics& o, const RayConst& rc, const Node& n, int w, float phase, float sphase,
                              float val[4]) {
    float ground[1], sground[1];
    ground_sums<1>(o, n, w, 1, ground, sground);
    first_light_value(o, rc, n, w, phase, sphase, ground[0], sground[0], val);
}

// Warm (multiple-scattering) value of one node for wavelength w from the current source: Rayleigh tensor of each
// corner rotated into the ray frame plus its aerosol SH source aero[c], bilinear in the corners, rescaled so that the
// trace follows the log-space (geometric) blend of the corner traces (numpy_reference.py:89-103,573-628).
SOS_HD void warm_value(const Optics& o, const RayConst& rc, const Node& n, const float* field, int w,
                       const float aero[4], float val[4]) {
    const int W = o.W;
    const float mix = o.mix;
    float logs = 0.0f, wg = 0.0f, am = 0.0f;
    for (int k = 0; k < 4; ++k) val[k] = 0.0f;
    for (int c = 0; c < 4; ++c) {
        const int cell = n.cell[c];
        const float* f = field + (size_t)cell * o.src * W + w;
        const float rm[4] = {f[0], f[W], f[2 * W], f[3 * W]};
        const float trace = (rm[0] + rm[1]) + rm[2];
        // an extended top's supports by the node's height (numpy_reference.py:604-609)
        const float dens = (n.above & 2) ? 0.0f : o.hr[n.ir + (c >> 1)];
        const float ae = (n.above & 1) ? 0.0f : aero[c];
        float tens[4];
        for (int k = 0; k < 4; ++k) {
            float rot = 0.0f;
            for (int u = 0; u < 4; ++u) rot += n.T[k][u] * rm[u];
            tens[k] = dens * (mix * rot + ((1.0f - mix) / 3.0f * trace) * rc.pu[k]);
            tens[k] += (ae * rc.pu[k]) / 2.0f;
            val[k] += n.sw[c] * tens[k];
        }
        const float tr = (tens[0] + tens[1]) + tens[2];
        if (tr >= TRACE_MIN) {  // subnormal or NaN traces do not enter the log-space blend
            logs += n.sw[c] * logf(tr);
            wg += n.sw[c];
            am += n.sw[c] * tr;
        }
    }
    if (wg > 0.0f && am >= TRACE_MIN) {
        const float scale = expf(logs - wg * logf(am / wg));
        for (int k = 0; k < 4; ++k) val[k] *= scale;
    }
}

// SH synthesis of one cell's plane at the ray direction: sum_m cos(m phi) sum_l Y_lm(mu) plane[k(l,m)], with the
// same FP32 recurrences as sh_contract and azimuth_sum, without keeping the per-m sums.
SOS_HD float sh_synth(const Optics& o, float mu, float st, float cp, const float* plane_cell, int wstride) {
    const int L = o.L;
    cp = clampf(cp, -1.0f, 1.0f);
    float pmm = 0.28209479177387814f;
    float c0 = 1.0f, c1 = cp;
    float total = 0.0f;
    for (int m = 0; m <= L; ++m) {
        float cm;
        if (m == 0) {
            cm = 1.0f;
        } else if (m == 1) {
            cm = cp;
        } else {
            const float c2 = (2.0f * cp) * c1 - c0;
            c0 = c1;
            c1 = c2;
            cm = c2;
        }
        if (m) pmm = (pmm * o.sh_d[m]) * st;
        const float scale = m ? 1.41421356237309515f : 1.0f;
        float p0 = pmm;
        int k = m * (m + 1) / 2 + m;
        float acc = (scale * p0) * plane_cell[(size_t)k * wstride];
        if (m < L) {
            float p1 = (sqrtf(2.0f * m + 3.0f) * mu) * p0;
            k = (m + 1) * (m + 2) / 2 + m;
            acc += (scale * p1) * plane_cell[(size_t)k * wstride];
            for (int l = m + 2; l <= L; ++l) {
                k = l * (l + 1) / 2 + m;
                const float p2 = (o.sh_a[k] * mu) * p1 - o.sh_b[k] * p0;
                acc += (scale * p2) * plane_cell[(size_t)k * wstride];
                p0 = p1;
                p1 = p2;
            }
        }
        total += cm * acc;
    }
    return total;
}

// The ray's SH basis at azimuth 0, Y[k] = scale_m P_lm(mu) (k = l(l+1)/2 + m), written by the lanes of a warp
// (lane m computes column m by the upward recurrence, the same FP32 steps as sh_synth).
SOS_HD void sh_basis_column(const Optics& o, float mu, float st, int m, float* Y) {
    const int L = o.L;
    float pmm = 0.28209479177387814f;
    for (int q = 1; q <= m; ++q) pmm = (pmm * o.sh_d[q]) * st;
    const float scale = m ? 1.41421356237309515f : 1.0f;
    float p0 = pmm;
    Y[m * (m + 1) / 2 + m] = scale * p0;
    if (m < L) {
        float p1 = (sqrtf(2.0f * m + 3.0f) * mu) * p0;
        Y[(m + 1) * (m + 2) / 2 + m] = scale * p1;
        for (int l = m + 2; l <= L; ++l) {
            const int k = l * (l + 1) / 2 + m;
            const float p2 = (o.sh_a[k] * mu) * p1 - o.sh_b[k] * p0;
            Y[k] = scale * p2;
            p0 = p1;
            p1 = p2;
        }
    }
}

// sum_m cos(m phi) sum_l Y[k(l,m)] plane_c[k] for the four corner planes at once.
SOS_HD void sh_synth4(int L, const float* Y, float cp, const float* const pc[4], int wstride, float out[4]) {
    cp = clampf(cp, -1.0f, 1.0f);
    float c0 = 1.0f, c1 = cp;
    for (int c = 0; c < 4; ++c) out[c] = 0.0f;
    for (int m = 0; m <= L; ++m) {
        float cm;
        if (m == 0) {
            cm = 1.0f;
        } else if (m == 1) {
            cm = cp;
        } else {
            const float c2 = (2.0f * cp) * c1 - c0;
            c0 = c1;
            c1 = c2;
            cm = c2;
        }
        float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
        int k = m * (m + 1) / 2 + m;
        for (int l = m; l <= L; ++l) {
            const float y = Y[k];
            const size_t off = (size_t)k * wstride;
            s0 += y * pc[0][off];
            s1 += y * pc[1][off];
            s2 += y * pc[2][off];
            s3 += y * pc[3][off];
            k += l + 1;
        }
        out[0] += cm * s0;
        out[1] += cm * s1;
        out[2] += cm * s2;
        out[3] += cm * s3;
    }
}

// m of SH index k = l (l + 1) / 2 + m.
SOS_HD constexpr int sh_m_of(int k) {
    int l = 0;
    while ((l + 1) * (l + 2) / 2 <= k) ++l;
    return k - l * (l + 1) / 2;
}

#if defined(__CUDACC__)
// acc[m] += Y[k] plane[k] over k = 4 V .. 4 V + 3 (< K), V = 0 .. ceil(K / 4) - 1: 16-byte loads of the basis and of
// one plane row, per-m sums in registers (k ascending, so each m sums its l in ascending order, as sh_synth4 does).
template <int L, int V>
struct ShStep {
    static __device__ __forceinline__ void run(const float4* y4, const float4* p4, float* acc) {
        constexpr int K = (L + 1) * (L + 2) / 2;
        const float4 y = y4[V];
        const float4 p = p4[V];
        if constexpr (4 * V + 0 < K) acc[sh_m_of(4 * V + 0)] += y.x * p.x;
        if constexpr (4 * V + 1 < K) acc[sh_m_of(4 * V + 1)] += y.y * p.y;
        if constexpr (4 * V + 2 < K) acc[sh_m_of(4 * V + 2)] += y.z * p.z;
        if constexpr (4 * V + 3 < K) acc[sh_m_of(4 * V + 3)] += y.w * p.w;
        // keep at most 8 loads of each operand in flight (registers), not the whole row
        if constexpr (V % 8 == 7) asm volatile("" ::: "memory");
        if constexpr (V + 1 < (K + 3) / 4) ShStep<L, V + 1>::run(y4, p4, acc);
    }
};

// sh_synth4 for a compile-time order L with 16-byte aligned basis and plane rows (padded to a multiple of 4).
template <int L>
__device__ __forceinline__ void sh_synth4_fixed(const float* Y, float cp, const float* const pc[4], float out[4]) {
    cp = clampf(cp, -1.0f, 1.0f);
    const float4* y4 = reinterpret_cast<const float4*>(Y);
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
        float acc[L + 1];
#pragma unroll
        for (int m = 0; m <= L; ++m) acc[m] = 0.0f;
        ShStep<L, 0>::run(y4, reinterpret_cast<const float4*>(pc[c]), acc);
        float c0 = 1.0f, c1 = cp;
        float s = acc[0];
        s += cp * acc[1];
#pragma unroll
        for (int m = 2; m <= L; ++m) {
            const float c2 = (2.0f * cp) * c1 - c0;
            s += c2 * acc[m];
            c0 = c1;
            c1 = c2;
        }
        out[c] = s;
    }
}
#endif

#if defined(__CUDACC__)
// sh_contract_basis for a compile-time order L (lane = wavelength, plane row stride W): rows l are unrolled by
// template recursion and the m of a row by a compile-time loop, so the per-m sums stay in registers and the loads
// of a row are issued together (instead of one dependent load per step); each m sums its l in ascending order, as
// sh_contract_basis does.
template <int L, int l>
struct ShWaveRow {
    static __device__ __forceinline__ void run(const float* Y, const float* plane_cell, int wstride, float* acc) {
#pragma unroll
        for (int m = 0; m <= l; ++m) {
            const int k = l * (l + 1) / 2 + m;
            acc[m] += Y[k] * plane_cell[(size_t)k * wstride];
        }
        // (no ordering barrier: a memory clobber would keep acc in local memory)
        if constexpr (l < L) ShWaveRow<L, l + 1>::run(Y, plane_cell, wstride, acc);
    }
};

template <int L>
__device__ __forceinline__ void sh_contract_wave(const float* Y, const float* plane_cell, int wstride, float* acc) {
#pragma unroll
    for (int m = 0; m <= L; ++m) acc[m] = 0.0f;
    ShWaveRow<L, 0>::run(Y, plane_cell, wstride, acc);
}
#endif

// Per-m sums of one cell from a shared basis (the cached form of sh_synth4).
SOS_HD void sh_contract_basis(int L, const float* Y, const float* plane_cell, int wstride, float* cache, int cstride) {
    for (int m = 0; m <= L; ++m) {
        float s = 0.0f;
        int k = m * (m + 1) / 2 + m;
        for (int l = m; l <= L; ++l) {
            s += Y[k] * plane_cell[(size_t)k * wstride];
            k += l + 1;
        }
        cache[m * cstride] = s;
    }
}

SOS_HD void boundary_term(const Optics& o, const Rays& b, const RayConst& rc, const float* boundary, int ray, int w,
                          float total[4]) {
    if (!boundary || !b.hits[ray]) return;
    const int W = o.W;
    const int j = b.end_j[ray];
    const float ef = rc.end_f;
    float E = (1.0f - ef) * boundary[j * W + w];
    E += ef * boundary[(j + 1) * W + w];
    const float* ec = b.end_col + 6 * (size_t)ray;
    float optical = 0.0f;
    for (int k = 0; k < 5; ++k) optical += ec[k] * o.ext[k * W + w];
    if (o.strato) optical += ec[5] * o.strato_ext[w];
    E *= expf(-optical);
    for (int k = 0; k < 4; ++k) total[k] += (E * rc.pu[k]) / 2.0f;
}

// Integrate one ray for wavelength w, node by node. `cache` holds 4 slots x (L+1) floats at stride `cstride`: the
// per-m SH sums of the cells at the current corners, recomputed only when a corner moves to another cell.
SOS_HD void transport_lane(const Optics& o, const Rays& b, const LaneInputs& in, int ray, int w, float* cache,
                           int cstride, float out[4]) {
    RayConst rc;
    ray_constants(b, ray, rc);
    const int W = o.W;
    const bool first = in.first != 0;
    float total[4] = {0, 0, 0, 0}, comp[4] = {0, 0, 0, 0};
    float tau = 0.0f, tauc = 0.0f;
    const float phase = hg_phase(rc.d32[2], o.g);
    const float sphase = (o.strato && first) ? legendre_phase(o, rc.d32[2], w) : 0.0f;
    int tag[4] = {-1, -1, -1, -1};  // cell held by each cache slot
    const int s0 = b.seg_off[ray], s1 = b.seg_off[ray + 1];
    for (int s = s0; s < s1; ++s) {
        const float4 sg = b.seg[s];
        const DS a = DS{sg.x, sg.y}, bb = DS{sg.z, sg.w};
        const bool lower = b.lower[s] != 0;
        DS t0 = a;
        float beta0 = beta_end(o, rc, t0, a, bb, w);
        float acc = 0.0f;
        for (int step = 0; step < in.nq; ++step) {
            Node n;
            sample_node(o, rc, a, bb, lower, DS{in.u_hi[step], in.u_lo[step]}, DS{in.wu_hi[step], in.wu_lo[step]},
                        n);
            const float beta1 = extinction(o, n.prof, n.st_prof, w);
            DS tm = ds_add(t0, n.t);
            tm = DS{tm.h * 0.5f, tm.l * 0.5f};
            const float wpan = ds_val(ds_sub(n.t, t0)) / 6.0f;
            acc = acc + wpan * ((beta0 + beta1) + 4.0f * beta_at(o, rc, tm, w));
            t0 = n.t;
            beta0 = beta1;
            const float att = n.ds * expf(-((tau - tauc) + acc));
            float val[4];
            if (first) {
                first_light_value(o, rc, n, w, phase, sphase, val);
            } else {
                // corner slots: reuse a slot whose cell is still a corner, recompute the others
                int slot_of[4];
                unsigned used = 0;
                for (int c = 0; c < 4; ++c) {
                    slot_of[c] = -1;
                    for (int q = 0; q < 4; ++q)
                        if (tag[q] == n.cell[c] && !(used & (1u << q))) {
                            slot_of[c] = q;
                            used |= 1u << q;
                            break;
                        }
                }
                for (int c = 0; c < 4; ++c) {
                    if (slot_of[c] >= 0) continue;
                    int q = 0;
                    while (used & (1u << q)) ++q;
                    used |= 1u << q;
                    slot_of[c] = q;
                    tag[q] = n.cell[c];
                    sh_contract(o, rc.d32[2], rc.st, in.plane + (size_t)n.cell[c] * o.K * W + w, W,
                                cache + (size_t)q * (o.L + 1) * cstride, cstride);
                }
                float aero[4];
                for (int c = 0; c < 4; ++c)
                    aero[c] = azimuth_sum(o.L, n.cp, cache + (size_t)slot_of[c] * (o.L + 1) * cstride, cstride);
                warm_value(o, rc, n, in.field, w, aero, val);
            }
            for (int k = 0; k < 4; ++k) kahan(total[k], comp[k], val[k] * att);
        }
        // closing panel to the segment end, then the segment's optical depth into tau (Kahan)
        DS tm = ds_add(t0, bb);
        tm = DS{tm.h * 0.5f, tm.l * 0.5f};
        const float wpan = ds_val(ds_sub(bb, t0)) / 6.0f;
        acc = acc + wpan * ((beta0 + beta_end(o, rc, bb, a, bb, w)) + 4.0f * beta_at(o, rc, tm, w));
        kahan(tau, tauc, acc);
    }
    boundary_term(o, b, rc, in.boundary, ray, w, total);
    for (int k = 0; k < 4; ++k) out[k] = total[k];
}

}  // namespace sos
