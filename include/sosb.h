/* C ABI of libsosb: the GB300 (sm_103a) successive-orders-of-scattering source iteration.
 *
 * The library is the drop-in for the transport/iteration boundary of cheek-walnut/sosfuse2: the `Kernel` object that
 * `create_configured` builds (src/sosfuse2/solve/source_solver.py:1109-1172) and the `Solver` that drives it
 * (src/sosfuse2/solve/source_iteration.py:100-663). Plain pointers and sizes only; no torch types.
 *
 * Conventions
 *   - Every entry point returns 0 on success, or a nonzero status whose message (prefixed with the reference's error
 *     code, e.g. "E_NONFINITE_SOURCE", "E_NOT_CONVERGED", "E_SHAPE") is read with sosb_last_error().
 *   - Host arrays passed to sosb_set_* are copied into device memory owned by the handle; the caller may free them
 *     after the call returns.
 *   - Pointers named *_dev are device pointers (e.g. torch tensors' data_ptr()) that the caller keeps alive for the
 *     duration of the call. All work is issued on the handle's stream (sosb_set_stream) and is complete when a call
 *     returns, unless stated otherwise.
 *   - One handle is used by one host thread at a time.
 *
 * Field layout (the reference's source layout, src/sosfuse2/backends/sh_layout.py:120-123):
 *   source[cell][slot][wave], cell = height_index * nc + chi_index, slot 0-3 Rayleigh coherency tensor
 *   (xx, yy, zz, xz), 4-9 Rayleigh SH coefficients, 10..10+K aerosol SH, then K stratospheric SH when enabled,
 *   K = (L+1)(L+2)/2, SH index k = l(l+1)/2 + m.
 */
#ifndef SOSB_H
#define SOSB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sosb_state *sosb_handle;

/* Sizes and scalar settings of one state (Kernel.setup constants, source_solver.py:1288-1312). */
typedef struct {
    int32_t L;            /* SH order, 2..48 */
    int32_t W;            /* wavelengths solved together, 1..64 */
    int32_t nh, nc;       /* height and solar-zenith grid sizes; cells = nh * nc */
    int32_t nq;           /* Gauss-Legendre nodes per segment, cell transport */
    int32_t nq_query;     /* nodes per segment, observer rays */
    int32_t strato;       /* stratospheric layer present: source has 10 + 2K slots */
    int32_t density_rows; /* rows of the density table (uniform profile grid) */
    int32_t density_mask; /* bit 0: tabulated air, bit 1: tabulated ozone */
    int32_t n_sun_h, n_sun_x; /* solar column table shape */
    int32_t monitors;     /* observer solar elevations used by the stop test (the first rows of the boxes) */
    int32_t n_monitor_rows; /* all observer solar elevations in the boxes (>= monitors) */
    int32_t n_dirs;       /* observer directions per elevation (7) */
    int32_t box_points;   /* Gauss-Legendre points per observer box (16) */
    double top_km, profile_step_km, mix, g, height, albedo, air_surface;
    double strato_center, strato_sigma, strato_norm;
    double lower_end_km;  /* extended top (above 80 km): support end of the components other than air, 0 for none */
    double air_end_km;    /* extended top: support end of the air (numpy_reference.py:158-183) */
} sosb_dims;

/* Host arrays of the per-state constants. Arrays of an absent layer may be NULL. */
typedef struct {
    const double *u, *wu;       /* [nq] nodes and weights on [0, 1] */
    const double *uq, *wuq;     /* [nq_query] */
    const float *h, *chi;       /* [nh] km, [nc] rad */
    const float *hr, *ha;       /* [nh] air and aerosol density shapes at the cell heights */
    const float *ext;           /* [5][W] extinction per unit profile: air, aerosol, O3, NO2, O4 */
    const float *asca;          /* [W] aerosol scattering */
    const float *density_table; /* [density_rows][3] air, ozone, NO2 */
    const float *sun_h;         /* [n_sun_h] */
    const float *sun_col;       /* [n_sun_h][n_sun_x][5] */
    const float *gm;            /* [nh*nc][4][W] first-light Rayleigh moments from the lit ground */
    const int64_t *goff;        /* [nh*nc + 1] ground directions of each cell */
    const float *gdir;          /* [goff[last]][3] */
    const float *gval;          /* [goff[last]][W] */
    const float *rf;            /* [6] Rayleigh SH factors */
    const float *af;            /* [K] aerosol phase eigenvalues (g^l) */
    const float *ext0;          /* [W] air extinction used by the composition */
    const double *solar;        /* [W] solar spectrum for the observer boxes */
    const double *box_ww;       /* [box_points] box quadrature weights */
    const float *strato_ext, *strato_sca; /* [W] */
    const float *strato_chi;    /* [33][W] Legendre moments of the stratospheric phase */
    const float *strato_density;/* [nh] stratospheric source density of each height */
    const float *strato_sun_col;/* [n_sun_h][n_sun_x] */
    const float *strato_eigen;  /* [K][W] */
    const float *strato_sca_source; /* [W] */
    const float *aer2;          /* [7] two-layer tropospheric aerosol profile (the AEROSOL_2L kernel vector of
                                 * atmosphere/tropo_profile.py:203-225: [bl_top - w/2, 1/w, a_bl, k_bl, a_ft, k_ft,
                                 * bl_top]), or NULL for the exponential profile exp(-h / height) */
    int32_t tropo_bins;         /* tabulated tropospheric phase (TROPO_MIE, atmosphere/tropo_mie.py:141-177): bins */
    const float *tropo_lut;     /* [tropo_bins + 1][W] phase per sr at u = -1 + 2 i / tropo_bins, linear in u; or NULL
                                 * for the Henyey-Greenstein phase of g */
    const float *tropo_eigen;   /* [K][W] its SH eigenvalues chi_l / (2l + 1), replacing af in the composition; or
                                 * NULL */
} sosb_constants;

/* Host arrays of one ray bundle (ray_geometry.Bundle, src/sosfuse2/solve/ray_geometry.py:290-392): destination
 * cells, their incoming rays and each ray's segments (only segments with b - a > 1e-8 are integrated). */
typedef struct {
    int32_t ncell;
    int64_t nray, nseg;
    const int64_t *cell_off;    /* [ncell+1] */
    const double *p;            /* [ncell][3] start point (km, Earth-centred, sun along +z) */
    const double *target;       /* [ncell][3][3] local frame */
    const double *d;            /* [nray][3] direction */
    const double *dloc;         /* [nray][3] direction in the local frame */
    const double *weight;       /* [nray] solid-angle weight */
    const int64_t *seg_off;     /* [nray+1] */
    const double *seg_a, *seg_b;/* [nseg] path coordinates of the segment ends */
    const uint8_t *seg_lower;   /* [nseg] 1 when the segment's lower end is at a */
    const int32_t *end_j;       /* [nray] solar-zenith interval of the ground end */
    const double *end_f;        /* [nray] fraction within it */
    const float *end_col;       /* [nray][5] component columns to the ground end */
    const float *end_st;        /* [nray] stratospheric column to the ground end (may be NULL) */
    const uint8_t *hits;        /* [nray] ray ends on the ground */
} sosb_bundle;

typedef struct {
    int32_t evaluations;
    int32_t converged;          /* 1 when every wavelength met the tolerance */
    double seconds;
    double observer_relative[64]; /* last evaluation, per wavelength */
    double source_relative[64];
    int32_t done[64];
    int64_t kernel_launches;    /* kernels this library launched during the call */
    int32_t start_fallback;     /* sosb_solve_warm: 1 when the supplied start was replaced by the fallback start */
} sosb_stats;

enum { SOSB_CELLS = 0, SOSB_OBSERVER = 1 };

/* Replaces: source_solver.Kernel.__init__ (source_solver.py:1110-1172) for backend 'b200'. */
int sosb_create(const sosb_dims *dims, sosb_handle *out);
int sosb_destroy(sosb_handle h);
/* Work stream (a cudaStream_t); 0 selects the handle's own stream. */
int sosb_set_stream(sosb_handle h, void *stream);
/* No reference counterpart. Node tables (default on): the first transport launch over a whole bundle after its rays
 * or the optics change stores each node's frame angles, corner fractions and attenuation (32 + 4 W bytes a node,
 * only within half the free device memory), and later warm launches read them instead of recomputing the
 * double-single geometry and the optical-depth prefix. 0 turns them off (every launch recomputes). */
int sosb_set_node_tables(sosb_handle h, int enable);
/* Projection form (no reference counterpart; the reference projects in compensated FP32 on CUDA cores):
 * 0 FP32 CUDA cores (compensated sums, the default), 1 bf16x3 tensor cores (split BF16 operands, three products,
 * FP32 accumulation), 2 TF32 tensor cores, 3 BF16 tensor cores. Forms 1-3 contract the SH rows per cell with
 * tcgen05.mma against a basis table built once per cell bundle; the Rayleigh rows and the ground flux stay FP32.
 * E_PROJECTION for an unknown form; E_TC_TIMEOUT when a tensor-core wait ran out. */
int sosb_set_projection(sosb_handle h, int mode);
/* No reference counterpart. Solve graphs (default on): a solve runs its first evaluation directly (it builds the node
 * tables and pair lists and tunes the launch shapes), then launches one CUDA graph whose WHILE node replays one
 * evaluation (Anderson mix, observer boxes, apply, residual feature and Gram column, and a control kernel that takes
 * the stop decision, the Gram solve and the next ring slot on the device) until the control kernel stops it: no host
 * round trip per evaluation. The graph is rebuilt when constants, bundles, modes or loop buffers change. Timing
 * (sosb_set_timing) or 0 here: the evaluations are launched one at a time, with the stop flag read after each. */
int sosb_set_graphs(sosb_handle h, int enable);
/* No reference counterpart. Autotuning (default on): the first table launch of each launch shape times 1, 2 and 4
 * warps per ray (two runs each, CUDA events) and keeps the fastest for the process; off (or during a graph capture of
 * an untuned shape): 4 warps from 96 nodes per ray, 2 from 48, else 1. Summation order follows the choice, so runs
 * with autotuning may differ from runs without it by rounding. */
int sosb_set_autotune(sosb_handle h, int enable);
/* No reference counterpart (its sos_vprod stage, kernel.cu:4568, contracts the same pairs). Pair contractions
 * (default on, more than four wavelengths): with the node tables, the distinct (ray, corner cell) pairs of each bundle
 * are listed once, every evaluation contracts each pair's plane row with the ray's basis once (per m and wavelength),
 * and the nodes add their azimuth series over the pair sums instead of each lane caching its corners. 0: off. */
int sosb_set_pairs(sosb_handle h, int enable);
/* No reference counterpart (its sos_vprod stage, kernel.cu:4568, computes the same corner sums on CUDA cores). Corner
 * values on the tensor cores (default on, more than four wavelengths; takes precedence over the pair form): with the
 * node tables, every node's four (node, corner cell) entries are bucketed by corner cell once per geometry; once per
 * plane, tiles of 128 entries of one cell form [128 x K] x [K x W] products of the nodes' basis rows
 * (Y_k(ray) cos(m phi_node)) with the cell's SH plane on tcgen05 (BF16 high and low parts, three products, FP32
 * accumulation in tensor memory), and the node pass reads each node's four corner values. 0: off (pair form).
 * E_TC_TIMEOUT when a tensor-core wait ran out. */
int sosb_set_corner_mma(sosb_handle h, int enable);
/* No reference counterpart (the first light's ground sums, numpy_reference.py:526-558, on CUDA cores there). Ground
 * sums on the tensor cores (default on, more than four wavelengths, Henyey-Greenstein tropospheric phase): the items
 * (node, corner pair) bucketed by the pair's first cell form, per tile of 128 items, [128 x directions] x [directions
 * x W] products of the pair phases times the corner weights with the ground values (BF16 high and low parts, three
 * products, FP32 accumulation in tensor memory); the stratospheric phase enters through the leading factors of its
 * table over the wavelengths (rank chosen at sosb_set_constants so that every table row is within 2e-6 of its
 * largest value; a table that needs more than 8 factors, or a tabulated tropospheric phase, keeps the CUDA-core
 * kernel). 0: off (CUDA cores). E_TC_TIMEOUT when a tensor-core wait ran out. */
int sosb_set_ground_mma(sosb_handle h, int enable);
/* No reference counterpart; host only (no GPU). The factorisation sosb_set_constants applies to the stratospheric
 * phase table for the tensor-core ground sums: lut [n][W] ~= U [n][r] V [r][W], V's rows the leading eigenvectors of
 * lut^T lut (cyclic Jacobi, FP64), U = lut V^T, r the smallest rank <= rmax with every row within tol of its largest
 * magnitude. Writes U (n * rmax doubles at most) and V (rmax * W) and returns r in *rank (0: none within tol). */
int sosb_phase_factors(const double *lut, int n, int W, int rmax, double tol, double *U, double *V, int *rank);
/* Replaces: Kernel.setup (source_solver.py:1243-1339) and constants_device (source_solver.py:2248). */
int sosb_set_constants(sosb_handle h, const sosb_constants *c);
/* Replaces: ray_geometry.upload_geometry / device_geometry (ray_geometry.py:205-287) of the cell bundle
 * (which = SOSB_CELLS) or of the observer rays of engine_core.Solver.boxes (which = SOSB_OBSERVER). */
int sosb_set_bundle(sosb_handle h, int which, const sosb_bundle *b);

/* Replaces: Kernel.launch (source_solver.py:2428-2456).
 *   phase 0: transport of every cell's rays (first light when first != 0, else warm with the optional ground
 *            boundary_dev [nc][W]) projected to moments_dev [cells][4+K][W] and flux_dev [cells][W];
 *   phase 1: ground pass over the nc surface cells: flux_dev [nc][W] only;
 *   phase 2: observer rays: radiance_dev [rays][W][4] (SOSB_OBSERVER bundle).
 * field_dev [cells][slots][W] is ignored for first light. Unused outputs may be NULL. */
int sosb_evaluate(sosb_handle h, int phase, int first, const float *field_dev, const float *boundary_dev,
                  float *moments_dev, float *flux_dev, float *radiance_dev);
/* Replaces: Solver.apply (source_iteration.py:161-216): ground pass, warm pass with the boundary, first-light moments
 * added, composition into the next source out_dev [cells][slots][W] (first call also runs first light). */
int sosb_apply(sosb_handle h, const float *field_dev, float *out_dev);
/* Allocation-free composition (no counterpart in the reference): the composition step of Solver.apply with the
 * reference's source metrics, for callers that must not allocate device memory once a state is set up - for example
 * a host loop that runs inside a service whose device memory is fully reserved by another allocator, or a pipeline
 * that cannot afford the device-wide synchronisation a cudaMalloc may cause. moments_dev [cells][4+K][W] (warm pass)
 * plus first_moments_dev (first light) are composed into out_dev [cells][slots][W]; wavelengths whose bit is set in
 * done_mask keep x_dev's values. Per wavelength it returns the count of non-finite composed values and
 * max|g - x| / max|g|. It calls no cudaMalloc, cudaFree or allocating library routine: its reduction scratch is a
 * file-scope device array of 3 x 64 words (W <= 64; larger W is rejected with E_SHAPE). Every call looks that array's
 * address up (cudaGetSymbolAddress) with the calling device current, so a device reset leaves no stale address; the
 * first call on a device may load the library's device code, so make it before any stream capture. Every call shares
 * the array and clears it first: calls that overlap on the GPU race. */
int sosb_compose_static(sosb_handle h, const float *moments_dev, const float *first_moments_dev, const float *x_dev,
                        uint64_t done_mask, float *out_dev, int64_t *nonfinite_host, double *source_relative_host);
/* Replaces: Solver.boxes (source_iteration.py:218-222): observer values [n_monitor_rows][n_dirs][W] to host. */
int sosb_boxes(sosb_handle h, const float *field_dev, double *out_host);
/* Replaces: Solver.solve (source_iteration.py:309-663): first light, then the fixed-point iteration from x0 (NULL:
 * zero) with Anderson depth 4 per wavelength. x_out is a host array [cells][slots][W] (x_out_is_device = 0) or a device pointer.
 * Returns nonzero with E_NOT_CONVERGED or E_NONFINITE_SOURCE like the reference. */
int sosb_solve(sosb_handle h, int max_eval, double tolerance, const float *x0_host, float *x_out,
               int x_out_is_device, sosb_stats *stats);
/* Replaces: the `history` list in the stats of Solver.solve (source_iteration.py:381-391): the per-evaluation
 * observer_relative and source_relative of the last solve on this handle (sosb_solve, sosb_solve_warm or a batch
 * member), row e = evaluation e + 1, [count][W] each. *count receives the evaluations recorded; at most `capacity`
 * rows are copied. */
int sosb_history(sosb_handle h, int capacity, int32_t *count, double *observer_relative, double *source_relative);
/* Kernel timing with CUDA events on the work stream (no counterpart in the reference's ABI; its Kernel.timed_launch,
 * source_solver.py:1478-1523, keeps a per-kind launch log). Classes: 0 transport with its geometry (first light,
 * node-table builds), 1 projection, 2 SH plane, 3 composition, 4 observer boxes, 5 Anderson, 6 other, 7 transport
 * from node tables. sosb_set_timing(h, 1) starts and clears the totals;
 * sosb_get_timing fills ms[k] and launches[k] for k < n. */
int sosb_set_timing(sosb_handle h, int on);
int sosb_get_timing(sosb_handle h, double *ms, int64_t *launches, int n);
/* Profile shapes of a synthetic atmosphere (sosfuse2_gb300.synth.Atmosphere) for sosb_column_table: air exp(-h/8),
 * aerosol exp(-h/aerosol_height), ozone exp(1 - z - exp(-z)) * ozone_norm with z = (h - ozone_peak) / 5, NO2
 * exp(-((h - no2_center) / 4)^2 / 2), O4 air^2, the first five on h clipped to [0, top]; the stratospheric layer
 * exp(-((h - strato_center) / strato_sigma)^2 / 2) / strato_norm when strato is nonzero. */
typedef struct {
    double top, aerosol_height, ozone_peak, ozone_norm, no2_center;
    int32_t strato;
    double strato_center, strato_sigma, strato_norm;
} sosb_profile_shape;
/* Solar column table of a synthetic state family (host, no device work; the project's counterpart of the reference's
 * sun geometry, src/sosfuse2/solve/engine_core.py:103-147): for every height h[i] and abscissa x[j] the six slant
 * columns (five profile shapes and the stratospheric one) along the upward ray of zenith cosine
 * mu = mg + (1 - mg) x^2 (mu = mg + 1e-9 at x = 0) into up[i][j][6] and along the downward ray
 * mu = max(mg - (1 + mg) x^2, -1) (mg - 1e-9 at x = 0) into down[i][j][6], mg the horizon cosine at that height; each
 * path cut at the shadow cylinder, the tangent point and the shells (at most 8) and integrated by the n_gl-point rule
 * (gl_u, gl_w on [0, 1]). threads: host threads (0: all cores). */
int sosb_column_table(int n_h, const double *h, int n_x, const double *x, const double *shells, int n_shells,
                      const double *gl_u, const double *gl_w, int n_gl, const sosb_profile_shape *shape, double *up,
                      double *down, int threads);
/* sosb_column_table on the device: one thread per (table, height, x), the same column function. h[n_h], x[n_x],
 * gl_u/gl_w[n_gl], up/down [n_h][n_x][6] are device pointers, shells[n_shells] host values; synchronises `stream`.
 * Returns 3 on a CUDA error. */
int sosb_column_table_device(int n_h, const double *h, int n_x, const double *x, const double *shells, int n_shells,
                             const double *gl_u, const double *gl_w, int n_gl, const sosb_profile_shape *shape,
                             double *up, double *down, void *stream);
/* A solar column table (sosb_column_table's output with its grids) for lookups: heights h[n_h] (ascending, to
 * top), abscissae x uniform on [0, 1] (n_x values), up/down [n_h][n_x][6]. */
typedef struct {
    int32_t n_h, n_x;
    double top;
    const double *h, *up, *down;
} sosb_column_grid;
/* Segments of n rays (the geometry CSR of a synthetic bundle, the project's counterpart of the reference's
 * ray_geometry.pack, src/sosfuse2/solve/ray_geometry.py:28-82; host threads): per ray from p[r][3] along d[r][3], the
 * 5 + 2 n_shells sorted cuts (edges[r][...], synth.ray_edges), for each consecutive pair whether it is a segment
 * (b - a > 1e-8) and whether its start is the lower end, the end's solar-zenith interval j and fraction, whether the
 * ray ends on the ground and, with a column table, the slant columns from the ray's start back to the ground along the
 * ray (end_col[r][5], end_st[r]; zero for rays that do not hit the ground). table may be NULL (no ground columns). */
int sosb_ray_segments(int64_t n, const double *p, const double *d, double top, const double *shells, int n_shells,
                      int n_chi, const double *chi, const sosb_column_grid *table, double *edges, uint8_t *valid,
                      uint8_t *lower, int32_t *end_j, double *end_f, float *end_col, float *end_st, uint8_t *hits,
                      int threads);
/* sosb_ray_segments on the device (the geometry CSR of ray_geometry.pack built by the GPU, one thread per ray): the
 * same arguments and outputs, every array a device pointer (`table`, when not NULL, is a host struct whose h, up and
 * down point to device arrays); asynchronous work on `stream` (a cudaStream_t, 0 the default stream), complete when
 * the call returns. FP64 arithmetic: the cuts equal the host function's to rounding (the device may contract
 * multiply-adds), so a segment whose length is within rounding of the 1e-8 threshold can differ. */
int sosb_ray_segments_device(int64_t n, const double *p, const double *d, double top, const double *shells,
                             int n_shells, int n_chi, const double *chi, const sosb_column_grid *table, double *edges,
                             uint8_t *valid, uint8_t *lower, int32_t *end_j, double *end_f, float *end_col,
                             float *end_st, uint8_t *hits, void *stream);
/* Incoming-direction quadratures of n_cells cells (host threads; the project's restatement of the reference's ring
 * rule, src/sosfuse2/rays/incoming_rings.py): cell c at radius r[c] and solar zenith chi[c], nphi + 1 azimuth
 * planes, in each a sinh-mapped (a) Gauss-Legendre rule (u, wu on [0, 1], nmu nodes) between the cuts at the
 * horizon, the shadow boundary, the forward direction and, with rings, the shadow rings of the n_heights shells.
 * counts[c] receives each cell's direction count; with loc (and w) not NULL the directions (local ex, ey, up) and
 * weights of all cells follow one another in cell order (capacity: directions loc and w can hold; 2 when short). */
int sosb_ring_quadrature(int n_cells, const double *r, const double *chi, int nmu, int nphi, const double *heights,
                         int n_heights, int rings, double a, const double *u, const double *wu, int64_t *counts,
                         double *loc, double *w, int64_t capacity, int threads);
/* Ground-illumination rays of every cell, the geometry of engine_core.Solver.prepare_ground
 * (src/sosfuse2/solve/engine_core.py:103-147) for the handle's grid: ray r belongs to cell[r] (ascending), arrives
 * from the local direction loc[r][3] with quadrature weight weight[r]; cols[r][6] are its slant columns (five
 * components and the stratospheric one) from the cell to the ground and on to the sun; cos_sun[r] = max(0, cosine
 * of the solar zenith at its ground point); ok[r] = 1 when that point is lit and the ray reaches the ground. */
typedef struct {
    int64_t n;
    const int32_t *cell;
    const double *loc, *weight, *cols, *cos_sun;
    const uint8_t *ok;
} sosb_ground_rays;
int sosb_set_ground_rays(sosb_handle h, const sosb_ground_rays *rays);
/* Solver.prepare_ground on the device (engine_core.py:103-147) for a state's optics over the rays of
 * sosb_set_ground_rays, replacing the ground arrays of sosb_set_constants (gm, goff, gdir, gval): per ray and
 * wavelength value = albedo / pi * cos_sun * exp(-(cols[0:5] . ext[:, w] + cols[5] strato_ext[w])) * ok * weight
 * in FP64; the rays with a positive value kept per cell in ray order; gm[cell][k][w] = sum over the cell's rays of
 * factor_k(loc) * value times 2 C ext[0][w] (C = 3 / (16 pi)). ext: [5][W] FP64 extinction, strato_ext: [W] FP64
 * (NULL without the stratospheric layer). */
int sosb_prepare_ground(sosb_handle h, double albedo, const double *ext, const double *strato_ext);
/* Warm-started Solver.solve (no counterpart in the reference; the learned start): iterate from the device field
 * x0_dev, reusing the first-light moments of the preceding sosb_apply on this handle. If the first evaluation's
 * largest source relative change max|g - x|/max|g| exceeds fallback_ss, the iteration restarts from fallback_dev
 * (e.g. the single-scattering source apply(0)); stats->start_fallback records it. */
int sosb_solve_warm(sosb_handle h, int max_eval, double tolerance, const float *x0_dev, double fallback_ss,
                    const float *fallback_dev, float *x_out, int x_out_is_device, sosb_stats *stats);
/* No reference counterpart. Warm history (default off): sosb_solve_warm (and its batch form) first enters the pair
 * (x = 0, g = fallback_dev) into the Anderson history - the single-scattering source apply(0) is the plain
 * iteration's first evaluation - with its observer boxes, residual feature and Gram entries (no evaluation counted),
 * so that the supplied start is the second iterate and the first warm evaluation already mixes with that direction
 * instead of restarting the history. */
int sosb_set_warm_history(sosb_handle h, int enable);
/* Batched form of Solver.solve (no single counterpart in the reference, whose pipeline runs one state per process,
 * src/sosfuse2/jobs/pipeline_execution.py): n independent states, each its own handle and stream, driven by one host
 * thread with up to `threads` solves in flight (0: all); each state's first evaluation and then its solve graph
 * (sosb_set_graphs) are enqueued on its stream, so that the states' evaluations overlap on the GPU with no host round
 * trip; a finished solve hands its place to the next state. status[i] is state i's sosb_solve result (its message
 * in sosb_last_error(hs[i])); returns nonzero when any state failed. */
int sosb_solve_batch(sosb_handle *hs, int n, int max_eval, double tolerance, const float *const *x0_host,
                     float *const *x_out, int x_out_is_device, sosb_stats *stats, int *status, int threads);
/* Tensor-core BF16 GEMM (tcgen05, TMA, TMEM; no counterpart in the reference, used by the learned warm start):
 * C[M x N] = A[M x K] * B[N x K]^T with A, B row-major BF16 device matrices (16-byte aligned), FP32 accumulation.
 * M and N multiples of 128, K of 64. epilogue 0: c_f32 = C; 1: c_f32 = C + bias[n] and c_bf16 = gelu(C + bias[n]);
 * 2: c_f32 = C + bias[n]. Asynchronous on `stream`; sosb_tc_check(stream) synchronises and reports a GEMM whose
 * pipeline wait ran out (E_TC_TIMEOUT). Messages of these calls: sosb_tc_last_error(). */
int sosb_gemm_bf16(const void *A, const void *B, int M, int N, int K, const float *bias, int epilogue, float *c_f32,
                   void *c_bf16, void *stream);
int sosb_tc_check(void *stream);
const char *sosb_tc_last_error(void);
/* Elementwise kernels of the warm-start MLP's training step (asynchronous on `stream`): GELU backward
 * (dz = dh * gelu'(z), BF16 and FP32 copies), transpose to BF16 (rows x cols -> cols x rows), column sums (bias
 * gradients), Adam on FP32 master weights with a BF16 copy, the mean squared error gradient with per-block partial
 * sums of squares, and FP32 -> BF16 conversion. */
int sosb_mlp_gelu_backward(const float *dh, const float *z, long long n, void *dz_bf16, float *dz_f32, void *stream);
int sosb_mlp_transpose(const void *in, int in_is_f32, int rows, int cols, void *out_bf16, void *stream);
int sosb_mlp_column_sum(const float *g, int rows, int cols, float *out, void *stream);
int sosb_mlp_adam(float *w, const float *g, float *m, float *v, long long n, float lr, float b1, float b2, float eps,
                  int step, float decay, void *w_bf16, void *stream);
int sosb_mlp_mse(const float *p, const float *y, long long n, float scale, float *d, float *partial, int blocks,
                 void *stream);
int sosb_mlp_to_bf16(const float *in, long long n, void *out, void *stream);
/* Batched forms of sosb_apply (n handles on `threads` host threads, 0: one per handle) and of sosb_solve_warm (the
 * one-thread graph driver of sosb_solve_batch, `threads` solves in flight) (no counterpart in the reference);
 * status[i] is handle i's result. */
int sosb_apply_batch(sosb_handle *hs, int n, const float *const *fields_dev, float *const *outs_dev, int *status,
                     int threads);
int sosb_solve_warm_batch(sosb_handle *hs, int n, int max_eval, double tolerance, const float *const *x0_dev,
                          double fallback_ss, const float *const *fallback_dev, float *const *x_out,
                          int x_out_is_device, sosb_stats *stats, int *status, int threads);
/* Message of the last failed call on this handle (empty when none). */
const char *sosb_last_error(sosb_handle h);
/* Sizes the handle was created with: cells, slots per cell, K. */
int sosb_shape(sosb_handle h, int64_t *cells, int32_t *slots, int32_t *K);
/* Library build identification: "sosb <version> sm_103a". */
const char *sosb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SOSB_H */
