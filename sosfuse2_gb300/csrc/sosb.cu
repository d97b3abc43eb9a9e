// libsosb: GB300 (sm_103a) kernels and C ABI of the successive-orders-of-scattering source iteration.
//
// Kernels (one evaluation = ground pass, warm pass, composition; plus two observer passes and Anderson mixing):
//   transport_kernel  one thread per (ray, wavelength): the ray's line-of-sight integral (sos_math.cuh)
//   plane_kernel      aerosol (+ stratospheric) SH plane of every cell, scaled by the cell's source density
//   project_kernel    one block per cell: weighted ray radiance onto 4 Rayleigh + K SH moments and ground flux
//   compose_kernel    moments -> next source (Solver.apply composition) fused with the convergence metrics
//   boxes_kernel      observer rays -> Gauss-Legendre box values
//   norm/feature/dot/mix kernels  Anderson depth-4 residual features, Gram columns (FP64) and the mixing
// The fixed-point loop (sosb_solve) runs on the host thread over device-resident buffers; per evaluation it reads
// back only per-wavelength scalars (metrics, box values, Gram columns).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>
#include <atomic>
#include <string>
#include <vector>

#include "sos_math.cuh"
#include "sos_pack.h"
#include "../../include/sosb.h"
#include "tc_ptx.cuh"

using namespace sos;

#define SOSB_VERSION "sosb 0.1 sm_103a"

// ------------------------------------------------------------------------------------------------ device buffers
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

// A device buffer owned by one host function: freed on every return, the error paths included.
struct LocalBuf : DevBuf {
    LocalBuf() = default;
    LocalBuf(const LocalBuf&) = delete;
    LocalBuf& operator=(const LocalBuf&) = delete;
    ~LocalBuf() {
        if (p) cudaFree(p);
    }
};

struct BundleDev {
    int ncell = 0;
    int64_t nray = 0, nseg = 0;
    DevBuf cell_off, ray_cell, p, frame, dir, dir_lo, dloc, pcp, seg_off, seg, lower, end_j, end_col, hits;
    std::vector<int64_t> host_cell_off, host_seg_off;
    int64_t host_seg_off_at(int64_t ray) const { return host_seg_off.empty() ? 0 : host_seg_off[(size_t)ray]; }
    // node table (NodeTable): valid once a launch over the whole bundle wrote it; too_big: over the memory budget
    DevBuf t_frame, t_misc, t_att;
    bool t_valid = false, t_too_big = false;
    // basis table of the tensor-core projection (BasisTable), built for projection mode b_mode (-1: none)
    DevBuf b_hi, b_lo;
    int b_mode = -1, b_kpad = 0, b_rpad = 0;
    // ray-cell pairs (PairTable): valid with the node table unless they exceed the memory budget; host copies of the
    // pair offsets at the ground-pass end and at the end
    DevBuf p_off, p_cell, p_ray, p_node, y_tab;
    DevBuf pair_A;  // the per-m contractions of the pairs
    bool p_valid = false;
    int64_t p_ground = 0, p_total = 0;
    int64_t a_version = -1;  // plane version pair_A was contracted from
    // (node, corner) entries bucketed by corner cell for the tensor-core corner values (CornerEntries), valid with
    // the node table unless over the memory budget; cv the corner values of plane version c_version
    DevBuf c_ray, c_cp, c_slot, c_tile, cv, node_ray, vbuf;
    bool c_valid = false;
    int c_ntiles = 0;
    int64_t c_version = -1;
};

// kernel classes timed by sosb_set_timing / sosb_get_timing
enum { K_TRANSPORT = 0, K_PROJECT, K_PLANE, K_COMPOSE, K_BOXES, K_ANDERSON, K_OTHER, K_TABLE, K_CORNER, K_CLASSES };

struct TimedLaunch {
    int cls;
    cudaEvent_t a, b;
};

struct EvalCtrl;
struct LoopDev;

struct sosb_state {
    sosb_dims d{};
    bool timing = false;
    std::vector<TimedLaunch> timed;
    std::vector<cudaEvent_t> event_pool;
    double timed_ms[K_CLASSES] = {0};
    int64_t timed_count[K_CLASSES] = {0};
    int K = 0, src = 0, ns = 0;
    cudaStream_t own = nullptr, stream = nullptr;
    std::string err;
    bool have_constants = false;
    // constants
    DevBuf h, chi, hr, ha, ext, asca, table, sun_h, sun_col, gm, goff, gdir, gval, rf, af, ext0;
    DevBuf t_lut, t_lut2;  // tabulated tropospheric phase and its (value, step) pairs
    DevBuf plane_tiles;    // the corner products' B tiles of the current plane (plane_tiles_kernel)
    const float* plane_field = nullptr;  // the field the current plane was built from
    bool plane_keep = false;  // one-shot: the next run_plane of plane_field keeps the current plane
    DevBuf s_ext, s_sca, s_chi, s_density, s_sun_col, s_eigen, s_sca_src, s_lut, s_lut2, gsame, gdir4;
    DevBuf sh_a, sh_b, sh_d;
    DevBuf u_hi, u_lo, wu_hi, wu_lo, uq_hi, uq_lo, wuq_hi, wuq_lo, box_ww, solar;
    BundleDev cells, obs;
    // work
    DevBuf rad, plane, moments, flux, first_moments, first_flux, boundary, metrics, boxes;
    DevBuf fx, fg, norms, partials, dots;
    DevBuf ring_g[4], ring_f[4];
    DevBuf fl_val0, fl_coef, fl_dir, fl_g, fl_cnt, fl_off, fl_cursor, fl_entries;  // staged first light
    // ground-illumination rays of every cell (sosb_set_ground_rays) and the scratch of sosb_prepare_ground
    DevBuf gr_off, gr_loc, gr_w, gr_cols, gr_cos, gr_ok, gr_value, gr_cnt, gr_cursor;
    int64_t gr_n = 0;
    int64_t plane_version = 0;  // incremented by every plane rebuild (the pair contractions follow it)
    bool have_first = false;
    bool tables = true;  // build and use node tables (sosb_set_node_tables)
    // fixed-point loop: evaluation control and report (device and pinned host copies), replayed evaluation graph
    // and loop state on the device (the control kernel's), the observer boxes of x and g, the residual's observer
    // features, the Gram matrices, the history and the norm maxima
    DevBuf ctrl_dev, loop_dev, box_old, box_new, obs_feat, gram, hist_dev, normmax;
    EvalCtrl* ctrl_host = nullptr;
    LoopDev* loop_host = nullptr;
    int feat_blocks = 0, feat_threads = 0;
    cudaGraphExec_t graph = nullptr;  // the solve graph: gate kernel, then a WHILE node over one evaluation
    cudaGraphConditionalHandle cond = 0;
    int64_t graph_launches = 0;       // kernels in one evaluation of the solve graph
    bool graphs = true;  // replay evaluations from a captured CUDA graph (sosb_set_graphs)
    bool autotune = true;  // time the table launch shapes once per shape (sosb_set_autotune)
    bool pairs = true;     // corner SH by ray-cell pair contractions (sosb_set_pairs)
    bool corner_mma = true;  // corner SH values on the tensor cores, more than four wavelengths (sosb_set_corner_mma)
    bool ground_mma = true;  // first-light ground sums on the tensor cores, more than four wavelengths
    int g_rank = 0;          // factors of the stratospheric phase table (strato_factors); 0: none within tolerance
    DevBuf g_su2, g_sv;      // their (value, step) table [STRATO_LUT_BINS][rank] and wavelength factors [rank][W]
    DevBuf gt_cnt, gt_off, gt_cursor, gt_tile;  // tiles of the ground-sum buckets
    bool corner_used = false;  // a corner GEMM ran since the last check of its bounded waits
    bool warm_history = false;  // sosb_solve_warm seeds the Anderson history with (0, fallback) (sosb_set_warm_history)
    int aer2_on = 0;     // two-layer tropospheric aerosol profile (sosb_constants.aer2)
    float aer2[7] = {};
    int tropo_bins = 0;  // tabulated tropospheric phase (sosb_constants.tropo_lut), 0 for Henyey-Greenstein
    int af_w = 0;        // af holds per-wavelength eigenvalues [K][W] (sosb_constants.tropo_eigen)
    int proj_mode = 0;   // projection form (sosb_set_projection): PROJ_FP32, PROJ_BF16X3, PROJ_TF32, PROJ_BF16
    int64_t launches = 0;
    // per-evaluation history of the last solve on this handle: [evaluation][W] observer and source relative changes
    std::vector<double> hist_obs, hist_src;
};

static int fail(sosb_state* s, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (s) s->err = buf;
    return 1;
}

#define CK(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            return fail(s, "E_CUDA: %s (%s:%d)", cudaGetErrorString(e_), __FILE__, __LINE__);          \
    } while (0)

#define TRY(call)          \
    do {                   \
        int r_ = (call);   \
        if (r_) return r_; \
    } while (0)

static int dfree(sosb_state* s, DevBuf& b) {
    if (b.p) CK(cudaFree(b.p));
    b.p = nullptr;
    b.bytes = 0;
    return 0;
}

static int dalloc(sosb_state* s, DevBuf& b, size_t bytes) {
    if (b.p && b.bytes >= bytes) return 0;
    TRY(dfree(s, b));
    if (bytes == 0) return 0;
    CK(cudaMalloc(&b.p, bytes));
    b.bytes = bytes;
    return 0;
}

static int dput(sosb_state* s, DevBuf& b, const void* host, size_t bytes) {
    TRY(dalloc(s, b, bytes));
    if (bytes) CK(cudaMemcpyAsync(b.p, host, bytes, cudaMemcpyHostToDevice, s->stream));
    return 0;
}

template <class T>
static int dput_vec(sosb_state* s, DevBuf& b, const std::vector<T>& v) {
    return dput(s, b, v.data(), v.size() * sizeof(T));
}

template <class T>
static T* P(const DevBuf& b) {
    return static_cast<T*>(b.p);
}

// Block size for element loops over [..][W] arrays: a multiple of W (at most 256), so that every thread of a
// grid-stride loop keeps one wavelength.
static int wave_threads(int W) { return W * std::max(1, 256 / std::max(W, 1)); }

static int grid_for(long long n, int threads) {
    long long g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > 152LL * 64) g = 152LL * 64;  // grid-stride loops beyond 64 blocks per SM
    return (int)g;
}

// ------------------------------------------------------------------------------------------------ kernels
constexpr int TRANSPORT_THREADS = 128;

// Per-node geometry and attenuation of one ray bundle (node id = segment * nq + step), written by the first launch
// over the whole bundle after the bundle or the optics change and read by every later warm launch, which then skips
// the double-single geometry, the profile lookups and the Simpson prefix. Null pointers: nothing is written.
struct NodeTable {
    float4* frame;  // [nodes] cos, sin of the interpolated cell angle; cos, sin of the node's longitude
    float4* misc;   // [nodes] height fraction, solar-zenith fraction, azimuth cosine, bits of (ir << 16 | j)
    float* att;     // [nodes][W] quadrature weight x attenuation from the ray's origin
};

// misc.w packs ir (bits 16-29), j (bits 0-15) and the node's support bits (30: above the lower components' end, 31:
// above the air's)
__device__ __forceinline__ float4 table_misc(const Node& n) {
    return make_float4(n.ah, n.ac, n.cp, __int_as_float((n.ir << 16) | n.j | (n.above << 30)));
}

__device__ __forceinline__ int misc_ir(int pk) { return (pk >> 16) & 0x3fff; }

// Node of a table entry: frame rotation, corners and azimuth cosine (what warm_value and the SH synthesis read).
__device__ __forceinline__ void table_node(const Optics& o, const RayConst& rc, const NodeTable& tab, long long id,
                                           Node& n) {
    const float4 fr = tab.frame[id];
    const float4 ms = tab.misc[id];
    node_frame(rc, fr.x, fr.y, fr.z, fr.w, n);
    const int pk = __float_as_int(ms.w);
    node_corners(o, misc_ir(pk), pk & 0xffff, ms.x, ms.y, n);
    n.cp = ms.z;
    n.above = (int)((unsigned)pk >> 30);
}

// First light of a cell bundle in stages (few wavelengths): a preparation launch stores per node the first-light
// value without its ground-scattered part (val0), the factors that scale the ground sums into it (coef: aerosol
// density x scattering, stratospheric profile x scattering) and the ray direction in the node's frame (dir); the
// ground sums G (aerosol, stratospheric) of each corner pair are then computed over node pairs bucketed by corner
// cell, and a last launch sums val0 + coef x G over each ray.
struct FirstLightBufs {
    float4* val0;  // [nodes][W]
    float2* coef;  // [nodes][W]
    float4* dir;   // [nodes] (mu, exd, |eyd|, 0)
    float2* g;     // [nodes][2 pairs][W] (ground, stratospheric ground)
};

constexpr unsigned FULL_MASK = 0xffffffffu;

// basis rows of the warps of a block, each padded to kp = K rounded up to 4
static size_t warp_smem(int K) { return sizeof(float) * (size_t)((K + 3) & ~3) * (TRANSPORT_THREADS / 32); }


// Sample-parallel transport for few wavelengths (W <= WM): one warp per ray, lane i takes the ray's node i (batches
// of 32 nodes, segment-major). Each lane evaluates its node's geometry and its Simpson panel [previous node, node]
// (plus the segment's closing panel on its last node); a warp prefix sum of the panel integrals gives every node's
// optical depth; each lane forms its node's value with the corner SH synthesised directly; a warp reduction sums the
// ray. Numerically this is transport_lane with the sums regrouped (panel and ray sums in tree order).
template <int WM, bool PREP>
__global__ void __launch_bounds__(TRANSPORT_THREADS)
    transport_warp_kernel(Optics o, Rays b, LaneInputs in, NodeTable tab, FirstLightBufs fl, int ray0, int nray,
                          float4* rad) {
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= nray) return;  // the whole warp leaves together
    const int ray = ray0 + (int)warp;
    const int W = o.W;
    RayConst rc;
    ray_constants(b, ray, rc);
    const bool first = in.first != 0;
    const int nq = in.nq;
    const int s0 = b.seg_off[ray], s1 = b.seg_off[ray + 1];
    const int nsamp = (s1 - s0) * nq;
    const float phase = hg_phase(rc.d32[2], o.g);
    extern __shared__ float warp_sm[];
    float* Y = warp_sm + (threadIdx.x >> 5) * in.kp;  // this ray's SH basis, shared by the warp
    if (!first) {
        for (int m = lane; m <= o.L; m += 32) sh_basis_column(o, rc.d32[2], rc.st, m, Y);
        __syncwarp();
    }
    float sphase[WM], tot[WM][4], cmp[WM][4], carry[WM], carry_beta[WM];
#pragma unroll
    for (int w = 0; w < WM; ++w) {
        sphase[w] = (o.strato && first && w < W) ? legendre_phase(o, rc.d32[2], w) : 0.0f;
        carry[w] = carry_beta[w] = 0.0f;
        for (int k = 0; k < 4; ++k) tot[w][k] = cmp[w][k] = 0.0f;
    }
    DS carry_t = DS{0.0f, 0.0f};
    for (int base = 0; base < nsamp; base += 32) {
        const int i = base + lane;
        const bool act = i < nsamp;
        Node n;
        n.t = DS{0.0f, 0.0f};
        float bnode[WM], e[WM], close[WM];
#pragma unroll
        for (int w = 0; w < WM; ++w) bnode[w] = e[w] = close[w] = 0.0f;
        int step = 0;
        DS a{0.0f, 0.0f}, bb{0.0f, 0.0f};
        if (act) {
            const int sl = i / nq;
            step = i - sl * nq;
            const float4 sg = b.seg[s0 + sl];
            a = DS{sg.x, sg.y};
            bb = DS{sg.z, sg.w};
            sample_node(o, rc, a, bb, b.lower[s0 + sl] != 0, DS{in.u_hi[step], in.u_lo[step]},
                        DS{in.wu_hi[step], in.wu_lo[step]}, n);
#pragma unroll
            for (int w = 0; w < WM; ++w)
                if (w < W) bnode[w] = extinction(o, n.prof, n.st_prof, w);
        }
        const float pth = __shfl_up_sync(FULL_MASK, n.t.h, 1), ptl = __shfl_up_sync(FULL_MASK, n.t.l, 1);
        float pbeta[WM];
#pragma unroll
        for (int w = 0; w < WM; ++w) pbeta[w] = __shfl_up_sync(FULL_MASK, bnode[w], 1);
        if (act) {
            DS t0;
            float beta0[WM];
            if (step == 0) {
                t0 = a;
                DS q[3], q2[3], r;
                path_point(rc, a, q, q2, r);
                const float h = segment_end_height(o, rc, path_height(o, r), a, bb);
                const Profile pa = profile_at(o, h);
                const float sa = o.strato ? strato_profile(o, h) : 0.0f;
#pragma unroll
                for (int w = 0; w < WM; ++w) beta0[w] = w < W ? extinction(o, pa, sa, w) : 0.0f;
            } else if (lane == 0) {
                t0 = carry_t;
#pragma unroll
                for (int w = 0; w < WM; ++w) beta0[w] = carry_beta[w];
            } else {
                t0 = DS{pth, ptl};
#pragma unroll
                for (int w = 0; w < WM; ++w) beta0[w] = pbeta[w];
            }
            {
                const DS tm = ds_half(ds_add(t0, n.t));
                DS q[3], q2[3], r;
                path_point(rc, tm, q, q2, r);
                const float h = path_height(o, r);
                const Profile pm = profile_at(o, h);
                const float sm = o.strato ? strato_profile(o, h) : 0.0f;
                const float wpan = ds_val(ds_sub(n.t, t0)) / 6.0f;
#pragma unroll
                for (int w = 0; w < WM; ++w)
                    if (w < W) e[w] = wpan * ((beta0[w] + bnode[w]) + 4.0f * extinction(o, pm, sm, w));
            }
            if (step == nq - 1) {
                DS q[3], q2[3], r;
                path_point(rc, bb, q, q2, r);
                float h = segment_end_height(o, rc, path_height(o, r), a, bb);
                const Profile pb = profile_at(o, h);
                const float sb = o.strato ? strato_profile(o, h) : 0.0f;
                const DS tm = ds_half(ds_add(n.t, bb));
                path_point(rc, tm, q, q2, r);
                h = path_height(o, r);
                const Profile pm = profile_at(o, h);
                const float sm = o.strato ? strato_profile(o, h) : 0.0f;
                const float wpan = ds_val(ds_sub(bb, n.t)) / 6.0f;
#pragma unroll
                for (int w = 0; w < WM; ++w)
                    if (w < W) {
                        close[w] = wpan * ((bnode[w] + extinction(o, pb, sb, w)) + 4.0f * extinction(o, pm, sm, w));
                        e[w] += close[w];
                    }
            }
        }
        float S[WM];
#pragma unroll
        for (int w = 0; w < WM; ++w) {
            float v = e[w];
#pragma unroll
            for (int dd = 1; dd < 32; dd <<= 1) {
                const float u = __shfl_up_sync(FULL_MASK, v, dd);
                if (lane >= dd) v += u;
            }
            S[w] = v;
        }
        if (act) {
            const long long id = (long long)s0 * nq + i;
            if (tab.frame) {
                tab.frame[id] = make_float4(n.fr[0], n.fr[1], n.fr[2], n.fr[3]);
                tab.misc[id] = table_misc(n);
            }
            if (PREP) fl.dir[id] = make_float4(n.mu, n.exd, fabsf(n.eyd), 0.0f);
            float ground[WM], sground[WM];
            if (first && !PREP) ground_sums<WM>(o, n, 0, W, ground, sground);
#pragma unroll
            for (int w = 0; w < WM; ++w) {
                if (w >= W) continue;
                const float att = n.ds * expf(-((carry[w] + S[w]) - close[w]));
                if (tab.att) tab.att[id * W + w] = att;
                float val[4];
                if (PREP) {
                    first_light_value(o, rc, n, w, phase, sphase[w], 0.0f, 0.0f, val);
                    fl.val0[id * W + w] = make_float4(val[0], val[1], val[2], val[3]);
                    fl.coef[id * W + w] = make_float2(n.prof.v[1] * o.asca[w],
                                                      o.strato ? n.st_prof * o.strato_sca[w] : 0.0f);
                    continue;
                }
                if (first) {
                    first_light_value(o, rc, n, w, phase, sphase[w], ground[w], sground[w], val);
                } else {
                    float aero[4];
                    const float* pc[4];
                    for (int c = 0; c < 4; ++c) pc[c] = in.plane + ((size_t)n.cell[c] * W + w) * in.kp;
                    sh_synth4(o.L, Y, n.cp, pc, 1, aero);
                    warm_value(o, rc, n, in.field, w, aero, val);
                }
                for (int k = 0; k < 4; ++k) kahan(tot[w][k], cmp[w][k], val[k] * att);
            }
        }
#pragma unroll
        for (int w = 0; w < WM; ++w) {
            carry[w] += __shfl_sync(FULL_MASK, S[w], 31);
            carry_beta[w] = __shfl_sync(FULL_MASK, bnode[w], 31);
        }
        carry_t = DS{__shfl_sync(FULL_MASK, n.t.h, 31), __shfl_sync(FULL_MASK, n.t.l, 31)};
    }
    if constexpr (!PREP) {
#pragma unroll
        for (int w = 0; w < WM; ++w) {
            float v[4];
            for (int k = 0; k < 4; ++k) {
                v[k] = tot[w][k] - cmp[w][k];
#pragma unroll
                for (int dd = 16; dd >= 1; dd >>= 1) v[k] += __shfl_xor_sync(FULL_MASK, v[k], dd);
            }
            if (lane == 0 && w < W) {
                boundary_term(o, b, rc, in.boundary, ray, w, v);
                rad[(size_t)ray * W + w] = make_float4(v[0], v[1], v[2], v[3]);
            }
        }
    }
}

// Node record shared by the lanes of one warp: everything the per-wavelength part of a node needs.
constexpr int REC_WORDS = 73;  // odd stride: the 32 lanes write their records without bank conflicts
struct NodeRec {
    float r_h, r_l, qz_h, qz_l, h, ds, cp, mu, exd, eyd, st_prof;
    float sw[4];
    int cell[4];
    int ir, flags;  // bit 0: first node of its segment, bit 1: last node of its segment
    float T[16];
    float prof[5];
    float pa[6];   // profiles (+ stratospheric) at the segment start (first node only)
    float pm[6];   // at the panel midpoint
    float pb[6];   // at the segment end (last node only)
    float pmc[6];  // at the closing panel's midpoint (last node only)
    float wpan, wpc;
};
static_assert(sizeof(NodeRec) <= REC_WORDS * 4, "node record exceeds its stride");

SOS_HD float ext6(const Optics& o, const float* p6, int w) {
    float b = 0.0f;
    for (int k = 0; k < 5; ++k) b += p6[k] * o.ext[k * o.W + w];
    if (o.strato) b += p6[5] * o.strato_ext[w];
    return b;
}

// Profiles at path coordinate t; at an end of segment [a, b] (end = true) with the support snap of an extended top.
SOS_HD void profile6(const Optics& o, const RayConst& rc, DS t, float* p6, bool end = false, DS a = DS{0.0f, 0.0f},
                     DS b = DS{0.0f, 0.0f}) {
    DS q[3], q2[3], r;
    path_point(rc, t, q, q2, r);
    const float h = end ? segment_end_height(o, rc, path_height(o, r), a, b) : path_height(o, r);
    const Profile p = profile_at(o, h);
    for (int k = 0; k < 5; ++k) p6[k] = p.v[k];
    p6[5] = o.strato ? strato_profile(o, h) : 0.0f;
}

// Transport for many wavelengths: one warp per (ray, chunk of 32 wavelengths). Phase A: lane j evaluates node
// base+j's geometry and the profiles its Simpson panels need, into a shared-memory record. Phase B: lane = wavelength
// walks the 32 records in order, exactly as transport_lane does (same per-wavelength operation order), with its own
// 4-slot corner SH cache in shared memory.
constexpr int WAVE_WARPS = 2;

template <bool PREP>
__global__ void __launch_bounds__(WAVE_WARPS * 32)
    transport_wave_kernel(Optics o, Rays b, LaneInputs in, NodeTable tab, FirstLightBufs fl, int ray0, int nray,
                          int wchunks, float4* rad) {
    extern __shared__ float wave_sm[];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const long long warp = (long long)blockIdx.x * WAVE_WARPS + wid;
    if (warp >= (long long)nray * wchunks) return;  // the whole warp leaves together
    const int ray = ray0 + (int)(warp / wchunks);
    const int w = (int)(warp % wchunks) * 32 + lane;
    const bool wok = w < o.W;
    const int wl = wok ? w : o.W - 1;  // idle lanes compute a valid wavelength and store nothing
    const int L1 = o.L + 1;
    float* recs = wave_sm + (size_t)wid * (32 * REC_WORDS + 4 * L1 * 32 + o.K);
    float* cache = recs + 32 * REC_WORDS + lane;  // [slot*(L+1) + m] * 32 + lane
    float* Y = recs + 32 * REC_WORDS + 4 * L1 * 32;  // this ray's SH basis, shared by the warp
    RayConst rc;
    ray_constants(b, ray, rc);
    const bool values = !in.table_only;
    if (in.first == 0 && values) {
        for (int m = lane; m <= o.L; m += 32) sh_basis_column(o, rc.d32[2], rc.st, m, Y);
        __syncwarp();
    }
    const bool first = in.first != 0;
    const int nq = in.nq;
    const int s0 = b.seg_off[ray], s1 = b.seg_off[ray + 1];
    const int nsamp = (s1 - s0) * nq;
    const float phase = hg_phase(rc.d32[2], o.g);
    const float sphase = (o.strato && first) ? legendre_phase(o, rc.d32[2], wl) : 0.0f;
    float total[4] = {0, 0, 0, 0}, comp[4] = {0, 0, 0, 0};
    float tau = 0.0f, tauc = 0.0f, acc = 0.0f, beta0 = 0.0f;
    int tag[4] = {-1, -1, -1, -1};
    DS carry_t = DS{0.0f, 0.0f};
    for (int base = 0; base < nsamp; base += 32) {
        const int i = base + lane;
        const int cnt = min(32, nsamp - base);
        DS tnode = DS{0.0f, 0.0f};
        __syncwarp();
        if (i < nsamp) {
            NodeRec* R = reinterpret_cast<NodeRec*>(recs + lane * REC_WORDS);
            const int sl = i / nq;
            const int step = i - sl * nq;
            const float4 sg = b.seg[s0 + sl];
            const DS a = DS{sg.x, sg.y}, bb = DS{sg.z, sg.w};
            Node n;
            sample_node(o, rc, a, bb, b.lower[s0 + sl] != 0, DS{in.u_hi[step], in.u_lo[step]},
                        DS{in.wu_hi[step], in.wu_lo[step]}, n);
            tnode = n.t;
            if (tab.frame) {
                const long long id = (long long)s0 * nq + i;
                tab.frame[id] = make_float4(n.fr[0], n.fr[1], n.fr[2], n.fr[3]);
                tab.misc[id] = table_misc(n);
            }
            if (PREP) fl.dir[(long long)s0 * nq + i] = make_float4(n.mu, n.exd, fabsf(n.eyd), 0.0f);
            R->r_h = n.r.h; R->r_l = n.r.l; R->qz_h = n.qz.h; R->qz_l = n.qz.l; R->h = n.h; R->ds = n.ds;
            R->cp = n.cp; R->mu = n.mu; R->exd = n.exd; R->eyd = n.eyd; R->st_prof = n.st_prof;
            for (int c = 0; c < 4; ++c) { R->sw[c] = n.sw[c]; R->cell[c] = n.cell[c]; }
            R->ir = n.ir;
            R->flags = (step == 0 ? 1 : 0) | (step == nq - 1 ? 2 : 0);
            for (int k = 0; k < 4; ++k)
                for (int u = 0; u < 4; ++u) R->T[4 * k + u] = n.T[k][u];
            for (int k = 0; k < 5; ++k) R->prof[k] = n.prof.v[k];
            R->wpan = 0.0f;  // set below, once the previous node's coordinate is known
            if (step == 0) profile6(o, rc, a, R->pa, true, a, bb);
            if (step == nq - 1) {
                profile6(o, rc, bb, R->pb, true, a, bb);
                profile6(o, rc, ds_half(ds_add(n.t, bb)), R->pmc);
                R->wpc = ds_val(ds_sub(bb, n.t)) / 6.0f;
            }
        }
        const float pth = __shfl_up_sync(FULL_MASK, tnode.h, 1), ptl = __shfl_up_sync(FULL_MASK, tnode.l, 1);
        if (i < nsamp) {
            NodeRec* R = reinterpret_cast<NodeRec*>(recs + lane * REC_WORDS);
            const int sl = i / nq;
            const int step = i - sl * nq;
            DS t0;
            if (step == 0) {
                const float4 sg = b.seg[s0 + sl];
                t0 = DS{sg.x, sg.y};
            } else {
                t0 = lane == 0 ? carry_t : DS{pth, ptl};
            }
            profile6(o, rc, ds_half(ds_add(t0, tnode)), R->pm);
            R->wpan = ds_val(ds_sub(tnode, t0)) / 6.0f;
        }
        carry_t = DS{__shfl_sync(FULL_MASK, tnode.h, 31), __shfl_sync(FULL_MASK, tnode.l, 31)};
        __syncwarp();
        // phase B: this lane's wavelength over the records in order
        for (int j = 0; j < cnt; ++j) {
            const NodeRec* R = reinterpret_cast<const NodeRec*>(recs + j * REC_WORDS);
            const int flags = R->flags;
            if (flags & 1) {
                acc = 0.0f;
                beta0 = ext6(o, R->pa, wl);
            }
            float beta1 = 0.0f;
            for (int k = 0; k < 5; ++k) beta1 += R->prof[k] * o.ext[k * o.W + wl];
            if (o.strato) beta1 += R->st_prof * o.strato_ext[wl];
            acc = acc + R->wpan * ((beta0 + beta1) + 4.0f * ext6(o, R->pm, wl));
            beta0 = beta1;
            const float att = R->ds * expf(-((tau - tauc) + acc));
            if (tab.att && wok) tab.att[((long long)s0 * nq + base + j) * o.W + w] = att;
            if (!values) {  // table only: the optical-depth prefix and nothing else
                if (flags & 2) {
                    acc = acc + R->wpc * ((beta0 + ext6(o, R->pb, wl)) + 4.0f * ext6(o, R->pmc, wl));
                    kahan(tau, tauc, acc);
                }
                continue;
            }
            Node n;
            n.r = DS{R->r_h, R->r_l};
            n.qz = DS{R->qz_h, R->qz_l};
            n.h = R->h;
            n.ds = R->ds;
            n.cp = R->cp;
            n.mu = R->mu;
            n.exd = R->exd;
            n.eyd = R->eyd;
            n.st_prof = R->st_prof;
            for (int c = 0; c < 4; ++c) { n.sw[c] = R->sw[c]; n.cell[c] = R->cell[c]; }
            n.ir = R->ir;
            for (int k = 0; k < 4; ++k)
                for (int u = 0; u < 4; ++u) n.T[k][u] = R->T[4 * k + u];
            for (int k = 0; k < 5; ++k) n.prof.v[k] = R->prof[k];
            float val[4];
            if (PREP) {
                // staged first light: the value without its ground-scattered part, and the ground-sum factors
                first_light_value(o, rc, n, wl, phase, sphase, 0.0f, 0.0f, val);
                if (wok) {
                    const long long id = ((long long)s0 * nq + base + j) * o.W + w;
                    fl.val0[id] = make_float4(val[0], val[1], val[2], val[3]);
                    fl.coef[id] = make_float2(n.prof.v[1] * o.asca[w], o.strato ? n.st_prof * o.strato_sca[w] : 0.0f);
                }
            } else if (first) {
                first_light_value(o, rc, n, wl, phase, sphase, val);
            } else {
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
                    sh_contract_basis(o.L, Y, in.plane + (size_t)n.cell[c] * o.K * o.W + wl, o.W,
                                      cache + (size_t)q * L1 * 32, 32);
                }
                float aero[4];
                for (int c = 0; c < 4; ++c) aero[c] = azimuth_sum(o.L, n.cp, cache + (size_t)slot_of[c] * L1 * 32, 32);
                warm_value(o, rc, n, in.field, wl, aero, val);
            }
            for (int k = 0; k < 4; ++k) kahan(total[k], comp[k], val[k] * att);
            if (flags & 2) {
                acc = acc + R->wpc * ((beta0 + ext6(o, R->pb, wl)) + 4.0f * ext6(o, R->pmc, wl));
                kahan(tau, tauc, acc);
            }
        }
    }
    if (wok && !PREP && values) {
        boundary_term(o, b, rc, in.boundary, ray, w, total);
        rad[(size_t)ray * o.W + w] = make_float4(total[0], total[1], total[2], total[3]);
    }
}

static size_t wave_smem(int L) {
    return sizeof(float) * (size_t)WAVE_WARPS * (32 * REC_WORDS + 4 * (L + 1) * 32 + (L + 1) * (L + 2) / 2);
}

// ------------------------------------------------------------------ ray-cell pairs
// The corner SH contraction by (ray, corner cell) pair, the form of the reference's sos_vprod, for many wavelengths:
// for every distinct corner cell a ray's nodes touch, A[pair][m][w] = sum_l Y_lm(ray) plane[cell][k(l, m)][w], once
// per plane and bundle (pair_contract_wave_kernel; the ground and the warm pass of one evaluation share them), and
// each node then adds its azimuth series over A[pair(node, corner)][m][w] (transport_pair_wave_kernel). Pairs, the
// ray basis table and each node's four pair indices are geometry and are built with the node table. With one to four
// wavelengths the per-node synthesis of transport_table_kernel is faster: on config 0 the rays' nodes are spread
// over long shell segments, so a node shares few corner cells with the ray's earlier nodes (1.53 M pairs for 0.51 M
// nodes) and a contraction per pair costs more than the per-node one it replaces (measured with one thread per pair:
// 55 us per node pass instead of 100 us, plus 80 us per contraction).
constexpr int PAIR_WINDOW = 16;  // recent distinct corner cells a ray's new corners are matched against

struct PairTable {
    const int* off;     // [nray + 1] first pair of each ray
    const int* cell;    // [pairs] corner cell
    const int* ray;     // [pairs] ray
    const int4* node;   // [nodes] pair index of each corner
    const float* y;     // [nray][kp] the ray's SH basis Y_k(mu) at azimuth 0
    float* A;           // [pairs][L + 1][W] per-m contractions of the current plane
};

// One thread per ray: the corner cells of the ray's nodes in node and corner order, each new one a pair unless it
// is among the ray's last PAIR_WINDOW pairs (a ray passes its cells in sequence, so this finds nearly every repeat;
// a repeat it misses costs one extra pair, not a wrong value). Pass 0 counts them (cnt[ray]), pass 1 writes the
// pairs and each node's four pair indices.
__global__ void pair_build_kernel(Optics o, Rays b, NodeTable tab, int nq, int pass, int* cnt, const int* off,
                                  int* p_cell, int* p_ray, int4* p_node) {
    for (int ray = blockIdx.x * blockDim.x + threadIdx.x; ray < b.nray; ray += gridDim.x * blockDim.x) {
        const int s0 = b.seg_off[ray];
        const long long node0 = (long long)s0 * nq;
        const int nn = (b.seg_off[ray + 1] - s0) * nq;
        const int base = pass == 1 ? off[ray] : 0;
        int win_cell[PAIR_WINDOW], win_idx[PAIR_WINDOW];
        int nwin = 0, head = 0, n = 0;
        for (int i = 0; i < nn; ++i) {
            const float4 ms = tab.misc[node0 + i];
            const int pk = __float_as_int(ms.w);
            const int cell0 = misc_ir(pk) * o.nc + (pk & 0xffff);
            int idx[4];
            for (int c = 0; c < 4; ++c) {
                const int cell = cell0 + (c & 1) + (c >> 1) * o.nc;
                int f = -1;
                for (int u = 0; u < nwin; ++u)
                    if (win_cell[u] == cell) {
                        f = win_idx[u];
                        break;
                    }
                if (f < 0) {
                    f = n++;
                    win_cell[head] = cell;
                    win_idx[head] = f;
                    head = (head + 1) % PAIR_WINDOW;
                    nwin = min(nwin + 1, PAIR_WINDOW);
                    if (pass == 1) {
                        p_cell[base + f] = cell;
                        p_ray[base + f] = ray;
                    }
                }
                idx[c] = f;
            }
            if (pass == 1) p_node[node0 + i] = make_int4(base + idx[0], base + idx[1], base + idx[2], base + idx[3]);
        }
        if (pass == 0) cnt[ray] = n;
    }
}

// One warp per ray: its basis row into the table (lane m computes column m).
__global__ void pair_basis_kernel(Optics o, Rays b, int kp, float* y_tab) {
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= b.nray) return;
    const float4 d = b.dir[warp];
    for (int m = lane; m <= o.L; m += 32) sh_basis_column(o, d.z, d.w, m, y_tab + (size_t)warp * kp);
}

// Many wavelengths (plane [cell][K][W]): one warp per (pair, chunk of 32 wavelengths), lane = wavelength.
template <int LT>
__global__ void pair_contract_wave_kernel(Optics o, PairTable pt, const float* __restrict__ plane, int np, int kp,
                                          int wchunks) {
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= (long long)np * wchunks) return;
    const int p = (int)(warp / wchunks);
    const int w = (int)(warp % wchunks) * 32 + lane;
    if (w >= o.W) return;
    const int W = o.W, L1 = o.L + 1;
    const float* Y = pt.y + (size_t)pt.ray[p] * kp;
    const float* P = plane + (size_t)pt.cell[p] * o.K * W + w;
    float* out = pt.A + (size_t)p * L1 * W + w;
    if constexpr (LT > 0) {
        float acc[LT + 1];
        sh_contract_wave<LT>(Y, P, W, acc);
#pragma unroll
        for (int m = 0; m <= LT; ++m) out[(size_t)m * W] = acc[m];
    } else {
        sh_contract_basis(o.L, Y, P, W, out, W);
    }
}

// ------------------------------------------------------------------ staged first light (W <= 4)
// Corner pair pr of a node (cells (ir + pr, j) and (ir + pr, j + 1)): its first cell, the key of its bucket.
__device__ __forceinline__ int pair_cell(const Optics& o, float4 ms, int pr) {
    const int pk = __float_as_int(ms.w);
    return (misc_ir(pk) + pr) * o.nc + (pk & 0xffff);
}

// Ground directions a pair visits: the first cell's, plus the second cell's unless the two share them.
__device__ __forceinline__ int pair_work(const Optics& o, int ca) {
    int n = o.goff[ca + 1] - o.goff[ca];
    if (!(o.gsame != nullptr && o.gsame[ca])) n += o.goff[ca + 2] - o.goff[ca + 1];
    return n;
}

// Bucket sizes: cnt[cell] += pairs with work whose first cell is `cell` (one atomic per group of equal keys in a
// warp). With `cursor`, the second pass writes the pair codes (node * 2 + pr) into their buckets.
__global__ void pair_bucket_kernel(Optics o, const float4* __restrict__ misc, long long nodes, int* cnt, int* cursor,
                                   int* entries) {
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < nodes;
         base += stride) {
        const long long node = base + lane;
        const bool ok = node < nodes;
        const float4 ms = ok ? misc[node] : make_float4(0.f, 0.f, 0.f, 0.f);
        for (int pr = 0; pr < 2; ++pr) {
            int key = -1;
            if (ok) {
                const int ca = pair_cell(o, ms, pr);
                if (pair_work(o, ca) > 0) key = ca;
            }
            const unsigned peers = __match_any_sync(FULL_MASK, key);
            const int leader = __ffs(peers) - 1;
            if (key < 0) continue;
            if (!cursor) {
                if (lane == leader) atomicAdd(&cnt[key], __popc(peers));
            } else {
                int at = 0;
                if (lane == leader) at = atomicAdd(&cursor[key], __popc(peers));
                at = __shfl_sync(peers, at, leader);
                const int rank = __popc(peers & ((1u << lane) - 1u));
                entries[at + rank] = (int)(node * 2 + pr);
            }
        }
    }
}

// Exclusive prefix sum of the bucket sizes (one block): off[0..n], and the scatter cursors.
__global__ void bucket_scan_kernel(const int* __restrict__ cnt, int n, int* off, int* cursor) {
    __shared__ int part[1024];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = i < n ? cnt[i] : 0;
        part[threadIdx.x] = v;
        __syncthreads();
        for (int d = 1; d < 1024; d <<= 1) {
            const int u = threadIdx.x >= d ? part[threadIdx.x - d] : 0;
            __syncthreads();
            part[threadIdx.x] += u;
            __syncthreads();
        }
        if (i < n) {
            off[i] = carry + part[threadIdx.x] - v;
            cursor[i] = off[i];
        }
        __syncthreads();
        if (threadIdx.x == 1023) carry += part[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) off[n] = carry;
}

// ------------------------------------------------------------------ ground preparation on the device
// engine_core.Solver.prepare_ground (src/sosfuse2/solve/engine_core.py:103-147) for a state's optics over the
// ground-illumination rays of every cell: per ray r and wavelength w
//   value = albedo / pi * cos_sun * exp(-(cols[0:5] . ext[:, w] + cols[5] strato_ext[w])) * ok * weight   (FP64),
// the rays with a positive value in some wavelength kept per cell in ray order (goff, gdir, gval), and
// gm[cell][k][w] = (sum over the cell's rays, in ray order, of factor_k(loc) value) * 2 C ext[0][w],
// factor = ((1 - lx^2) / 2, (1 - ly^2) / 2, (1 - lz^2) / 2, -lx lz / 2), C = 3 / (16 pi).
struct GroundRays {
    const int* off;       // [cells + 1] first ray of each cell
    const double* loc;    // [n][3]
    const double* w;      // [n]
    const double* cols;   // [n][6]
    const double* cos;    // [n]
    const uint8_t* ok;    // [n]
    long long n;
};

// One thread per ray: its values for every wavelength and whether it is kept; cnt[cell] counts the kept rays.
__global__ void ground_value_kernel(GroundRays g, int ns, int W, double albedo, const double* __restrict__ ext,
                                    const double* __restrict__ strato_ext, double* __restrict__ value,
                                    int* __restrict__ cnt, const int* __restrict__ ray_cell) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.n) return;
    const double* c = g.cols + r * 6;
    bool take = false;
    for (int w = 0; w < W; ++w) {
        double od = c[0] * ext[w];
        for (int k = 1; k < 5; ++k) od += c[k] * ext[k * W + w];
        if (strato_ext) od += c[5] * strato_ext[w];
        const double v = (((albedo / M_PI) * g.cos[r]) * exp(-od)) * (double)g.ok[r] * g.w[r];
        value[r * W + w] = v;
        take |= v > 0.0;
    }
    if (take) atomicAdd(&cnt[ray_cell[r]], 1);
}

// One block per cell: warp j sums gm's (k, w) entries q = j, j + warps, ... over the cell's rays (lanes stride the
// rays, FP64, then a shuffle tree; the order differs from a sequential sum only far below the FP32 result's last
// bit), then warp 0 writes the kept rays' directions and values in ray order from goff[cell].
__global__ void __launch_bounds__(256)
    ground_cell_kernel(GroundRays g, int W, const double* __restrict__ ext0, const double* __restrict__ value,
                       const int* __restrict__ goff, float* __restrict__ gm, float* __restrict__ gdir,
                       float4* __restrict__ gdir4, float* __restrict__ gval) {
    const int cell = blockIdx.x;
    const int r0 = g.off[cell], r1 = g.off[cell + 1];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int q = wid; q < 4 * W; q += nw) {
        const int k = q / W, w = q % W;
        double acc = 0.0;
        for (int r = r0 + lane; r < r1; r += 32) {
            const double* l = g.loc + (size_t)r * 3;
            double f;
            if (k == 0) f = (1.0 - l[0] * l[0]) / 2.0;
            else if (k == 1) f = (1.0 - l[1] * l[1]) / 2.0;
            else if (k == 2) f = (1.0 - l[2] * l[2]) / 2.0;
            else f = (-l[0] * l[2]) / 2.0;
            acc += f * value[(size_t)r * W + w];
        }
#pragma unroll
        for (int dd = 16; dd >= 1; dd >>= 1) acc += __shfl_xor_sync(FULL_MASK, acc, dd);
        if (lane == 0) gm[((size_t)cell * 4 + k) * W + w] = (float)(acc * ((2.0 * (3.0 / (16.0 * M_PI))) * ext0[w]));
    }
    if (wid != 0) return;
    int pos = goff[cell];
    for (int base = r0; base < r1; base += 32) {
        const int r = base + lane;
        bool take = false;
        if (r < r1)
            for (int w = 0; w < W; ++w) take |= value[(size_t)r * W + w] > 0.0;
        const unsigned bal = __ballot_sync(FULL_MASK, take);
        if (take) {
            const int at = pos + __popc(bal & ((1u << lane) - 1u));
            const double* l = g.loc + (size_t)r * 3;
            const float x = (float)l[0], y = (float)l[1], z = (float)l[2];
            gdir[(size_t)at * 3] = x;
            gdir[(size_t)at * 3 + 1] = y;
            gdir[(size_t)at * 3 + 2] = z;
            gdir4[at] = make_float4(x, y, z, 0.0f);
            for (int w = 0; w < W; ++w) gval[(size_t)at * W + w] = (float)value[(size_t)r * W + w];
        }
        pos += __popc(bal);
    }
}

// gsame[cell]: the next solar-zenith cell of the same height keeps the same ground directions, bit for bit (one
// warp per cell comparing the two direction blocks).
__global__ void ground_same_kernel(const int* __restrict__ goff, const float* __restrict__ gdir, int ns, int nc,
                                   uint8_t* __restrict__ same) {
    const int lane = threadIdx.x & 31;
    const int cell = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (cell >= ns) return;  // the whole warp leaves together
    bool v = false;
    if (cell % nc != nc - 1) {
        const int n0 = goff[cell + 1] - goff[cell], n1 = goff[cell + 2] - goff[cell + 1];
        if (n0 > 0 && n0 == n1) {
            const unsigned* a = reinterpret_cast<const unsigned*>(gdir) + (size_t)goff[cell] * 3;
            const unsigned* b = reinterpret_cast<const unsigned*>(gdir) + (size_t)goff[cell + 1] * 3;
            bool differ = false;
            for (int i = lane; i < n0 * 3; i += 32) differ |= a[i] != b[i];
            v = !__any_sync(FULL_MASK, differ);
        }
    }
    if (lane == 0) same[cell] = v ? 1 : 0;
}

// Ground sums of the bucketed pairs: lane = pair, pairs of one bucket visit the same ground directions, so the
// lanes of a warp run the same loop over warp-uniform direction loads (numpy_reference.py:548-566; the
// per-direction arithmetic of ground_sums).
template <int WM>
__global__ void __launch_bounds__(256)
    ground_pairs_kernel(Optics o, const float4* __restrict__ misc, const float4* __restrict__ dir,
                        const int* __restrict__ entries, const int* __restrict__ total, float2* g) {
    const int W = o.W;
    const int n_entries = *total;
    const HgPair hk = hg_pair_constants(o.g);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n_entries; e += gridDim.x * blockDim.x) {
        const int code = entries[e];
        const long long node = code >> 1;
        const int pr = code & 1;
        const float4 ms = misc[node];
        const float4 dv = dir[node];
        const float ah = ms.x, ac = ms.y;
        const float wa = pr ? ah * (1.0f - ac) : (1.0f - ah) * (1.0f - ac);
        const float wb = pr ? ah * ac : (1.0f - ah) * ac;
        const int ca = pair_cell(o, ms, pr), cb = ca + 1;
        const bool merged = o.gsame != nullptr && o.gsame[ca] != 0;
        float ground[WM], sground[WM];
#pragma unroll
        for (int w = 0; w < WM; ++w) ground[w] = sground[w] = 0.0f;
        for (int side = 0; side < (merged ? 1 : 2); ++side) {
            const int cell = side ? cb : ca;
            const float wc = side ? wb : wa;
            const int g0 = o.goff[cell], g1 = o.goff[cell + 1];
            const int shift = merged ? o.goff[cb] - g0 : 0;
#pragma unroll 2
            for (int gi = g0; gi < g1; ++gi) {
                const float4 gd = o.gdir4[gi];
                const float m0 = dv.x * gd.z + dv.y * gd.x;
                const float m1 = dv.z * gd.y;
                const float up = clampf(m0 + m1, -1.0f, 1.0f), dn = clampf(m0 - m1, -1.0f, 1.0f);
                const float ph = o.tropo_bins ? 0.0f : hg_pair(hk, up, dn);
                int iu = 0, id = 0, tu = 0, td = 0;
                float fu = 0.0f, fd = 0.0f, gu = 0.0f, gd_ = 0.0f;
                if (o.strato) {
                    strato_lut_pos_clamped(up, iu, fu);
                    strato_lut_pos_clamped(dn, id, fd);
                }
                if (o.tropo_bins) {
                    tropo_lut_pos(o, up, tu, gu);
                    tropo_lut_pos(o, dn, td, gd_);
                }
#pragma unroll
                for (int w = 0; w < WM; ++w) {
                    if (w >= W) break;
                    float gv = wc * o.gval[(size_t)gi * W + w];
                    if (merged) gv += wb * o.gval[(size_t)(gi + shift) * W + w];
                    const float phw =
                        o.tropo_bins ? (tropo_lut_at(o, tu, gu, w) + tropo_lut_at(o, td, gd_, w)) * 0.5f : ph;
                    ground[w] += phw * gv;
                    if (o.strato) {
                        const float sph = (strato_lut_at(o, iu, fu, w) + strato_lut_at(o, id, fd, w)) * 0.5f;
                        sground[w] += sph * gv;
                    }
                }
            }
        }
#pragma unroll
        for (int w = 0; w < WM; ++w)
            if (w < W) g[((size_t)node * 2 + pr) * W + w] = make_float2(ground[w], sground[w]);
    }
}

// Per-ray sum of the staged first light: val0 + coef x (G pair 0 + G pair 1), attenuated, in the node-to-lane
// assignment and Kahan order of transport_warp_kernel.
template <int WM>
__global__ void __launch_bounds__(TRANSPORT_THREADS)
    first_light_sum_kernel(Optics o, Rays b, LaneInputs in, NodeTable tab, FirstLightBufs fl, int ray0, int nray,
                           float4* rad) {
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= nray) return;  // the whole warp leaves together
    const int ray = ray0 + (int)warp;
    const int W = o.W;
    RayConst rc;
    ray_constants(b, ray, rc);
    const int nq = in.nq;
    const int s0 = b.seg_off[ray];
    const long long node0 = (long long)s0 * nq;
    const int nn = (b.seg_off[ray + 1] - s0) * nq;
    float tot[WM][4], cmp[WM][4];
#pragma unroll
    for (int w = 0; w < WM; ++w)
        for (int k = 0; k < 4; ++k) tot[w][k] = cmp[w][k] = 0.0f;
    for (int i = lane; i < nn; i += 32) {
        const long long id = node0 + i;
#pragma unroll
        for (int w = 0; w < WM; ++w) {
            if (w >= W) continue;
            const float att = tab.att[id * W + w];
            const float4 v0 = fl.val0[id * W + w];
            const float2 cf = fl.coef[id * W + w];
            const float2 g0 = fl.g[(size_t)id * 2 * W + w], g1 = fl.g[((size_t)id * 2 + 1) * W + w];
            const float ga = cf.x * (g0.x + g1.x), gs = cf.y * (g0.y + g1.y);
            const float val[4] = {v0.x, v0.y, v0.z, v0.w};
            for (int k = 0; k < 4; ++k) {
                float v = val[k] + ga * rc.pu[k] / 2.0f;
                if (o.strato) v += (gs * rc.pu[k]) / 2.0f;
                kahan(tot[w][k], cmp[w][k], v * att);
            }
        }
    }
#pragma unroll
    for (int w = 0; w < WM; ++w) {
        float v[4];
        for (int k = 0; k < 4; ++k) {
            v[k] = tot[w][k] - cmp[w][k];
#pragma unroll
            for (int dd = 16; dd >= 1; dd >>= 1) v[k] += __shfl_xor_sync(FULL_MASK, v[k], dd);
        }
        if (lane == 0 && w < W) {
            boundary_term(o, b, rc, in.boundary, ray, w, v);
            rad[(size_t)ray * W + w] = make_float4(v[0], v[1], v[2], v[3]);
        }
    }
}

// Ground sums of the bucketed pairs, many wavelengths: one thread per (pair, wavelength), wavelengths fastest, so the
// lanes of a warp share a pair (or two of one bucket) and run the same direction loop; each recomputes the pair's
// phases (the arithmetic of ground_pairs_kernel) and adds its own wavelength's ground values and table phase.
__global__ void __launch_bounds__(256)
    ground_pairs_wave_kernel(Optics o, const float4* __restrict__ misc, const float4* __restrict__ dir,
                             const int* __restrict__ entries, const int* __restrict__ total, float2* g) {
    const int W = o.W;
    const long long n_items = (long long)(*total) * W;
    const HgPair hk = hg_pair_constants(o.g);
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n_items;
         t += (long long)gridDim.x * blockDim.x) {
        const int code = entries[t / W];
        const int w = (int)(t % W);
        const long long node = code >> 1;
        const int pr = code & 1;
        const float4 ms = misc[node];
        const float4 dv = dir[node];
        const float ah = ms.x, ac = ms.y;
        const float wa = pr ? ah * (1.0f - ac) : (1.0f - ah) * (1.0f - ac);
        const float wb = pr ? ah * ac : (1.0f - ah) * ac;
        const int ca = pair_cell(o, ms, pr), cb = ca + 1;
        const bool merged = o.gsame != nullptr && o.gsame[ca] != 0;
        float ground = 0.0f, sground = 0.0f;
        for (int side = 0; side < (merged ? 1 : 2); ++side) {
            const int cell = side ? cb : ca;
            const float wc = side ? wb : wa;
            const int g0 = o.goff[cell], g1 = o.goff[cell + 1];
            const int shift = merged ? o.goff[cb] - g0 : 0;
            for (int gi = g0; gi < g1; ++gi) {
                const float4 gd = o.gdir4[gi];
                const float m0 = dv.x * gd.z + dv.y * gd.x;
                const float m1 = dv.z * gd.y;
                const float up = clampf(m0 + m1, -1.0f, 1.0f), dn = clampf(m0 - m1, -1.0f, 1.0f);
                float gv = wc * o.gval[(size_t)gi * W + w];
                if (merged) gv += wb * o.gval[(size_t)(gi + shift) * W + w];
                const float ph = o.tropo_bins
                                     ? (tropo_phase_at(o, up, w) + tropo_phase_at(o, dn, w)) * 0.5f
                                     : hg_pair(hk, up, dn);
                ground += ph * gv;
                if (o.strato) {
                    int iu, id;
                    float fu, fd;
                    strato_lut_pos_clamped(up, iu, fu);
                    strato_lut_pos_clamped(dn, id, fd);
                    const float sph = (strato_lut_at(o, iu, fu, w) + strato_lut_at(o, id, fd, w)) * 0.5f;
                    sground += sph * gv;
                }
            }
        }
        g[((size_t)node * 2 + pr) * W + w] = make_float2(ground, sground);
    }
}

// Ground sums of the bucketed pairs, many wavelengths, with the wavelength-independent work done once: one warp per
// pair; per batch of 32 ground directions, lane j computes direction j's cosine pair, its Henyey-Greenstein pair
// phase and its stratospheric table positions into shared memory, then lane = wavelength (two chunks above 32) adds
// the batch's directions in order with its own ground values and table phase. The sums are those of
// ground_pairs_wave_kernel, term for term and in the same order.
constexpr int GPW_WARPS = 8;

__global__ void __launch_bounds__(GPW_WARPS * 32)
    ground_pairs_warp_kernel(Optics o, const float4* __restrict__ misc, const float4* __restrict__ dir,
                             const int* __restrict__ entries, const int* __restrict__ total, float2* g) {
    // per staged direction: Henyey-Greenstein pair phase, the two stratospheric table fractions and bins (16 bits
    // each); with the tabulated tropospheric phase, its two fractions and bins in s_tro
    __shared__ float4 s_dir[GPW_WARPS][32];
    __shared__ float4 s_tro[GPW_WARPS][32];
    const int W = o.W;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int items = *total;
    const HgPair hk = hg_pair_constants(o.g);
    const int w0 = lane, w1 = lane + 32;
    for (int item = blockIdx.x * GPW_WARPS + wid; item < items; item += gridDim.x * GPW_WARPS) {
        const int code = entries[item];
        const long long node = code >> 1;
        const int pr = code & 1;
        const float4 ms = misc[node];
        const float4 dv = dir[node];
        const float ah = ms.x, ac = ms.y;
        const float wa = pr ? ah * (1.0f - ac) : (1.0f - ah) * (1.0f - ac);
        const float wb = pr ? ah * ac : (1.0f - ah) * ac;
        const int ca = pair_cell(o, ms, pr), cb = ca + 1;
        const bool merged = o.gsame != nullptr && o.gsame[ca] != 0;
        float ground0 = 0.0f, sground0 = 0.0f, ground1 = 0.0f, sground1 = 0.0f;
        for (int side = 0; side < (merged ? 1 : 2); ++side) {
            const int cell = side ? cb : ca;
            const float wc = side ? wb : wa;
            const int g0 = o.goff[cell], g1 = o.goff[cell + 1];
            const int shift = merged ? o.goff[cb] - g0 : 0;
            for (int base = g0; base < g1; base += 32) {
                const int gi = base + lane;
                __syncwarp();
                if (gi < g1) {
                    const float4 gd = o.gdir4[gi];
                    const float m0 = dv.x * gd.z + dv.y * gd.x;
                    const float m1 = dv.z * gd.y;
                    const float up = clampf(m0 + m1, -1.0f, 1.0f), dn = clampf(m0 - m1, -1.0f, 1.0f);
                    int iu = 0, id = 0;
                    float fu = 0.0f, fd = 0.0f;
                    if (o.strato) {
                        strato_lut_pos_clamped(up, iu, fu);
                        strato_lut_pos_clamped(dn, id, fd);
                    }
                    if (o.tropo_bins) {
                        int tu, td;
                        float gu, gd_;
                        tropo_lut_pos(o, up, tu, gu);
                        tropo_lut_pos(o, dn, td, gd_);
                        s_tro[wid][lane] = make_float4(gu, gd_, __int_as_float(tu), __int_as_float(td));
                    }
                    s_dir[wid][lane] =
                        make_float4(o.tropo_bins ? 0.0f : hg_pair(hk, up, dn), fu, fd, __int_as_float(iu | (id << 16)));
                }
                __syncwarp();
                const int cnt = min(32, g1 - base);
                for (int j = 0; j < cnt; ++j) {
                    const int gj = base + j;
                    const float4 sd = s_dir[wid][j];
                    const float hg = sd.x;
                    const int bins = __float_as_int(sd.w), iu = bins & 0xffff, id = bins >> 16;
                    float4 st = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    if (o.tropo_bins) st = s_tro[wid][j];
                    if (w0 < W) {
                        float gv = wc * o.gval[(size_t)gj * W + w0];
                        if (merged) gv += wb * o.gval[(size_t)(gj + shift) * W + w0];
                        const float ph = o.tropo_bins ? (tropo_lut_at(o, __float_as_int(st.z), st.x, w0) +
                                                         tropo_lut_at(o, __float_as_int(st.w), st.y, w0)) * 0.5f
                                                      : hg;
                        ground0 += ph * gv;
                        if (o.strato) {
                            const float sph = (strato_lut_at(o, iu, sd.y, w0) + strato_lut_at(o, id, sd.z, w0)) * 0.5f;
                            sground0 += sph * gv;
                        }
                    }
                    if (w1 < W) {
                        float gv = wc * o.gval[(size_t)gj * W + w1];
                        if (merged) gv += wb * o.gval[(size_t)(gj + shift) * W + w1];
                        const float ph = o.tropo_bins ? (tropo_lut_at(o, __float_as_int(st.z), st.x, w1) +
                                                         tropo_lut_at(o, __float_as_int(st.w), st.y, w1)) * 0.5f
                                                      : hg;
                        ground1 += ph * gv;
                        if (o.strato) {
                            const float sph = (strato_lut_at(o, iu, sd.y, w1) + strato_lut_at(o, id, sd.z, w1)) * 0.5f;
                            sground1 += sph * gv;
                        }
                    }
                }
            }
        }
        if (w0 < W) g[((size_t)node * 2 + pr) * W + w0] = make_float2(ground0, sground0);
        if (w1 < W) g[((size_t)node * 2 + pr) * W + w1] = make_float2(ground1, sground1);
    }
}

// Per-ray sum of the staged first light, many wavelengths: one warp per (ray, chunk of 32 wavelengths), lane =
// wavelength walking the ray's nodes in order (the Kahan order of transport_wave_kernel).
__global__ void __launch_bounds__(128)
    first_light_sum_wave_kernel(Optics o, Rays b, LaneInputs in, NodeTable tab, FirstLightBufs fl, int ray0,
                                int nray, int wchunks, float4* rad) {
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= (long long)nray * wchunks) return;  // the whole warp leaves together
    const int ray = ray0 + (int)(warp / wchunks);
    const int w = (int)(warp % wchunks) * 32 + lane;
    if (w >= o.W) return;
    const int W = o.W;
    RayConst rc;
    ray_constants(b, ray, rc);
    const int s0 = b.seg_off[ray];
    const long long node0 = (long long)s0 * in.nq;
    const int nn = (b.seg_off[ray + 1] - s0) * in.nq;
    float total[4] = {0, 0, 0, 0}, comp[4] = {0, 0, 0, 0};
    for (int i = 0; i < nn; ++i) {
        const long long id = node0 + i;
        const float att = tab.att[id * W + w];
        const float4 v0 = fl.val0[id * W + w];
        const float2 cf = fl.coef[id * W + w];
        const float2 g0 = fl.g[(size_t)id * 2 * W + w], g1 = fl.g[((size_t)id * 2 + 1) * W + w];
        const float ga = cf.x * (g0.x + g1.x), gs = cf.y * (g0.y + g1.y);
        const float val[4] = {v0.x, v0.y, v0.z, v0.w};
        for (int k = 0; k < 4; ++k) {
            float v = val[k] + ga * rc.pu[k] / 2.0f;
            if (o.strato) v += (gs * rc.pu[k]) / 2.0f;
            kahan(total[k], comp[k], v * att);
        }
    }
    boundary_term(o, b, rc, in.boundary, ray, w, total);
    rad[(size_t)ray * W + w] = make_float4(total[0], total[1], total[2], total[3]);
}

// Warm pass from the node table, few wavelengths (W <= WM): `wpr` warps (1, 2 or 4) per ray, lane l of warp q takes
// nodes 32 q + l, 32 (q + wpr) + l, ... with its own Kahan sums; the warps' sums are added in warp order. Each node's
// corner SH is synthesised from the ray's basis (sh_synth4; for L = 16 and 32, sh_synth4_fixed with 16-byte loads).
// Several warps per ray serve bundles of long rays (observer rays) that would otherwise leave most SMs idle.
// Contracting each distinct corner cell of a batch once
// (per-m sums in shared memory) measured slower on the config-0 warm pass in three forms (0.30-1.3 ms against
// 0.24 ms): the per-batch ballots, deduplication and synchronisation cost more than the 16-byte row loads they save.
template <int WM, int LT>
__global__ void __launch_bounds__(TRANSPORT_THREADS)
    transport_table_kernel(Optics o, Rays b, LaneInputs in, NodeTable tab, int ray0, int nray, int wpr,
                           float4* rad) {
    constexpr int WARPS = TRANSPORT_THREADS / 32;
    __shared__ float red[WARPS][WM][4];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int q = wid % wpr;
    const long long rr = (long long)blockIdx.x * (WARPS / wpr) + wid / wpr;
    const bool live = rr < nray;  // uniform over each warp
    const int ray = ray0 + (int)(live ? rr : 0);
    const int W = o.W;
    RayConst rc;
    float v[WM][4];
    if (live) {
        ray_constants(b, ray, rc);
        const int nq = in.nq;
        const int s0 = b.seg_off[ray];
        const long long node0 = (long long)s0 * nq;
        const int nn = (b.seg_off[ray + 1] - s0) * nq;
        extern __shared__ float warp_sm[];
        float* Y = warp_sm + wid * in.kp;
        for (int m = lane; m <= o.L; m += 32) sh_basis_column(o, rc.d32[2], rc.st, m, Y);
        __syncwarp();
        float tot[WM][4], cmp[WM][4];
#pragma unroll
        for (int w = 0; w < WM; ++w)
            for (int k = 0; k < 4; ++k) tot[w][k] = cmp[w][k] = 0.0f;
        for (int i = q * 32 + lane; i < nn; i += 32 * wpr) {
            const long long id = node0 + i;
            Node n;
            table_node(o, rc, tab, id, n);
#pragma unroll
            for (int w = 0; w < WM; ++w) {
                if (w >= W) continue;
                const float att = tab.att[id * W + w];
                float aero[4];
                const float* pc[4];
                for (int c = 0; c < 4; ++c) pc[c] = in.plane + ((size_t)n.cell[c] * W + w) * in.kp;
                if constexpr (LT > 0)
                    sh_synth4_fixed<LT>(Y, n.cp, pc, aero);
                else
                    sh_synth4(o.L, Y, n.cp, pc, 1, aero);
                float val[4];
                warm_value(o, rc, n, in.field, w, aero, val);
                for (int k = 0; k < 4; ++k) kahan(tot[w][k], cmp[w][k], val[k] * att);
            }
        }
#pragma unroll
        for (int w = 0; w < WM; ++w)
            for (int k = 0; k < 4; ++k) {
                v[w][k] = tot[w][k] - cmp[w][k];
#pragma unroll
                for (int dd = 16; dd >= 1; dd >>= 1) v[w][k] += __shfl_xor_sync(FULL_MASK, v[w][k], dd);
            }
    }
    if (wpr > 1) {
        if (live && lane == 0)
            for (int w = 0; w < WM; ++w)
                for (int k = 0; k < 4; ++k) red[wid][w][k] = v[w][k];
        __syncthreads();
        if (live && q == 0 && lane == 0)
            for (int w = 0; w < WM; ++w)
                for (int k = 0; k < 4; ++k) {
                    float t = red[wid][w][k];
                    for (int u = 1; u < wpr; ++u) t += red[wid + u][w][k];
                    v[w][k] = t;
                }
    }
    if (live && q == 0 && lane == 0)
        for (int w = 0; w < WM; ++w) {
            if (w >= W) break;
            boundary_term(o, b, rc, in.boundary, ray, w, v[w]);
            rad[(size_t)ray * W + w] = make_float4(v[w][0], v[w][1], v[w][2], v[w][3]);
        }
}

// Node record of the table wave kernel: what warm_value and the corner cache read.
constexpr int TREC_WORDS = 27;  // odd stride: the 32 lanes write their records without bank conflicts
struct TableRec {
    float T[16];
    float sw[4];
    int cell[4];
    int ir;
    float cp;
};
static_assert(sizeof(TableRec) <= TREC_WORDS * 4, "table record exceeds its stride");

// Warm pass from the node table, many wavelengths: one warp per (ray, chunk of 32 wavelengths). Lane j rebuilds
// node base+j's record into shared memory; then lane = wavelength walks the records in order with its 4-slot corner
// SH cache (the operation order of transport_wave_kernel's warm branch).
template <int LT>
__global__ void __launch_bounds__(WAVE_WARPS * 32)
    transport_table_wave_kernel(Optics o, Rays b, LaneInputs in, NodeTable tab, int ray0, int nray, int wchunks,
                                float4* rad) {
    extern __shared__ float wave_sm[];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const long long warp = (long long)blockIdx.x * WAVE_WARPS + wid;
    if (warp >= (long long)nray * wchunks) return;  // the whole warp leaves together
    const int ray = ray0 + (int)(warp / wchunks);
    const int w = (int)(warp % wchunks) * 32 + lane;
    const bool wok = w < o.W;
    const int wl = wok ? w : o.W - 1;  // idle lanes compute a valid wavelength and store nothing
    const int L1 = o.L + 1;
    float* recs = wave_sm + (size_t)wid * (32 * TREC_WORDS + 4 * L1 * 32 + o.K);
    float* cache = recs + 32 * TREC_WORDS + lane;
    float* Y = recs + 32 * TREC_WORDS + 4 * L1 * 32;
    RayConst rc;
    ray_constants(b, ray, rc);
    for (int m = lane; m <= o.L; m += 32) sh_basis_column(o, rc.d32[2], rc.st, m, Y);
    const int nq = in.nq;
    const int s0 = b.seg_off[ray];
    const long long node0 = (long long)s0 * nq;
    const int nn = (b.seg_off[ray + 1] - s0) * nq;
    float total[4] = {0, 0, 0, 0}, comp[4] = {0, 0, 0, 0};
    int tag[4] = {-1, -1, -1, -1};
    for (int base = 0; base < nn; base += 32) {
        const int i = base + lane;
        const int cnt = min(32, nn - base);
        __syncwarp();
        if (i < nn) {
            TableRec* R = reinterpret_cast<TableRec*>(recs + lane * TREC_WORDS);
            Node n;
            table_node(o, rc, tab, node0 + i, n);
            for (int k = 0; k < 4; ++k)
                for (int u = 0; u < 4; ++u) R->T[4 * k + u] = n.T[k][u];
            for (int c = 0; c < 4; ++c) {
                R->sw[c] = n.sw[c];
                R->cell[c] = n.cell[c];
            }
            R->ir = n.ir;
            R->cp = n.cp;
        }
        __syncwarp();
        for (int j = 0; j < cnt; ++j) {
            const TableRec* R = reinterpret_cast<const TableRec*>(recs + j * TREC_WORDS);
            const float att = tab.att[(node0 + base + j) * o.W + wl];
            Node n;
            for (int k = 0; k < 4; ++k)
                for (int u = 0; u < 4; ++u) n.T[k][u] = R->T[4 * k + u];
            for (int c = 0; c < 4; ++c) {
                n.sw[c] = R->sw[c];
                n.cell[c] = R->cell[c];
            }
            n.ir = R->ir;
            n.cp = R->cp;
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
                if constexpr (LT > 0) {
                    float acc[LT + 1];
                    sh_contract_wave<LT>(Y, in.plane + (size_t)n.cell[c] * o.K * o.W + wl, o.W, acc);
                    float* cq = cache + (size_t)q * L1 * 32;
#pragma unroll
                    for (int m = 0; m <= LT; ++m) cq[m * 32] = acc[m];
                } else {
                    sh_contract_basis(o.L, Y, in.plane + (size_t)n.cell[c] * o.K * o.W + wl, o.W,
                                      cache + (size_t)q * L1 * 32, 32);
                }
            }
            float aero[4];
            for (int c = 0; c < 4; ++c) aero[c] = azimuth_sum(o.L, n.cp, cache + (size_t)slot_of[c] * L1 * 32, 32);
            float val[4];
            warm_value(o, rc, n, in.field, wl, aero, val);
            for (int k = 0; k < 4; ++k) kahan(total[k], comp[k], val[k] * att);
        }
    }
    if (wok) {
        boundary_term(o, b, rc, in.boundary, ray, w, total);
        rad[(size_t)ray * o.W + w] = make_float4(total[0], total[1], total[2], total[3]);
    }
}

// Warm pass from the node table and the pair contractions, many wavelengths: one warp per (ray, chunk of 32
// wavelengths); lane j rebuilds node base+j's record (with its four pair indices) into shared memory, then lane =
// wavelength walks the records in order reading the per-m contractions of its corner pairs (coalesced over lanes).
constexpr int PREC_WORDS = 31;  // TableRec + 4 pair indices, odd stride
constexpr int PAIR_WAVE_WARPS = 4;

__global__ void __launch_bounds__(PAIR_WAVE_WARPS * 32)
    transport_pair_wave_kernel(Optics o, Rays b, LaneInputs in, NodeTable tab, PairTable pt, int ray0, int nray,
                               int wchunks, float4* rad) {
    __shared__ float recs_all[PAIR_WAVE_WARPS][32 * PREC_WORDS];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const long long warp = (long long)blockIdx.x * PAIR_WAVE_WARPS + wid;
    if (warp >= (long long)nray * wchunks) return;  // the whole warp leaves together
    const int ray = ray0 + (int)(warp / wchunks);
    const int w = (int)(warp % wchunks) * 32 + lane;
    const bool wok = w < o.W;
    const int wl = wok ? w : o.W - 1;  // idle lanes compute a valid wavelength and store nothing
    const int W = o.W, L1 = o.L + 1;
    float* recs = recs_all[wid];
    RayConst rc;
    ray_constants(b, ray, rc);
    const int nq = in.nq;
    const int s0 = b.seg_off[ray];
    const long long node0 = (long long)s0 * nq;
    const int nn = (b.seg_off[ray + 1] - s0) * nq;
    float total[4] = {0, 0, 0, 0}, comp[4] = {0, 0, 0, 0};
    for (int base = 0; base < nn; base += 32) {
        const int i = base + lane;
        const int cnt = min(32, nn - base);
        __syncwarp();
        if (i < nn) {
            TableRec* R = reinterpret_cast<TableRec*>(recs + lane * PREC_WORDS);
            Node n;
            table_node(o, rc, tab, node0 + i, n);
            for (int k = 0; k < 4; ++k)
                for (int u = 0; u < 4; ++u) R->T[4 * k + u] = n.T[k][u];
            for (int c = 0; c < 4; ++c) {
                R->sw[c] = n.sw[c];
                R->cell[c] = n.cell[c];
            }
            R->ir = n.ir;
            R->cp = n.cp;
            const int4 pn = pt.node[node0 + i];
            int* pr = reinterpret_cast<int*>(recs + lane * PREC_WORDS + TREC_WORDS);
            pr[0] = pn.x;
            pr[1] = pn.y;
            pr[2] = pn.z;
            pr[3] = pn.w;
        }
        __syncwarp();
        for (int j = 0; j < cnt; ++j) {
            const TableRec* R = reinterpret_cast<const TableRec*>(recs + j * PREC_WORDS);
            const int* pr = reinterpret_cast<const int*>(recs + j * PREC_WORDS + TREC_WORDS);
            const float att = tab.att[(node0 + base + j) * W + wl];
            Node n;
            for (int k = 0; k < 4; ++k)
                for (int u = 0; u < 4; ++u) n.T[k][u] = R->T[4 * k + u];
            for (int c = 0; c < 4; ++c) {
                n.sw[c] = R->sw[c];
                n.cell[c] = R->cell[c];
            }
            n.ir = R->ir;
            n.cp = R->cp;
            float aero[4];
            for (int c = 0; c < 4; ++c) aero[c] = azimuth_sum(o.L, n.cp, pt.A + (size_t)pr[c] * L1 * W + wl, W);
            float val[4];
            warm_value(o, rc, n, in.field, wl, aero, val);
            for (int k = 0; k < 4; ++k) kahan(total[k], comp[k], val[k] * att);
        }
    }
    if (wok) {
        boundary_term(o, b, rc, in.boundary, ray, w, total);
        rad[(size_t)ray * W + w] = make_float4(total[0], total[1], total[2], total[3]);
    }
}

static size_t table_wave_smem(int L) {
    return sizeof(float) * (size_t)WAVE_WARPS * (32 * TREC_WORDS + 4 * (L + 1) * 32 + (L + 1) * (L + 2) / 2);
}

// Index (a, b, c) of element i of an [.][nb][nc] array for a grid-stride loop: set once by division, then advanced
// by the stride's own (a, b, c) digits with carries, so that the loop divides nothing per element.
struct StrideIndex {
    long long a, da;
    int b, c, db, dc, nb, nc;
    __device__ StrideIndex(long long i, long long stride, int nb_, int nc_) : nb(nb_), nc(nc_) {
        c = (int)(i % nc);
        const long long r = i / nc;
        b = (int)(r % nb);
        a = r / nb;
        dc = (int)(stride % nc);
        const long long rs = stride / nc;
        db = (int)(rs % nb);
        da = rs / nb;
    }
    __device__ __forceinline__ void next() {
        c += dc;
        const int c1 = c >= nc;
        c -= c1 ? nc : 0;
        b += db + c1;
        const int c2 = b >= nb;
        b -= c2 ? nb : 0;
        a += da + c2;
    }
};

// plane = SH slots x cell density (+ stratospheric slots x their density): [cell][k][w] (kp = 0), or
// [cell][w][kp] with zero padding k = K .. kp - 1 (few wavelengths: 16-byte aligned rows for sh_synth4_fixed).
__global__ void plane_kernel(const float* __restrict__ field, const float* __restrict__ ha,
                             const float* __restrict__ sd, int nc, int K, int src, int W, int strato, int kp,
                             long long n, float* __restrict__ plane) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    // kp: (cell, w, k) over [cell][W][kp]; otherwise (cell, k, w) over [cell][K][W]
    StrideIndex ix(i, stride, kp ? W : K, kp ? kp : W);
    for (; i < n; i += stride, ix.next()) {
        const int cell = (int)ix.a;
        const int w = kp ? ix.b : ix.c, k = kp ? ix.c : ix.b;
        if (k >= K) {
            plane[i] = 0.0f;
            continue;
        }
        const int hi = cell / nc;
        const float* f = field + (size_t)cell * src * W + w;
        // each product and the sum rounded on its own (sh_layout.combined_coefficients)
        float v = __fmul_rn(f[(size_t)(10 + k) * W], ha[hi]);
        if (strato) v = __fadd_rn(v, __fmul_rn(f[(size_t)(10 + K + k) * W], sd[hi]));
        plane[i] = v;
    }
}

constexpr int PROJ_THREADS = 512;
constexpr int PROJ_RAYS = 16;
constexpr int PROJ_OWN = 16;

static size_t project_smem(int K, int W) { return sizeof(float) * (size_t)PROJ_RAYS * (K + 6 * W); }

// One block per cell. Output (slot, w) pairs are owned by threads (registers, Kahan-compensated FP32 over ray
// chunks); the basis row Y_lm(mu) cos(m phi) of PROJ_RAYS rays is staged in shared memory per chunk
// (numpy_reference.py:689-711: moments[0:4] = sum wt rad, moments[4+k] = sum (wt trace) (Y_k cos m phi),
// flux = sum trace wt max(0, dloc_z) * albedo / pi).
__global__ void __launch_bounds__(PROJ_THREADS)
    project_kernel(Optics o, Rays b, const float4* __restrict__ rad, int cell0, int ground_only, int rayleigh_only,
                   int out_base, float* __restrict__ moments, float* __restrict__ flux, float flux_scale) {
    extern __shared__ float sm[];
    const int W = o.W, K = o.K, L = o.L;
    const int cell = cell0 + blockIdx.x;
    const int r0 = b.cell_off[cell], r1 = b.cell_off[cell + 1];
    const int nout = (4 + K) * W;
    const int nown = rayleigh_only ? 4 * W : nout;  // outputs this launch computes (the SH rows elsewhere)
    float* basis = sm;                    // [PROJ_RAYS][K]
    float* wtr = basis + PROJ_RAYS * K;   // [PROJ_RAYS][W]  weight * trace
    float* wr = wtr + PROJ_RAYS * W;      // [PROJ_RAYS][4][W] weight * radiance
    float* wgr = wr + PROJ_RAYS * 4 * W;  // [PROJ_RAYS][W] trace * weight * max(0, dloc_z)
    float acc[PROJ_OWN], cmp[PROJ_OWN];
#pragma unroll
    for (int i = 0; i < PROJ_OWN; ++i) acc[i] = cmp[i] = 0.0f;
    float facc = 0.0f, fcmp = 0.0f;
    const bool do_flux = out_base == 0 && (int)threadIdx.x < W && flux != nullptr;
    for (int rb = r0; rb < r1; rb += PROJ_RAYS) {
        const int nr = min(PROJ_RAYS, r1 - rb);
        __syncthreads();
        if (!ground_only && !rayleigh_only) {
            for (int it = threadIdx.x; it < nr * (L + 1); it += blockDim.x) {
                const int r = it / (L + 1), m = it % (L + 1);
                const int ray = rb + r;
                const float4 dv = b.dir[ray];
                const float mu = dv.z, st = dv.w;
                const float cp = clampf(b.pcp[ray], -1.0f, 1.0f);
                float c0 = 1.0f, c1 = cp, cm = 1.0f;
                if (m == 1) cm = cp;
                for (int q = 2; q <= m; ++q) {
                    float c2 = (2.0f * cp) * c1 - c0;
                    c0 = c1;
                    c1 = c2;
                    cm = c2;
                }
                float pmm = 0.28209479177387814f;
                for (int q = 1; q <= m; ++q) pmm = (pmm * o.sh_d[q]) * st;
                const float scale = m ? 1.41421356237309515f : 1.0f;
                float* row = basis + r * K;
                float p0 = pmm;
                row[m * (m + 1) / 2 + m] = (scale * p0) * cm;
                if (m < L) {
                    float p1 = (sqrtf(2.0f * m + 3.0f) * mu) * p0;
                    row[(m + 1) * (m + 2) / 2 + m] = (scale * p1) * cm;
                    for (int l = m + 2; l <= L; ++l) {
                        const int k = l * (l + 1) / 2 + m;
                        float p2 = (o.sh_a[k] * mu) * p1 - o.sh_b[k] * p0;
                        row[k] = (scale * p2) * cm;
                        p0 = p1;
                        p1 = p2;
                    }
                }
            }
        }
        for (int it = threadIdx.x; it < nr * W; it += blockDim.x) {
            const int r = it / W, w = it % W;
            const int ray = rb + r;
            const float4 v = rad[(size_t)ray * W + w];
            const float wt = b.dir_lo[ray].w;
            const float tr = (v.x + v.y) + v.z;
            wtr[r * W + w] = tr * wt;
            wr[(r * 4 + 0) * W + w] = v.x * wt;
            wr[(r * 4 + 1) * W + w] = v.y * wt;
            wr[(r * 4 + 2) * W + w] = v.z * wt;
            wr[(r * 4 + 3) * W + w] = v.w * wt;
            wgr[r * W + w] = tr * (wt * fmaxf(0.0f, b.dloc[ray].z));
        }
        __syncthreads();
        if (!ground_only) {
#pragma unroll
            for (int i = 0; i < PROJ_OWN; ++i) {
                const int oi = out_base + threadIdx.x + i * PROJ_THREADS;
                if (oi < nown) {
                    const int slot = oi / W, w = oi % W;
                    float part = 0.0f;
                    if (slot < 4) {
                        for (int r = 0; r < nr; ++r) part += wr[(r * 4 + slot) * W + w];
                    } else {
                        const int k = slot - 4;
                        for (int r = 0; r < nr; ++r) part += wtr[r * W + w] * basis[r * K + k];
                    }
                    kahan(acc[i], cmp[i], part);
                }
            }
        }
        if (do_flux) {
            float part = 0.0f;
            for (int r = 0; r < nr; ++r) part += wgr[r * W + threadIdx.x];
            kahan(facc, fcmp, part);
        }
    }
    if (!ground_only && moments) {
#pragma unroll
        for (int i = 0; i < PROJ_OWN; ++i) {
            const int oi = out_base + threadIdx.x + i * PROJ_THREADS;
            if (oi < nown) moments[(size_t)cell * nout + oi] = acc[i];
        }
    }
    if (do_flux) flux[(size_t)cell * W + threadIdx.x] = facc * flux_scale;
}

// ------------------------------------------------------------------ tensor-core projection
// The SH rows of the projection as a dense contraction per cell: moments[4 + k][w] = sum_r B[k][r] V[r][w] with
// B[k][r] = Y_k(mu_r) cos(m phi_r) (geometry only, a table built once per cell bundle) and V[r][w] = weight_r x
// trace_r,w (from the radiance). One CTA per (cell, 128 rows of k): the tile of B (128 rows x one 128-byte chunk of
// rays) and of V^T (N = W rounded up to 16 rows) are written to shared memory in the 128-byte swizzle, one thread
// issues tcgen05.mma into an FP32 accumulator in tensor memory, the four warps read it back. Precision forms:
// BF16 (one product), TF32 (kind::tf32), bf16x3 (B = Bh + Bl, V = Vh + Vl; Bh Vh + Bh Vl + Bl Vh).
enum { PROJ_FP32 = 0, PROJ_BF16X3 = 1, PROJ_TF32 = 2, PROJ_BF16 = 3 };

__device__ unsigned g_proj_error;  // bounded-wait flags of the tensor-core projection

struct BasisTable {
    void* hi;  // [cells][kpad][rpad]: BF16 (BF16, bf16x3) or FP32 (TF32)
    void* lo;  // bf16x3: BF16 of (basis - hi)
    int kpad, rpad;
};

// One thread per (ray, m): column m of the ray's basis row (the FP32 recurrences of project_kernel), stored at
// [cell][k][ray - first ray of the cell].
template <int MODE>
__global__ void basis_table_kernel(Optics o, Rays b, BasisTable bt) {
    const int L = o.L;
    const long long n = (long long)b.nray * (L + 1);
    for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < n;
         it += (long long)gridDim.x * blockDim.x) {
        const int ray = (int)(it / (L + 1)), m = (int)(it % (L + 1));
        const int cell = b.ray_cell[ray];
        const int j = ray - b.cell_off[cell];
        const float4 dv = b.dir[ray];
        const float mu = dv.z, st = dv.w;
        const float cp = clampf(b.pcp[ray], -1.0f, 1.0f);
        float c0 = 1.0f, c1 = cp, cm = 1.0f;
        if (m == 1) cm = cp;
        for (int q = 2; q <= m; ++q) {
            const float c2 = (2.0f * cp) * c1 - c0;
            c0 = c1;
            c1 = c2;
            cm = c2;
        }
        float pmm = 0.28209479177387814f;
        for (int q = 1; q <= m; ++q) pmm = (pmm * o.sh_d[q]) * st;
        const float scale = m ? 1.41421356237309515f : 1.0f;
        const size_t base = (size_t)cell * bt.kpad * bt.rpad + j;
        auto put = [&](int k, float v) {
            const size_t at = base + (size_t)k * bt.rpad;
            if (MODE == PROJ_TF32) {
                static_cast<float*>(bt.hi)[at] = v;
            } else {
                const __nv_bfloat16 h = __float2bfloat16_rn(v);
                static_cast<__nv_bfloat16*>(bt.hi)[at] = h;
                if (MODE == PROJ_BF16X3) static_cast<__nv_bfloat16*>(bt.lo)[at] = __float2bfloat16_rn(v - __bfloat162float(h));
            }
        };
        float p0 = pmm;
        put(m * (m + 1) / 2 + m, (scale * p0) * cm);
        if (m < L) {
            float p1 = (sqrtf(2.0f * m + 3.0f) * mu) * p0;
            put((m + 1) * (m + 2) / 2 + m, (scale * p1) * cm);
            for (int l = m + 2; l <= L; ++l) {
                const int k = l * (l + 1) / 2 + m;
                const float p2 = (o.sh_a[k] * mu) * p1 - o.sh_b[k] * p0;
                put(k, (scale * p2) * cm);
                p0 = p1;
                p1 = p2;
            }
        }
    }
}

static size_t project_tc_smem(int mode, int np) {
    const int na = mode == PROJ_BF16X3 ? 2 : 1;
    return 1024 + (size_t)na * 16384 + (size_t)na * np * 128 + 64;
}

template <int MODE>
__global__ void __launch_bounds__(128)
    project_tc_kernel(BasisTable bt, Rays b, const float4* __restrict__ rad, int W, int K, int np, uint32_t idesc,
                      uint32_t tmem_cols, float* __restrict__ moments) {
    constexpr int ESZ = MODE == PROJ_TF32 ? 4 : 2;  // operand bytes
    constexpr int CH = 128 / ESZ;                   // rays per 128-byte chunk
    constexpr int NT = MODE == PROJ_BF16X3 ? 2 : 1; // operand tiles (high, low parts)
    extern __shared__ uint8_t proj_raw[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(proj_raw) + 1023) & ~(uintptr_t)1023);
    uint8_t* at0 = sm;
    uint8_t* at1 = sm + 16384;
    uint8_t* vt0 = sm + NT * 16384;
    uint8_t* vt1 = vt0 + np * 128;
    uint64_t* bar = reinterpret_cast<uint64_t*>(vt0 + NT * np * 128);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
    const int cell = blockIdx.y, mt = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r0 = b.cell_off[cell], nr = b.cell_off[cell + 1] - r0;
    if (threadIdx.x == 0) {
        tcx::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tcx::tmem_alloc(tslot, tmem_cols);
    tcx::fence_before();
    __syncthreads();
    tcx::fence_after();
    const uint32_t tmem = *tslot;
    const int nchunk = (nr + CH - 1) / CH;
    bool ok = true;
    for (int ch = 0; ch < nchunk && ok; ++ch) {
        for (int pc = threadIdx.x; pc < 128 * 8; pc += 128) {  // basis tile: 128 rows x 8 pieces of 16 bytes
            const int row = pc >> 3, piece = pc & 7;
            const size_t src =
                ((((size_t)cell * bt.kpad + mt * 128 + row) * bt.rpad) + (size_t)ch * CH) * ESZ + piece * 16;
            *reinterpret_cast<uint4*>(at0 + tcx::sw128_offset(row, piece)) =
                *reinterpret_cast<const uint4*>(static_cast<const uint8_t*>(bt.hi) + src);
            if (NT == 2)
                *reinterpret_cast<uint4*>(at1 + tcx::sw128_offset(row, piece)) =
                    *reinterpret_cast<const uint4*>(static_cast<const uint8_t*>(bt.lo) + src);
        }
        for (int pc = threadIdx.x; pc < np * 8; pc += 128) {  // V^T tile: np rows (wavelengths) x 8 pieces
            const int w = pc >> 3, piece = pc & 7;
            constexpr int PER = 16 / ESZ;
            float v[PER];
#pragma unroll
            for (int e = 0; e < PER; ++e) {
                const int j = ch * CH + piece * PER + e;
                v[e] = 0.0f;
                if (w < W && j < nr) {
                    const int ray = r0 + j;
                    const float4 q = rad[(size_t)ray * W + w];
                    v[e] = ((q.x + q.y) + q.z) * b.dir_lo[ray].w;
                }
            }
            if (MODE == PROJ_TF32) {
                *reinterpret_cast<float4*>(vt0 + tcx::sw128_offset(w, piece)) = make_float4(v[0], v[1], v[2], v[3]);
            } else {
                __align__(16) __nv_bfloat16 h[8], l[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    h[e] = __float2bfloat16_rn(v[e % PER]);
                    l[e] = __float2bfloat16_rn(v[e % PER] - __bfloat162float(h[e]));
                }
                *reinterpret_cast<uint4*>(vt0 + tcx::sw128_offset(w, piece)) = *reinterpret_cast<const uint4*>(h);
                if (NT == 2)
                    *reinterpret_cast<uint4*>(vt1 + tcx::sw128_offset(w, piece)) = *reinterpret_cast<const uint4*>(l);
            }
        }
        tcx::fence_proxy_async();
        __syncthreads();
        if (threadIdx.x == 0) {
            tcx::fence_after();
            const uint32_t a0 = tcx::smem_u32(at0), a1 = tcx::smem_u32(at1);
            const uint32_t v0 = tcx::smem_u32(vt0), v1 = tcx::smem_u32(vt1);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {  // four K steps of 32 bytes cover the chunk
                const uint32_t acc = (ch > 0 || kk > 0) ? 1u : 0u;
                if (MODE == PROJ_TF32) {
                    tcx::mma_tf32(tmem, tcx::sw128_desc(a0 + kk * 32), tcx::sw128_desc(v0 + kk * 32), idesc, acc);
                } else {
                    tcx::mma_f16(tmem, tcx::sw128_desc(a0 + kk * 32), tcx::sw128_desc(v0 + kk * 32), idesc, acc);
                    if (NT == 2) {
                        tcx::mma_f16(tmem, tcx::sw128_desc(a0 + kk * 32), tcx::sw128_desc(v1 + kk * 32), idesc, 1u);
                        tcx::mma_f16(tmem, tcx::sw128_desc(a1 + kk * 32), tcx::sw128_desc(v0 + kk * 32), idesc, 1u);
                    }
                }
            }
            tcx::mma_commit(bar);
        }
        ok = tcx::mbar_wait(bar, ch & 1, 1u, &g_proj_error);  // the tiles may be overwritten once the MMAs are done
        ok = __all_sync(FULL_MASK, ok);
        tcx::fence_after();
    }
    const int k = mt * 128 + warp * 32 + lane;
    if (ok) {
        for (int c0 = 0; c0 < np; c0 += 16) {
            float v[16];
            if (nchunk > 0) {
                tcx::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            } else {
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = 0.0f;
            }
            if (k < K)
#pragma unroll
                for (int i = 0; i < 16; ++i)
                    if (c0 + i < W) moments[((size_t)cell * (4 + K) + 4 + k) * W + c0 + i] = v[i];
        }
    }
    tcx::fence_before();
    __syncthreads();
    if (warp == 0) tcx::tmem_dealloc(tmem, tmem_cols);
}

// ------------------------------------------------------------------ corner SH values on the tensor cores (W > 4)
// The corner SH value of a node at one of its four corner cells c is
//     V[node, c][w] = sum_m cos(m phi_node) sum_l Y_lm(mu_ray) plane[c][k(l, m)][w] = sum_k B[node][k] plane[c][k][w]
// with the node's basis row B[node][k] = Y_k(ray) cos(m(k) phi_node) (the per-m contraction of a ray-cell pair
// followed by the node's azimuth series, folded into one K-long dot product). The (node, corner) entries of a bundle
// are bucketed by corner cell once per geometry; for every cell, tiles of 128 entries form the GEMM
// [128 x K] x [K x W] against the cell's plane on tcgen05 (BF16 operands split into high and low parts, three
// products, FP32 accumulation in tensor memory: the bf16x3 form), once per plane and bundle; the node pass then reads
// the four corner values of each node (transport_corner_wave_kernel).
struct CornerEntries {
    const int* ray;    // [entries] ray of the entry's node
    const float* cp;   // [entries] the node's azimuth cosine
    const int* slot;   // [entries] node * 4 + corner: the row of the output
    const int4* tile;  // [tiles] (cell, first entry, entries, 0)
};

// One thread per ray: the four corner cells of each of its nodes. Pass 0 counts the entries of each cell (cnt),
// pass 1 writes them at the cell's cursor (the order within a cell does not matter: each output row is its own dot
// product).
__global__ void corner_entries_kernel(Optics o, Rays b, NodeTable tab, int nq, int pass, int* cnt, int* cursor,
                                      int* e_ray, float* e_cp, int* e_slot) {
    for (int ray = blockIdx.x * blockDim.x + threadIdx.x; ray < b.nray; ray += gridDim.x * blockDim.x) {
        const int s0 = b.seg_off[ray];
        const long long node0 = (long long)s0 * nq;
        const int nn = (b.seg_off[ray + 1] - s0) * nq;
        for (int i = 0; i < nn; ++i) {
            const float4 ms = tab.misc[node0 + i];
            const int pk = __float_as_int(ms.w);
            const int cell0 = misc_ir(pk) * o.nc + (pk & 0xffff);
            for (int c = 0; c < 4; ++c) {
                const int cell = cell0 + (c & 1) + (c >> 1) * o.nc;
                if (pass == 0) {
                    atomicAdd(&cnt[cell], 1);
                } else {
                    const int at = atomicAdd(&cursor[cell], 1);
                    e_ray[at] = ray;
                    e_cp[at] = ms.z;
                    e_slot[at] = (int)((node0 + i) * 4 + c);
                }
            }
        }
    }
}

// B tiles of the corner products for every cell and chunk of 64 SH coefficients, once per plane: the plane rows
// [k][w] split into BF16 high and low parts in the 128-byte-swizzled K-major layout of the tile (np wavelength rows of
// 8 pieces), high tile then low tile, so that a CTA copies a chunk's 2 np x 128 bytes as they are. One thread per
// (cell, chunk, piece, wavelength row), wavelengths fastest (coalesced plane reads).
__global__ void plane_tiles_kernel(const float* __restrict__ plane, int ns, int K, int W, int np, int nchunk,
                                   uint8_t* __restrict__ tiles) {
    const long long n = (long long)ns * nchunk * 8 * np;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int w = (int)(i % np);
        const long long r = i / np;
        const int p = (int)(r % 8);
        const long long cc = r / 8;  // cell * nchunk + chunk
        const int ch = (int)(cc % nchunk);
        const long long cell = cc / nchunk;
        const float* pc = plane + (size_t)cell * K * W;
        __align__(16) __nv_bfloat16 h[8], lo[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int k = ch * 64 + p * 8 + e;
            const float x = (w < W && k < K) ? pc[(size_t)k * W + w] : 0.0f;
            h[e] = __float2bfloat16_rn(x);
            lo[e] = __float2bfloat16_rn(x - __bfloat162float(h[e]));
        }
        uint8_t* base = tiles + (size_t)cc * (2 * (size_t)np * 128);
        *reinterpret_cast<uint4*>(base + tcx::sw128_offset(w, p)) = *reinterpret_cast<const uint4*>(h);
        *reinterpret_cast<uint4*>(base + (size_t)np * 128 + tcx::sw128_offset(w, p)) = *reinterpret_cast<const uint4*>(lo);
    }
}

// Pass 1 of the entries, one warp per ray, lanes over its nodes 32 at a time: the entries of one cell from one batch
// take consecutive positions (one atomic per distinct cell and corner), so the rows of a tile that share a ray are
// neighbours and a warp's loads of their basis rows hit few distinct addresses.
__global__ void corner_entries_fill_kernel(Optics o, Rays b, NodeTable tab, int nq, int* cursor, int* e_ray,
                                           float* e_cp, int* e_slot) {
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long ray = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ray < b.nray; ray += nwarps) {
        const int s0 = b.seg_off[ray];
        const long long node0 = (long long)s0 * nq;
        const int nn = (b.seg_off[ray + 1] - s0) * nq;
        for (int base = 0; base < nn; base += 32) {
            const int i = base + lane;
            const bool act = i < nn;
            const float4 ms = act ? tab.misc[node0 + i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            const int pk = __float_as_int(ms.w);
            const int cell0 = misc_ir(pk) * o.nc + (pk & 0xffff);
            for (int c = 0; c < 4; ++c) {
                const int cell = act ? cell0 + (c & 1) + (c >> 1) * o.nc : -1;
                const unsigned peers = __match_any_sync(FULL_MASK, cell);
                const int leader = __ffs(peers) - 1;
                int at = 0;
                if (act && lane == leader) at = atomicAdd(&cursor[cell], __popc(peers));
                at = __shfl_sync(FULL_MASK, at, leader);
                if (act) {
                    const int k = at + __popc(peers & ((1u << lane) - 1u));
                    e_ray[k] = (int)ray;
                    e_cp[k] = ms.z;
                    e_slot[k] = (int)((node0 + i) * 4 + c);
                }
            }
        }
    }
}

constexpr int CORNER_ROWS = 128;     // entries per tile (the MMA's M)
constexpr int CORNER_THREADS = 256;  // two threads per row build the A tile (four 16-byte pieces each)
constexpr int CORNER_STAGES = 1;     // shared-memory stages of the A and B tiles
constexpr int CORNER_ROW_BATCH = 4;  // A-tile steps (two rows each) whose basis loads a warp issues together

static size_t corner_tc_smem(int np, int L) {
    // CORNER_STAGES stages of A high/low tiles (2 x 16 KB) and B high/low tiles (2 x np rows of 128 bytes), cos(m phi)
    // rows, the rows' rays and output slots, the order m of every coefficient (bytes, rounded up to 16), the stages'
    // barriers and the tensor-memory slot; 1 KB of alignment slack
    const size_t K = (size_t)(L + 1) * (L + 2) / 2;
    return 1024 + CORNER_STAGES * (2 * 16384 + 2 * (size_t)np * 128) + (size_t)CORNER_ROWS * (L + 1) * 4 +
           2 * CORNER_ROWS * 4 + ((K + 15) & ~(size_t)15) + 64;
}

// One CTA per tile of 128 entries of one corner cell, chunks of 64 SH coefficients in CORNER_STAGES shared-memory
// stages: the block builds chunk ch (the A tile a row per warp at a time, lanes over the row's coefficients: the
// entry's basis row times its cos(m phi), split into BF16 high and low parts; the B tile, the cell's plane for np
// wavelength rows, split likewise; both in the 128-byte swizzle); one thread issues the 12 MMAs of a chunk (four K
// steps of 16, three products each) and commits them to the stage's barrier, which the block waits on (bounded)
// before it rebuilds that stage. The epilogue moves the rows through shared memory and writes each row's W FP32
// values at its slot, lanes over the wavelengths.
__global__ void __launch_bounds__(CORNER_THREADS, 4)
    corner_tc_kernel(Optics o, CornerEntries ce, const float* __restrict__ y_tab, int kp,
                     const uint4* __restrict__ btiles, int np, uint32_t idesc, uint32_t tmem_cols,
                     float* __restrict__ out) {
    extern __shared__ uint8_t corner_raw[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(corner_raw) + 1023) & ~(uintptr_t)1023);
    const size_t stage_bytes = 2 * 16384 + 2 * (size_t)np * 128;  // stage st: A high, A low, B high, B low
    float* cm = reinterpret_cast<float*>(sm + CORNER_STAGES * stage_bytes);  // [CORNER_ROWS][L + 1]
    const int L1 = o.L + 1;
    int* rays_s = reinterpret_cast<int*>(cm + CORNER_ROWS * L1);  // [CORNER_ROWS] the rows' rays
    int* slots_s = rays_s + CORNER_ROWS;                              // [CORNER_ROWS] the rows' output slots
    uint8_t* mk = reinterpret_cast<uint8_t*>(slots_s + CORNER_ROWS);  // [K] the order m of each coefficient
    uint64_t* bar = reinterpret_cast<uint64_t*>(mk + ((o.K + 15) & ~15));  // [stages], 8-byte aligned
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + CORNER_STAGES);
    const int4 tile = ce.tile[blockIdx.x];
    const int cell = tile.x, e0 = tile.y, ne = tile.z;
    const int t = threadIdx.x, warp = t >> 5;
    const int row = t & (CORNER_ROWS - 1), half = t >> 7;
    const int W = o.W, K = o.K;
    if (t == 0) {
        for (int q = 0; q < CORNER_STAGES; ++q) tcx::mbar_init(&bar[q], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tcx::tmem_alloc(tslot, tmem_cols);
    // the row's entry: its ray and its cos(m phi) series (the Chebyshev recurrence of azimuth_sum)
    const bool valid = row < ne;
    if (half == 0) {
        rays_s[row] = valid ? ce.ray[e0 + row] : 0;
        slots_s[row] = valid ? ce.slot[e0 + row] : 0;
        const float cpv = valid ? clampf(ce.cp[e0 + row], -1.0f, 1.0f) : 0.0f;
        float* crow = cm + row * L1;
        float c0 = 1.0f, c1 = cpv;
        crow[0] = valid ? 1.0f : 0.0f;
        if (L1 > 1) crow[1] = valid ? c1 : 0.0f;
        for (int m = 2; m < L1; ++m) {
            const float c2 = (2.0f * cpv) * c1 - c0;
            c0 = c1;
            c1 = c2;
            crow[m] = valid ? c2 : 0.0f;
        }
    }
    for (int k = t; k < K; k += CORNER_THREADS) {  // k = l (l + 1) / 2 + m
        int l = (int)((sqrtf(8.0f * k + 1.0f) - 1.0f) * 0.5f);
        while ((l + 1) * (l + 2) / 2 <= k) ++l;
        while (l * (l + 1) / 2 > k) --l;
        mk[k] = (uint8_t)(k - l * (l + 1) / 2);
    }
    tcx::fence_before();
    __syncthreads();
    tcx::fence_after();
    const uint32_t tmem = *tslot;
    const int lane = t & 31;
    const int nchunk_all = (K + 63) / 64;
    const uint4* bcell = btiles + (size_t)cell * nchunk_all * (16 * np);  // the cell's B tiles, 16 np pieces a chunk
    const int nchunk = (K + 63) / 64;
    bool ok = true;
    for (int ch = 0; ch < nchunk && ok; ++ch) {
        const int st = ch % CORNER_STAGES;
        uint8_t* const ahi = sm + st * stage_bytes;
        uint8_t* const alo = ahi + 16384;
        uint8_t* const bhi = ahi + 32768;
        uint8_t* const blo = bhi + np * 128;
        if (ch >= CORNER_STAGES) {
            // the MMAs of chunk ch - CORNER_STAGES read this stage: wait for them before it is rebuilt
            // one thread waits (bounded) on the barrier, the block on it
            const unsigned parity = ((ch - CORNER_STAGES) / CORNER_STAGES) & 1;
            ok = t == 0 ? tcx::mbar_wait(&bar[st], parity, 2u, &g_proj_error) : true;
            ok = __syncthreads_and(ok);
            if (!ok) break;
            tcx::fence_after();
        }
        const int k0 = ch * 64;
        // A tile: warp `warp` builds rows warp, warp + 8, ..., two rows per step: lanes 0-15 one row, lanes 16-31
        // the next, lane l taking coefficients k0 + 4 (l mod 16) .. + 3 of its row (one coalesced 16-byte load from the
        // row's basis row), times cos(m phi) of the row, split into BF16 high and low parts, one 8-byte store per
        // part: a warp writes two 128-byte tile rows a step. The loads of CORNER_ROW_BATCH steps are issued first.
        {
            constexpr int WARPS = CORNER_THREADS / 32;
            const int hl = lane >> 4, q = lane & 15;
            const int ka = k0 + 4 * q;
            int mq[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) mq[e] = ka + e < K ? mk[ka + e] : 0;
            const int piece = q >> 1, sub = (q & 1) * 8;
#pragma unroll 1
            for (int s0 = 0; s0 < CORNER_ROWS / (2 * WARPS); s0 += CORNER_ROW_BATCH) {
                float4 y[CORNER_ROW_BATCH];
#pragma unroll
                for (int u = 0; u < CORNER_ROW_BATCH; ++u) {
                    const int r = warp + WARPS * (2 * (s0 + u) + hl);
                    y[u] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    if (r < ne) {
                        const float* yr = y_tab + (size_t)rays_s[r] * kp + ka;
                        if (ka + 3 < K) {
                            y[u] = *reinterpret_cast<const float4*>(yr);
                        } else {
                            if (ka < K) y[u].x = yr[0];
                            if (ka + 1 < K) y[u].y = yr[1];
                            if (ka + 2 < K) y[u].z = yr[2];
                        }
                    }
                }
#pragma unroll
                for (int u = 0; u < CORNER_ROW_BATCH; ++u) {
                    const int r = warp + WARPS * (2 * (s0 + u) + hl);
                    const float* cr = cm + r * L1;
                    const float x0 = y[u].x * cr[mq[0]], x1 = y[u].y * cr[mq[1]];
                    const float x2 = y[u].z * cr[mq[2]], x3 = y[u].w * cr[mq[3]];
                    __align__(8) __nv_bfloat162 h[2], lo[2];
                    h[0] = __floats2bfloat162_rn(x0, x1);
                    h[1] = __floats2bfloat162_rn(x2, x3);
                    const float2 f0 = __bfloat1622float2(h[0]), f1 = __bfloat1622float2(h[1]);
                    lo[0] = __floats2bfloat162_rn(x0 - f0.x, x1 - f0.y);
                    lo[1] = __floats2bfloat162_rn(x2 - f1.x, x3 - f1.y);
                    const uint32_t off = tcx::sw128_offset(r, piece) + sub;
                    *reinterpret_cast<uint2*>(ahi + off) = *reinterpret_cast<const uint2*>(h);
                    *reinterpret_cast<uint2*>(alo + off) = *reinterpret_cast<const uint2*>(lo);
                }
            }
        }
        // B tile: the chunk's high and low tiles of the cell's plane, already split and swizzled (plane_tiles_kernel),
        // copied in 16-byte pieces
        {
            const uint4* src = bcell + (size_t)ch * (16 * np);
            uint4* dst = reinterpret_cast<uint4*>(bhi);
            for (int q = t; q < 16 * np; q += CORNER_THREADS) dst[q] = src[q];
        }
        tcx::fence_proxy_async();
        __syncthreads();
        if (t == 0) {
            tcx::fence_after();
            const uint32_t ah = tcx::smem_u32(ahi), al = tcx::smem_u32(alo);
            const uint32_t bh = tcx::smem_u32(bhi), bl = tcx::smem_u32(blo);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                const uint32_t acc = (ch > 0 || kk > 0) ? 1u : 0u;
                tcx::mma_f16(tmem, tcx::sw128_desc(ah + kk * 32), tcx::sw128_desc(bh + kk * 32), idesc, acc);
                tcx::mma_f16(tmem, tcx::sw128_desc(ah + kk * 32), tcx::sw128_desc(bl + kk * 32), idesc, 1u);
                tcx::mma_f16(tmem, tcx::sw128_desc(al + kk * 32), tcx::sw128_desc(bh + kk * 32), idesc, 1u);
            }
            tcx::mma_commit(&bar[st]);
        }
    }
    if (ok) {
        // the last commit covers every MMA issued before it
        const int last = nchunk - 1;
        const unsigned parity = (last / CORNER_STAGES) & 1;
        ok = t == 0 ? tcx::mbar_wait(&bar[last % CORNER_STAGES], parity, 2u, &g_proj_error) : true;
        ok = __syncthreads_and(ok);
        tcx::fence_after();
    }
    // epilogue: warps 0-3 (one tensor-memory lane quarter each) move the rows into shared memory (stage 0, free once
    // the last MMAs are done; row stride np + 1 keeps the lanes' stores on distinct banks), then every warp writes
    // whole rows at their slots, lanes over the wavelengths (coalesced)
    float* stage = reinterpret_cast<float*>(sm);
    const int sp = np + 1;
    if (ok && warp < 4) {
        for (int c0 = 0; c0 < np; c0 += 16) {
            float v[16];
            tcx::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);  // warp-wide
#pragma unroll
            for (int i = 0; i < 16; ++i) stage[row * sp + c0 + i] = v[i];
        }
    }
    tcx::fence_before();
    __syncthreads();
    if (ok)
        for (int r = warp; r < ne; r += CORNER_THREADS / 32) {
            float* dst = out + (size_t)slots_s[r] * W;
            for (int w = lane; w < W; w += 32) dst[w] = stage[r * sp + w];
        }
    if (warp == 0) tcx::tmem_dealloc(tmem, tmem_cols);
}

// ------------------------------------------------------------------ first-light ground sums on the tensor cores
// The ground sums of the items (node, corner pair) of one bucket (the pair's first cell ca; its second is ca + 1)
// are products over the pair's ground directions k in [goff[ca], goff[ca + 2]), contiguous in the CSR:
//   ground[item][w]  = sum_k hg_pair(item, k) wgt(item, k) gval[k][w]
//   sground[item][w] = sum_k sum_r U_r(item, k) wgt(item, k) V_r[w] gval[k][w]
// with wgt the corner weight of the side k belongs to and the stratospheric pair phase written as
// (sph(up, w) + sph(dn, w)) / 2 = sum_r (U_r(up) + U_r(dn)) / 2 V_r[w], the leading factors of its table
// (strato_factors). Each is a [items x directions] x [directions x W] product: A rows are built from the item's
// direction and the ground directions, B from the ground values (times V_r), both split into BF16 high and low parts
// (three MMAs, FP32 accumulation in tensor memory).
constexpr int GTC_ROWS = 128;     // items per tile (the MMA's M)
constexpr int GTC_THREADS = 256;  // two threads per row build the A tile
constexpr int GTC_MAX_RANK = 8;   // most stratospheric phase factors the product takes

struct GroundTc {
    const int* entries;  // item codes node * 2 + pr, bucketed by the pair's first cell
    const int4* tile;    // [tiles] (first cell ca, first item, items, 0)
    const int* ntiles;   // number of tiles (device)
    const float2* su2;   // [STRATO_LUT_BINS][rank] (value, next value - value) of the factors U_r on the table's grid
    const float* sv;     // [rank][W] the factors V_r
    int rank;
};

static size_t ground_tc_smem(int np) { return 1024 + 2 * 16384 + 2 * (size_t)np * 128 + 64; }

// Tiles of at most GTC_ROWS items of one bucket: pass 0 counts each bucket's tiles, pass 1 writes them at the offsets
// bucket_scan_kernel made of the counts.
__global__ void ground_tiles_kernel(const int* __restrict__ off, int ns, int pass, int* cnt, const int* toff,
                                    int4* tile) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ns; c += gridDim.x * blockDim.x) {
        const int e0 = off[c], n = off[c + 1] - e0;
        const int nt = (n + GTC_ROWS - 1) / GTC_ROWS;
        if (pass == 0) {
            cnt[c] = nt;
            continue;
        }
        const int at = toff[c];
        for (int i = 0; i < nt; ++i)
            tile[at + i] = make_int4(c, e0 + i * GTC_ROWS, min(GTC_ROWS, n - i * GTC_ROWS), 0);
    }
}

// One CTA per tile of 128 items of one bucket, one shared-memory stage; steps = (chunk of 64 directions) x (part:
// 0 the Henyey-Greenstein product into accumulator 0, r + 1 the stratospheric factor r into accumulator 1). Per step
// threads r and r + 128 build row r of the A tile (four 16-byte pieces each), all threads the B tile (np wavelength
// rows), thread 0 issues the 12 MMAs (four K steps of 16, three products each) and commits them to the stage's
// barrier, which the block waits on (bounded) before the next step rebuilds the stage. The epilogue (warps 0-3, one
// tensor-memory lane quarter each) stores (ground, sground) of each valid row's np wavelengths.
__global__ void __launch_bounds__(GTC_THREADS)
    ground_tc_kernel(Optics o, const float4* __restrict__ misc, const float4* __restrict__ dir, GroundTc gt, int np,
                     uint32_t idesc, uint32_t tmem_cols, float2* __restrict__ g) {
    if ((int)blockIdx.x >= *gt.ntiles) return;  // the whole CTA leaves before any barrier or tensor-memory use
    extern __shared__ uint8_t gtc_raw[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(gtc_raw) + 1023) & ~(uintptr_t)1023);
    uint8_t* const ahi = sm;
    uint8_t* const alo = sm + 16384;
    uint8_t* const bhi = sm + 32768;
    uint8_t* const blo = bhi + np * 128;
    uint64_t* bar = reinterpret_cast<uint64_t*>(blo + np * 128);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
    const int4 tile = gt.tile[blockIdx.x];
    const int ca = tile.x, e0 = tile.y, ne = tile.z;
    const int t = threadIdx.x, warp = t >> 5;
    const int row = t & (GTC_ROWS - 1), half = t >> 7;
    const int W = o.W;
    if (t == 0) {
        tcx::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tcx::tmem_alloc(tslot, tmem_cols);
    // the row's item: its direction terms and corner weights (the arithmetic of ground_pairs_warp_kernel)
    const bool valid = row < ne;
    const int code = valid ? gt.entries[e0 + row] : 0;
    float4 dv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float wa = 0.0f, wb = 0.0f;
    if (valid) {
        const long long node = code >> 1;
        const int pr = code & 1;
        const float4 ms = misc[node];
        dv = dir[node];
        const float ah = ms.x, ac = ms.y;
        wa = pr ? ah * (1.0f - ac) : (1.0f - ah) * (1.0f - ac);
        wb = pr ? ah * ac : (1.0f - ah) * ac;
    }
    const int k0 = o.goff[ca], k1 = o.goff[ca + 1], k2 = o.goff[ca + 2];
    const int parts = 1 + (o.strato ? gt.rank : 0);
    const int steps = (k2 - k0 + 63) / 64 * parts;
    const HgPair hk = hg_pair_constants(o.g);
    tcx::fence_before();
    __syncthreads();
    tcx::fence_after();
    const uint32_t tmem = *tslot;
    bool ok = true;
    for (int s = 0; s < steps && ok; ++s) {
        const int ch = s / parts, part = s - ch * parts;
        if (s > 0) {
            // the MMAs of step s - 1 read the stage: wait for them before it is rebuilt
            ok = t == 0 ? tcx::mbar_wait(bar, (s - 1) & 1, 4u, &g_proj_error) : true;
            ok = __syncthreads_and(ok);
            if (!ok) break;
            tcx::fence_after();
        }
        const int kc = k0 + ch * 64;
        const int r = part - 1;
#pragma unroll
        for (int pp = 0; pp < 4; ++pp) {
            const int p = half * 4 + pp;
            float x[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int k = kc + p * 8 + e;
                float v = 0.0f;
                if (valid && k < k2) {
                    const float4 gd = o.gdir4[k];
                    const float m0 = dv.x * gd.z + dv.y * gd.x;
                    const float m1 = dv.z * gd.y;
                    const float up = clampf(m0 + m1, -1.0f, 1.0f), dn = clampf(m0 - m1, -1.0f, 1.0f);
                    float ph;
                    if (part == 0) {
                        ph = hg_pair(hk, up, dn);
                    } else {
                        int iu, id;
                        float fu, fd;
                        strato_lut_pos_clamped(up, iu, fu);
                        strato_lut_pos_clamped(dn, id, fd);
                        const float2 a = gt.su2[(size_t)iu * gt.rank + r], b = gt.su2[(size_t)id * gt.rank + r];
                        ph = ((a.x + fu * a.y) + (b.x + fd * b.y)) * 0.5f;
                    }
                    v = ph * (k < k1 ? wa : wb);
                }
                x[e] = v;
            }
            __align__(16) __nv_bfloat162 h[4], lo[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                h[e] = __floats2bfloat162_rn(x[2 * e], x[2 * e + 1]);
                const float2 hf = __bfloat1622float2(h[e]);
                lo[e] = __floats2bfloat162_rn(x[2 * e] - hf.x, x[2 * e + 1] - hf.y);
            }
            *reinterpret_cast<uint4*>(ahi + tcx::sw128_offset(row, p)) = *reinterpret_cast<const uint4*>(h);
            *reinterpret_cast<uint4*>(alo + tcx::sw128_offset(row, p)) = *reinterpret_cast<const uint4*>(lo);
        }
        // B tile: np rows (wavelengths) x 8 pieces; consecutive threads take consecutive wavelengths (coalesced)
        for (int q = t; q < np * 8; q += GTC_THREADS) {
            const int p = q / np, w = q - p * np;
            const float vs = (part == 0 || w >= W) ? 1.0f : gt.sv[r * W + w];
            __align__(16) __nv_bfloat16 h[8], lo[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int k = kc + p * 8 + e;
                const float x = (w < W && k < k2) ? o.gval[(size_t)k * W + w] * vs : 0.0f;
                h[e] = __float2bfloat16_rn(x);
                lo[e] = __float2bfloat16_rn(x - __bfloat162float(h[e]));
            }
            *reinterpret_cast<uint4*>(bhi + tcx::sw128_offset(w, p)) = *reinterpret_cast<const uint4*>(h);
            *reinterpret_cast<uint4*>(blo + tcx::sw128_offset(w, p)) = *reinterpret_cast<const uint4*>(lo);
        }
        tcx::fence_proxy_async();
        __syncthreads();
        if (t == 0) {
            tcx::fence_after();
            const uint32_t ah = tcx::smem_u32(ahi), al = tcx::smem_u32(alo);
            const uint32_t bh = tcx::smem_u32(bhi), bl = tcx::smem_u32(blo);
            const uint32_t acc_col = part == 0 ? 0u : (uint32_t)np;
            const bool fresh = ch == 0 && part <= 1;  // the first product into this accumulator
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                const uint32_t acc = (fresh && kk == 0) ? 0u : 1u;
                tcx::mma_f16(tmem + acc_col, tcx::sw128_desc(ah + kk * 32), tcx::sw128_desc(bh + kk * 32), idesc, acc);
                tcx::mma_f16(tmem + acc_col, tcx::sw128_desc(ah + kk * 32), tcx::sw128_desc(bl + kk * 32), idesc, 1u);
                tcx::mma_f16(tmem + acc_col, tcx::sw128_desc(al + kk * 32), tcx::sw128_desc(bh + kk * 32), idesc, 1u);
            }
            tcx::mma_commit(bar);
        }
    }
    if (ok && steps > 0) {
        // the last commit covers every MMA issued before it
        ok = t == 0 ? tcx::mbar_wait(bar, (steps - 1) & 1, 4u, &g_proj_error) : true;
        ok = __syncthreads_and(ok);
        tcx::fence_after();
    }
    if (ok && warp < 4) {
        float2* dst = valid ? g + (size_t)code * W : nullptr;
        if (steps == 0) {  // no ground directions: the accumulators were never written
            if (valid)
                for (int w = 0; w < W; ++w) dst[w] = make_float2(0.0f, 0.0f);
        } else {
            for (int c0 = 0; c0 < np; c0 += 16) {
                float vg[16], vs[16];
                tcx::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, vg);  // warp-wide
                if (parts > 1)
                    tcx::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(np + c0), vs);
                else
#pragma unroll
                    for (int i = 0; i < 16; ++i) vs[i] = 0.0f;
                if (valid)
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                        if (c0 + i < W) dst[c0 + i] = make_float2(vg[i], vs[i]);
            }
        }
    }
    tcx::fence_before();
    __syncthreads();
    if (warp == 0) tcx::tmem_dealloc(tmem, tmem_cols);
}

// Warm pass from the node table and the corner values (many wavelengths): transport_pair_wave_kernel with each
// corner's SH value read from V[node * 4 + corner][w] instead of summed from the pair contractions.
__global__ void __launch_bounds__(PAIR_WAVE_WARPS * 32)
    transport_corner_wave_kernel(Optics o, Rays b, LaneInputs in, NodeTable tab, const float* __restrict__ cv,
                                 int ray0, int nray, int wchunks, float4* rad) {
    __shared__ float recs_all[PAIR_WAVE_WARPS][32 * TREC_WORDS];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const long long warp = (long long)blockIdx.x * PAIR_WAVE_WARPS + wid;
    if (warp >= (long long)nray * wchunks) return;  // the whole warp leaves together
    const int ray = ray0 + (int)(warp / wchunks);
    const int w = (int)(warp % wchunks) * 32 + lane;
    const bool wok = w < o.W;
    const int wl = wok ? w : o.W - 1;  // idle lanes compute a valid wavelength and store nothing
    const int W = o.W;
    float* recs = recs_all[wid];
    RayConst rc;
    ray_constants(b, ray, rc);
    const int nq = in.nq;
    const int s0 = b.seg_off[ray];
    const long long node0 = (long long)s0 * nq;
    const int nn = (b.seg_off[ray + 1] - s0) * nq;
    float total[4] = {0, 0, 0, 0}, comp[4] = {0, 0, 0, 0};
    for (int base = 0; base < nn; base += 32) {
        const int i = base + lane;
        const int cnt = min(32, nn - base);
        __syncwarp();
        if (i < nn) {
            TableRec* R = reinterpret_cast<TableRec*>(recs + lane * TREC_WORDS);
            Node n;
            table_node(o, rc, tab, node0 + i, n);
            for (int k = 0; k < 4; ++k)
                for (int u = 0; u < 4; ++u) R->T[4 * k + u] = n.T[k][u];
            for (int c = 0; c < 4; ++c) {
                R->sw[c] = n.sw[c];
                R->cell[c] = n.cell[c];
            }
            R->ir = n.ir;
            R->cp = n.cp;
        }
        __syncwarp();
        for (int j = 0; j < cnt; ++j) {
            const TableRec* R = reinterpret_cast<const TableRec*>(recs + j * TREC_WORDS);
            const long long node = node0 + base + j;
            const float att = tab.att[node * W + wl];
            Node n;
            for (int k = 0; k < 4; ++k)
                for (int u = 0; u < 4; ++u) n.T[k][u] = R->T[4 * k + u];
            for (int c = 0; c < 4; ++c) {
                n.sw[c] = R->sw[c];
                n.cell[c] = R->cell[c];
            }
            n.ir = R->ir;
            n.cp = R->cp;
            float aero[4];
            for (int c = 0; c < 4; ++c) aero[c] = cv[(size_t)(node * 4 + c) * W + wl];
            float val[4];
            warm_value(o, rc, n, in.field, wl, aero, val);
            for (int k = 0; k < 4; ++k) kahan(total[k], comp[k], val[k] * att);
        }
    }
    if (wok) {
        boundary_term(o, b, rc, in.boundary, ray, w, total);
        rad[(size_t)ray * W + w] = make_float4(total[0], total[1], total[2], total[3]);
    }
}


// The warm pass from the corner values split in two launches for many wavelengths, so that the per-node work has the
// whole grid's memory parallelism: corner_node_kernel (one thread per node and wavelength, consecutive threads the
// wavelengths of one node) forms each node's value with its four corner values (warm_value) times its attenuation
// into vbuf[node][w]; ray_sum_kernel (one thread per ray and wavelength) adds the nodes of the ray in node order
// (Kahan), then the ground boundary term, as transport_corner_wave_kernel does in one launch.
__global__ void __launch_bounds__(256)
    corner_node_kernel(Optics o, Rays b, NodeTable tab, const int* __restrict__ node_ray, const float* __restrict__ cv,
                       const float* __restrict__ field, long long node0, long long nodes, float4* __restrict__ vbuf) {
    const int W = o.W;
    const long long n = nodes * W;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long node = node0 + i / W;
        const int w = (int)(i - (i / W) * W);
        RayConst rc;
        ray_constants(b, node_ray[node], rc);
        Node nd;
        table_node(o, rc, tab, node, nd);
        float aero[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) aero[c] = cv[(size_t)(node * 4 + c) * W + w];
        float val[4];
        warm_value(o, rc, nd, field, w, aero, val);
        const float att = tab.att[node * W + w];
        vbuf[node * W + w] = make_float4(val[0] * att, val[1] * att, val[2] * att, val[3] * att);
    }
}

__global__ void __launch_bounds__(256)
    ray_sum_kernel(Optics o, Rays b, LaneInputs in, const float4* __restrict__ vbuf, int ray0, int nray,
                   float4* __restrict__ rad) {
    const int W = o.W;
    const long long n = (long long)nray * W;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int ray = ray0 + (int)(i / W);
        const int w = (int)(i - (i / W) * W);
        const int s0 = b.seg_off[ray];
        const long long nd0 = (long long)s0 * in.nq;
        const int nn = (b.seg_off[ray + 1] - s0) * in.nq;
        float total[4] = {0, 0, 0, 0}, comp[4] = {0, 0, 0, 0};
        const float4* v = vbuf + nd0 * W + w;
        int j = 0;
        for (; j + 4 <= nn; j += 4) {  // four nodes' loads in flight, added in node order
            float4 q[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) q[u] = v[(size_t)(j + u) * W];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                kahan(total[0], comp[0], q[u].x);
                kahan(total[1], comp[1], q[u].y);
                kahan(total[2], comp[2], q[u].z);
                kahan(total[3], comp[3], q[u].w);
            }
        }
        for (; j < nn; ++j) {
            const float4 q = v[(size_t)j * W];
            kahan(total[0], comp[0], q.x);
            kahan(total[1], comp[1], q.y);
            kahan(total[2], comp[2], q.z);
            kahan(total[3], comp[3], q.w);
        }
        RayConst rc;
        ray_constants(b, ray, rc);
        boundary_term(o, b, rc, in.boundary, ray, w, total);
        rad[(size_t)ray * W + w] = make_float4(total[0], total[1], total[2], total[3]);
    }
}

// Node -> ray index of a bundle (one thread per ray).
__global__ void node_ray_kernel(Rays b, int nq, int* __restrict__ node_ray) {
    for (int ray = blockIdx.x * blockDim.x + threadIdx.x; ray < b.nray; ray += gridDim.x * blockDim.x) {
        const long long a = (long long)b.seg_off[ray] * nq, e = (long long)b.seg_off[ray + 1] * nq;
        for (long long node = a; node < e; ++node) node_ray[node] = ray;
    }
}

__global__ void add_kernel(const float* a, const float* b, float* out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] + b[i];
}

// metrics layout: [0][W] nonfinite count, [1][W] max |g| bits, [2][W] max |g - x| bits (uint32)
__global__ void compose_kernel(const float* __restrict__ warm, const float* __restrict__ first, const float* __restrict__ x,
                               const float* __restrict__ rf, const float* __restrict__ af, const float* __restrict__ asca,
                               const float* __restrict__ ext0, const float* __restrict__ s_eigen,
                               const float* __restrict__ s_sca, int K, int src, int W, int af_w, long long n,
                               unsigned long long done_mask, const unsigned long long* __restrict__ done_dev,
                               float* __restrict__ out, unsigned* __restrict__ metrics) {
    __shared__ unsigned sm_bad[64], sm_mag[64], sm_dif[64];
    if (done_dev) done_mask = *done_dev;  // frozen wavelengths from the evaluation control block
    for (int i = threadIdx.x; i < 64; i += blockDim.x) sm_bad[i] = sm_mag[i] = sm_dif[i] = 0u;
    __syncthreads();
    const int nm = 4 + K;
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    StrideIndex ix(i, stride, src, W);  // (cell, slot, w)
    // the metrics of this thread's elements, per wavelength it meets (one unless the stride is not a multiple of W)
    unsigned bad = 0u, mag = 0u, dif = 0u;
    int wcur = -1;
    auto flush = [&]() {
        if (wcur < 0) return;
        if (bad) atomicAdd(&sm_bad[wcur], bad);
        atomicMax(&sm_mag[wcur], mag);
        atomicMax(&sm_dif[wcur], dif);
        bad = mag = dif = 0u;
    };
    for (; i < n; i += stride, ix.next()) {
        const int w = ix.c, slot = ix.b;
        const long long cell = ix.a;
        if (w != wcur) {
            flush();
            wcur = w;
        }
        const size_t mb = ((size_t)cell * nm) * W + w;
        float v;
        if (slot < 4) {
            const float m = warm[mb + (size_t)slot * W] + first[mb + (size_t)slot * W];
            v = m * (C_3_8PI * ext0[w]);
        } else if (slot < 10) {
            const float m = warm[mb + (size_t)slot * W] + first[mb + (size_t)slot * W];
            v = (m * rf[slot - 4]) * ext0[w];
        } else if (slot < 10 + K) {
            const int k = slot - 10;
            const float m = warm[mb + (size_t)(4 + k) * W] + first[mb + (size_t)(4 + k) * W];
            v = (m * af[af_w ? k * W + w : k]) * asca[w];  // af_w: per-wavelength eigenvalues [K][W] (TROPO_MIE)
        } else {
            const int k = slot - 10 - K;
            const float m = warm[mb + (size_t)(4 + k) * W] + first[mb + (size_t)(4 + k) * W];
            v = (m * s_eigen[k * W + w]) * s_sca[w];
        }
        if (fabsf(v) < TRACE_MIN) v = 0.0f;
        bad += isfinite(v) ? 0u : 1u;
        const float xv = x ? x[i] : 0.0f;
        if ((done_mask >> w) & 1ull) v = xv;
        out[i] = v;
        mag = max(mag, __float_as_uint(fabsf(v)));
        dif = max(dif, __float_as_uint(fabsf(v - xv)));
    }
    flush();
    __syncthreads();
    for (int w = threadIdx.x; w < W; w += blockDim.x) {
        if (sm_bad[w]) atomicAdd(&metrics[w], sm_bad[w]);
        atomicMax(&metrics[W + w], sm_mag[w]);
        atomicMax(&metrics[2 * W + w], sm_dif[w]);
    }
}

// Observer boxes: out[row][dir][w] = solar[w] sum_n ww[n] (rad_xx + rad_yy + rad_zz)[row, dir, n, w] in FP64.
__global__ void boxes_kernel(const float4* __restrict__ rad, const double* __restrict__ ww,
                             const double* __restrict__ solar, int rows, int dirs, int pts, int W, double* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * dirs * W) return;
    const int w = i % W;
    const int rd = i / W;
    double s = 0.0;
    for (int n = 0; n < pts; ++n) {
        const float4 v = rad[((size_t)rd * pts + n) * W + w];
        s += ww[n] * (((double)v.x + (double)v.y) + (double)v.z);
    }
    out[i] = s * solar[w];
}

// Norm of each cell's source per wavelength, ||g[cell, :, w]||_2, one block per cell: the block size is a multiple
// of W, thread t keeps wavelength t % W and, as member t / W of its wavelength's group of G, sums the squares of
// the slots k = member, member + G, ... (contiguous loads across the block); the members' sums are added by a
// pairwise tree in member order. mx[w] collects the maximum norm (bits of a non-negative float order as unsigned
// integers).
__global__ void norm_kernel(const float* __restrict__ g, long long ns, int src, int W, float* __restrict__ norms,
                            unsigned* __restrict__ mx) {
    extern __shared__ float part[];  // [blockDim.x]
    const int B = blockDim.x, t = threadIdx.x;
    const int w = t % W, G = B / W, mem = t / W;
    for (long long cell = blockIdx.x; cell < ns; cell += gridDim.x) {
        const float* row = g + (size_t)cell * src * W;
        float acc = 0.0f;
        for (int k = mem; k < src; k += G) {
            const float v = row[(size_t)k * W + w];
            acc += v * v;
        }
        part[t] = acc;
        __syncthreads();
        for (int h = 1; h < G; h <<= 1) {
            if ((mem & (2 * h - 1)) == 0 && mem + h < G) part[t] += part[t + h * W];
            __syncthreads();
        }
        if (mem == 0) {
            const float nv = sqrtf(part[w]);
            norms[cell * W + w] = nv;
            atomicMax(&mx[w], __float_as_uint(nv));
        }
        __syncthreads();
    }
}

// Per-evaluation control of the fixed-point loop, written by the host (pinned) and copied to the device at the start
// of every evaluation, so that one evaluation's launches are the same every time (a CUDA graph replays them).
struct EvalCtrl {
    int slot;      // ring slot receiving this evaluation's g and residual feature
    int m;         // ring slots after adding it (1..4)
    int order[4];  // those slots, oldest first
    int mix;       // 1: x = Anderson mix of the previous ring (mix_m, mix_order, weights, use); 0: x as it is
    int mix_m;
    int mix_order[4];
    int use[64];                 // per wavelength: 1 mix, 0 take g (frozen or no valid weights)
    float weights[4 * 64];       // [j][w] over mix_order
    unsigned long long done;     // converged wavelengths, frozen by the composition
    int restart;                 // 1: x = *fallback (the warm start's fallback), no mix
    const float* fallback;       // the fallback start of a warm-started solve (device field), or null
};

struct Ring4 {
    float* p[4];
};

// Residual feature f = (g - x) / max(norm, 1e-8 max norm) into ring slot ctrl->slot, and FP64 partial dots of f
// with the ring slots ctrl->order[0 .. m-1] (the new slot among them): partials[block][j][w]. Blocks walk whole
// cells; the block size is a multiple of W, so thread t keeps wavelength t % W over all its elements (FP32 products
// in compensated FP32 sums), and the per-thread sums of a wavelength are added in FP64 by a pairwise tree in thread
// order (no atomics: the dots are reproducible run to run).
// One cell's elements for thread t with NS ring slots dotted: four elements' loads are issued before any of them is
// used (the kernel is latency-bound otherwise), and every element is summed in the same order as a plain loop.
template <int NS>
__device__ __forceinline__ void feature_cell(const float* __restrict__ g, const float* __restrict__ x, float* dst,
                                             const float* const* rj, const bool* self, size_t base, int row, int t,
                                             int B, float scale, float* loc, float* lcm) {
    int e = t;
    for (; e + 3 * B < row; e += 4 * B) {
        float gv[4], xv[4], ov[NS > 0 ? NS : 1][4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const size_t i = base + e + u * B;
            gv[u] = g[i];
            xv[u] = x[i];
#pragma unroll
            for (int j = 0; j < NS; ++j) ov[j][u] = self[j] ? 0.0f : rj[j][i];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const float f = (gv[u] - xv[u]) / scale;
            dst[base + e + u * B] = f;
#pragma unroll
            for (int j = 0; j < NS; ++j) kahan(loc[j], lcm[j], f * (self[j] ? f : ov[j][u]));
        }
    }
    for (; e < row; e += B) {
        const size_t i = base + e;
        const float f = (g[i] - x[i]) / scale;
        dst[i] = f;
#pragma unroll
        for (int j = 0; j < NS; ++j) kahan(loc[j], lcm[j], f * (self[j] ? f : rj[j][i]));
    }
}

__global__ void __launch_bounds__(256, 4) feature_kernel(const float* __restrict__ g, const float* __restrict__ x,
                               const float* __restrict__ norms, const unsigned* __restrict__ mx, long long ns, int src,
                               int W, Ring4 ring, const EvalCtrl* __restrict__ ctrl, double* __restrict__ partials) {
    extern __shared__ double sd[];  // [blockDim.x][4]
    const int B = blockDim.x;
    const int t = threadIdx.x;
    const int w = t % W;
    const int row = src * W;
    const int nslot = ctrl->m;
    float* dst = ring.p[ctrl->slot];
    const float* rj[4];
    bool self[4];
    for (int j = 0; j < 4; ++j) {
        rj[j] = ring.p[ctrl->order[j & 3]];
        self[j] = rj[j] == dst;
    }
    const float floor_w = __uint_as_float(mx[w]) * 1e-8f;
    // per-thread dots in compensated FP32 (FP32 products, Kahan sums), combined in FP64 below
    float loc[4] = {0.0f, 0.0f, 0.0f, 0.0f}, lcm[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (long long cell = blockIdx.x; cell < ns; cell += gridDim.x) {
        const float scale = fmaxf(norms[cell * W + w], floor_w);
        const size_t base = (size_t)cell * row;
        switch (nslot) {
            case 1: feature_cell<1>(g, x, dst, rj, self, base, row, t, B, scale, loc, lcm); break;
            case 2: feature_cell<2>(g, x, dst, rj, self, base, row, t, B, scale, loc, lcm); break;
            case 3: feature_cell<3>(g, x, dst, rj, self, base, row, t, B, scale, loc, lcm); break;
            default: feature_cell<4>(g, x, dst, rj, self, base, row, t, B, scale, loc, lcm); break;
        }
    }
    for (int j = 0; j < 4; ++j) sd[t * 4 + j] = (double)loc[j] - (double)lcm[j];
    __syncthreads();
    // thread t is member t / W of its wavelength's group of G = B / W; pairwise tree over the members
    const int G = B / W, mem = t / W;
    for (int h = 1; h < G; h <<= 1) {
        if ((mem & (2 * h - 1)) == 0 && mem + h < G)
            for (int j = 0; j < 4; ++j) sd[t * 4 + j] += sd[(t + h * W) * 4 + j];
        __syncthreads();
    }
    for (int q = t; q < 4 * W; q += B) {
        const int j = q / W, ww = q % W;
        partials[(size_t)blockIdx.x * 4 * W + q] = j < nslot ? sd[ww * 4 + j] : 0.0;
    }
}

// ring.p[ctrl->slot] = g
__global__ void ring_copy_kernel(const float* __restrict__ g, Ring4 ring, const EvalCtrl* __restrict__ ctrl,
                                 long long n) {
    float* dst = ring.p[ctrl->slot];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = g[i];
}

__global__ void sum_partials_kernel(const double* __restrict__ partials, int blocks, int n, double* out) {
    const int lane = threadIdx.x & 31;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= n) return;  // the whole warp leaves together
    double acc = 0.0;
    for (int b = lane; b < blocks; b += 32) acc += partials[(size_t)b * n + i];
    for (int dd = 16; dd >= 1; dd >>= 1) acc += __shfl_xor_sync(FULL_MASK, acc, dd);
    if (lane == 0) out[i] = acc;
}

// When ctrl->mix: x[i] = sum_j weights[j][w] ring[mix_order j][i] for wavelengths with valid weights, else g[i]
// (the previous evaluation's g). Without ctrl->mix, x stays as it is.
// x[i] = sum_j weights[j][w] q_j[i] over M ring slots for the mixed wavelengths, g[i] for the others; four elements
// a thread, loads issued first. The block size is a multiple of W, so a thread keeps one wavelength.
template <int M>
__device__ __forceinline__ void mix_elements(const float* __restrict__ g, const float* const* q,
                                             const EvalCtrl* __restrict__ ctrl, int W, long long n,
                                             float* __restrict__ x) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += 4 * stride) {
        float qv[M][4], gv[4];
        int wv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const long long i = i0 + u * stride;
            wv[u] = -1;
            if (i >= n) continue;
            wv[u] = (int)(i0 % W);  // the stride is a multiple of W
            if (ctrl->use[wv[u]]) {
#pragma unroll
                for (int j = 0; j < M; ++j) qv[j][u] = q[j][i];
            } else {
                gv[u] = g[i];
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int w = wv[u];
            if (w < 0) continue;
            const long long i = i0 + u * stride;
            if (!ctrl->use[w]) {
                x[i] = gv[u];
                continue;
            }
            float acc = ctrl->weights[w] * qv[0][u];
#pragma unroll
            for (int j = 1; j < M; ++j) acc += ctrl->weights[j * 64 + w] * qv[j][u];
            x[i] = acc;
        }
    }
}

__global__ void mix_kernel(const float* __restrict__ g, Ring4 ring, const EvalCtrl* __restrict__ ctrl, int W,
                           long long n, float* __restrict__ x) {
    if (ctrl->restart) {
        const float* __restrict__ f = ctrl->fallback;
        for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
            x[i] = f[i];
        return;
    }
    if (!ctrl->mix) return;
    const float* q[4];
    for (int j = 0; j < 4; ++j) q[j] = ring.p[ctrl->mix_order[j]];
    switch (ctrl->mix_m) {
        case 1: mix_elements<1>(g, q, ctrl, W, n, x); break;
        case 2: mix_elements<2>(g, q, ctrl, W, n, x); break;
        case 3: mix_elements<3>(g, q, ctrl, W, n, x); break;
        default: mix_elements<4>(g, q, ctrl, W, n, x); break;
    }
}

// ------------------------------------------------------------------------------------------------ host helpers
static Optics optics_of(const sosb_state* s) {
    Optics o{};
    const sosb_dims& d = s->d;
    o.L = d.L;
    o.K = s->K;
    o.W = d.W;
    o.nh = d.nh;
    o.nc = d.nc;
    o.ns = s->ns;
    o.src = s->src;
    o.strato = d.strato;
    o.top_km = (float)d.top_km;
    o.mix = (float)d.mix;
    o.g = (float)d.g;
    o.height = (float)d.height;
    o.air_surface = (float)d.air_surface;
    o.inv_step = (float)(1.0 / d.profile_step_km);
    o.density_last = d.density_rows - 2;
    o.density_mask = d.density_mask;
    o.strato_center = (float)d.strato_center;
    o.strato_sigma = (float)d.strato_sigma;
    o.strato_norm = (float)d.strato_norm;
    o.h = P<float>(s->h);
    o.chi = P<float>(s->chi);
    o.hr = P<float>(s->hr);
    o.ext = P<float>(s->ext);
    o.asca = P<float>(s->asca);
    o.table = P<float>(s->table);
    o.n_sun_h = d.n_sun_h;
    o.n_sun_x = d.n_sun_x;
    o.sun_h = P<float>(s->sun_h);
    o.sun_col = P<float>(s->sun_col);
    o.strato_sun_col = P<float>(s->s_sun_col);
    o.gm = P<float>(s->gm);
    o.goff = P<int>(s->goff);
    o.gdir = P<float>(s->gdir);
    o.gval = P<float>(s->gval);
    o.strato_ext = P<float>(s->s_ext);
    o.strato_sca = P<float>(s->s_sca);
    o.strato_chi = P<float>(s->s_chi);
    o.sh_a = P<float>(s->sh_a);
    o.sh_b = P<float>(s->sh_b);
    o.sh_d = P<float>(s->sh_d);
    o.strato_lut = P<float>(s->s_lut);
    o.gsame = P<uint8_t>(s->gsame);
    o.strato_lut2 = P<float2>(s->s_lut2);
    o.gdir4 = P<float4>(s->gdir4);
    o.aer2_on = s->aer2_on;
    for (int i = 0; i < 7; ++i) o.aer2[i] = s->aer2[i];
    o.support = d.lower_end_km > 0.0 ? 1 : 0;
    o.lower_end = (float)d.lower_end_km;
    o.air_end = (float)d.air_end_km;
    o.tropo_bins = s->tropo_bins;
    o.tropo_lut = s->tropo_bins ? P<float>(s->t_lut) : nullptr;
    o.tropo_lut2 = s->tropo_bins ? P<float2>(s->t_lut2) : nullptr;
    return o;
}

static Rays rays_of(const BundleDev& b) {
    Rays r{};
    r.ncell = b.ncell;
    r.nray = (int)b.nray;
    r.cell_off = P<int>(b.cell_off);
    r.ray_cell = P<int>(b.ray_cell);
    r.p = P<float>(b.p);
    r.frame = P<float>(b.frame);
    r.dir = P<float4>(b.dir);
    r.dir_lo = P<float4>(b.dir_lo);
    r.dloc = P<float4>(b.dloc);
    r.seg_off = P<int>(b.seg_off);
    r.seg = P<float4>(b.seg);
    r.lower = P<uint8_t>(b.lower);
    r.end_j = P<int>(b.end_j);
    r.end_col = P<float>(b.end_col);
    r.hits = P<uint8_t>(b.hits);
    r.pcp = P<float>(b.pcp);
    return r;
}

// Drops the captured evaluation graph (its launches hold the handle's constants, pointers and modes).
static void graph_reset(sosb_state* s) {
    if (s->graph) cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
}

static int launch_check(sosb_state* s) {
    s->launches++;
    CK(cudaGetLastError());
    return 0;
}

static int take_event(sosb_state* s, cudaEvent_t& e) {
    if (!s->event_pool.empty()) {
        e = s->event_pool.back();
        s->event_pool.pop_back();
        return 0;
    }
    CK(cudaEventCreate(&e));
    return 0;
}

// Brackets one kernel launch with events on the work stream when timing is on.
struct Timer {
    sosb_state* s;
    int cls;
    cudaEvent_t a = nullptr, b = nullptr;
    Timer(sosb_state* st, int c) : s(st), cls(c) {
        if (s->timing && take_event(s, a) == 0 && take_event(s, b) == 0) cudaEventRecord(a, s->stream);
    }
    ~Timer() {
        if (s->timing && a && b) {
            cudaEventRecord(b, s->stream);
            s->timed.push_back(TimedLaunch{cls, a, b});
        }
    }
};

// Folds finished event pairs into the per-class totals.
static int collect_timing(sosb_state* s) {
    if (s->timed.empty()) return 0;
    CK(cudaStreamSynchronize(s->stream));
    for (const TimedLaunch& t : s->timed) {
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, t.a, t.b));
        s->timed_ms[t.cls] += ms;
        s->timed_count[t.cls] += 1;
        s->event_pool.push_back(t.a);
        s->event_pool.push_back(t.b);
    }
    s->timed.clear();
    return 0;
}

// Node table of bundle `b` for a launch: `read` when a valid table serves a warm launch; `write` when this launch
// covers the whole bundle and should build it (within half the free device memory).
static int table_for(sosb_state* s, BundleDev& b, int nq, bool whole, int first, NodeTable& write, bool& read) {
    write = NodeTable{nullptr, nullptr, nullptr};
    read = false;
    if (!s->tables || b.t_too_big) return 0;
    if (b.t_valid) {
        read = !first;
        return 0;
    }
    if (!whole) return 0;
    const sosb_dims& d = s->d;
    if (d.nh > 16384 || d.nc > 65536) {  // (ir << 16 | j) packing with two support bits above ir
        b.t_too_big = true;
        return 0;
    }
    const size_t nodes = (size_t)b.nseg * nq;
    const size_t need = nodes * (2 * sizeof(float4) + (size_t)d.W * sizeof(float));
    const size_t have = b.t_frame.bytes + b.t_misc.bytes + b.t_att.bytes;
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    if (need > have && need - have > (free_b + have) / 2) {
        b.t_too_big = true;
        return 0;
    }
    TRY(dalloc(s, b.t_frame, std::max<size_t>(nodes, 1) * sizeof(float4)));
    TRY(dalloc(s, b.t_misc, std::max<size_t>(nodes, 1) * sizeof(float4)));
    TRY(dalloc(s, b.t_att, std::max<size_t>(nodes * d.W, 1) * sizeof(float)));
    write = NodeTable{P<float4>(b.t_frame), P<float4>(b.t_misc), P<float>(b.t_att)};
    return 0;
}

using TableKernel = void (*)(Optics, Rays, LaneInputs, NodeTable, int, int, int, float4*);

// The table kernel instance for (W, L): one wavelength or up to four, the order unrolled for L = 16 and 32.
static TableKernel table_kernel_for(int W, int L) {
    if (W == 1) return L == 16 ? transport_table_kernel<1, 16> : (L == 32 ? transport_table_kernel<1, 32>
                                                                          : transport_table_kernel<1, 0>);
    return L == 16 ? transport_table_kernel<4, 16> : (L == 32 ? transport_table_kernel<4, 32> : transport_table_kernel<4, 0>);
}

// Row length of the padded plane layout (W <= 4), 0 for the wavelength-fastest layout of the wave kernels.
static int plane_kp(const sosb_state* s) { return s->d.W <= 4 ? (s->K + 3) & ~3 : 0; }

// Node tables hold the optics (attenuation) and must be rebuilt when the constants change; the ray-cell pairs are
// geometry only and survive new constants (`geometry` false).
static void invalidate_tables(BundleDev& b, bool geometry = true) {
    b.t_valid = false;
    b.t_too_big = false;
    if (geometry) {
        b.p_valid = false;
        b.c_valid = false;
    }
}

// (node, corner) entries of bundle b bucketed by corner cell (geometry only), the tiles of 128 entries within a cell,
// the rays' basis table and the corner-value buffer; over half the free memory: the bundle stays on the pair form.
static int build_corners(sosb_state* s, BundleDev& b, int nq) {
    b.c_valid = false;
    if (!s->corner_mma || b.nray == 0 || s->d.W <= 4) return 0;
    const sosb_dims& d = s->d;
    const int64_t nray = b.nray;
    const int64_t entries = (int64_t)b.nseg * nq * 4;
    const int kp = (s->K + 3) & ~3;
    if (entries >= (int64_t)1 << 31) return 0;
    const size_t nodes = (size_t)b.nseg * nq;
    const size_t need = (size_t)entries * (12 + (size_t)d.W * 4) + (size_t)nray * kp * sizeof(float) +
                        nodes * (4 + (size_t)d.W * 16);
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    if (need > free_b / 2) return 0;
    const int ns = s->ns;
    LocalBuf cnt, off, cursor;
    TRY(dalloc(s, cnt, (size_t)(ns + 1) * sizeof(int)));
    TRY(dalloc(s, off, (size_t)(ns + 1) * sizeof(int)));
    TRY(dalloc(s, cursor, (size_t)(ns + 1) * sizeof(int)));
    CK(cudaMemsetAsync(cnt.p, 0, (size_t)(ns + 1) * sizeof(int), s->stream));
    const NodeTable tab{P<float4>(b.t_frame), P<float4>(b.t_misc), P<float>(b.t_att)};
    const int blocks = grid_for(nray, 128);
    corner_entries_kernel<<<blocks, 128, 0, s->stream>>>(optics_of(s), rays_of(b), tab, nq, 0, P<int>(cnt), nullptr,
                                                        nullptr, nullptr, nullptr);
    TRY(launch_check(s));
    bucket_scan_kernel<<<1, 1024, 0, s->stream>>>(P<int>(cnt), ns, P<int>(off), P<int>(cursor));
    TRY(launch_check(s));
    TRY(dalloc(s, b.c_ray, (size_t)entries * sizeof(int)));
    TRY(dalloc(s, b.c_cp, (size_t)entries * sizeof(float)));
    TRY(dalloc(s, b.c_slot, (size_t)entries * sizeof(int)));
    corner_entries_fill_kernel<<<(unsigned)std::min<int64_t>((nray + 3) / 4, 152LL * 64), 128, 0, s->stream>>>(
        optics_of(s), rays_of(b), tab, nq, P<int>(cursor), P<int>(b.c_ray), P<float>(b.c_cp), P<int>(b.c_slot));
    TRY(launch_check(s));
    std::vector<int> hoff(ns + 1);
    CK(cudaMemcpyAsync(hoff.data(), off.p, (size_t)(ns + 1) * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    std::vector<int4> tiles;
    for (int c = 0; c < ns; ++c)
        for (int e = hoff[c]; e < hoff[c + 1]; e += 128) tiles.push_back(make_int4(c, e, std::min(128, hoff[c + 1] - e), 0));
    TRY(dalloc(s, b.c_tile, std::max<size_t>(tiles.size(), 1) * sizeof(int4)));
    if (!tiles.empty()) CK(cudaMemcpyAsync(b.c_tile.p, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice,
                                           s->stream));
    TRY(dalloc(s, b.y_tab, (size_t)nray * kp * sizeof(float)));
    pair_basis_kernel<<<(unsigned)((nray * 32 + 127) / 128), 128, 0, s->stream>>>(optics_of(s), rays_of(b), kp,
                                                                                 P<float>(b.y_tab));
    TRY(launch_check(s));
    TRY(dalloc(s, b.cv, (size_t)entries * d.W * sizeof(float)));
    TRY(dalloc(s, b.node_ray, std::max<size_t>(nodes, 1) * sizeof(int)));
    TRY(dalloc(s, b.vbuf, std::max<size_t>(nodes, 1) * d.W * sizeof(float4)));
    node_ray_kernel<<<blocks, 128, 0, s->stream>>>(rays_of(b), nq, P<int>(b.node_ray));
    TRY(launch_check(s));
    CK(cudaStreamSynchronize(s->stream));  // the host tile list outlives no call
    b.c_ntiles = (int)tiles.size();
    b.c_version = -1;
    b.c_valid = true;
    return 0;
}

// Ray-cell pairs of bundle b from its node table (geometry only): per-ray counts, offsets, the pairs, each node's
// four pair indices and the ray basis table. Pairs over half the free memory leave the bundle on per-node synthesis.
static int build_pairs(sosb_state* s, BundleDev& b, int nq) {
    b.p_valid = false;
    if (!s->pairs || b.nray == 0 || s->d.W <= 4) return 0;
    const sosb_dims& d = s->d;
    const int64_t nray = b.nray;
    const size_t nodes = (size_t)b.nseg * nq;
    const int kp = (s->K + 3) & ~3;
    LocalBuf cnt, cursor;
    TRY(dalloc(s, cnt, (size_t)(nray + 1) * sizeof(int)));
    TRY(dalloc(s, cursor, (size_t)(nray + 1) * sizeof(int)));
    TRY(dalloc(s, b.p_off, (size_t)(nray + 1) * sizeof(int)));
    const NodeTable tab{P<float4>(b.t_frame), P<float4>(b.t_misc), P<float>(b.t_att)};
    const int blocks = grid_for(nray, 128);
    pair_build_kernel<<<blocks, 128, 0, s->stream>>>(optics_of(s), rays_of(b), tab, nq, 0, P<int>(cnt), nullptr,
                                                     nullptr, nullptr, nullptr);
    TRY(launch_check(s));
    bucket_scan_kernel<<<1, 1024, 0, s->stream>>>(P<int>(cnt), (int)nray, P<int>(b.p_off), P<int>(cursor));
    TRY(launch_check(s));
    int total = 0, ground = 0;
    CK(cudaMemcpyAsync(&total, P<int>(b.p_off) + nray, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    const int64_t r_gnd = (int64_t)b.host_cell_off.size() > d.nc ? b.host_cell_off[d.nc] : 0;
    CK(cudaMemcpyAsync(&ground, P<int>(b.p_off) + r_gnd, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    TRY(dfree(s, cnt));
    TRY(dfree(s, cursor));
    const size_t a_bytes = (size_t)total * (d.L + 1) * d.W * sizeof(float);
    const size_t need = (size_t)total * 8 + nodes * sizeof(int4) + (size_t)nray * kp * sizeof(float) +
                        (a_bytes > b.pair_A.bytes ? a_bytes - b.pair_A.bytes : 0);
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    if (need > free_b / 2) return 0;
    TRY(dalloc(s, b.p_cell, std::max<size_t>(total, 1) * sizeof(int)));
    TRY(dalloc(s, b.p_ray, std::max<size_t>(total, 1) * sizeof(int)));
    TRY(dalloc(s, b.p_node, std::max<size_t>(nodes, 1) * sizeof(int4)));
    TRY(dalloc(s, b.pair_A, std::max<size_t>(a_bytes, 16)));
    pair_build_kernel<<<blocks, 128, 0, s->stream>>>(optics_of(s), rays_of(b), tab, nq, 1, nullptr, P<int>(b.p_off),
                                                     P<int>(b.p_cell), P<int>(b.p_ray), P<int4>(b.p_node));
    TRY(launch_check(s));
    TRY(dalloc(s, b.y_tab, (size_t)nray * kp * sizeof(float)));
    pair_basis_kernel<<<(unsigned)((nray * 32 + 127) / 128), 128, 0, s->stream>>>(optics_of(s), rays_of(b), kp,
                                                                                 P<float>(b.y_tab));
    TRY(launch_check(s));
    b.a_version = -1;
    b.p_total = total;
    b.p_ground = ground;
    b.p_valid = true;
    return 0;
}

// ------------------------------------------------------------------------------------------------ autotuner
// Warps per ray of the table launches (1, 2 or 4): with autotuning on, the first table launch of a shape (rays of
// the launch, segments, nodes per segment, W, L, cells) times each choice twice with CUDA events on the work stream
// and keeps the fastest for the process; otherwise (or while a graph is being captured) the choice follows the mean
// nodes per ray (4 warps from 96, 2 from 48). The launch that follows uses the chosen value, so results do not
// depend on which candidate ran last.
struct TuneKey {
    int64_t nray, nseg;
    int nq, W, L, ns, kind;  // kind: 0 table kernel
    bool operator<(const TuneKey& o) const {
        return std::tie(nray, nseg, nq, W, L, ns, kind) < std::tie(o.nray, o.nseg, o.nq, o.W, o.L, o.ns, o.kind);
    }
};
static std::mutex g_tune_lock;
static std::map<TuneKey, int> g_tuned;

template <class Launch>
static int tuned_wpr(sosb_state* s, const BundleDev& b, int nq, int64_t nray, int kind, Launch launch, int& wpr) {
    const double mean_nodes = (double)b.nseg * nq / std::max<int64_t>(b.nray, 1);
    wpr = mean_nodes >= 96.0 ? 4 : (mean_nodes >= 48.0 ? 2 : 1);
    if (!s->autotune) return 0;
    const TuneKey key{nray, b.nseg, nq, s->d.W, s->d.L, s->ns, kind};
    {
        std::lock_guard<std::mutex> guard(g_tune_lock);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) {
            wpr = it->second;
            return 0;
        }
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(s->stream, &cap));
    if (cap != cudaStreamCaptureStatusNone) return 0;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best = 1e30f;
    int best_wpr = wpr;
    for (int cand : {1, 2, 4}) {
        float t = 1e30f;
        for (int rep = 0; rep < 2; ++rep) {
            CK(cudaEventRecord(e0, s->stream));
            launch(cand);
            CK(cudaGetLastError());
            CK(cudaEventRecord(e1, s->stream));
            CK(cudaEventSynchronize(e1));
            float ms = 0.0f;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            t = std::min(t, ms);
        }
        if (t < best) {
            best = t;
            best_wpr = cand;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    s->launches += 6;
    wpr = best_wpr;
    std::lock_guard<std::mutex> guard(g_tune_lock);
    g_tuned[key] = wpr;
    return 0;
}

// Staged first light of the whole cell bundle (FirstLightBufs). Returns 0 with `done` false when the scratch does
// not fit, leaving the single-launch path to the caller.
static int run_first_light_staged(sosb_state* s, BundleDev& b, const LaneInputs& in, const NodeTable& table,
                                  bool& done) {
    done = false;
    const sosb_dims& d = s->d;
    const int W = d.W;
    const long long nodes = (long long)b.nseg * in.nq;
    if (nodes >= (1LL << 30)) return 0;  // pair codes node * 2 + pr are int
    const size_t need = (size_t)nodes * ((size_t)W * (16 + 8 + 16) + 16 + 8) + (size_t)(3 * s->ns + 2) * 4;
    const size_t have = s->fl_val0.bytes + s->fl_coef.bytes + s->fl_dir.bytes + s->fl_g.bytes + s->fl_entries.bytes;
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    if (need > have && need - have > (free_b + have) / 2) return 0;
    const size_t n1 = std::max<long long>(nodes, 1);
    TRY(dalloc(s, s->fl_val0, n1 * W * sizeof(float4)));
    TRY(dalloc(s, s->fl_coef, n1 * W * sizeof(float2)));
    TRY(dalloc(s, s->fl_dir, n1 * sizeof(float4)));
    TRY(dalloc(s, s->fl_g, n1 * 2 * W * sizeof(float2)));
    TRY(dalloc(s, s->fl_entries, n1 * 2 * sizeof(int)));
    TRY(dalloc(s, s->fl_cnt, (size_t)(s->ns + 1) * sizeof(int)));
    TRY(dalloc(s, s->fl_off, (size_t)(s->ns + 1) * sizeof(int)));
    TRY(dalloc(s, s->fl_cursor, (size_t)(s->ns + 1) * sizeof(int)));
    const FirstLightBufs fl{P<float4>(s->fl_val0), P<float2>(s->fl_coef), P<float4>(s->fl_dir), P<float2>(s->fl_g)};
    const Optics o = optics_of(s);
    const Rays r = rays_of(b);
    const long long blocks = (b.nray * 32 + TRANSPORT_THREADS - 1) / TRANSPORT_THREADS;
    const int nb = (int)std::min<long long>((nodes + 255) / 256, 152LL * 8);
    const int wchunks = (W + 31) / 32;
    const long long wave_blocks = (b.nray * wchunks + WAVE_WARPS - 1) / WAVE_WARPS;
    Timer timer(s, K_TRANSPORT);
    if (W == 1)
        transport_warp_kernel<1, true><<<(unsigned)blocks, TRANSPORT_THREADS, warp_smem(s->K), s->stream>>>(
            o, r, in, table, fl, 0, (int)b.nray, P<float4>(s->rad));
    else if (W <= 4)
        transport_warp_kernel<4, true><<<(unsigned)blocks, TRANSPORT_THREADS, warp_smem(s->K), s->stream>>>(
            o, r, in, table, fl, 0, (int)b.nray, P<float4>(s->rad));
    else
        transport_wave_kernel<true><<<(unsigned)wave_blocks, WAVE_WARPS * 32, wave_smem(d.L), s->stream>>>(
            o, r, in, table, fl, 0, (int)b.nray, wchunks, P<float4>(s->rad));
    TRY(launch_check(s));
    CK(cudaMemsetAsync(s->fl_cnt.p, 0, (size_t)(s->ns + 1) * sizeof(int), s->stream));
    CK(cudaMemsetAsync(s->fl_g.p, 0, (size_t)nodes * 2 * W * sizeof(float2), s->stream));
    pair_bucket_kernel<<<std::max(nb, 1), 256, 0, s->stream>>>(o, table.misc, nodes, P<int>(s->fl_cnt), nullptr,
                                                               nullptr);
    TRY(launch_check(s));
    bucket_scan_kernel<<<1, 1024, 0, s->stream>>>(P<int>(s->fl_cnt), s->ns, P<int>(s->fl_off), P<int>(s->fl_cursor));
    TRY(launch_check(s));
    pair_bucket_kernel<<<std::max(nb, 1), 256, 0, s->stream>>>(o, table.misc, nodes, nullptr, P<int>(s->fl_cursor),
                                                               P<int>(s->fl_entries));
    TRY(launch_check(s));
    if (W <= 4) {
        const int gb = (int)((2 * nodes + 255) / 256);  // one pair per thread at most
        if (W == 1)
            ground_pairs_kernel<1><<<std::max(gb, 1), 256, 0, s->stream>>>(o, table.misc, fl.dir,
                                                                           P<int>(s->fl_entries),
                                                                           P<int>(s->fl_off) + s->ns, fl.g);
        else
            ground_pairs_kernel<4><<<std::max(gb, 1), 256, 0, s->stream>>>(o, table.misc, fl.dir,
                                                                           P<int>(s->fl_entries),
                                                                           P<int>(s->fl_off) + s->ns, fl.g);
    } else if (s->ground_mma && !s->tropo_bins && (!d.strato || s->g_rank > 0)) {
        // tiles of the buckets on the device (no host round trip), then one CTA per tile; CTAs beyond the count
        // leave at once (at most one partial tile per bucket above items / 128)
        TRY(dalloc(s, s->gt_cnt, (size_t)(s->ns + 1) * sizeof(int)));
        TRY(dalloc(s, s->gt_off, (size_t)(s->ns + 1) * sizeof(int)));
        TRY(dalloc(s, s->gt_cursor, (size_t)(s->ns + 1) * sizeof(int)));
        const long long max_tiles = (2 * nodes + GTC_ROWS - 1) / GTC_ROWS + s->ns;
        TRY(dalloc(s, s->gt_tile, (size_t)max_tiles * sizeof(int4)));
        const int tb = (s->ns + 255) / 256;
        ground_tiles_kernel<<<tb, 256, 0, s->stream>>>(P<int>(s->fl_off), s->ns, 0, P<int>(s->gt_cnt), nullptr,
                                                      nullptr);
        TRY(launch_check(s));
        bucket_scan_kernel<<<1, 1024, 0, s->stream>>>(P<int>(s->gt_cnt), s->ns, P<int>(s->gt_off),
                                                       P<int>(s->gt_cursor));
        TRY(launch_check(s));
        ground_tiles_kernel<<<tb, 256, 0, s->stream>>>(P<int>(s->fl_off), s->ns, 1, nullptr, P<int>(s->gt_off),
                                                      P<int4>(s->gt_tile));
        TRY(launch_check(s));
        const int np = (W + 15) / 16 * 16;
        const int acc_cols = d.strato ? 2 * np : np;
        const uint32_t cols = acc_cols <= 32 ? 32u : (acc_cols <= 64 ? 64u : 128u);
        const GroundTc gt{P<int>(s->fl_entries), P<int4>(s->gt_tile), P<int>(s->gt_off) + s->ns,
                          P<float2>(s->g_su2), P<float>(s->g_sv), s->g_rank};
        ground_tc_kernel<<<(unsigned)max_tiles, GTC_THREADS, ground_tc_smem(np), s->stream>>>(
            o, table.misc, fl.dir, gt, np, tcx::idesc_bf16(128, np), cols, fl.g);
        s->corner_used = true;  // the bounded waits' flags are read by proj_check
    } else {
        const int gb = (int)std::min<long long>((2 * nodes + GPW_WARPS - 1) / GPW_WARPS, 152LL * 32);
        ground_pairs_warp_kernel<<<std::max(gb, 1), GPW_WARPS * 32, 0, s->stream>>>(
            o, table.misc, fl.dir, P<int>(s->fl_entries), P<int>(s->fl_off) + s->ns, fl.g);
    }
    TRY(launch_check(s));
    if (W == 1)
        first_light_sum_kernel<1><<<(unsigned)blocks, TRANSPORT_THREADS, 0, s->stream>>>(o, r, in, table, fl, 0,
                                                                                          (int)b.nray,
                                                                                          P<float4>(s->rad));
    else if (W <= 4)
        first_light_sum_kernel<4><<<(unsigned)blocks, TRANSPORT_THREADS, 0, s->stream>>>(o, r, in, table, fl, 0,
                                                                                          (int)b.nray,
                                                                                          P<float4>(s->rad));
    else
        first_light_sum_wave_kernel<<<(unsigned)((b.nray * wchunks * 32 + 127) / 128), 128, 0, s->stream>>>(
            o, r, in, table, fl, 0, (int)b.nray, wchunks, P<float4>(s->rad));
    TRY(launch_check(s));
    b.t_valid = true;
    if (!b.c_valid) TRY(build_corners(s, b, in.nq));
    if (!b.c_valid && !b.p_valid) TRY(build_pairs(s, b, in.nq));
    done = true;
    return 0;
}

// transport of rays [ray0, ray0 + nray) of bundle `b` into s->rad
static int run_transport(sosb_state* s, BundleDev& b, int64_t ray0, int64_t nray, const float* field,
                         const float* boundary, int first, bool query) {
    if (nray <= 0) return 0;
    const sosb_dims& d = s->d;
    TRY(dalloc(s, s->rad, (size_t)b.nray * d.W * sizeof(float4)));
    LaneInputs in{};
    in.field = field;
    in.plane = P<float>(s->plane);
    in.kp = plane_kp(s);
    in.boundary = boundary;
    in.first = first;
    if (query) {
        in.u_hi = P<float>(s->uq_hi);
        in.u_lo = P<float>(s->uq_lo);
        in.wu_hi = P<float>(s->wuq_hi);
        in.wu_lo = P<float>(s->wuq_lo);
        in.nq = d.nq_query;
    } else {
        in.u_hi = P<float>(s->u_hi);
        in.u_lo = P<float>(s->u_lo);
        in.wu_hi = P<float>(s->wu_hi);
        in.wu_lo = P<float>(s->wu_lo);
        in.nq = d.nq;
    }
    NodeTable write;
    bool read = false;
    TRY(table_for(s, b, in.nq, ray0 == 0 && nray == b.nray, first, write, read));
    const NodeTable table{P<float4>(b.t_frame), P<float4>(b.t_misc), P<float>(b.t_att)};
    if (first && !query && ray0 == 0 && nray == b.nray && (write.frame || b.t_valid)) {
        bool done = false;
        TRY(run_first_light_staged(s, b, in, table, done));
        if (done) return 0;
    }
    const FirstLightBufs no_fl{nullptr, nullptr, nullptr, nullptr};
    bool table_only = false;
    if (d.W <= 4) {
        // sample-parallel: one warp per ray
        const long long blocks = (nray * 32 + TRANSPORT_THREADS - 1) / TRANSPORT_THREADS;
        const size_t smem = warp_smem(s->K);
        Timer timer(s, read ? K_TABLE : K_TRANSPORT);
        if (read) {
            const TableKernel kernel = table_kernel_for(d.W, d.L);
            auto launch = [&](int wpr) {
                const long long tblocks = (nray * wpr + TRANSPORT_THREADS / 32 - 1) / (TRANSPORT_THREADS / 32);
                kernel<<<(unsigned)tblocks, TRANSPORT_THREADS, smem, s->stream>>>(optics_of(s), rays_of(b), in, table,
                                                                                 (int)ray0, (int)nray, wpr,
                                                                                 P<float4>(s->rad));
            };
            int wpr = 0;
            TRY(tuned_wpr(s, b, in.nq, nray, 0, launch, wpr));
            launch(wpr);
        } else if (d.W == 1)
            transport_warp_kernel<1, false><<<(unsigned)blocks, TRANSPORT_THREADS, smem, s->stream>>>(
                optics_of(s), rays_of(b), in, write, no_fl, (int)ray0, (int)nray, P<float4>(s->rad));
        else
            transport_warp_kernel<4, false><<<(unsigned)blocks, TRANSPORT_THREADS, smem, s->stream>>>(
                optics_of(s), rays_of(b), in, write, no_fl, (int)ray0, (int)nray, P<float4>(s->rad));
    } else {
        // many wavelengths: one warp per (ray, chunk of 32 wavelengths), geometry shared through shared memory
        const int wchunks = (d.W + 31) / 32;
        const long long warps = (long long)nray * wchunks;
        const long long blocks = (warps + WAVE_WARPS - 1) / WAVE_WARPS;
        Timer timer(s, read ? K_TABLE : K_TRANSPORT);
        if (read && b.c_valid) {
            if (b.c_version != s->plane_version) {
                // corner values of every (node, corner) entry of the bundle against the current plane (reused by the
                // launches that follow on the same plane: the ground and the warm pass of one apply)
                const int np = (d.W + 15) / 16 * 16;
                const uint32_t cols = np <= 32 ? 32u : 64u;
                const size_t smem = corner_tc_smem(np, d.L);
                const CornerEntries ce{P<int>(b.c_ray), P<float>(b.c_cp), P<int>(b.c_slot), P<int4>(b.c_tile)};
                if (b.c_ntiles > 0) {
                    Timer ct(s, K_CORNER);
                    corner_tc_kernel<<<(unsigned)b.c_ntiles, CORNER_THREADS, smem, s->stream>>>(
                        optics_of(s), ce, P<float>(b.y_tab), (s->K + 3) & ~3, P<uint4>(s->plane_tiles), np,
                        tcx::idesc_bf16(128, np), cols, P<float>(b.cv));
                    TRY(launch_check(s));
                    s->corner_used = true;
                }
                b.c_version = s->plane_version;
            }
            const long long nd0 = (long long)b.host_seg_off_at(ray0) * in.nq;
            const long long nd1 = (long long)b.host_seg_off_at(ray0 + nray) * in.nq;
            corner_node_kernel<<<grid_for((nd1 - nd0) * d.W, 256), 256, 0, s->stream>>>(
                optics_of(s), rays_of(b), table, P<int>(b.node_ray), P<float>(b.cv), field, nd0, nd1 - nd0,
                P<float4>(b.vbuf));
            TRY(launch_check(s));
            ray_sum_kernel<<<grid_for(nray * d.W, 256), 256, 0, s->stream>>>(optics_of(s), rays_of(b), in,
                                                                          P<float4>(b.vbuf), (int)ray0, (int)nray,
                                                                          P<float4>(s->rad));
        } else if (read && b.p_valid) {
            const PairTable pt{P<int>(b.p_off), P<int>(b.p_cell), P<int>(b.p_ray), P<int4>(b.p_node),
                               P<float>(b.y_tab), P<float>(b.pair_A)};
            if (b.a_version != s->plane_version) {
                // contractions of every pair of the bundle against the current plane (reused by the launches that
                // follow on the same plane: the ground and the warm pass of one apply)
                const int kp = (s->K + 3) & ~3;
                if (b.p_total > 0) {
                    const unsigned cg = (unsigned)((b.p_total * wchunks * 32 + 127) / 128);
                    const auto contract = d.L == 16 ? pair_contract_wave_kernel<16>
                                                    : (d.L == 32 ? pair_contract_wave_kernel<32>
                                                                 : pair_contract_wave_kernel<0>);
                    contract<<<cg, 128, 0, s->stream>>>(optics_of(s), pt, in.plane, (int)b.p_total, kp, wchunks);
                    TRY(launch_check(s));
                }
                b.a_version = s->plane_version;
            }
            const unsigned pb = (unsigned)((warps + PAIR_WAVE_WARPS - 1) / PAIR_WAVE_WARPS);
            transport_pair_wave_kernel<<<pb, PAIR_WAVE_WARPS * 32, 0, s->stream>>>(
                optics_of(s), rays_of(b), in, table, pt, (int)ray0, (int)nray, wchunks, P<float4>(s->rad));
        } else if (read) {
            auto kernel = d.L == 16 ? transport_table_wave_kernel<16>
                                    : (d.L == 32 ? transport_table_wave_kernel<32> : transport_table_wave_kernel<0>);
            kernel<<<(unsigned)blocks, WAVE_WARPS * 32, table_wave_smem(d.L), s->stream>>>(
                optics_of(s), rays_of(b), in, table, (int)ray0, (int)nray, wchunks, P<float4>(s->rad));
        } else {
            // a warm launch that writes the table: with the corner values on the tensor cores it writes the table
            // only, then the bundle's corner entries are built and the launch is served by the corner path below
            LaneInputs win = in;
            win.table_only = write.frame && !first && s->corner_mma ? 1 : 0;
            table_only = win.table_only != 0;
            transport_wave_kernel<false><<<(unsigned)blocks, WAVE_WARPS * 32, wave_smem(d.L), s->stream>>>(
                optics_of(s), rays_of(b), win, write, no_fl, (int)ray0, (int)nray, wchunks, P<float4>(s->rad));
        }
    }
    TRY(launch_check(s));
    if (write.frame) {
        b.t_valid = true;
        if (!b.c_valid) TRY(build_corners(s, b, in.nq));
        if (table_only && !b.c_valid) {
            // no room for the corner entries: the pairs or the per-lane synthesis from the table serve the launch
            if (!b.p_valid) TRY(build_pairs(s, b, in.nq));
            return run_transport(s, b, ray0, nray, field, boundary, first, query);
        }
        if (!b.c_valid && !b.p_valid) TRY(build_pairs(s, b, in.nq));
        if (table_only) return run_transport(s, b, ray0, nray, field, boundary, first, query);
    }
    return 0;
}

// Basis table of the tensor-core projection for the cell bundle in the current projection mode.
static int ensure_basis(sosb_state* s, BundleDev& b) {
    const int mode = s->proj_mode;
    if (b.b_mode == mode) return 0;
    const sosb_dims& d = s->d;
    const int esz = mode == PROJ_TF32 ? 4 : 2, ch = 128 / esz;
    int64_t rmax = 0;
    for (int c = 0; c < b.ncell; ++c) rmax = std::max(rmax, b.host_cell_off[c + 1] - b.host_cell_off[c]);
    const int kpad = (s->K + 127) / 128 * 128;
    const int rpad = (int)std::max<int64_t>(ch, (rmax + ch - 1) / ch * ch);
    const size_t bytes = (size_t)b.ncell * kpad * rpad * esz;
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    if (bytes * (mode == PROJ_BF16X3 ? 2 : 1) > (free_b + b.b_hi.bytes + b.b_lo.bytes) / 2)
        return fail(s, "E_MEMORY: projection basis table of %zu bytes", bytes);
    TRY(dalloc(s, b.b_hi, bytes));
    CK(cudaMemsetAsync(b.b_hi.p, 0, bytes, s->stream));
    if (mode == PROJ_BF16X3) {
        TRY(dalloc(s, b.b_lo, bytes));
        CK(cudaMemsetAsync(b.b_lo.p, 0, bytes, s->stream));
    }
    const BasisTable bt{b.b_hi.p, b.b_lo.p, kpad, rpad};
    const int blocks = grid_for(b.nray * (int64_t)(d.L + 1), 256);
    if (mode == PROJ_BF16X3)
        basis_table_kernel<PROJ_BF16X3><<<blocks, 256, 0, s->stream>>>(optics_of(s), rays_of(b), bt);
    else if (mode == PROJ_TF32)
        basis_table_kernel<PROJ_TF32><<<blocks, 256, 0, s->stream>>>(optics_of(s), rays_of(b), bt);
    else
        basis_table_kernel<PROJ_BF16><<<blocks, 256, 0, s->stream>>>(optics_of(s), rays_of(b), bt);
    TRY(launch_check(s));
    b.b_mode = mode;
    b.b_kpad = kpad;
    b.b_rpad = rpad;
    return 0;
}

// Moments of `ncell` cells from s->rad: Rayleigh rows and ground flux on the CUDA cores (compensated FP32); the SH
// rows there too (PROJ_FP32) or on the tensor cores (the other projection forms).
static int run_project(sosb_state* s, BundleDev& b, int ncell, bool ground_only, float* moments, float* flux) {
    if (ncell <= 0) return 0;
    const sosb_dims& d = s->d;
    const bool tc = s->proj_mode != PROJ_FP32 && !ground_only;
    if (tc) TRY(ensure_basis(s, b));
    const int nout = tc ? 4 * d.W : (4 + s->K) * d.W;
    const size_t smem = project_smem(s->K, d.W);
    const float flux_scale = (float)(d.albedo / M_PI);
    const int per_pass = PROJ_THREADS * PROJ_OWN;
    const int passes = ground_only ? 1 : (nout + per_pass - 1) / per_pass;
    for (int pass = 0; pass < passes; ++pass) {
        Timer timer(s, K_PROJECT);
        project_kernel<<<ncell, PROJ_THREADS, smem, s->stream>>>(optics_of(s), rays_of(b), P<float4>(s->rad), 0,
                                                                 ground_only ? 1 : 0, tc ? 1 : 0, pass * per_pass,
                                                                 moments, pass == 0 ? flux : nullptr, flux_scale);
        TRY(launch_check(s));
    }
    if (tc) {
        const int np = (d.W + 15) / 16 * 16;
        const uint32_t cols = np <= 32 ? 32u : 64u;
        const uint32_t idesc = s->proj_mode == PROJ_TF32 ? tcx::idesc_tf32(128, np) : tcx::idesc_bf16(128, np);
        const BasisTable bt{b.b_hi.p, b.b_lo.p, b.b_kpad, b.b_rpad};
        const dim3 grid(b.b_kpad / 128, ncell);
        const size_t tsm = project_tc_smem(s->proj_mode, np);
        Timer timer(s, K_PROJECT);
        if (s->proj_mode == PROJ_BF16X3)
            project_tc_kernel<PROJ_BF16X3><<<grid, 128, tsm, s->stream>>>(bt, rays_of(b), P<float4>(s->rad), d.W,
                                                                          s->K, np, idesc, cols, moments);
        else if (s->proj_mode == PROJ_TF32)
            project_tc_kernel<PROJ_TF32><<<grid, 128, tsm, s->stream>>>(bt, rays_of(b), P<float4>(s->rad), d.W, s->K,
                                                                        np, idesc, cols, moments);
        else
            project_tc_kernel<PROJ_BF16><<<grid, 128, tsm, s->stream>>>(bt, rays_of(b), P<float4>(s->rad), d.W, s->K,
                                                                        np, idesc, cols, moments);
        TRY(launch_check(s));
    }
    return 0;
}

// Bounded waits of the tensor-core projection that ran out since the last check (synchronises the stream).
static int proj_check(sosb_state* s) {
    if (s->proj_mode == PROJ_FP32 && !s->corner_used) return 0;
    s->corner_used = false;
    unsigned flags = 0;
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaMemcpyFromSymbol(&flags, g_proj_error, sizeof flags));
    if (flags) {
        const unsigned zero = 0;
        CK(cudaMemcpyToSymbol(g_proj_error, &zero, sizeof zero));
        return fail(s, "E_TC_TIMEOUT: a tensor-core wait ran out (flags %u: 1 projection, 2 corner values, 4 ground sums)",
                    flags);
    }
    return 0;
}

static int run_plane(sosb_state* s, const float* field) {
    if (s->plane_keep && s->plane_field == field) {  // the plane of this field is current (eval_body)
        s->plane_keep = false;
        return 0;
    }
    s->plane_keep = false;
    s->plane_field = field;
    const sosb_dims& d = s->d;
    const int kp = plane_kp(s);
    const long long n = (long long)s->ns * (kp ? kp : s->K) * d.W;
    TRY(dalloc(s, s->plane, n * sizeof(float)));
    ++s->plane_version;
    Timer timer(s, K_PLANE);
    plane_kernel<<<grid_for(n, 256), 256, 0, s->stream>>>(field, P<float>(s->ha), P<float>(s->s_density), d.nc, s->K,
                                                          s->src, d.W, d.strato, kp, n, P<float>(s->plane));
    TRY(launch_check(s));
    if (s->corner_mma && d.W > 4) {
        // the corner products' B tiles of this plane
        const int np = (d.W + 15) / 16 * 16, nchunk = (s->K + 63) / 64;
        TRY(dalloc(s, s->plane_tiles, (size_t)s->ns * nchunk * 2 * np * 128));
        const long long nt = (long long)s->ns * nchunk * 8 * np;
        plane_tiles_kernel<<<grid_for(nt, 256), 256, 0, s->stream>>>(P<float>(s->plane), s->ns, s->K, d.W, np, nchunk,
                                                                     P<uint8_t>(s->plane_tiles));
        TRY(launch_check(s));
    }
    return 0;
}

static int check_ready(sosb_state* s, bool need_obs) {
    if (!s->have_constants) return fail(s, "E_STATE: constants not set");
    if (s->cells.nray == 0) return fail(s, "E_STATE: cell bundle not set");
    if (need_obs && s->obs.nray == 0) return fail(s, "E_STATE: observer bundle not set");
    return 0;
}

static int evaluate_impl(sosb_state* s, int phase, int first, const float* field, const float* boundary,
                         float* moments, float* flux, float* radiance) {
    const sosb_dims& d = s->d;
    TRY(check_ready(s, phase == 2));
    if (phase == 2) {
        if (!first) TRY(run_plane(s, field));
        TRY(run_transport(s, s->obs, 0, s->obs.nray, field, nullptr, first, true));
        if (radiance)
            CK(cudaMemcpyAsync(radiance, s->rad.p, (size_t)s->obs.nray * d.W * sizeof(float4), cudaMemcpyDeviceToDevice,
                               s->stream));
        return 0;
    }
    if (!first) TRY(run_plane(s, field));
    if (phase == 1) {
        const int64_t nray = s->cells.host_cell_off[d.nc];
        TRY(run_transport(s, s->cells, 0, nray, field, nullptr, first, false));
        TRY(run_project(s, s->cells, d.nc, true, nullptr, flux));
        return 0;
    }
    TRY(run_transport(s, s->cells, 0, s->cells.nray, field, boundary, first, false));
    TRY(run_project(s, s->cells, s->ns, false, moments, flux));
    if (radiance)
        CK(cudaMemcpyAsync(radiance, s->rad.p, (size_t)s->cells.nray * d.W * sizeof(float4), cudaMemcpyDeviceToDevice,
                           s->stream));
    return 0;
}

static int ensure_first(sosb_state* s) {
    if (s->have_first) return 0;
    const sosb_dims& d = s->d;
    TRY(dalloc(s, s->first_moments, (size_t)s->ns * (4 + s->K) * d.W * sizeof(float)));
    TRY(dalloc(s, s->first_flux, (size_t)s->ns * d.W * sizeof(float)));
    TRY(evaluate_impl(s, 0, 1, nullptr, nullptr, P<float>(s->first_moments), P<float>(s->first_flux), nullptr));
    s->have_first = true;
    return 0;
}

// Solver.apply: returns metrics on device in s->metrics (reset here)
static int apply_impl(sosb_state* s, const float* field, float* out, unsigned long long done_mask,
                      const unsigned long long* done_dev = nullptr) {
    const sosb_dims& d = s->d;
    TRY(check_ready(s, false));
    TRY(ensure_first(s));
    const size_t nmom = (size_t)s->ns * (4 + s->K) * d.W;
    TRY(dalloc(s, s->moments, nmom * sizeof(float)));
    TRY(dalloc(s, s->flux, (size_t)s->ns * d.W * sizeof(float)));
    TRY(dalloc(s, s->boundary, (size_t)d.nc * d.W * sizeof(float)));
    TRY(dalloc(s, s->metrics, 3 * 64 * sizeof(unsigned)));
    // ground pass over the surface cells, then the boundary = ground flux + first-light flux
    TRY(evaluate_impl(s, 1, 0, field, nullptr, nullptr, P<float>(s->flux), nullptr));
    const int nb = d.nc * d.W;
    {
    Timer timer(s, K_OTHER);
    add_kernel<<<(nb + 255) / 256, 256, 0, s->stream>>>(P<float>(s->flux), P<float>(s->first_flux), P<float>(s->boundary),
                                                        nb);
    }
    TRY(launch_check(s));
    // warm pass (the plane of `field` is already current)
    TRY(run_transport(s, s->cells, 0, s->cells.nray, field, P<float>(s->boundary), 0, false));
    TRY(run_project(s, s->cells, s->ns, false, P<float>(s->moments), P<float>(s->flux)));
    CK(cudaMemsetAsync(s->metrics.p, 0, 3 * 64 * sizeof(unsigned), s->stream));
    const long long n = (long long)s->ns * s->src * d.W;
    Timer timer(s, K_COMPOSE);
    compose_kernel<<<grid_for(n, wave_threads(d.W)), wave_threads(d.W), 0, s->stream>>>(
        P<float>(s->moments), P<float>(s->first_moments), field, P<float>(s->rf), P<float>(s->af), P<float>(s->asca),
        P<float>(s->ext0), P<float>(s->s_eigen), P<float>(s->s_sca_src), s->K, s->src, d.W, s->af_w, n, done_mask, done_dev,
        out,
        P<unsigned>(s->metrics));
    return launch_check(s);
}

// Observer boxes of `field` into device memory (engine_core.Solver.boxes), no synchronisation.
static int boxes_dev(sosb_state* s, const float* field, double* out_dev) {
    const sosb_dims& d = s->d;
    TRY(check_ready(s, true));
    if (s->obs.nray < (int64_t)d.n_monitor_rows * d.n_dirs * d.box_points)
        return fail(s, "E_SHAPE: %lld observer rays for %d x %d boxes of %d points", (long long)s->obs.nray,
                    d.n_monitor_rows, d.n_dirs, d.box_points);
    TRY(run_plane(s, field));
    TRY(run_transport(s, s->obs, 0, s->obs.nray, field, nullptr, 0, true));
    const int n = d.n_monitor_rows * d.n_dirs * d.W;
    Timer timer(s, K_BOXES);
    boxes_kernel<<<(n + 127) / 128, 128, 0, s->stream>>>(P<float4>(s->rad), P<double>(s->box_ww), P<double>(s->solar),
                                                        d.n_monitor_rows, d.n_dirs, d.box_points, d.W, out_dev);
    return launch_check(s);
}

static int boxes_impl(sosb_state* s, const float* field, double* out_host) {
    const sosb_dims& d = s->d;
    const int n = d.n_monitor_rows * d.n_dirs * d.W;
    TRY(dalloc(s, s->boxes, n * sizeof(double)));
    TRY(boxes_dev(s, field, P<double>(s->boxes)));
    CK(cudaMemcpyAsync(out_host, s->boxes.p, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return collect_timing(s);
}

// Runs fn(i) for i < n on `threads` host threads with the caller's device current.
template <class F>
static void run_parallel(int n, int threads, F fn) {
    int dev = 0;
    cudaGetDevice(&dev);
    const int nt = std::max(1, std::min(threads > 0 ? threads : n, n));
    std::atomic<int> next(0);
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&]() {
            cudaSetDevice(dev);
            for (int i = next++; i < n; i = next++) fn(i);
        });
    for (auto& t : pool) t.join();
}

// ------------------------------------------------------------------------------------------------ C ABI
extern "C" {

const char* sosb_version(void) { return SOSB_VERSION; }

const char* sosb_last_error(sosb_handle h) { return h ? h->err.c_str() : "E_HANDLE: null handle"; }

int sosb_create(const sosb_dims* dims, sosb_handle* out) {
    if (!dims || !out) return 1;
    *out = nullptr;
    const sosb_dims& d = *dims;
    if (d.L < 2 || d.L > MAX_L || d.W < 1 || d.W > 64 || d.nh < 2 || d.nc < 2 || d.nq < 1 || d.nq_query < 1 ||
        d.density_rows < 2 || d.n_sun_h < 2 || d.n_sun_x < 2 || d.n_dirs < 1 || d.box_points < 1 || d.monitors < 1 ||
        d.n_monitor_rows < d.monitors)
        return 2;
    sosb_state* s = new sosb_state();
    s->d = d;
    s->K = (d.L + 1) * (d.L + 2) / 2;
    s->src = 10 + s->K * (d.strato ? 2 : 1);
    s->ns = d.nh * d.nc;
    cudaError_t e = cudaStreamCreateWithFlags(&s->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete s;
        return 3;
    }
    s->stream = s->own;
    {
        // Dynamic shared memory of the kernels whose needs depend on L, K and W: every handle's sizes must fit the
        // device's opt-in limit, and the limit itself is what the attributes are set to, so that handles of
        // different sizes in one process never lower a bound another handle relies on.
        int dev = 0, optin = 0;
        const int K = (d.L + 1) * (d.L + 2) / 2;
        const size_t need = std::max({table_wave_smem(d.L), project_smem(K, d.W), wave_smem(d.L), warp_smem(K)});
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
            need > (size_t)optin) {
            cudaStreamDestroy(s->own);
            delete s;
            return 5;
        }
        const void* fns[] = {(const void*)transport_table_wave_kernel<16>, (const void*)transport_table_wave_kernel<32>,
                             (const void*)transport_table_wave_kernel<0>, (const void*)project_kernel,
                             (const void*)transport_wave_kernel<false>, (const void*)transport_wave_kernel<true>,
                             (const void*)transport_warp_kernel<1, false>, (const void*)transport_warp_kernel<4, false>,
                             (const void*)transport_warp_kernel<1, true>, (const void*)transport_warp_kernel<4, true>,
                             (const void*)corner_tc_kernel, (const void*)ground_tc_kernel,
                             (const void*)project_tc_kernel<PROJ_BF16X3>,
                             (const void*)project_tc_kernel<PROJ_TF32>, (const void*)project_tc_kernel<PROJ_BF16>};
        for (const void* fn : fns)
            if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin) != cudaSuccess) {
                cudaStreamDestroy(s->own);
                delete s;
                return 5;
            }
    }
    // FP32 SH recurrence constants
    std::vector<float> a, b, dd;
    sh_recurrence(d.L, a, b, dd);
    if (dput_vec(s, s->sh_a, a) || dput_vec(s, s->sh_b, b) || dput_vec(s, s->sh_d, dd)) {
        sosb_destroy(s);
        return 4;
    }
    *out = s;
    return 0;
}

int sosb_destroy(sosb_handle s) {
    if (!s) return 0;
    cudaStreamSynchronize(s->stream);
    DevBuf* bufs[] = {&s->h, &s->chi, &s->hr, &s->ha, &s->ext, &s->asca, &s->table, &s->sun_h, &s->sun_col, &s->gm,
                      &s->goff, &s->gdir, &s->gval, &s->rf, &s->af, &s->ext0, &s->s_ext, &s->s_sca, &s->s_chi,
                      &s->s_density, &s->s_sun_col, &s->s_eigen, &s->s_sca_src, &s->s_lut, &s->s_lut2, &s->gsame,
                      &s->gdir4, &s->sh_a, &s->sh_b, &s->sh_d, &s->u_hi, &s->u_lo, &s->wu_hi, &s->wu_lo, &s->uq_hi,
                      &s->uq_lo, &s->wuq_hi, &s->wuq_lo, &s->box_ww, &s->solar, &s->rad, &s->plane, &s->moments,
                      &s->flux, &s->first_moments, &s->first_flux, &s->boundary, &s->metrics, &s->boxes, &s->fx,
                      &s->fg, &s->norms, &s->partials, &s->dots, &s->ctrl_dev, &s->loop_dev, &s->box_old, &s->box_new,
                      &s->obs_feat, &s->gram, &s->hist_dev, &s->normmax, &s->ring_g[0],
                      &s->ring_g[1], &s->ring_g[2], &s->ring_g[3], &s->ring_f[0], &s->ring_f[1], &s->ring_f[2],
                      &s->ring_f[3], &s->fl_val0, &s->fl_coef, &s->fl_dir, &s->fl_g, &s->fl_cnt, &s->fl_off,
                      &s->fl_cursor, &s->fl_entries, &s->gr_off, &s->gr_loc, &s->gr_w, &s->gr_cols, &s->gr_cos,
                      &s->gr_ok, &s->gr_value, &s->gr_cnt, &s->gr_cursor, &s->t_lut, &s->t_lut2, &s->g_su2,
                      &s->g_sv, &s->gt_cnt, &s->gt_off, &s->gt_cursor, &s->gt_tile, &s->plane_tiles};
    for (DevBuf* b : bufs) dfree(s, *b);
    for (BundleDev* bd : {&s->cells, &s->obs}) {
        DevBuf* bb[] = {&bd->cell_off, &bd->ray_cell, &bd->p, &bd->frame, &bd->dir, &bd->dir_lo, &bd->dloc, &bd->pcp,
                        &bd->seg_off, &bd->seg, &bd->lower, &bd->end_j, &bd->end_col, &bd->hits,
                        &bd->t_frame, &bd->t_misc, &bd->t_att, &bd->b_hi, &bd->b_lo, &bd->p_off, &bd->p_cell,
                        &bd->p_ray, &bd->p_node, &bd->y_tab, &bd->pair_A, &bd->c_ray, &bd->c_cp, &bd->c_slot,
                        &bd->c_tile, &bd->cv, &bd->node_ray, &bd->vbuf};
        for (DevBuf* b : bb) dfree(s, *b);
    }
    collect_timing(s);
    graph_reset(s);
    if (s->ctrl_host) cudaFreeHost(s->ctrl_host);
    if (s->loop_host) cudaFreeHost(s->loop_host);
    for (cudaEvent_t e : s->event_pool) cudaEventDestroy(e);
    if (s->own) cudaStreamDestroy(s->own);
    delete s;
    return 0;
}

int sosb_set_timing(sosb_handle s, int on) {
    if (!s) return 1;
    TRY(collect_timing(s));
    s->timing = on != 0;
    for (int k = 0; k < K_CLASSES; ++k) {
        s->timed_ms[k] = 0.0;
        s->timed_count[k] = 0;
    }
    return 0;
}

int sosb_get_timing(sosb_handle s, double* ms, int64_t* launches, int n) {
    if (!s || !ms || !launches) return 1;
    TRY(collect_timing(s));
    for (int k = 0; k < n && k < K_CLASSES; ++k) {
        ms[k] = s->timed_ms[k];
        launches[k] = s->timed_count[k];
    }
    return 0;
}

int sosb_set_projection(sosb_handle s, int mode) {
    if (!s) return 1;
    if (mode < PROJ_FP32 || mode > PROJ_BF16) return fail(s, "E_PROJECTION: unknown form %d", mode);
    s->proj_mode = mode;
    graph_reset(s);
    return 0;
}

int sosb_set_node_tables(sosb_handle s, int enable) {
    if (!s) return 1;
    s->tables = enable != 0;
    invalidate_tables(s->cells);
    invalidate_tables(s->obs);
    graph_reset(s);
    return 0;
}

int sosb_set_stream(sosb_handle s, void* stream) {
    if (!s) return 1;
    s->stream = stream ? (cudaStream_t)stream : s->own;
    return 0;
}

int sosb_shape(sosb_handle s, int64_t* cells, int32_t* slots, int32_t* K) {
    if (!s) return 1;
    if (cells) *cells = s->ns;
    if (slots) *slots = s->src;
    if (K) *K = s->K;
    return 0;
}

static int put_ds(sosb_state* s, DevBuf& hi, DevBuf& lo, const double* v, int n) {
    std::vector<float> h, l;
    split_nodes(v, n, h, l);
    TRY(dput_vec(s, hi, h));
    return dput_vec(s, lo, l);
}

// Leading factors of a phase table lut[i][w] (rows i < n, W wavelengths): lut ~= U V with V's rows the eigenvectors
// of lut^T lut of the largest eigenvalues (cyclic Jacobi in FP64) and U = lut V^T; the smallest rank r <= rmax whose
// error in every row is at most tol times that row's largest magnitude (the phase varies over orders of magnitude in
// u, little across wavelengths at one u). Returns r, 0 when no rank up to rmax is within tol.
static int strato_factors(const std::vector<double>& lut, int n, int W, int rmax, double tol, std::vector<double>& U,
                          std::vector<double>& V) {
    std::vector<double> G((size_t)W * W, 0.0), E((size_t)W * W, 0.0);
    for (int i = 0; i < n; ++i)
        for (int a = 0; a < W; ++a)
            for (int b = a; b < W; ++b) G[(size_t)a * W + b] += lut[(size_t)i * W + a] * lut[(size_t)i * W + b];
    for (int a = 0; a < W; ++a) {
        for (int b = 0; b < a; ++b) G[(size_t)a * W + b] = G[(size_t)b * W + a];
        E[(size_t)a * W + a] = 1.0;
    }
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = 0.0, diag = 0.0;
        for (int a = 0; a < W; ++a) {
            diag += G[(size_t)a * W + a] * G[(size_t)a * W + a];
            for (int b = a + 1; b < W; ++b) off += G[(size_t)a * W + b] * G[(size_t)a * W + b];
        }
        if (off <= 1e-30 * diag) break;
        for (int p = 0; p < W; ++p)
            for (int q = p + 1; q < W; ++q) {
                const double gpq = G[(size_t)p * W + q];
                if (std::fabs(gpq) < 1e-300) continue;
                const double theta = (G[(size_t)q * W + q] - G[(size_t)p * W + p]) / (2.0 * gpq);
                const double tt = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(tt * tt + 1.0), sn = tt * c;
                for (int k = 0; k < W; ++k) {  // G <- J^T G J, E <- E J
                    const double gkp = G[(size_t)k * W + p], gkq = G[(size_t)k * W + q];
                    G[(size_t)k * W + p] = c * gkp - sn * gkq;
                    G[(size_t)k * W + q] = sn * gkp + c * gkq;
                }
                for (int k = 0; k < W; ++k) {
                    const double gpk = G[(size_t)p * W + k], gqk = G[(size_t)q * W + k];
                    G[(size_t)p * W + k] = c * gpk - sn * gqk;
                    G[(size_t)q * W + k] = sn * gpk + c * gqk;
                }
                for (int k = 0; k < W; ++k) {
                    const double ekp = E[(size_t)k * W + p], ekq = E[(size_t)k * W + q];
                    E[(size_t)k * W + p] = c * ekp - sn * ekq;
                    E[(size_t)k * W + q] = sn * ekp + c * ekq;
                }
            }
    }
    std::vector<int> order(W);
    for (int a = 0; a < W; ++a) order[a] = a;
    std::sort(order.begin(), order.end(),
              [&](int x, int y) { return G[(size_t)x * W + x] > G[(size_t)y * W + y]; });
    for (int r = 1; r <= std::min(rmax, W); ++r) {
        V.assign((size_t)r * W, 0.0);
        for (int j = 0; j < r; ++j)
            for (int w = 0; w < W; ++w) V[(size_t)j * W + w] = E[(size_t)w * W + order[j]];
        U.assign((size_t)n * r, 0.0);
        bool within = true;
        for (int i = 0; i < n && within; ++i) {
            const double* row = &lut[(size_t)i * W];
            double big = 0.0;
            for (int w = 0; w < W; ++w) big = std::max(big, std::fabs(row[w]));
            for (int j = 0; j < r; ++j) {
                double u = 0.0;
                for (int w = 0; w < W; ++w) u += row[w] * V[(size_t)j * W + w];
                U[(size_t)i * r + j] = u;
            }
            for (int w = 0; w < W && within; ++w) {
                double v = 0.0;
                for (int j = 0; j < r; ++j) v += U[(size_t)i * r + j] * V[(size_t)j * W + w];
                within = std::fabs(v - row[w]) <= tol * big;
            }
        }
        if (within) return r;
    }
    return 0;
}

int sosb_phase_factors(const double* lut, int n, int W, int rmax, double tol, double* U, double* V, int* rank) {
    if (!lut || !U || !V || !rank || n < 1 || W < 1 || rmax < 1) return 1;
    std::vector<double> l(lut, lut + (size_t)n * W), u, v;
    *rank = strato_factors(l, n, W, rmax, tol, u, v);
    std::copy(u.begin(), u.end(), U);
    std::copy(v.begin(), v.end(), V);
    return 0;
}

int sosb_set_constants(sosb_handle s, const sosb_constants* c) {
    if (!s || !c) return 1;
    const sosb_dims& d = s->d;
    const int W = d.W, K = s->K, ns = s->ns;
    if (!c->u || !c->wu || !c->uq || !c->wuq || !c->h || !c->chi || !c->hr || !c->ha || !c->ext || !c->asca ||
        !c->density_table || !c->sun_h || !c->sun_col || !c->gm || !c->goff || !c->rf || !c->af || !c->ext0 ||
        !c->solar || !c->box_ww)
        return fail(s, "E_CONSTANTS: missing array");
    if (d.strato && (!c->strato_ext || !c->strato_sca || !c->strato_chi || !c->strato_density || !c->strato_sun_col ||
                     !c->strato_eigen || !c->strato_sca_source))
        return fail(s, "E_CONSTANTS: missing stratospheric array");
    TRY(put_ds(s, s->u_hi, s->u_lo, c->u, d.nq));
    TRY(put_ds(s, s->wu_hi, s->wu_lo, c->wu, d.nq));
    TRY(put_ds(s, s->uq_hi, s->uq_lo, c->uq, d.nq_query));
    TRY(put_ds(s, s->wuq_hi, s->wuq_lo, c->wuq, d.nq_query));
    TRY(dput(s, s->h, c->h, d.nh * 4));
    TRY(dput(s, s->chi, c->chi, d.nc * 4));
    TRY(dput(s, s->hr, c->hr, d.nh * 4));
    TRY(dput(s, s->ha, c->ha, d.nh * 4));
    TRY(dput(s, s->ext, c->ext, 5 * W * 4));
    TRY(dput(s, s->asca, c->asca, W * 4));
    TRY(dput(s, s->table, c->density_table, (size_t)d.density_rows * 3 * 4));
    TRY(dput(s, s->sun_h, c->sun_h, d.n_sun_h * 4));
    TRY(dput(s, s->sun_col, c->sun_col, (size_t)d.n_sun_h * d.n_sun_x * 5 * 4));
    TRY(dput(s, s->gm, c->gm, (size_t)ns * 4 * W * 4));
    std::vector<int> goff(ns + 1);
    for (int i = 0; i <= ns; ++i) goff[i] = (int)c->goff[i];
    const int ng = goff[ns];
    TRY(dput_vec(s, s->goff, goff));
    if (ng > 0) {
        if (!c->gdir || !c->gval) return fail(s, "E_CONSTANTS: missing ground directions");
        TRY(dput(s, s->gdir, c->gdir, (size_t)ng * 3 * 4));
        std::vector<float4> g4(ng);
        for (int i = 0; i < ng; ++i) g4[i] = make_float4(c->gdir[3 * i], c->gdir[3 * i + 1], c->gdir[3 * i + 2], 0.0f);
        TRY(dput_vec(s, s->gdir4, g4));
        TRY(dput(s, s->gval, c->gval, (size_t)ng * W * 4));
    } else {
        TRY(dalloc(s, s->gdir, 16));
        TRY(dalloc(s, s->gdir4, 16));
        TRY(dalloc(s, s->gval, 16));
    }
    {
        // cells whose next solar-zenith neighbour (same height) has the same ground directions, bit for bit
        std::vector<uint8_t> same(ns, 0);
        for (int cell = 0; cell < ns; ++cell) {
            if (cell % d.nc == d.nc - 1) continue;
            const int n0 = goff[cell + 1] - goff[cell], n1 = goff[cell + 2] - goff[cell + 1];
            same[cell] = n0 > 0 && n0 == n1 &&
                         std::memcmp(c->gdir + 3 * (size_t)goff[cell], c->gdir + 3 * (size_t)goff[cell + 1],
                                     (size_t)n0 * 3 * sizeof(float)) == 0;
        }
        TRY(dput_vec(s, s->gsame, same));
    }
    s->aer2_on = c->aer2 != nullptr;
    for (int i = 0; i < 7; ++i) s->aer2[i] = c->aer2 ? c->aer2[i] : 0.0f;
    TRY(dput(s, s->rf, c->rf, 6 * 4));
    s->af_w = c->tropo_eigen != nullptr;
    TRY(dput(s, s->af, c->tropo_eigen ? c->tropo_eigen : c->af, (size_t)K * (s->af_w ? W : 1) * 4));
    s->tropo_bins = 0;
    if (c->tropo_lut) {
        if (c->tropo_bins < 2 || c->tropo_bins > (1 << 24)) return fail(s, "E_CONSTANTS: tropo_bins %d", c->tropo_bins);
        const size_t nb = (size_t)c->tropo_bins;
        TRY(dput(s, s->t_lut, c->tropo_lut, (nb + 1) * W * 4));
        std::vector<float2> lut2(nb * W);
        for (size_t i = 0; i < nb * W; ++i)
            lut2[i] = make_float2(c->tropo_lut[i], c->tropo_lut[i + W] - c->tropo_lut[i]);
        TRY(dput_vec(s, s->t_lut2, lut2));
        s->tropo_bins = c->tropo_bins;
    }
    TRY(dput(s, s->ext0, c->ext0, W * 4));
    TRY(dput(s, s->solar, c->solar, W * 8));
    TRY(dput(s, s->box_ww, c->box_ww, d.box_points * 8));
    if (d.strato) {
        TRY(dput(s, s->s_ext, c->strato_ext, W * 4));
        TRY(dput(s, s->s_sca, c->strato_sca, W * 4));
        TRY(dput(s, s->s_chi, c->strato_chi, 33 * W * 4));
        TRY(dput(s, s->s_density, c->strato_density, d.nh * 4));
        TRY(dput(s, s->s_sun_col, c->strato_sun_col, (size_t)d.n_sun_h * d.n_sun_x * 4));
        TRY(dput(s, s->s_eigen, c->strato_eigen, (size_t)K * W * 4));
        TRY(dput(s, s->s_sca_src, c->strato_sca_source, W * 4));
        // phase table on u in [-1, 1] from the 33 Legendre moments (FP64 recurrence, per sr)
        std::vector<float> lut((size_t)(STRATO_LUT_BINS + 1) * W);
        for (int i = 0; i <= STRATO_LUT_BINS; ++i) {
            const double u = -1.0 + 2.0 * i / STRATO_LUT_BINS;
            for (int w = 0; w < W; ++w) {
                double p0 = 1.0, p1 = u;
                double v = c->strato_chi[w] + u * c->strato_chi[W + w];
                for (int l = 2; l < 33; ++l) {
                    const double pn = ((2.0 * l - 1) * u * p1 - (l - 1.0) * p0) / l;
                    v += pn * c->strato_chi[l * W + w];
                    p0 = p1;
                    p1 = pn;
                }
                lut[(size_t)i * W + w] = (float)(v / (4.0 * M_PI));
            }
        }
        TRY(dput_vec(s, s->s_lut, lut));
        std::vector<float2> lut2((size_t)STRATO_LUT_BINS * W);
        for (size_t i = 0; i < (size_t)STRATO_LUT_BINS * W; ++i)
            lut2[i] = make_float2(lut[i], lut[i + W] - lut[i]);
        TRY(dput_vec(s, s->s_lut2, lut2));
        // factors of the table for the tensor-core ground sums
        std::vector<double> lut64((size_t)(STRATO_LUT_BINS + 1) * W);
        for (size_t i = 0; i < lut64.size(); ++i) lut64[i] = lut[i];
        std::vector<double> U, V;
        s->g_rank = strato_factors(lut64, STRATO_LUT_BINS + 1, W, GTC_MAX_RANK, 2e-6, U, V);
        if (s->g_rank > 0) {
            const int R = s->g_rank;
            std::vector<float2> su2((size_t)STRATO_LUT_BINS * R);
            for (int i = 0; i < STRATO_LUT_BINS; ++i)
                for (int r = 0; r < R; ++r) {
                    const float a = (float)U[(size_t)i * R + r], b = (float)U[(size_t)(i + 1) * R + r];
                    su2[(size_t)i * R + r] = make_float2(a, b - a);
                }
            std::vector<float> sv((size_t)R * W);
            for (size_t i = 0; i < sv.size(); ++i) sv[i] = (float)V[i];
            TRY(dput_vec(s, s->g_su2, su2));
            TRY(dput_vec(s, s->g_sv, sv));
        }
    }
    CK(cudaStreamSynchronize(s->stream));
    s->have_constants = true;
    s->have_first = false;
    invalidate_tables(s->cells, false);
    invalidate_tables(s->obs, false);
    graph_reset(s);
    return 0;
}

// Slant columns of the solar column table (host; the synthetic family's counterpart of the reference's sun geometry,
// src/sosfuse2/solve/engine_core.py:103-147 and S/precompute): from radius r0 along zenith cosine mu to the top of
// the atmosphere or the ground, the path cut at the shadow cylinder, the tangent point and the shells, each piece
// integrated by an n-point Gauss-Legendre rule of the five profile shapes (clipped to [0, top]) and the
// stratospheric shape; the operations of the NumPy restatement in order, in FP64.
// Sorted path coordinates where a ray from p along d is cut (synth.ray_edges): start, tangent point, the shadow
// cylinder's two roots, the shells' crossings, and the end at the top or the ground (each absent cut repeats the end).
// Returns the count (5 + 2 nshell) and whether the ray ends on the ground.
constexpr int MAX_CUTS = 5 + 2 * 8;
SOS_HD int ray_cuts(const double p[3], const double d[3], double top, const double* shells, int nshell,
                    double cols[MAX_CUTS], bool* ground_out) {
    const double R = 6371.0;
    const double px = p[0], py = p[1], pz = p[2], dx = d[0], dy = d[1], dz = d[2];
    const double b = (px * dx + py * dy) + pz * dz;
    const double pp = (px * px + py * py) + pz * pz;
    double end = -b + sqrt(fmax(b * b - pp + (R + top) * (R + top), 0.0));
    const double disc = b * b - pp + R * R;
    const double hit = -b - sqrt(fmax(disc, 0.0));
    const bool ground = disc >= 0.0 && b < 0.0 && hit >= -1e-7;
    end = fmax(ground ? fmax(hit, 0.0) : end, 0.0);
    const double tangent = (-b > 0.0 && -b < end) ? -b : end;
    const double aa = dx * dx + dy * dy, bb = px * dx + py * dy, cc = px * px + py * py - R * R;
    const double ds = bb * bb - aa * cc;
    int nc = 0;
    cols[nc++] = 0.0;
    cols[nc++] = tangent;
    cols[nc++] = end;
    for (int sign = -1; sign <= 1; sign += 2) {
        const double root = (-bb + sign * sqrt(fmax(ds, 0.0))) / fmax(aa, 1e-30);
        const bool ok = aa > 1e-20 && ds >= 0.0 && root > 0.0 && root < end && pz + root * dz < 0.0;
        cols[nc++] = ok ? root : end;
    }
    for (int k = 0; k < nshell && k < 8; ++k) {
        const double disc2 = b * b - pp + (R + shells[k]) * (R + shells[k]);
        for (int sign = -1; sign <= 1; sign += 2) {
            const double root = -b + sign * sqrt(fmax(disc2, 0.0));
            cols[nc++] = (disc2 > 0.0 && root > 0.0 && root < end) ? root : end;
        }
    }
    for (int i = 1; i < nc; ++i) {  // insertion sort (at most 21 cuts)
        const double v = cols[i];
        int j = i - 1;
        while (j >= 0 && cols[j] > v) {
            cols[j + 1] = cols[j];
            --j;
        }
        cols[j + 1] = v;
    }
    if (ground_out) *ground_out = ground;
    return nc;
}

SOS_HD void column_along(double r0, double mu, const sosb_profile_shape& a, const double* shells, int nshell,
                         const double* u, const double* wu, int n, double out[6]) {
    const double R = 6371.0;
    const double px = 0.0, py = 0.0, pz = r0;
    const double dx = sqrt(fmax(1.0 - mu * mu, 0.0)), dy = 0.0, dz = mu;
    const double pv[3] = {px, py, pz}, dv[3] = {dx, dy, dz};
    double cols[MAX_CUTS];
    const int nc = ray_cuts(pv, dv, a.top, shells, nshell, cols, nullptr);
    for (int k = 0; k < 6; ++k) out[k] = 0.0;
    for (int k = 0; k + 1 < nc; ++k) {
        const double s0 = cols[k], s1 = cols[k + 1];
        double seg[5] = {0.0, 0.0, 0.0, 0.0, 0.0}, sst = 0.0;
        for (int q = 0; q < n; ++q) {
            const double t = s0 + (s1 - s0) * u[q];
            const double qx = px + t * dx, qy = py + t * dy, qz = pz + t * dz;
            const double h = sqrt((qx * qx + qy * qy) + qz * qz) - R;
            const double w = (s1 - s0) * wu[q];
            const double hc = fmin(fmax(h, 0.0), a.top);
            const double air = exp(-hc / 8.0);
            const double z = (hc - a.ozone_peak) / 5.0;
            const double no2 = (hc - a.no2_center) / 4.0;
            const double prof[5] = {air, exp(-hc / a.aerosol_height), exp(1.0 - z - exp(-z)) * a.ozone_norm,
                                    exp(-0.5 * (no2 * no2)), air * air};
            for (int c = 0; c < 5; ++c) seg[c] += w * prof[c];
            if (a.strato) {
                const double v = (h - a.strato_center) / a.strato_sigma;
                sst += w * (exp(-0.5 * (v * v)) / a.strato_norm);
            }
        }
        for (int c = 0; c < 5; ++c) out[c] += seg[c];
        out[5] += sst;
    }
}

int sosb_column_table(int n_h, const double* h, int n_x, const double* x, const double* shells, int n_shells,
                      const double* gl_u, const double* gl_w, int n_gl, const sosb_profile_shape* shape, double* up,
                      double* down, int threads) {
    if (n_h < 1 || n_x < 1 || !h || !x || !gl_u || !gl_w || n_gl < 1 || !shape || !up || !down) return 1;
    if (n_shells < 0 || n_shells > 8 || (n_shells > 0 && !shells)) return 1;
    const double R = 6371.0;
    const sosb_profile_shape a = *shape;
    auto row = [&](int i) {
        const double r = R + h[i];
        const double mg = -std::sqrt(std::max(0.0, 1.0 - (R / r) * (R / r)));
        for (int j = 0; j < n_x; ++j) {
            double mu = mg + (1.0 - mg) * (x[j] * x[j]);
            if (j == 0) mu = mg + 1e-9;
            column_along(r, mu, a, shells, n_shells, gl_u, gl_w, n_gl, up + ((size_t)i * n_x + j) * 6);
            double mud = mg - (1.0 + mg) * (x[j] * x[j]);
            if (j == 0) mud = mg - 1e-9;
            column_along(r, std::max(mud, -1.0), a, shells, n_shells, gl_u, gl_w, n_gl, down + ((size_t)i * n_x + j) * 6);
        }
    };
    const int nt = std::max(1, std::min(threads > 0 ? threads : (int)std::thread::hardware_concurrency(), n_h));
    std::atomic<int> next(0);
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&]() {
            for (int i = next++; i < n_h; i = next++) row(i);
        });
    for (auto& t : pool) t.join();
    return 0;
}

// The solar column table on the device: one thread per (up or down table, height, x), the column function of
// sosb_column_table (the same FP64 operations; a compiler may contract them differently on the two sides).
struct ColArgs {
    int n_h, n_x, n_gl, nshell;
    const double *h, *x, *gl_u, *gl_w;
    double shells[8];
    sosb_profile_shape a;
    double *up, *down;
};

__global__ void column_table_kernel(ColArgs g) {
    const long long nhx = (long long)g.n_h * g.n_x, n = 2 * nhx;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int dn = t >= nhx ? 1 : 0;
        const long long ij = t - dn * nhx;
        const int i = (int)(ij / g.n_x), j = (int)(ij - (long long)i * g.n_x);
        const double R = 6371.0, r = R + g.h[i];
        const double mg = -sqrt(fmax(0.0, 1.0 - (R / r) * (R / r)));
        double mu;
        if (!dn) {
            mu = mg + (1.0 - mg) * (g.x[j] * g.x[j]);
            if (j == 0) mu = mg + 1e-9;
        } else {
            mu = mg - (1.0 + mg) * (g.x[j] * g.x[j]);
            if (j == 0) mu = mg - 1e-9;
            mu = fmax(mu, -1.0);
        }
        column_along(r, mu, g.a, g.shells, g.nshell, g.gl_u, g.gl_w, g.n_gl, (dn ? g.down : g.up) + ij * 6);
    }
}

int sosb_column_table_device(int n_h, const double* h, int n_x, const double* x, const double* shells, int n_shells,
                             const double* gl_u, const double* gl_w, int n_gl, const sosb_profile_shape* shape,
                             double* up, double* down, void* stream) {
    if (n_h < 1 || n_x < 1 || !h || !x || !gl_u || !gl_w || n_gl < 1 || !shape || !up || !down) return 1;
    if (n_shells < 0 || n_shells > 8 || (n_shells > 0 && !shells)) return 1;
    ColArgs g{};
    g.n_h = n_h;
    g.n_x = n_x;
    g.n_gl = n_gl;
    g.nshell = n_shells;
    g.h = h;
    g.x = x;
    g.gl_u = gl_u;
    g.gl_w = gl_w;
    for (int k = 0; k < n_shells; ++k) g.shells[k] = shells[k];  // host values
    g.a = *shape;
    g.up = up;
    g.down = down;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    column_table_kernel<<<grid_for(2LL * n_h * n_x, 128), 128, 0, st>>>(g);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? 0 : 3;
}

// Bilinear lookup of a solar column table (synth.ColumnTable.lookup): columns [6] at height h (clipped to [0, top])
// along zenith cosine mu from the up table when the ray escapes (mu >= the horizon cosine), else the down table.
// index of the last grid value <= x (std::upper_bound - 1)
SOS_HD int upper_index(const double* g, int n, double x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (g[mid] <= x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo - 1;
}

SOS_HD void column_lookup(const sosb_column_grid& t, double h, double mu, double out[6]) {
    const double R = 6371.0;
    h = fmin(fmax(h, 0.0), t.top);
    const double r = R + h;
    const double rr = fmax(r, R);
    const double mg = -sqrt(fmax(0.0, 1.0 - (R / rr) * (R / rr)));
    const bool escape = mu >= mg;
    const double x = escape ? sqrt(fmin(fmax((mu - mg) / (1.0 - mg), 0.0), 1.0))
                            : sqrt(fmin(fmax((mg - mu) / (1.0 + mg), 0.0), 1.0));
    // i = clip(searchsorted(h_grid, h, 'right') - 1, 0, n_h - 2)
    int i = upper_index(t.h, t.n_h, h);
    i = i < 0 ? 0 : (i > t.n_h - 2 ? t.n_h - 2 : i);
    const double a = (h - t.h[i]) / (t.h[i + 1] - t.h[i]);
    const double f = x * (double)(t.n_x - 1);
    int j = (int)f;
    j = j < 0 ? 0 : (j > t.n_x - 2 ? t.n_x - 2 : j);
    const double bb = f - (double)j;
    const double* tab = escape ? t.up : t.down;
    const double* t00 = tab + ((size_t)i * t.n_x + j) * 6;
    const double* t10 = tab + ((size_t)(i + 1) * t.n_x + j) * 6;
    const double* t01 = t00 + 6;
    const double* t11 = t10 + 6;
    for (int k = 0; k < 6; ++k)
        out[k] = (((1.0 - a) * (1.0 - bb) * t00[k] + a * (1.0 - bb) * t10[k]) + (1.0 - a) * bb * t01[k]) +
                 a * bb * t11[k];
}

// The segments and ray-end quantities of ray r (sosb_ray_segments; host threads or one device thread per ray).
struct SegArgs {
    const double *p, *d;
    double top;
    const double* shells;
    int n_shells, n_chi;
    const double* chi;
    sosb_column_grid grid;  // the column table (its arrays on the side that runs the segments)
    int has_grid;           // 0: no ground columns
    double* edges;
    uint8_t *valid, *lower, *hits;
    int32_t* end_j;
    double* end_f;
    float *end_col, *end_st;
};

SOS_HD void ray_segments_one(const SegArgs& g, int64_t r) {
    const double R = 6371.0;
    const int ncut = 5 + 2 * g.n_shells;
    const double* pr = g.p + r * 3;
    const double* dr = g.d + r * 3;
    double* e = g.edges + r * ncut;
    double cuts[MAX_CUTS];
    ray_cuts(pr, dr, g.top, g.shells, g.n_shells, cuts, nullptr);
    for (int k = 0; k < ncut; ++k) e[k] = cuts[k];
    for (int k = 0; k + 1 < ncut; ++k) {
        const double a = cuts[k], b = cuts[k + 1];
        g.valid[r * (ncut - 1) + k] = (b - a) > 1e-8;
        double qa[3], qb[3];
        for (int c = 0; c < 3; ++c) {
            qa[c] = pr[c] + a * dr[c];
            qb[c] = pr[c] + b * dr[c];
        }
        g.lower[r * (ncut - 1) + k] =
            ((qa[0] * qa[0] + qa[1] * qa[1]) + qa[2] * qa[2]) <= ((qb[0] * qb[0] + qb[1] * qb[1]) + qb[2] * qb[2]);
    }
    const double end = cuts[ncut - 1];
    double qe[3];
    for (int c = 0; c < 3; ++c) qe[c] = pr[c] + end * dr[c];
    const double re = sqrt((qe[0] * qe[0] + qe[1] * qe[1]) + qe[2] * qe[2]);
    const double ch = acos(fmin(fmax(qe[2] / re, -1.0), 1.0));
    int j = upper_index(g.chi, g.n_chi, ch);
    j = j < 0 ? 0 : (j > g.n_chi - 2 ? g.n_chi - 2 : j);
    g.end_j[r] = j;
    g.end_f[r] = fmin(fmax((ch - g.chi[j]) / (g.chi[j + 1] - g.chi[j]), 0.0), 1.0);
    const bool hit = re < R + 1e-5;
    g.hits[r] = hit;
    if (g.has_grid) {
        double cols[6] = {0, 0, 0, 0, 0, 0};
        if (hit) {
            const double r0 = sqrt((pr[0] * pr[0] + pr[1] * pr[1]) + pr[2] * pr[2]);
            const double mu = ((pr[0] * dr[0] + pr[1] * dr[1]) + pr[2] * dr[2]) / r0;
            column_lookup(g.grid, r0 - R, mu, cols);
        }
        for (int k = 0; k < 5; ++k) g.end_col[r * 5 + k] = (float)cols[k];
        g.end_st[r] = (float)cols[5];
    }
}

__global__ void ray_segments_kernel(SegArgs g, int64_t n) {
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        ray_segments_one(g, r);
}

int sosb_ray_segments(int64_t n, const double* p, const double* d, double top, const double* shells, int n_shells,
                      int n_chi, const double* chi, const sosb_column_grid* table, double* edges, uint8_t* valid,
                      uint8_t* lower, int32_t* end_j, double* end_f, float* end_col, float* end_st, uint8_t* hits,
                      int threads) {
    if (n < 0 || (n > 0 && (!p || !d || !edges || !valid || !lower || !end_j || !end_f || !hits)) || n_chi < 2 ||
        !chi || n_shells < 0 || n_shells > 8 || (n_shells > 0 && !shells))
        return 1;
    if (table && (!end_col || !end_st || table->n_h < 2 || table->n_x < 2)) return 1;
    const SegArgs g{p, d, top, shells, n_shells, n_chi, chi, table ? *table : sosb_column_grid{}, table ? 1 : 0,
                    edges, valid, lower, hits, end_j, end_f, end_col, end_st};
    auto ray = [&](int64_t r) { ray_segments_one(g, r); };
    const int64_t chunk = 4096;
    const int64_t nchunk = (n + chunk - 1) / chunk;
    const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(threads > 0 ? threads : (int)std::thread::hardware_concurrency(), nchunk));
    std::atomic<int64_t> next(0);
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&]() {
            for (int64_t c = next++; c < nchunk; c = next++)
                for (int64_t r = c * chunk; r < std::min(n, (c + 1) * chunk); ++r) ray(r);
        });
    for (auto& t : pool) t.join();
    return 0;
}

int sosb_ray_segments_device(int64_t n, const double* p, const double* d, double top, const double* shells,
                             int n_shells, int n_chi, const double* chi, const sosb_column_grid* table, double* edges,
                             uint8_t* valid, uint8_t* lower, int32_t* end_j, double* end_f, float* end_col,
                             float* end_st, uint8_t* hits, void* stream) {
    if (n < 0 || (n > 0 && (!p || !d || !edges || !valid || !lower || !end_j || !end_f || !hits)) || n_chi < 2 ||
        !chi || n_shells < 0 || n_shells > 8 || (n_shells > 0 && !shells))
        return 1;
    if (table && (!end_col || !end_st || table->n_h < 2 || table->n_x < 2 || !table->h || !table->up ||
                  !table->down))
        return 1;
    if (n == 0) return 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const SegArgs g{p, d, top, shells, n_shells, n_chi, chi, table ? *table : sosb_column_grid{}, table ? 1 : 0,
                    edges, valid, lower, hits, end_j, end_f, end_col, end_st};
    ray_segments_kernel<<<grid_for(n, 128), 128, 0, st>>>(g, n);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? 0 : 3;
}

// Incoming-direction quadrature of one cell (synth.ring_quadrature, the reference's ring rule restated: per azimuth
// plane a sinh-mapped Gauss-Legendre rule in mu between the cuts at the horizon, the shadow boundary and the shells'
// shadow rings). Writes the directions (local ex, ey, up) and weights when loc is not NULL; returns the count.
static int64_t ring_cell(double r, double chi, int nmu, int nphi, const double* heights, int nh, bool rings, double a,
                         const double* u, const double* wu, double* loc, double* wout) {
    const double R = 6371.0, PI = 3.141592653589793;
    const double mg = -std::sqrt(std::max(0.0, 1.0 - (R / r) * (R / r)));
    const double sa = std::sinh(a);
    const double sinchi = std::sin(chi), coschi = std::cos(chi);
    const double rp = r * sinchi;
    const double up[3] = {sinchi, 0.0, coschi}, ex[3] = {-coschi, 0.0, sinchi};
    const double p[3] = {r * up[0], r * up[1], r * up[2]};
    const double ey[3] = {up[1] * ex[2] - up[2] * ex[1], up[2] * ex[0] - up[0] * ex[2], up[0] * ex[1] - up[1] * ex[0]};
    const double step = PI / (double)nphi;
    int64_t count = 0;
    std::vector<double> edges, tt;
    for (int j = 0; j <= nphi; ++j) {
        const double phi = j == nphi ? PI : (double)j * step;
        const double cphi = std::cos(phi), sphi = std::sin(phi);
        edges.assign({-1.0, 1.0, mg, 0.0, mg - 0.05234, mg + 0.05234, mg - 0.0061, mg + 0.0061});
        if (rp > R + 1e-8 && std::fabs(sinchi) > 1e-8) {
            const double kk = R / std::sqrt(rp * rp - R * R);
            for (int sign = -1; sign <= 1; sign += 2) {
                const double t = cphi * coschi / sinchi + sign * sphi / (kk * sinchi);
                const double mu = t / std::sqrt(1.0 + t * t);
                const double st = std::sqrt(1.0 - mu * mu);
                const double dx = mu * sinchi - st * cphi * coschi;
                const double dy = -st * sphi;
                const double dz = mu * coschi + st * cphi * sinchi;
                const double tmin = -rp * dx / std::max(dx * dx + dy * dy, 1e-25);
                if (std::fabs(dx) + std::fabs(dy) < 1e-10 || (tmin > 0.0 && r * coschi + tmin * dz < 0.0))
                    edges.push_back(mu);
            }
        }
        if (phi < PI / 6.0) {
            const double mu = coschi / std::sqrt(coschi * coschi + cphi * cphi * (sinchi * sinchi) + 1e-300);
            edges.push_back(mu);
            edges.push_back(mu - 0.012);
            edges.push_back(mu + 0.012);
        }
        if (rings) {
            double hz[3];
            for (int c = 0; c < 3; ++c) hz[c] = cphi * ex[c] + sphi * ey[c];
            const double nrm[3] = {up[1] * hz[2] - up[2] * hz[1], up[2] * hz[0] - up[0] * hz[2],
                                   up[0] * hz[1] - up[1] * hz[0]};
            const double amp = R * std::hypot(nrm[0], nrm[1]);
            if (amp >= 1e-10) {
                const double angle = std::atan2(nrm[1], nrm[0]);
                for (int k = 0; k < nh; ++k) {
                    const double z = -std::sqrt(std::max(0.0, (R + heights[k]) * (R + heights[k]) - R * R));
                    const double target = -nrm[2] * z / amp;
                    if (std::fabs(target) > 1.0) continue;
                    const double delta = std::acos(target);
                    for (int side = 0; side < 2; ++side) {
                        const double az = side == 0 ? angle - delta : angle + delta;
                        double d[3] = {R * std::cos(az) - p[0], R * std::sin(az) - p[1], z - p[2]};
                        const double length = std::sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
                        if (length < 1e-8) continue;
                        for (int c = 0; c < 3; ++c) d[c] /= length;
                        if ((d[0] * hz[0] + d[1] * hz[1]) + d[2] * hz[2] <= 1e-10) continue;
                        const double b = (p[0] * d[0] + p[1] * d[1]) + p[2] * d[2];
                        const double disc = b * b - r * r + R * R;
                        const double hit = -b - std::sqrt(std::max(0.0, disc));
                        if (disc >= 0.0 && b < 0.0 && hit >= -1e-7 && hit < length - 1e-5) continue;
                        edges.push_back((d[0] * up[0] + d[1] * up[1]) + d[2] * up[2]);
                    }
                }
            }
        }
        for (double& e : edges) e = std::min(std::max(e, -1.0), 1.0);
        std::sort(edges.begin(), edges.end());
        edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
        tt.resize(edges.size());
        for (size_t k = 0; k < edges.size(); ++k) {
            const double dl = edges[k] - mg;
            const double sg = dl > 0.0 ? 1.0 : (dl < 0.0 ? -1.0 : 0.0);
            tt[k] = sg * std::asinh(std::fabs(dl) / (dl < 0.0 ? 1.0 + mg : 1.0 - mg) * sa) / a;
        }
        const double half = (j == 0 || j == nphi) ? 0.5 : 1.0;
        for (size_t k = 0; k + 1 < tt.size(); ++k) {
            const double left = tt[k], right = tt[k + 1];
            if (!(right - left >= 1e-10)) continue;
            for (int q = 0; q < nmu; ++q) {
                if (loc) {
                    const double t = left + (right - left) * u[q];
                    const double den = t < 0.0 ? 1.0 + mg : 1.0 - mg;
                    const double sg = t > 0.0 ? 1.0 : (t < 0.0 ? -1.0 : 0.0);
                    const double mu = mg + sg * den * std::sinh(a * std::fabs(t)) / sa;
                    const double st = std::sqrt(std::max(0.0, 1.0 - mu * mu));
                    loc[count * 3] = st * cphi;
                    loc[count * 3 + 1] = st * sphi;
                    loc[count * 3 + 2] = mu;
                    wout[count] = (right - left) * wu[q] * den * a * std::cosh(a * std::fabs(t)) / sa *
                                  (2.0 * PI / (double)nphi) * half;
                }
                ++count;
            }
        }
    }
    return count;
}

int sosb_ring_quadrature(int n_cells, const double* r, const double* chi, int nmu, int nphi, const double* heights,
                         int n_heights, int rings, double a, const double* u, const double* wu, int64_t* counts,
                         double* loc, double* w, int64_t capacity, int threads) {
    if (n_cells < 0 || (n_cells > 0 && (!r || !chi || !counts)) || nmu < 1 || nphi < 1 || !u || !wu ||
        n_heights < 0 || (n_heights > 0 && !heights) || (loc && !w))
        return 1;
    auto run = [&](bool fill, const std::vector<int64_t>& off) {
        const int nt = std::max(1, std::min(threads > 0 ? threads : (int)std::thread::hardware_concurrency(),
                                            std::max(n_cells, 1)));
        std::atomic<int> next(0);
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t)
            pool.emplace_back([&]() {
                for (int c = next++; c < n_cells; c = next++) {
                    if (fill)
                        ring_cell(r[c], chi[c], nmu, nphi, heights, n_heights, rings != 0, a, u, wu, loc + off[c] * 3,
                                  w + off[c]);
                    else
                        counts[c] = ring_cell(r[c], chi[c], nmu, nphi, heights, n_heights, rings != 0, a, u, wu,
                                              nullptr, nullptr);
                }
            });
        for (auto& th : pool) th.join();
    };
    const std::vector<int64_t> none;
    run(false, none);
    if (!loc) return 0;
    std::vector<int64_t> off((size_t)n_cells + 1, 0);
    for (int c = 0; c < n_cells; ++c) off[c + 1] = off[c] + counts[c];
    if (off[n_cells] > capacity) return 2;
    run(true, off);
    return 0;
}

int sosb_set_ground_rays(sosb_handle s, const sosb_ground_rays* g) {
    if (!s || !g) return 1;
    if (g->n < 0 || (g->n > 0 && (!g->cell || !g->loc || !g->weight || !g->cols || !g->cos_sun || !g->ok)))
        return fail(s, "E_GROUND: missing ground-ray array");
    if (g->n >= (1LL << 31)) return fail(s, "E_GROUND: %lld ground rays", (long long)g->n);
    std::vector<int> off((size_t)s->ns + 1, 0);
    for (int64_t r = 0; r < g->n; ++r) {
        const int c = g->cell[r];
        if (c < 0 || c >= s->ns || (r > 0 && c < g->cell[r - 1]))
            return fail(s, "E_GROUND: ground-ray cells must ascend within 0..%lld", (long long)s->ns - 1);
        ++off[(size_t)c + 1];
    }
    for (int64_t c = 0; c < s->ns; ++c) off[c + 1] += off[c];
    const size_t n = (size_t)std::max<int64_t>(g->n, 1);
    TRY(dput_vec(s, s->gr_off, off));
    TRY(dalloc(s, s->gr_loc, n * 3 * sizeof(double)));
    TRY(dalloc(s, s->gr_w, n * sizeof(double)));
    TRY(dalloc(s, s->gr_cols, n * 6 * sizeof(double)));
    TRY(dalloc(s, s->gr_cos, n * sizeof(double)));
    TRY(dalloc(s, s->gr_ok, n));
    TRY(dalloc(s, s->gr_cursor, n * sizeof(int)));  // ray -> cell
    if (g->n > 0) {
        std::vector<int> cell(g->cell, g->cell + g->n);
        CK(cudaMemcpyAsync(s->gr_loc.p, g->loc, (size_t)g->n * 3 * sizeof(double), cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(s->gr_w.p, g->weight, (size_t)g->n * sizeof(double), cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(s->gr_cols.p, g->cols, (size_t)g->n * 6 * sizeof(double), cudaMemcpyHostToDevice,
                           s->stream));
        CK(cudaMemcpyAsync(s->gr_cos.p, g->cos_sun, (size_t)g->n * sizeof(double), cudaMemcpyHostToDevice,
                           s->stream));
        CK(cudaMemcpyAsync(s->gr_ok.p, g->ok, (size_t)g->n, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(s->gr_cursor.p, cell.data(), cell.size() * sizeof(int), cudaMemcpyHostToDevice,
                           s->stream));
    }
    CK(cudaStreamSynchronize(s->stream));
    s->gr_n = g->n;
    return 0;
}

int sosb_prepare_ground(sosb_handle s, double albedo, const double* ext, const double* strato_ext) {
    if (!s || !ext) return 1;
    if (!s->have_constants) return fail(s, "E_STATE: constants not set");
    if (!s->gr_off.p) return fail(s, "E_STATE: ground rays not set");
    if (s->d.strato && !strato_ext) return fail(s, "E_CONSTANTS: missing stratospheric extinction");
    const int W = s->d.W, ns = s->ns;
    const size_t n = (size_t)std::max<int64_t>(s->gr_n, 1);
    LocalBuf dext, dsext;
    TRY(dput(s, dext, ext, 5 * (size_t)W * sizeof(double)));
    if (s->d.strato) TRY(dput(s, dsext, strato_ext, (size_t)W * sizeof(double)));
    TRY(dalloc(s, s->gr_value, n * W * sizeof(double)));
    TRY(dalloc(s, s->gr_cnt, ((size_t)ns + 1) * sizeof(int)));
    TRY(dalloc(s, s->gm, (size_t)ns * 4 * W * sizeof(float)));
    TRY(dalloc(s, s->goff, ((size_t)ns + 1) * sizeof(int)));
    TRY(dalloc(s, s->gdir, n * 3 * sizeof(float)));
    TRY(dalloc(s, s->gdir4, n * sizeof(float4)));
    TRY(dalloc(s, s->gval, n * W * sizeof(float)));
    TRY(dalloc(s, s->gsame, (size_t)ns));
    const GroundRays g{P<int>(s->gr_off), P<double>(s->gr_loc), P<double>(s->gr_w), P<double>(s->gr_cols),
                       P<double>(s->gr_cos), P<uint8_t>(s->gr_ok), (long long)s->gr_n};
    LocalBuf cursor;
    TRY(dalloc(s, cursor, ((size_t)ns + 1) * sizeof(int)));
    CK(cudaMemsetAsync(s->gr_cnt.p, 0, ((size_t)ns + 1) * sizeof(int), s->stream));
    {
        Timer t(s, K_OTHER);
        if (s->gr_n > 0)
            ground_value_kernel<<<(unsigned)((s->gr_n + 127) / 128), 128, 0, s->stream>>>(
                g, ns, W, albedo, P<double>(dext), s->d.strato ? P<double>(dsext) : nullptr, P<double>(s->gr_value),
                P<int>(s->gr_cnt), P<int>(s->gr_cursor));
        TRY(launch_check(s));
        bucket_scan_kernel<<<1, 1024, 0, s->stream>>>(P<int>(s->gr_cnt), ns, P<int>(s->goff), P<int>(cursor));
        TRY(launch_check(s));
        ground_cell_kernel<<<ns, 256, 0, s->stream>>>(g, W, P<double>(dext), P<double>(s->gr_value), P<int>(s->goff),
                                                      P<float>(s->gm), P<float>(s->gdir), P<float4>(s->gdir4),
                                                      P<float>(s->gval));
        TRY(launch_check(s));
        ground_same_kernel<<<(unsigned)(((long long)ns * 32 + 127) / 128), 128, 0, s->stream>>>(
            P<int>(s->goff), P<float>(s->gdir), ns, s->d.nc, P<uint8_t>(s->gsame));
        TRY(launch_check(s));
    }
    CK(cudaStreamSynchronize(s->stream));
    TRY(dfree(s, dext));
    TRY(dfree(s, dsext));
    TRY(dfree(s, cursor));
    s->have_first = false;  // the first light's ground term uses these arrays
    graph_reset(s);
    return 0;
}

int sosb_set_bundle(sosb_handle s, int which, const sosb_bundle* b) {
    if (!s || !b) return 1;
    if (which != SOSB_CELLS && which != SOSB_OBSERVER) return fail(s, "E_BUNDLE: unknown bundle %d", which);
    if (which == SOSB_CELLS && b->ncell != s->ns)
        return fail(s, "E_SHAPE: cell bundle has %d cells, state %d", b->ncell, s->ns);
    PackedBundle pk;
    const std::string msg = pack_bundle(b, s->d.nc, pk);
    if (!msg.empty()) return fail(s, "%s", msg.c_str());
    BundleDev& bd = which == SOSB_CELLS ? s->cells : s->obs;
    invalidate_tables(bd);
    bd.b_mode = -1;
    graph_reset(s);
    bd.ncell = pk.ncell;
    bd.nray = pk.nray;
    bd.nseg = pk.nseg;
    bd.host_cell_off.assign(b->cell_off, b->cell_off + b->ncell + 1);
    bd.host_seg_off.assign(pk.seg_off.begin(), pk.seg_off.end());
    TRY(dput_vec(s, bd.cell_off, pk.cell_off));
    TRY(dput_vec(s, bd.ray_cell, pk.ray_cell));
    TRY(dput_vec(s, bd.p, pk.p));
    TRY(dput_vec(s, bd.frame, pk.frame));
    TRY(dput_vec(s, bd.dir, pk.dir));
    TRY(dput_vec(s, bd.dir_lo, pk.dir_lo));
    TRY(dput_vec(s, bd.dloc, pk.dloc));
    TRY(dput_vec(s, bd.pcp, pk.pcp));
    TRY(dput_vec(s, bd.seg_off, pk.seg_off));
    TRY(dput_vec(s, bd.seg, pk.seg));
    TRY(dput_vec(s, bd.lower, pk.lower));
    TRY(dput_vec(s, bd.end_j, pk.end_j));
    TRY(dput_vec(s, bd.end_col, pk.end_col));
    TRY(dput_vec(s, bd.hits, pk.hits));
    CK(cudaStreamSynchronize(s->stream));
    if (which == SOSB_CELLS) s->have_first = false;
    return 0;
}

int sosb_evaluate(sosb_handle s, int phase, int first, const float* field_dev, const float* boundary_dev,
                  float* moments_dev, float* flux_dev, float* radiance_dev) {
    if (!s) return 1;
    if (phase < 0 || phase > 2) return fail(s, "E_PHASE: %d", phase);
    if (!first && !field_dev) return fail(s, "E_FIELD: warm transport needs a field");
    if (first && phase == 1) return fail(s, "E_PHASE: first light has no ground pass");
    s->err.clear();
    TRY(evaluate_impl(s, phase, first, field_dev, boundary_dev, moments_dev, flux_dev, radiance_dev));
    CK(cudaStreamSynchronize(s->stream));
    return proj_check(s);
}

int sosb_apply(sosb_handle s, const float* field_dev, float* out_dev) {
    if (!s) return 1;
    if (!field_dev || !out_dev) return fail(s, "E_FIELD: null field");
    s->err.clear();
    TRY(apply_impl(s, field_dev, out_dev, 0ull));
    CK(cudaStreamSynchronize(s->stream));
    return proj_check(s);
}

// ------------------------------------------------------------------------ allocation-free composition
// Scratch of sosb_compose_static: the composition kernel's per-wavelength reduction words (nonfinite count, max |g|,
// max |g - x|), 3 x SOSB_STATIC_WAVES words. It lives in a file-scope device array, so this entry point never
// allocates; every GPU that loads the library holds these 768 bytes until the process exits.
#define SOSB_STATIC_WAVES 64
static __device__ __align__(256) unsigned g_compose_scratch[3 * SOSB_STATIC_WAVES];

// The array's name is only a host-side stand-in for it; its device address is looked up on every call, with the
// calling device current, so that a context torn down and created again (cudaDeviceReset) never leaves a stale
// address behind. The lookup is a host-side query next to the kernel's cost.
static int compose_scratch_address(sosb_state* s, unsigned** out) {
    void* ptr = nullptr;
    CK(cudaGetSymbolAddress(&ptr, g_compose_scratch));
    *out = static_cast<unsigned*>(ptr);
    return 0;
}

int sosb_compose_static(sosb_handle s, const float* moments_dev, const float* first_moments_dev, const float* x_dev,
                        uint64_t done_mask, float* out_dev, int64_t* nonfinite_host, double* source_relative_host) {
    if (!s) return 1;
    s->err.clear();
    const sosb_dims& d = s->d;
    if (!s->have_constants) return fail(s, "E_STATE: constants not set");
    if (!moments_dev || !first_moments_dev || !x_dev || !out_dev || !nonfinite_host || !source_relative_host)
        return fail(s, "E_FIELD: null pointer");
    if (d.W > SOSB_STATIC_WAVES)
        return fail(s, "E_SHAPE: %d wavelengths exceed the static composition scratch (%d)", d.W, SOSB_STATIC_WAVES);
    unsigned* scratch = nullptr;
    TRY(compose_scratch_address(s, &scratch));
    // the scratch keeps the previous call's words: clear the part this call accumulates into
    CK(cudaMemsetAsync(scratch, 0, 3 * SOSB_STATIC_WAVES * sizeof(unsigned), s->stream));
    const long long n = (long long)s->ns * s->src * d.W;
    compose_kernel<<<grid_for(n, wave_threads(d.W)), wave_threads(d.W), 0, s->stream>>>(
        moments_dev, first_moments_dev, x_dev, P<float>(s->rf), P<float>(s->af), P<float>(s->asca), P<float>(s->ext0),
        P<float>(s->s_eigen), P<float>(s->s_sca_src), s->K, s->src, d.W, s->af_w, n, (unsigned long long)done_mask, nullptr,
        out_dev, scratch);
    TRY(launch_check(s));
    unsigned words[3 * SOSB_STATIC_WAVES];
    CK(cudaMemcpyAsync(words, scratch, 3 * d.W * sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    for (int w = 0; w < d.W; ++w) {
        float mg, df;
        std::memcpy(&mg, &words[d.W + w], 4);
        std::memcpy(&df, &words[2 * d.W + w], 4);
        nonfinite_host[w] = words[w];
        source_relative_host[w] = (double)(df / std::max(mg, 1e-30f));
    }
    return 0;
}

int sosb_boxes(sosb_handle s, const float* field_dev, double* out_host) {
    if (!s) return 1;
    if (!field_dev || !out_host) return fail(s, "E_FIELD: null pointer");
    s->err.clear();
    return boxes_impl(s, field_dev, out_host);
}

// Solve the regularised Gram system (FP64, partial pivoting); weights normalised to sum 1 and rejected unless finite
// with max |w| < 8 (source_iteration.py:25-33). Returns false when singular or rejected. One thread per wavelength.
__device__ bool anderson_weights(int n, const double* G, float* out) {
    double A[4][5];
    double tr = 0.0;
    for (int i = 0; i < n; ++i) tr += G[i * n + i];
    const double reg = fmax(tr * 1e-10, 1e-30);
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) A[i][j] = G[i * n + j] + (i == j ? reg : 0.0);
        A[i][n] = 1.0;
    }
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (fabs(A[r][c]) > fabs(A[piv][c])) piv = r;
        if (A[piv][c] == 0.0) return false;
        if (piv != c)
            for (int j = 0; j <= n; ++j) {
                const double t = A[c][j];
                A[c][j] = A[piv][j];
                A[piv][j] = t;
            }
        for (int r = c + 1; r < n; ++r) {
            const double f = A[r][c] / A[c][c];
            for (int j = c; j <= n; ++j) A[r][j] -= f * A[c][j];
        }
    }
    double x[4];
    for (int i = n - 1; i >= 0; --i) {
        double v = A[i][n];
        for (int j = i + 1; j < n; ++j) v -= A[i][j] * x[j];
        x[i] = v / A[i][i];
    }
    double sum = 0.0;
    for (int i = 0; i < n; ++i) sum += x[i];
    double mx = 0.0;
    for (int i = 0; i < n; ++i) {
        x[i] /= sum;
        if (!isfinite(x[i])) return false;
        mx = fmax(mx, fabs(x[i]));
    }
    if (!(mx < 8.0)) return false;
    for (int i = 0; i < n; ++i) out[i] = (float)x[i];
    return true;
}

// ------------------------------------------------------------------------------------------------ the fixed-point loop
// Loop state of one solve on the device (Solver.solve, source_iteration.py:309-663): the evaluation count, the stop
// flag and outcome, the per-wavelength convergence marks and measures, and the Anderson ring order. The control
// kernel at the end of every evaluation updates it and the evaluation control block, so that one evaluation follows
// another without a host round trip; a CUDA graph's WHILE node replays the evaluation until the control kernel
// clears its condition.
enum { LOOP_RUNNING = 0, LOOP_CONVERGED = 1, LOOP_BUDGET = 2, LOOP_NONFINITE = 3 };

struct LoopDev {
    int it;        // evaluations completed
    int max_eval;
    int go;        // 1 while another evaluation follows
    int status;    // LOOP_*
    int fell_back; // the supplied start was replaced by the fallback start
    int has_fallback;
    int norder;    // ring slots of the Anderson history, oldest first
    int order[4];
    int nfeat;     // observer features of the residual: stop rows x directions
    int W;
    unsigned long long bad;  // non-finite composed values of the last evaluation
    double tol, fallback_ss, obs_scale;
    int done[64];
    double rr[64], ss[64];
};

// End of one evaluation (one block of CONTROL_THREADS): the observer change rr = max |new - old| / |new| over the stop
// rows' boxes and the source change ss = max |g - x| / max |g| from the composition's metrics ([0][W] non-finite
// counts, [1][W] max |g| bits, [2][W] max |g - x| bits); a wavelength is done from the second evaluation on when
// max(rr, ss) <= tol (source_iteration.py:353-376); the history row; the warm start's fallback check after the first
// evaluation; then per active wavelength the observer part of the residual feature, the new Gram row and column
// (FP64: the feature kernel's dots plus the observer products, one warp per entry with a fixed shuffle tree) and the
// Anderson weights of the next mix (source_iteration.py:401-635); last, the ring slot of the next evaluation (the
// oldest slot once four are held) and the condition of the enclosing WHILE node. The (feature, wavelength) loops are
// spread over the block; the per-wavelength decisions take one thread each.
constexpr int CONTROL_THREADS = 256;

__global__ void __launch_bounds__(CONTROL_THREADS)
control_kernel(LoopDev* __restrict__ L, EvalCtrl* __restrict__ ctrl, const unsigned* __restrict__ met,
               const double* __restrict__ old_b, const double* __restrict__ new_b, const double* __restrict__ dots,
               float* __restrict__ obs, double* __restrict__ gram, double* __restrict__ hist,
               unsigned* __restrict__ normmax, cudaGraphConditionalHandle cond, int set_cond, int seed) {
    __shared__ unsigned long long s_rr[64];  // bits of non-negative doubles order as unsigned integers
    __shared__ double s_ss[64];
    __shared__ int s_done[64];
    __shared__ unsigned long long s_bad;
    __shared__ int s_anderson, s_restart, s_stop, s_m, s_slot, s_order[4];
    const int t = threadIdx.x;
    const int W = L->W;
    const int it = L->it + 1;
    const int nobs = L->nfeat;
    if (t < 64) {
        s_rr[t] = 0ull;
        s_ss[t] = 0.0;
        s_done[t] = t < W ? L->done[t] : 1;
    }
    if (t == 0) s_bad = 0ull;
    __syncthreads();
    if (seed) {
        // history seed (no evaluation counted): the pair in ring slot ctrl->slot enters the Anderson history with
        // its observer features and Gram entries; the next evaluation takes the next slot without a mix
        if (t == 0) {
            s_anderson = 1;
            s_restart = 0;
            s_stop = 0;
            s_m = ctrl->m;
            s_slot = ctrl->slot;
            for (int j = 0; j < 4; ++j) s_order[j] = ctrl->order[j];
        }
        __syncthreads();
    }
    for (int q = t; q < nobs * W && !seed; q += CONTROL_THREADS) {
        const double nv = new_b[q], ov = old_b[q];  // [feature][W], q = i * W + w
        const double r = fabs(nv - ov) / fmax(fabs(nv), 1e-30);
        atomicMax(&s_rr[q % W], (unsigned long long)__double_as_longlong(r));
    }
    __syncthreads();
    if (t < W && !seed) {
        const double r = __longlong_as_double((long long)s_rr[t]);
        const float mg = __uint_as_float(met[W + t]), df = __uint_as_float(met[2 * W + t]);
        const double ss = (double)(df / fmaxf(mg, 1e-30f));
        L->rr[t] = r;
        L->ss[t] = ss;
        s_ss[t] = ss;
        if (it >= 2 && fmax(r, ss) <= L->tol) {
            L->done[t] = 1;
            s_done[t] = 1;
        }
        if (it <= L->max_eval) {
            hist[((size_t)(it - 1) * 2) * W + t] = r;
            hist[((size_t)(it - 1) * 2 + 1) * W + t] = ss;
        }
        if (met[t]) atomicAdd(&s_bad, (unsigned long long)met[t]);
    }
    __syncthreads();
    if (t == 0 && !seed) {
        L->it = it;
        L->bad = s_bad;
        int stop = 0, anderson = 0, restart = 0;
        if (s_bad) {
            L->status = LOOP_NONFINITE;
            stop = 1;
        } else {
            double mx = 0.0;
            for (int w = 0; w < W; ++w) mx = fmax(mx, s_ss[w]);
            if (it == 1 && L->has_fallback && !L->fell_back && mx > L->fallback_ss) {
                // the supplied start is further from the fixed point than the fallback start: restart from it
                L->fell_back = 1;
                L->norder = 0;
                restart = 1;
                if (it >= L->max_eval) {
                    stop = 1;
                    L->status = LOOP_BUDGET;
                }
            } else {
                int all = 1;
                for (int w = 0; w < W; ++w) all &= s_done[w];
                if (all) {
                    stop = 1;
                    L->status = LOOP_CONVERGED;
                } else {
                    anderson = 1;
                }
            }
        }
        s_anderson = anderson;
        s_restart = restart;
        s_stop = stop;
        // this evaluation's g and residual feature are in ring slot ctrl->slot; the ring order after it is the order
        // its evaluation was issued with (ctrl->order[0 .. ctrl->m - 1])
        s_m = ctrl->m;
        s_slot = ctrl->slot;
        for (int j = 0; j < 4; ++j) s_order[j] = ctrl->order[j];
    }
    __syncthreads();
    if (s_anderson) {
        const int m = s_m, slot = s_slot;
        for (int q = t; q < nobs * W; q += CONTROL_THREADS) {
            const int i = q / W, w = q - i * W;
            if (s_done[w]) continue;
            const double nv = new_b[q], ov = old_b[q];
            obs[((size_t)slot * W + w) * nobs + i] = (float)((nv - ov) / fmax(fabs(nv), 1e-20) * L->obs_scale);
        }
        __syncthreads();
        const int lane = t & 31, warp = t >> 5;
        for (int e = warp; e < W * m; e += CONTROL_THREADS / 32) {
            const int w = e / m, j = e - w * m;
            if (s_done[w]) continue;  // the whole warp skips
            const int oj = s_order[j];
            const float* a = obs + ((size_t)slot * W + w) * nobs;
            const float* q = obs + ((size_t)oj * W + w) * nobs;
            double acc = 0.0;
            for (int i = lane; i < nobs; i += 32) acc += (double)a[i] * (double)q[i];
            for (int dd = 16; dd >= 1; dd >>= 1) acc += __shfl_xor_sync(FULL_MASK, acc, dd);
            if (lane == 0) {
                const double v = dots[j * W + w] + acc;
                gram[(size_t)w * 16 + slot * 4 + oj] = v;
                gram[(size_t)w * 16 + oj * 4 + slot] = v;
            }
        }
        __syncthreads();
        if (t < 64) {
            const int w = t;
            int use = 0;
            float wt[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            if (w < W && !s_done[w] && m > 1) {
                const double* gw = gram + (size_t)w * 16;
                double G[16];
                for (int i = 0; i < m; ++i)
                    for (int j = 0; j < m; ++j) G[i * m + j] = gw[s_order[i] * 4 + s_order[j]];
                use = anderson_weights(m, G, wt) ? 1 : 0;
            }
            ctrl->use[w] = use;
            for (int j = 0; j < 4; ++j) ctrl->weights[j * 64 + w] = (use && j < m) ? wt[j] : 0.0f;
        }
    }
    __syncthreads();
    if (t == 0) {
        int stop = s_stop;
        if (s_anderson) {
            const int m = s_m;
            L->norder = m;
            for (int j = 0; j < 4; ++j) L->order[j] = s_order[j];
            ctrl->mix = seed ? 0 : 1;  // after a seed the next evaluation starts from the supplied x
            ctrl->mix_m = m;
            for (int j = 0; j < 4; ++j) ctrl->mix_order[j] = j < m ? s_order[j] : s_order[m - 1];
            if (!seed && it >= L->max_eval) {
                stop = 1;
                L->status = LOOP_BUDGET;
            }
        } else if (s_restart) {
            ctrl->mix = 0;
        }
        ctrl->restart = s_restart;
        if (!stop) {
            // the next evaluation's ring slot: a new one while fewer than four are held, else the oldest
            int pend[4], np = L->norder;
            for (int j = 0; j < 4; ++j) pend[j] = L->order[j];
            int nslot;
            if (np < 4) {
                nslot = np;
            } else {
                nslot = pend[0];
                for (int j = 0; j < 3; ++j) pend[j] = pend[j + 1];
                np = 3;
            }
            pend[np++] = nslot;
            ctrl->slot = nslot;
            ctrl->m = np;
            for (int j = 0; j < 4; ++j) ctrl->order[j] = j < np ? pend[j] : nslot;
            unsigned long long mask = 0ull;
            for (int v = 0; v < W; ++v)
                if (s_done[v]) mask |= 1ull << v;
            ctrl->done = mask;
        }
        L->go = stop ? 0 : 1;
        if (set_cond && !seed) cudaGraphSetConditional(cond, stop ? 0u : 1u);
    }
    if (t < 64) normmax[t] = 0u;  // the next evaluation's norm pass collects its maxima from zero
}

// First node of a solve graph: the WHILE node runs while the eager first evaluation left the loop going.
__global__ void gate_kernel(const LoopDev* __restrict__ L, cudaGraphConditionalHandle cond) {
    cudaGraphSetConditional(cond, L->go ? 1u : 0u);
}

// Buffers of the loop: iterate x and g, the Anderson rings, norms, Gram partials and dots, the observer boxes of x
// and g, the residual's observer features and the Gram matrices, the history, control and loop state. A buffer
// that moves drops the captured solve graph.
static int loop_alloc(sosb_state* s, int max_eval) {
    const int W = s->d.W;
    const size_t bytes = (size_t)s->ns * s->src * W * sizeof(float);
    DevBuf* bufs[] = {&s->fx, &s->fg, &s->ring_g[0], &s->ring_g[1], &s->ring_g[2], &s->ring_g[3], &s->ring_f[0],
                      &s->ring_f[1], &s->ring_f[2], &s->ring_f[3], &s->norms, &s->partials, &s->dots, &s->box_old,
                      &s->box_new, &s->obs_feat, &s->gram, &s->hist_dev, &s->normmax, &s->metrics, &s->ctrl_dev,
                      &s->loop_dev};
    void* before[sizeof bufs / sizeof bufs[0]];
    for (size_t i = 0; i < sizeof bufs / sizeof bufs[0]; ++i) before[i] = bufs[i]->p;
    TRY(dalloc(s, s->fx, bytes));
    TRY(dalloc(s, s->fg, bytes));
    for (int j = 0; j < 4; ++j) {
        TRY(dalloc(s, s->ring_g[j], bytes));
        TRY(dalloc(s, s->ring_f[j], bytes));
    }
    TRY(dalloc(s, s->norms, (size_t)s->ns * W * sizeof(float)));
    // feature kernel: blocks of a multiple of W threads (one wavelength per thread), whole cells per block
    s->feat_threads = W * std::max(1, 256 / W);
    // cells of at least four elements a thread: one cell per block, up to 8 blocks an SM; smaller cells: 4 an SM
    const bool long_rows = (long long)s->src * W >= 4LL * s->feat_threads;
    s->feat_blocks = (int)std::min<long long>(s->ns, 152LL * (long_rows ? 8 : 4));
    TRY(dalloc(s, s->partials, (size_t)s->feat_blocks * 4 * W * sizeof(double)));
    TRY(dalloc(s, s->dots, (size_t)4 * W * sizeof(double)));
    const size_t nbox = (size_t)s->d.n_monitor_rows * s->d.n_dirs * W;
    TRY(dalloc(s, s->box_old, nbox * sizeof(double)));
    TRY(dalloc(s, s->box_new, nbox * sizeof(double)));
    const int nfeat = s->d.monitors * s->d.n_dirs;
    TRY(dalloc(s, s->obs_feat, (size_t)4 * W * std::max(nfeat, 1) * sizeof(float)));
    TRY(dalloc(s, s->gram, (size_t)W * 16 * sizeof(double)));
    TRY(dalloc(s, s->hist_dev, (size_t)std::max(max_eval, 64) * 2 * W * sizeof(double)));
    TRY(dalloc(s, s->normmax, 64 * sizeof(unsigned)));
    TRY(dalloc(s, s->metrics, 3 * 64 * sizeof(unsigned)));
    TRY(dalloc(s, s->ctrl_dev, sizeof(EvalCtrl)));
    TRY(dalloc(s, s->loop_dev, sizeof(LoopDev)));
    if (!s->ctrl_host) CK(cudaMallocHost(&s->ctrl_host, sizeof(EvalCtrl)));
    if (!s->loop_host) CK(cudaMallocHost(&s->loop_host, sizeof(LoopDev)));
    for (size_t i = 0; i < sizeof bufs / sizeof bufs[0]; ++i)
        if (before[i] != bufs[i]->p) {
            graph_reset(s);
            break;
        }
    return 0;
}

// One evaluation on the device, the same launches every time (the control block and the loop state carry what
// changes): x = Anderson mix of the previous ring (or the fallback start after a restart); boxes(x); g = apply(x)
// with the composition metrics; boxes(g); g into the ring; residual feature and FP64 Gram column; the control kernel
// (source_iteration.py:309-635, one evaluation of the loop). set_cond: the control kernel sets the enclosing WHILE
// node's condition.
// The end of an evaluation after g: g into ring slot ctrl->slot, the residual feature (g - x) / norm and its FP64
// Gram column against the ring's slots, then the control kernel (seed: a history seed, see control_kernel).
static int residual_tail(sosb_state* s, bool set_cond, bool seed) {
    const int W = s->d.W;
    const long long n = (long long)s->ns * s->src * W;
    float* x = P<float>(s->fx);
    float* g = P<float>(s->fg);
    EvalCtrl* ctrl = P<EvalCtrl>(s->ctrl_dev);
    const Ring4 rg{{P<float>(s->ring_g[0]), P<float>(s->ring_g[1]), P<float>(s->ring_g[2]), P<float>(s->ring_g[3])}};
    const Ring4 rf{{P<float>(s->ring_f[0]), P<float>(s->ring_f[1]), P<float>(s->ring_f[2]), P<float>(s->ring_f[3])}};
    {
        Timer t(s, K_ANDERSON);
        ring_copy_kernel<<<grid_for(n, 256), 256, 0, s->stream>>>(g, rg, ctrl, n);
    }
    TRY(launch_check(s));
    {
        Timer t(s, K_ANDERSON);
        norm_kernel<<<(unsigned)std::min<long long>(s->ns, 152LL * 16), s->feat_threads,
                      (size_t)s->feat_threads * sizeof(float), s->stream>>>(g, (long long)s->ns, s->src, W,
                                                                            P<float>(s->norms), P<unsigned>(s->normmax));
    }
    TRY(launch_check(s));
    {
        Timer t(s, K_ANDERSON);
        feature_kernel<<<s->feat_blocks, s->feat_threads, (size_t)s->feat_threads * 4 * sizeof(double),
                         s->stream>>>(g, x, P<float>(s->norms), P<unsigned>(s->normmax), (long long)s->ns, s->src, W,
                                      rf, ctrl, P<double>(s->partials));
    }
    TRY(launch_check(s));
    {
        Timer t(s, K_ANDERSON);
        sum_partials_kernel<<<(4 * W * 32 + 127) / 128, 128, 0, s->stream>>>(P<double>(s->partials), s->feat_blocks,
                                                                             4 * W, P<double>(s->dots));
    }
    TRY(launch_check(s));
    {
        Timer t(s, K_ANDERSON);
        control_kernel<<<1, CONTROL_THREADS, 0, s->stream>>>(P<LoopDev>(s->loop_dev), ctrl, P<unsigned>(s->metrics),
                                                             P<double>(s->box_old), P<double>(s->box_new),
                                                             P<double>(s->dots), P<float>(s->obs_feat),
                                                             P<double>(s->gram), P<double>(s->hist_dev),
                                                             P<unsigned>(s->normmax), s->cond, set_cond ? 1 : 0,
                                                             seed ? 1 : 0);
    }
    return launch_check(s);
}

// One evaluation on the device, the same launches every time (the control block and the loop state carry what
// changes): x = Anderson mix of the previous ring (or the fallback start after a restart); boxes(x); g = apply(x)
// with the composition metrics; boxes(g); then residual_tail (source_iteration.py:309-635, one evaluation of the
// loop). set_cond: the control kernel sets the enclosing WHILE node's condition.
static int eval_body(sosb_state* s, bool set_cond) {
    const int W = s->d.W;
    const long long n = (long long)s->ns * s->src * W;
    float* x = P<float>(s->fx);
    float* g = P<float>(s->fg);
    EvalCtrl* ctrl = P<EvalCtrl>(s->ctrl_dev);
    const Ring4 rg{{P<float>(s->ring_g[0]), P<float>(s->ring_g[1]), P<float>(s->ring_g[2]), P<float>(s->ring_g[3])}};
    {
        Timer t(s, K_ANDERSON);
        mix_kernel<<<grid_for(n, wave_threads(W)), wave_threads(W), 0, s->stream>>>(g, rg, ctrl, W, n, x);
    }
    TRY(launch_check(s));
    TRY(boxes_dev(s, x, P<double>(s->box_old)));
    s->plane_keep = true;  // apply(x) reads the plane boxes(x) just built: nothing writes x in between
    TRY(apply_impl(s, x, g, 0ull, &ctrl->done));
    TRY(boxes_dev(s, g, P<double>(s->box_new)));
    return residual_tail(s, set_cond, false);
}

// The solve graph of the handle: a gate kernel (the condition from the loop state) and a WHILE node whose body is
// one evaluation (eval_body with its control kernel). Built after an eager first evaluation, once tables, pair
// lists and launch shapes exist; dropped when constants, bundles, modes or loop buffers change. A capture that fails
// (an allocation, or a call that a conditional body cannot hold) turns graphs off for the handle.
static int build_solve_graph(sosb_state* s) {
    if (s->graph) return 0;
    cudaGraph_t gph = nullptr;
    cudaError_t e = cudaGraphCreate(&gph, 0);
    cudaGraphConditionalHandle cond = 0;
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&cond, gph, 0, 0);
    cudaGraphNode_t gate = nullptr, loop = nullptr;
    cudaGraph_t body = nullptr;
    const LoopDev* ld = P<LoopDev>(s->loop_dev);
    if (e == cudaSuccess) {
        cudaKernelNodeParams kp{};
        void* args[] = {(void*)&ld, (void*)&cond};
        kp.func = (void*)gate_kernel;
        kp.gridDim = dim3(1);
        kp.blockDim = dim3(1);
        kp.kernelParams = args;
        e = cudaGraphAddKernelNode(&gate, gph, nullptr, 0, &kp);
    }
    if (e == cudaSuccess) {
        cudaGraphNodeParams np{};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = cond;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        e = cudaGraphAddNode(&loop, gph, &gate, nullptr, 1, &np);
        if (e == cudaSuccess) body = np.conditional.phGraph_out[0];
    }
    int rc = 1;
    int64_t captured = 0;
    if (e == cudaSuccess) {
        s->cond = cond;
        const int64_t l0 = s->launches;
        e = cudaStreamBeginCaptureToGraph(s->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            rc = eval_body(s, true);
            cudaGraph_t out = nullptr;
            const cudaError_t e1 = cudaStreamEndCapture(s->stream, &out);
            if (e1 != cudaSuccess) e = e1;
        }
        captured = s->launches - l0;  // kernels recorded into the body, counted while capturing
        s->launches = l0;
    }
    cudaGraphExec_t exec = nullptr;
    if (rc == 0 && e == cudaSuccess) e = cudaGraphInstantiate(&exec, gph, 0);
    if (gph) cudaGraphDestroy(gph);
    if (rc != 0 || e != cudaSuccess || !exec) {
        cudaGetLastError();
        if (exec) cudaGraphExecDestroy(exec);
        s->graphs = false;
        s->err.clear();
        return 0;
    }
    s->graph = exec;
    s->graph_launches = captured;
    return 0;
}

// Host side of one solve (Solver.solve, source_iteration.py:309-663). The loop itself runs on the device: begin()
// sets the start and the loop state, first() enqueues the first evaluation directly (it builds node tables, pair
// lists and tunes launch shapes), rest() enqueues the solve graph (the WHILE node runs the remaining evaluations
// until the control kernel stops it) or, with graphs off, one evaluation at a time with a read of the stop flag,
// and end() reads the outcome, the statistics and the history back once.
struct SolveRun {
    sosb_state* s = nullptr;
    int max_eval = 0;
    std::chrono::steady_clock::time_point t0;
    int64_t launches0 = 0;
    bool graphed = false;

    // Sets the start x (NULL: zero; host or device field), the control block and the loop state.
    int begin(sosb_state* st, int max_eval_, double tol, const float* x0, int x0_device, bool keep_first,
              double fallback_ss, const float* fallback_dev) {
        s = st;
        max_eval = max_eval_;
        s->err.clear();
        t0 = std::chrono::steady_clock::now();
        launches0 = s->launches;
        TRY(check_ready(s, true));
        if (!keep_first) s->have_first = false;  // a solve includes its first-light pass unless told otherwise
        TRY(loop_alloc(s, max_eval));
        const int W = s->d.W;
        const size_t bytes = (size_t)s->ns * s->src * W * sizeof(float);
        // evaluation 1: ring slot 0, no mix (x is the start)
        EvalCtrl& c = *s->ctrl_host;
        std::memset(&c, 0, sizeof c);
        c.slot = 0;
        c.m = 1;
        c.fallback = fallback_dev;
        LoopDev& L = *s->loop_host;
        std::memset(&L, 0, sizeof L);
        L.max_eval = max_eval;
        L.go = 1;
        L.has_fallback = fallback_dev ? 1 : 0;
        L.nfeat = s->d.monitors * s->d.n_dirs;
        L.W = W;
        L.tol = tol;
        L.fallback_ss = fallback_ss;
        L.obs_scale = std::sqrt((double)((size_t)s->ns * s->src) / (double)std::max(L.nfeat, 1));
        CK(cudaMemcpyAsync(s->ctrl_dev.p, &c, sizeof c, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(s->loop_dev.p, &L, sizeof L, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemsetAsync(s->gram.p, 0, (size_t)W * 16 * sizeof(double), s->stream));
        CK(cudaMemsetAsync(s->normmax.p, 0, 64 * sizeof(unsigned), s->stream));
        if (fallback_dev && s->warm_history) {
            // the pair (x = 0, g = the fallback start, the single-scattering source) enters the Anderson history
            // first, so that the supplied start is the second iterate of the plain iteration, not a restart
            CK(cudaMemsetAsync(s->fx.p, 0, bytes, s->stream));
            CK(cudaMemcpyAsync(s->fg.p, fallback_dev, bytes, cudaMemcpyDeviceToDevice, s->stream));
            TRY(boxes_dev(s, P<float>(s->fx), P<double>(s->box_old)));
            TRY(boxes_dev(s, P<float>(s->fg), P<double>(s->box_new)));
            TRY(residual_tail(s, false, true));
        }
        if (x0)
            CK(cudaMemcpyAsync(s->fx.p, x0, bytes, x0_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                               s->stream));
        else
            CK(cudaMemsetAsync(s->fx.p, 0, bytes, s->stream));
        return 0;
    }

    int first() { return eval_body(s, false); }

    // The remaining evaluations: the solve graph (no host round trip), or the launches one evaluation at a time.
    int rest() {
        graphed = false;
        if (s->graphs && !s->timing) TRY(build_solve_graph(s));
        if (s->graph && s->graphs && !s->timing) {
            CK(cudaGraphLaunch(s->graph, s->stream));
            graphed = true;
            return 0;
        }
        for (;;) {
            CK(cudaMemcpyAsync(&s->loop_host->go, &P<LoopDev>(s->loop_dev)->go, sizeof(int), cudaMemcpyDeviceToHost,
                               s->stream));
            CK(cudaStreamSynchronize(s->stream));
            if (!s->loop_host->go) return 0;
            TRY(eval_body(s, false));
        }
    }

    // The result (g when converged, else the mix the next evaluation would have started with: the reference leaves
    // its last mix in x), the statistics and the history; the reference's error codes.
    int end(float* x_out, int x_out_is_device, sosb_stats* stats) {
        CK(cudaMemcpyAsync(s->loop_host, s->loop_dev.p, sizeof(LoopDev), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        TRY(proj_check(s));
        const LoopDev& L = *s->loop_host;
        const int W = s->d.W;
        const int n_it = std::min(L.it, max_eval);
        if (graphed) s->launches += 1 + s->graph_launches * std::max(L.it - 1, 0);
        std::vector<double> h((size_t)n_it * 2 * W);
        if (n_it) CK(cudaMemcpy(h.data(), s->hist_dev.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost));
        s->hist_obs.assign((size_t)n_it * W, 0.0);
        s->hist_src.assign((size_t)n_it * W, 0.0);
        for (int e = 0; e < n_it; ++e)
            for (int w = 0; w < W; ++w) {
                s->hist_obs[(size_t)e * W + w] = h[((size_t)e * 2) * W + w];
                s->hist_src[(size_t)e * W + w] = h[((size_t)e * 2 + 1) * W + w];
            }
        if (L.status == LOOP_NONFINITE)
            return fail(s, "E_NONFINITE_SOURCE: %llu values after evaluation %d", L.bad, L.it);
        const bool converged = L.status == LOOP_CONVERGED;
        const size_t bytes = (size_t)s->ns * s->src * W * sizeof(float);
        float* result = P<float>(converged ? s->fg : s->fx);
        if (!converged) {
            const long long n = (long long)s->ns * s->src * W;
            const Ring4 rg{{P<float>(s->ring_g[0]), P<float>(s->ring_g[1]), P<float>(s->ring_g[2]),
                            P<float>(s->ring_g[3])}};
            mix_kernel<<<grid_for(n, wave_threads(W)), wave_threads(W), 0, s->stream>>>(
                P<float>(s->fg), rg, P<EvalCtrl>(s->ctrl_dev), W, n, result);
            TRY(launch_check(s));
        }
        CK(cudaMemcpyAsync(x_out, result, bytes, x_out_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                           s->stream));
        CK(cudaStreamSynchronize(s->stream));
        if (stats) {
            std::memset(stats, 0, sizeof *stats);
            stats->evaluations = n_it;
            stats->converged = converged ? 1 : 0;
            stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            for (int w = 0; w < W; ++w) {
                stats->observer_relative[w] = L.rr[w];
                stats->source_relative[w] = L.ss[w];
                stats->done[w] = L.done[w];
            }
            stats->kernel_launches = s->launches - launches0;
            stats->start_fallback = L.fell_back;
        }
        if (!converged) {
            int nd = 0;
            for (int w = 0; w < W; ++w) nd += L.done[w] != 0;
            return fail(s, "E_NOT_CONVERGED: %d/%d within %g", nd, W, L.tol);
        }
        return 0;
    }
};

// The fixed-point loop of one handle. x0: NULL (zero start), a host (x0_device = 0) or device field. keep_first:
// reuse the first-light moments already computed on this handle. fallback_dev: when the first evaluation's largest
// source relative change exceeds fallback_ss, the iteration restarts from this device field.
static int solve_impl(sosb_state* s, int max_eval, double tol, const float* x0, int x0_device, bool keep_first,
                      double fallback_ss, const float* fallback_dev, float* x_out, int x_out_is_device,
                      sosb_stats* stats) {
    if (!x_out) return fail(s, "E_FIELD: null output");
    if (max_eval < 1) return fail(s, "E_FIELD: max_eval %d", max_eval);
    SolveRun run;
    TRY(run.begin(s, max_eval, tol, x0, x0_device, keep_first, fallback_ss, fallback_dev));
    TRY(run.first());
    TRY(run.rest());
    return run.end(x_out, x_out_is_device, stats);
}

// Many solves from one host thread: every state's first evaluation and then its solve graph are enqueued on the
// state's own stream, up to `concurrency` states in flight; the thread only waits for streams to finish (no
// per-evaluation round trip), and a finished state hands its place to the next one. With graphs off, every state
// runs its evaluations one at a time (SolveRun::rest).
static int batch_drive(sosb_handle* hs, int n, int max_eval, double tol, const float* const* x0, int x0_device,
                       bool keep_first, double fallback_ss, const float* const* fallback_dev, float* const* x_out,
                       int x_out_is_device, sosb_stats* stats, int* status, int concurrency) {
    if (n <= 0) return 0;
    const int cap = std::max(1, std::min(concurrency > 0 ? concurrency : n, n));
    std::vector<SolveRun> runs(n);
    std::vector<int> active;
    int next = 0;
    auto start = [&]() {
        while (next < n && (int)active.size() < cap) {
            const int i = next++;
            if (!hs[i] || !x_out[i]) {
                status[i] = 1;
                continue;
            }
            if (keep_first && !hs[i]->have_first) {
                status[i] = fail(hs[i], "E_STATE: no first light on this handle (run an apply first)");
                continue;
            }
            status[i] = runs[i].begin(hs[i], max_eval, tol, x0 ? x0[i] : nullptr, x0_device, keep_first, fallback_ss,
                                      fallback_dev ? fallback_dev[i] : nullptr);
            if (status[i] == 0) status[i] = runs[i].first();
            if (status[i] == 0) status[i] = runs[i].rest();
            if (status[i] == 0) active.push_back(i);
        }
    };
    start();
    while (!active.empty()) {
        std::vector<int> keep;
        bool finished = false;
        for (int i : active) {
            const cudaError_t q = cudaStreamQuery(hs[i]->stream);
            if (q == cudaErrorNotReady) {
                keep.push_back(i);
                continue;
            }
            finished = true;
            if (q != cudaSuccess)
                status[i] = fail(hs[i], "E_CUDA: %s", cudaGetErrorString(q));
            else
                status[i] = runs[i].end(x_out[i], x_out_is_device, stats ? &stats[i] : nullptr);
        }
        active = keep;
        start();
        if (!finished) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    int failed = 0;
    for (int i = 0; i < n; ++i) failed += status[i] != 0;
    return failed ? 3 : 0;
}

int sosb_solve(sosb_handle s, int max_eval, double tol, const float* x0_host, float* x_out, int x_out_is_device,
               sosb_stats* stats) {
    if (!s) return 1;
    return solve_impl(s, max_eval, tol, x0_host, 0, false, 0.0, nullptr, x_out, x_out_is_device, stats);
}

int sosb_history(sosb_handle s, int capacity, int32_t* count, double* observer_relative, double* source_relative) {
    if (!s) return 1;
    if (!count) return fail(s, "E_FIELD: null pointer");
    const int W = s->d.W;
    const int n = W ? (int)(s->hist_obs.size() / W) : 0;
    *count = n;
    const int m = std::min(n, std::max(capacity, 0));
    if (m && (!observer_relative || !source_relative)) return fail(s, "E_FIELD: null pointer");
    std::copy(s->hist_obs.begin(), s->hist_obs.begin() + (size_t)m * W, observer_relative);
    std::copy(s->hist_src.begin(), s->hist_src.begin() + (size_t)m * W, source_relative);
    return 0;
}

int sosb_solve_warm(sosb_handle s, int max_eval, double tol, const float* x0_dev, double fallback_ss,
                    const float* fallback_dev, float* x_out, int x_out_is_device, sosb_stats* stats) {
    if (!s) return 1;
    if (!x0_dev) return fail(s, "E_FIELD: null start");
    if (!s->have_first) return fail(s, "E_STATE: no first light on this handle (run an apply first)");
    return solve_impl(s, max_eval, tol, x0_dev, 1, true, fallback_ss, fallback_dev, x_out, x_out_is_device, stats);
}

int sosb_solve_batch(sosb_handle* hs, int n, int max_eval, double tol, const float* const* x0_host,
                     float* const* x_out, int x_out_is_device, sosb_stats* stats, int* status, int threads) {
    if (!hs || !x_out || !status || n < 0) return 1;
    return batch_drive(hs, n, max_eval, tol, x0_host, 0, false, 0.0, nullptr, x_out, x_out_is_device, stats, status,
                       threads);
}

int sosb_apply_batch(sosb_handle* hs, int n, const float* const* fields, float* const* outs, int* status,
                     int threads) {
    if (!hs || !fields || !outs || !status || n < 0) return 1;
    run_parallel(n, threads, [&](int i) { status[i] = sosb_apply(hs[i], fields[i], outs[i]); });
    for (int i = 0; i < n; ++i)
        if (status[i]) return 3;
    return 0;
}

int sosb_solve_warm_batch(sosb_handle* hs, int n, int max_eval, double tol, const float* const* x0_dev,
                          double fallback_ss, const float* const* fallback_dev, float* const* x_out,
                          int x_out_is_device, sosb_stats* stats, int* status, int threads) {
    if (!hs || !x0_dev || !x_out || !status || n < 0) return 1;
    return batch_drive(hs, n, max_eval, tol, x0_dev, 1, true, fallback_ss, fallback_dev, x_out, x_out_is_device,
                       stats, status, threads);
}

int sosb_set_pairs(sosb_handle s, int enable) {
    if (!s) return 1;
    s->pairs = enable != 0;
    invalidate_tables(s->cells);
    invalidate_tables(s->obs);
    graph_reset(s);
    return 0;
}

int sosb_set_warm_history(sosb_handle s, int enable) {
    if (!s) return 1;
    s->warm_history = enable != 0;
    return 0;
}

int sosb_set_ground_mma(sosb_handle s, int enable) {
    if (!s) return 1;
    s->ground_mma = enable != 0;
    s->have_first = false;  // the next apply recomputes its first light with the chosen kernel
    graph_reset(s);
    return 0;
}

int sosb_set_corner_mma(sosb_handle s, int enable) {
    if (!s) return 1;
    s->corner_mma = enable != 0;
    invalidate_tables(s->cells);
    invalidate_tables(s->obs);
    graph_reset(s);
    return 0;
}

int sosb_set_autotune(sosb_handle s, int enable) {
    if (!s) return 1;
    graph_reset(s);
    s->autotune = enable != 0;
    return 0;
}

int sosb_set_graphs(sosb_handle s, int enable) {
    if (!s) return 1;
    graph_reset(s);
    s->graphs = enable != 0;
    return 0;
}

}  // extern "C"
