// Host-side packing of a state into the device layout of sos_math.cuh (shared by libsosb and its host build).
//
// FP64 inputs become double-single (hi, lo) FP32 pairs where the transport computes in double-single (start points,
// directions, segment ends, quadrature nodes: numpy_reference.py:294-311 splits them the same way), FP32 elsewhere.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/sosb.h"

namespace sos {

inline void split_ds(double x, float& hi, float& lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

struct PackedBundle {
    int ncell = 0;
    int64_t nray = 0, nseg = 0;
    std::vector<int> cell_off, ray_cell, seg_off, end_j;
    std::vector<float> p, frame, dir, dir_lo, dloc, pcp, seg, end_col;
    std::vector<uint8_t> lower, hits;
};

// Validates and packs one bundle; returns an error message ("" on success).
inline std::string pack_bundle(const sosb_bundle* b, int nc, PackedBundle& out) {
    char msg[256];
    if (b->ncell < 1 || b->nray <= 0 || b->nray >= (1LL << 31) || b->nseg < 0 || b->nseg >= (1LL << 31)) {
        snprintf(msg, sizeof msg, "E_SHAPE: %d cells, %lld rays, %lld segments", b->ncell, (long long)b->nray,
                 (long long)b->nseg);
        return msg;
    }
    if (!b->cell_off || !b->p || !b->target || !b->d || !b->dloc || !b->weight || !b->seg_off || !b->seg_a ||
        !b->seg_b || !b->seg_lower || !b->end_j || !b->end_f || !b->end_col || !b->hits)
        return "E_SHAPE: missing bundle array";
    if (b->cell_off[0] != 0 || b->cell_off[b->ncell] != b->nray || b->seg_off[0] != 0 || b->seg_off[b->nray] != b->nseg)
        return "E_SHAPE: offsets do not cover the rays and segments";
    const int64_t nr = b->nray, ne = b->nseg;
    out.ncell = b->ncell;
    out.nray = nr;
    out.nseg = ne;
    out.cell_off.resize(b->ncell + 1);
    out.ray_cell.resize(nr);
    out.seg_off.resize(nr + 1);
    out.end_j.resize(nr);
    out.p.resize(6 * (size_t)b->ncell);
    out.frame.resize(9 * (size_t)b->ncell);
    out.dir.resize(4 * nr);
    out.dir_lo.resize(4 * nr);
    out.dloc.resize(4 * nr);
    out.pcp.resize(nr);
    out.seg.resize(4 * ne);
    out.end_col.resize(6 * nr);
    out.lower.assign(b->seg_lower, b->seg_lower + ne);
    out.hits.assign(b->hits, b->hits + nr);
    for (int i = 0; i <= b->ncell; ++i) out.cell_off[i] = (int)b->cell_off[i];
    for (int i = 0; i < b->ncell; ++i) {
        if (b->cell_off[i + 1] < b->cell_off[i]) return "E_SHAPE: cell offsets decrease";
        for (int k = 0; k < 3; ++k) split_ds(b->p[3 * i + k], out.p[6 * i + k], out.p[6 * i + 3 + k]);
        for (int k = 0; k < 9; ++k) out.frame[9 * i + k] = (float)b->target[9 * i + k];
        for (int64_t r = b->cell_off[i]; r < b->cell_off[i + 1]; ++r) out.ray_cell[r] = i;
    }
    for (int64_t r = 0; r < nr; ++r) {
        if (b->seg_off[r + 1] < b->seg_off[r]) return "E_SHAPE: segment offsets decrease";
        if (b->hits[r] && (b->end_j[r] < 0 || b->end_j[r] > nc - 2)) {
            snprintf(msg, sizeof msg, "E_SHAPE: ray %lld ends outside the solar-zenith grid", (long long)r);
            return msg;
        }
        const double* dv = b->d + 3 * r;
        const double st = std::sqrt(std::fmax(0.0, 1.0 - dv[2] * dv[2]));
        for (int k = 0; k < 3; ++k) split_ds(dv[k], out.dir[4 * r + k], out.dir_lo[4 * r + k]);
        out.dir[4 * r + 3] = (float)st;
        out.dir_lo[4 * r + 3] = (float)b->weight[r];
        for (int k = 0; k < 3; ++k) out.dloc[4 * r + k] = (float)b->dloc[3 * r + k];
        out.dloc[4 * r + 3] = (float)b->end_f[r];
        out.pcp[r] = (float)(st > 1e-12 ? dv[0] / std::fmax(st, 1e-30) : 1.0);
        out.seg_off[r] = (int)b->seg_off[r];
        out.end_j[r] = b->hits[r] ? b->end_j[r] : 0;
        for (int k = 0; k < 5; ++k) out.end_col[6 * r + k] = b->end_col[5 * r + k];
        out.end_col[6 * r + 5] = b->end_st ? b->end_st[r] : 0.0f;
    }
    out.seg_off[nr] = (int)b->seg_off[nr];
    for (int64_t e = 0; e < ne; ++e) {
        split_ds(b->seg_a[e], out.seg[4 * e + 0], out.seg[4 * e + 1]);
        split_ds(b->seg_b[e], out.seg[4 * e + 2], out.seg[4 * e + 3]);
    }
    return "";
}

// FP32 coefficients of the normalised associated-Legendre recurrence (arithmetic.py:69-83):
// a[k], b[k] for k = l(l+1)/2 + m and the diagonal factors d[m].
inline void sh_recurrence(int L, std::vector<float>& a, std::vector<float>& b, std::vector<float>& d) {
    const int K = (L + 1) * (L + 2) / 2;
    a.assign(K, 0.0f);
    b.assign(K, 0.0f);
    d.assign(L + 1, 0.0f);
    for (int m = 1; m <= L; ++m) d[m] = (float)(-std::sqrt((2.0 * m + 1) / (2.0 * m)));
    for (int l = 1; l <= L; ++l)
        for (int m = 0; m < l; ++m) {
            const int k = l * (l + 1) / 2 + m;
            a[k] = (float)std::sqrt((4.0 * l * l - 1) / (double)(l * l - m * m));
            if (l > m + 1)
                b[k] = (float)std::sqrt((2.0 * l + 1) * ((l - 1.0) * (l - 1.0) - m * m) /
                                        ((2.0 * l - 3) * (double)(l * l - m * m)));
        }
}

inline void split_nodes(const double* v, int n, std::vector<float>& hi, std::vector<float>& lo) {
    hi.resize(n);
    lo.resize(n);
    for (int i = 0; i < n; ++i) split_ds(v[i], hi[i], lo[i]);
}

}  // namespace sos
