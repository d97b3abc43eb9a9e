// Host (CPU) build of the device transport in sos_math.cuh, for tests without a GPU.
//
// Runs `transport_lane` for every (ray, wavelength) of a bundle, exactly as transport_kernel does on the device,
// over host arrays packed by the library's own sos_pack.h. The caller sets the FPU flush-to-zero mode (the device
// build computes with -ftz=true). Built by the tests with g++ -ffp-contract=off.
#include <cstring>
#include <vector>

#include "../../sosfuse2_gb300/csrc/sos_math.cuh"
#include "../../sosfuse2_gb300/csrc/sos_pack.h"

using namespace sos;

extern "C" int host_transport(const sosb_dims* d, const sosb_constants* c, const sosb_bundle* b, int first,
                              int query, const float* field, const float* boundary, float* rad_out, char* err,
                              int nerr) {
    PackedBundle pk;
    std::string msg = pack_bundle(b, d->nc, pk);
    if (!msg.empty()) {
        snprintf(err, nerr, "%s", msg.c_str());
        return 1;
    }
    const int L = d->L, K = (L + 1) * (L + 2) / 2, W = d->W, ns = d->nh * d->nc;
    const int src = 10 + K * (d->strato ? 2 : 1);
    std::vector<float> sa, sb, sdg;
    sh_recurrence(L, sa, sb, sdg);
    std::vector<int> goff(ns + 1);
    for (int i = 0; i <= ns; ++i) goff[i] = (int)c->goff[i];
    Optics o{};
    o.L = L; o.K = K; o.W = W; o.nh = d->nh; o.nc = d->nc; o.ns = ns; o.src = src; o.strato = d->strato;
    o.top_km = (float)d->top_km; o.mix = (float)d->mix; o.g = (float)d->g; o.height = (float)d->height;
    o.air_surface = (float)d->air_surface; o.inv_step = (float)(1.0 / d->profile_step_km);
    o.density_last = d->density_rows - 2; o.density_mask = d->density_mask;
    o.strato_center = (float)d->strato_center; o.strato_sigma = (float)d->strato_sigma;
    o.strato_norm = (float)d->strato_norm;
    o.h = c->h; o.chi = c->chi; o.hr = c->hr; o.ext = c->ext; o.asca = c->asca; o.table = c->density_table;
    o.n_sun_h = d->n_sun_h; o.n_sun_x = d->n_sun_x; o.sun_h = c->sun_h; o.sun_col = c->sun_col;
    o.strato_sun_col = c->strato_sun_col; o.gm = c->gm; o.goff = goff.data(); o.gdir = c->gdir; o.gval = c->gval;
    o.strato_ext = c->strato_ext; o.strato_sca = c->strato_sca; o.strato_chi = c->strato_chi;
    o.sh_a = sa.data(); o.sh_b = sb.data(); o.sh_d = sdg.data();
    o.support = d->lower_end_km > 0.0 ? 1 : 0;
    o.lower_end = (float)d->lower_end_km;
    o.air_end = (float)d->air_end_km;
    o.aer2_on = c->aer2 != nullptr;
    for (int i = 0; i < 7; ++i) o.aer2[i] = c->aer2 ? c->aer2[i] : 0.0f;
    o.tropo_bins = c->tropo_lut ? c->tropo_bins : 0;
    o.tropo_lut = c->tropo_lut;
    std::vector<float> lut;
    if (d->strato) {
        lut.resize((size_t)(STRATO_LUT_BINS + 1) * W);
        for (int i = 0; i <= STRATO_LUT_BINS; ++i) {
            const double u = -1.0 + 2.0 * i / STRATO_LUT_BINS;
            for (int w = 0; w < W; ++w) {
                double p0 = 1.0, p1 = u, v = c->strato_chi[w] + u * c->strato_chi[W + w];
                for (int l = 2; l < 33; ++l) {
                    const double pn = ((2.0 * l - 1) * u * p1 - (l - 1.0) * p0) / l;
                    v += pn * c->strato_chi[l * W + w];
                    p0 = p1;
                    p1 = pn;
                }
                lut[(size_t)i * W + w] = (float)(v / (4.0 * 3.14159265358979323846));
            }
        }
    }
    o.strato_lut = lut.data();
    Rays r{};
    r.ncell = pk.ncell; r.nray = (int)pk.nray; r.cell_off = pk.cell_off.data(); r.ray_cell = pk.ray_cell.data();
    r.p = pk.p.data(); r.frame = pk.frame.data(); r.dir = reinterpret_cast<const float4*>(pk.dir.data());
    r.dir_lo = reinterpret_cast<const float4*>(pk.dir_lo.data());
    r.dloc = reinterpret_cast<const float4*>(pk.dloc.data()); r.seg_off = pk.seg_off.data();
    r.seg = reinterpret_cast<const float4*>(pk.seg.data()); r.lower = pk.lower.data(); r.end_j = pk.end_j.data();
    r.end_col = pk.end_col.data(); r.hits = pk.hits.data(); r.pcp = pk.pcp.data();
    // SH plane of the field, as plane_kernel builds it
    std::vector<float> plane;
    if (!first) {
        plane.resize((size_t)ns * K * W);
        for (int cell = 0; cell < ns; ++cell)
            for (int k = 0; k < K; ++k)
                for (int w = 0; w < W; ++w) {
                    const int hi = cell / d->nc;
                    const float* f = field + (size_t)cell * src * W + w;
                    float v = f[(size_t)(10 + k) * W] * c->ha[hi];
                    if (d->strato) v += f[(size_t)(10 + K + k) * W] * c->strato_density[hi];
                    plane[((size_t)cell * K + k) * W + w] = v;
                }
    }
    std::vector<float> uh, ul, wh, wl;
    split_nodes(query ? c->uq : c->u, query ? d->nq_query : d->nq, uh, ul);
    split_nodes(query ? c->wuq : c->wu, query ? d->nq_query : d->nq, wh, wl);
    LaneInputs in{};
    in.field = field; in.plane = plane.data(); in.boundary = boundary;
    in.u_hi = uh.data(); in.u_lo = ul.data(); in.wu_hi = wh.data(); in.wu_lo = wl.data();
    in.nq = query ? d->nq_query : d->nq; in.first = first;
    std::vector<float> cache(4 * (L + 1));
    for (int ray = 0; ray < r.nray; ++ray)
        for (int w = 0; w < W; ++w) {
            float out[4];
            transport_lane(o, r, in, ray, w, cache.data(), 1, out);
            std::memcpy(rad_out + ((size_t)ray * W + w) * 4, out, sizeof out);
        }
    return 0;
}
