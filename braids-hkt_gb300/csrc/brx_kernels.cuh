// Kernels of one SSPRK(2,2) substep of the augmented f-wave river step.
//
// Included by one translation unit per arithmetic form. Each includer
// defines BRX_NS (the namespace its kernel copies live in) so the FP64
// unit (-fmad=false, reference operation order) and the mixed unit (FP32
// fluxes, FMA on) never share a symbol. Kernels whose arithmetic differs
// between the forms are templates on the flux type F; with F = double they
// evaluate exactly the FP64 expressions of the reference.
#pragma once
#include "brx_common.cuh"

#ifndef BRX_NS
#error "define BRX_NS before including brx_kernels.cuh"
#endif

namespace BRX_NS {
using namespace brx;
// ---------------------------------------------------------------------------
// Drag: cell-local implicit Manning/Chezy friction over dt_scale * trial.
// src/braids_core/sediment/river_hydraulic_drag.h:3-16
// ---------------------------------------------------------------------------
template <class F>
__device__ __forceinline__ F chezy(int method, F depth, F value)
{
    if (method == 1) return value;
    if (method == 2) return pow(depth, F(1.) / F(6.)) / value;
    if (method == 3) return sqrt(F(9.81)) / F(.41) * log1p(F(30.) * depth / (exp(F(1.)) * value));
    return F(18.) * log10(F(12.) * fmax(F(.5), depth / value));
}

// Depth stays FP64; the friction factor is evaluated in F.
template <class F>
__device__ __forceinline__ void drag_cell(const Ctrl &ct, double dt, double &h, double &hu, double &hv)
{
    if (h <= ct.dry) { hu = 0.; hv = 0.; return; }
    const F hf = F(h), uf = F(hu), vf = F(hv);
    const F c = chezy<F>(ct.roughness_mode, hf, F(ct.roughness_value));
    const F speed = sqrt(uf * uf + vf * vf) / hf;
    const F factor = F(1.) / (F(1.) + F(dt) * F(ct.grav) * speed / (c * c * hf));
    hu *= factor;
    hv *= factor;
}

// work = drag(accepted, trial/2)
template <class F>
__global__ void k_open_drag(MeshDev m, StateDev s, Ctrl *ctrl)
{
    const int nc = m.nc;
    FOR_ACTIVE_CELLS(m.act, c) {
        const Ctrl &ct = ctrl[m.cell_sid[c]];
        if (!ct.active || ct.done) continue;
        const double *q = ct.cur ? s.q[1] : s.q[0];
        double h = q[c], hu = q[nc + c], hv = q[2 * nc + c];
        drag_cell<F>(ct, .5 * ct.trial, h, hu, hv);
        s.work[c] = h; s.work[nc + c] = hu; s.work[2 * nc + c] = hv;
    }
}

// ---------------------------------------------------------------------------
// Boundary: one CTA per scenario evaluates its open segments (stage sums,
// conveyance weights, exterior traces/fluxes) and caps outlet outflow by the
// owners' stage-start stock. Sums use the reference's fixed tree: 64-face
// tiles from each segment start, then the tiles in order.
// ---------------------------------------------------------------------------
template <class F>
__device__ __forceinline__ F exterior_chezy(int mode, F h, F parameter, F floor_, F gravity, int waqua)
{
    const F d = fmax(h, floor_);
    if (mode == 1) return parameter;
    if (mode == 2) return pow(d, F(1.) / F(6.)) / parameter;
    return waqua ? F(18.) * log10(F(12.) * fmax(F(.5), d / parameter))
                 : sqrt(gravity) / F(.41) * log1p(F(30.) * d / (exp(F(1.)) * parameter));
}

__device__ __forceinline__ void stage_wave(double h, double un, double target, double gravity, double &depth,
                                           double &velocity)
{
    const double c = sqrt(gravity * h);
    depth = h; velocity = un;
    if (target > h) {
        const double k = sqrt(.5 * gravity * (1. / target + 1. / h));
        const double shock = un - target * k;
        if (shock >= 0.) return;
        depth = target; velocity = un - (target - h) * k;
        return;
    }
    if (un - c >= 0.) return;
    const double cb = sqrt(gravity * target), ub = un + 2. * (c - cb);
    if (ub - cb > 0. || target == 0.) {
        velocity = (un + 2. * c) / 3.; depth = velocity * velocity / gravity;
        return;
    }
    depth = target; velocity = ub;
}

__device__ __forceinline__ bool is_outlet(int mode)
{
    return mode == 2 || mode == 3 || mode == 4 || mode == 5 || mode == 10 || mode == 11;
}

// Sums of field `row` of b.terms over each segment of the scenario, in the
// 64-tile tree. Called by all threads of the CTA; result in b.seg_sums[out_row].
__device__ void segment_sums(const BoundaryDev &b, int s0, int s1, int row, int out_row, double *tile_buf)
{
    // tile partials: one thread per (segment, tile)
    int ntile_total = 0;
    for (int s = s0; s < s1; ++s) ntile_total += max(1, (b.seg_off[s + 1] - b.seg_off[s] + 63) / 64);
    for (int t = threadIdx.x; t < ntile_total; t += blockDim.x) {
        int s = s0, rem = t;
        while (rem >= max(1, (b.seg_off[s + 1] - b.seg_off[s] + 63) / 64)) {
            rem -= max(1, (b.seg_off[s + 1] - b.seg_off[s] + 63) / 64);
            ++s;
        }
        const int start = b.seg_off[s] + 64 * rem, end = min(b.seg_off[s + 1], start + 64);
        double sum = 0.;
        for (int k = start; k < end; ++k) sum += b.terms[(size_t)row * b.nslot + k];
        tile_buf[t] = sum;
    }
    __syncthreads();
    for (int s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
        int first = 0;
        for (int u = s0; u < s; ++u) first += max(1, (b.seg_off[u + 1] - b.seg_off[u] + 63) / 64);
        const int nt = max(1, (b.seg_off[s + 1] - b.seg_off[s] + 63) / 64);
        double total = 0.;
        for (int t = 0; t < nt; ++t) total += tile_buf[first + t];
        b.seg_sums[(size_t)out_row * b.nseg + s] = total;
    }
    __syncthreads();
}


// ---------------------------------------------------------------------------
// Q-H rating outlet (mode 11): the common water elevation at which the
// outgoing characteristic discharge of the opening equals the rating curve,
// then each face's trace (river_rating_outlet.h:15-102). One thread per
// segment, faces in boundary order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double rating_velocity(double h, double hi, double u, double g)
{
    return h > hi ? u - (h - hi) * sqrt(.5 * g * (1. / h + 1. / hi)) : u + 2. * (sqrt(g * hi) - sqrt(g * h));
}

__device__ double rating_q(const BoundaryDev &b, int sg, double eta)
{
    const int a = b.rt_off[sg], end = b.rt_off[sg + 1];
    if (eta <= b.rt_eta[a]) return b.rt_q[a];
    if (eta >= b.rt_eta[end - 1]) return b.rt_q[end - 1];
    int lo = a, hi = end - 1;
    while (hi - lo > 1) { const int mid = (lo + hi) / 2; if (b.rt_eta[mid] <= eta) lo = mid; else hi = mid; }
    const double w = (eta - b.rt_eta[lo]) / (b.rt_eta[hi] - b.rt_eta[lo]);
    return (1. - w) * b.rt_q[lo] + w * b.rt_q[hi];
}

__device__ double rating_residual(const MeshDev &m, const BoundaryDev &b, int sg, double eta, double g, double dry,
                                  const double *q, const double *z, double &actual)
{
    const int nc = m.nc, nf = m.nf;
    double Q = 0.;
    for (int k = b.seg_off[sg]; k < b.seg_off[sg + 1]; ++k) {
        const int f = b.slot_face[k], c = m.owner[f];
        const double bed = b.ext_bed[k], hc = q[c], hi = fmax(hc + z[c] - bed, 0.);
        if (hc <= dry || hi <= dry) continue;
        const double u = (q[nc + c] * m.normal[f] + q[2 * nc + c] * m.normal[nf + f]) / hc;
        if (u >= sqrt(g * hi)) { Q += hi * u * m.length[f]; continue; }
        const double h = fmax(eta - bed, 0.);
        if (h > dry) Q += h * fmax(rating_velocity(h, hi, u, g), 0.) * m.length[f];
    }
    actual = Q;
    return Q - rating_q(b, sg, eta);
}

// 0, or the section failure: 1 no bracket, 2 residual, 3 a fictitious zero-flow root.
__device__ int rating_section(const MeshDev &m, const BoundaryDev &b, int sg, double g, double dry, double speed,
                              const double *q, const double *z, bool &bad)
{
    const int nc = m.nc, nf = m.nf;
    double lo = b.rt_eta[b.rt_off[sg]], hi = b.rt_eta[b.rt_off[sg + 1] - 1];
    int wet = 0;
    for (int k = b.seg_off[sg]; k < b.seg_off[sg + 1]; ++k) {
        const int f = b.slot_face[k], c = m.owner[f];
        const double h0 = q[c], h = fmax(h0 + z[c] - b.ext_bed[k], 0.);
        if (h0 <= dry || h <= dry) continue;
        const double u = (q[nc + c] * m.normal[f] + q[2 * nc + c] * m.normal[nf + f]) / h0;
        if (u >= sqrt(g * h)) continue;
        double left = dry, right = fmax(h, 1.);
        for (int it = 0; it < 60 && rating_velocity(right, h, u, g) > sqrt(g * right); ++it) right *= 2.;
        for (int it = 0; it < 60; ++it) {
            const double mid = .5 * (left + right);
            if (rating_velocity(mid, h, u, g) > sqrt(g * mid)) left = mid; else right = mid;
        }
        lo = fmax(lo, b.ext_bed[k] + right);
        ++wet;
    }
    double level = 0., actual = 0.;
    if (wet) {
        if (!(lo <= hi)) return 1;
        const double rlo = rating_residual(m, b, sg, lo, g, dry, q, z, actual);
        const double rhi = rating_residual(m, b, sg, hi, g, dry, q, z, actual);
        if (!isfinite(rlo) || !isfinite(rhi) || rlo < 0. || rhi > 0.) return 1;
        for (int it = 0; it < 90; ++it) {
            const double mid = .5 * (lo + hi);
            if (mid == lo || mid == hi) break;
            if (rating_residual(m, b, sg, mid, g, dry, q, z, actual) > 0.) lo = mid; else hi = mid;
        }
        level = .5 * (lo + hi);
        const double r = rating_residual(m, b, sg, level, g, dry, q, z, actual);
        if (!isfinite(r) || fabs(r) > 1e-10 * fmax(1., fabs(actual))) return 2;
        if (actual <= 1e-14)
            for (int k = b.seg_off[sg]; k < b.seg_off[sg + 1]; ++k) {
                const int f = b.slot_face[k], c = m.owner[f];
                const double hc = q[c], hh = fmax(hc + z[c] - b.ext_bed[k], 0.);
                if (hc <= dry || hh <= dry) continue;
                const double ui = (q[nc + c] * m.normal[f] + q[2 * nc + c] * m.normal[nf + f]) / hc;
                const double h = fmax(level - b.ext_bed[k], 0.);
                if (h > dry && ui < sqrt(g * hh) && rating_velocity(h, hh, ui, g) < -1e-12) return 3;
            }
    }
    const size_t ns = b.nslot;
    for (int k = b.seg_off[sg]; k < b.seg_off[sg + 1]; ++k) {
        const int f = b.slot_face[k], c = m.owner[f];
        const double bed = b.ext_bed[k], h0 = q[c], geom = fmax(h0 + z[c] - bed, 0.);
        const double nx = m.normal[f], ny = m.normal[nf + f];
        double ux = 0., uy = 0.;
        if (h0 > dry) { ux = q[nc + c] / h0; uy = q[2 * nc + c] / h0; }
        double un = ux * nx + uy * ny, h = geom;
        const double tx = ux - un * nx, ty = uy - un * ny;
        if (h0 <= dry || geom <= dry) { h = 0.; un = 0.; }
        else if (!(un >= sqrt(g * geom))) {     // subcritical: the common level; supercritical keeps its own
            const double incoming = un;
            h = fmax(level - bed, 0.);
            un = h > dry ? rating_velocity(h, geom, incoming, g) : 0.;
            if (un <= 0.) {                      // reflected: the stagnation depth of the incoming stream
                double left = dry, right = fmax(geom, 1.);
                for (int it = 0; it < 60 && rating_velocity(right, geom, incoming, g) > 0.; ++it) right *= 2.;
                for (int it = 0; it < 80; ++it) {
                    const double mid = .5 * (left + right);
                    if (rating_velocity(mid, geom, incoming, g) > 0.) left = mid; else right = mid;
                }
                h = .5 * (left + right);
                un = 0.;
            }
        }
        if (!isfinite(h) || !isfinite(un) || sqrt(un * un + tx * tx + ty * ty) > speed) { bad = true; continue; }
        double water = 0., fx = 0., fy = 0., t0 = 0., t1 = 0., t2 = 0.;
        if (h > dry) {
            t0 = h; t1 = h * (un * nx + tx); t2 = h * (un * ny + ty);
            water = h * un;
            fx = water * (un * nx + tx) + .5 * g * h * h * nx;
            fy = water * (un * ny + ty) + .5 * g * h * h * ny;
        }
        const double pressure = h0 > dry ? .5 * g * (h0 * h0 - geom * geom) : 0.;
        b.trace[k] = t0; b.trace[ns + k] = t1; b.trace[2 * ns + k] = t2;
        b.flux[k] = water; b.flux[ns + k] = fx + pressure * nx; b.flux[2 * ns + k] = fy + pressure * ny;
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Normal-depth outlet (mode 10): per connected face chain, the level at which
// the outgoing characteristic discharge equals the uniform-flow conveyance
// at the chain's bed slope (river_normal_outlet.h:17-134). One thread per
// chain; dry faces close with their owner's pressure.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double nout_chezy(int law, double r, double value, double g)
{
    if (law == 1) return value;
    if (law == 2) return pow(r, 1. / 6.) / value;
    if (law == 3) return sqrt(g) / .41 * log1p(30. * r / (exp(1.) * value));
    return 18. * log10(12. * fmax(.5, r / value));
}

__device__ double nout_residual(const MeshDev &m, const BoundaryDev &b, const int *slots, int start, int end,
                                double eta, double slope, double g, double dry, int law, double rough,
                                const double *q, const double *z, double &area_out, double &q_out)
{
    const int nc = m.nc, nf = m.nf;
    double area = 0., perimeter = 0., rate = 0., drag = 0., prev = 0.;
    for (int k = start; k < end; ++k) {
        const int sl = slots[k], f = b.slot_face[sl];
        const double h = fmax(eta - b.ext_bed[sl], 0.);
        area += h * m.length[f];
        perimeter += h > dry ? m.length[f] : 0.;
        if (k == start) perimeter += h; else perimeter += fabs(h - prev);
        prev = h;
    }
    perimeter += prev;
    if (area <= 0. || perimeter <= 0.) { area_out = 0.; q_out = 0.; return 0.; }
    const double radius = area / perimeter;
    const double manning_radius = law == 2 ? pow(radius, 1. / 6.) : 0.;
    for (int k = start; k < end; ++k) {
        const int sl = slots[k], f = b.slot_face[sl], c = m.owner[f];
        const double bed = b.ext_bed[sl], h0 = q[c], hi = fmax(h0 + z[c] - bed, 0.), h = fmax(eta - bed, 0.);
        double face_rate = 0.;
        if (h0 > dry && hi > dry) {
            const double ui = (q[nc + c] * m.normal[f] + q[2 * nc + c] * m.normal[nf + f]) / h0;
            if (ui >= sqrt(g * hi)) face_rate = ui * hi;
            else {
                const double invariant = fmax(ui + 2. * sqrt(g * hi), 0.), sonic = invariant * invariant / (9. * g);
                if (h < sonic) face_rate = sonic * sqrt(g * sonic);
                else if (h > dry) face_rate = h * fmax(rating_velocity(h, hi, ui, g), 0.);
            }
        }
        rate += face_rate * m.length[f];
        if (h <= dry) continue;
        const double left = k == start ? 0. : fmax(eta - b.ext_bed[slots[k - 1]], 0.);
        const double right = k + 1 == end ? 0. : fmax(eta - b.ext_bed[slots[k + 1]], 0.);
        const double p = m.length[f] + fmax(h - left, 0.) + fmax(h - right, 0.);
        const double C = law == 2 ? manning_radius / rough : nout_chezy(law, radius, rough, g);
        drag += p / (C * C);
    }
    area_out = area; q_out = rate;
    return rate - (drag > 0. ? area * sqrt(area * slope / drag) : 0.);
}

// 0, or the chain's failure (a trial rejection in the reference).
__device__ int normal_chain(const MeshDev &m, const BoundaryDev &b, int ch, double g, double dry, double speed,
                            int law, double rough, const double *q, const double *z, bool &bad)
{
    const int nc = m.nc, nf = m.nf;
    const size_t ns = b.nslot;
    const int *slots = b.chain_slot;
    const double slope = b.chain_slope[ch];
    int cursor = b.chain_off[ch];
    const int stop = b.chain_off[ch + 1];
    while (cursor < stop) {
        const int fsl = slots[cursor], ff = b.slot_face[fsl], fc = m.owner[ff];
        const double fh = q[fc], fgeom = fmax(fh + z[fc] - b.ext_bed[fsl], 0.);
        if (fh <= dry || fgeom <= dry) {
            const double pressure = fh > dry ? .5 * g * fh * fh : 0.;
            b.trace[fsl] = 0.; b.trace[ns + fsl] = 0.; b.trace[2 * ns + fsl] = 0.;
            b.flux[fsl] = 0.; b.flux[ns + fsl] = pressure * m.normal[ff]; b.flux[2 * ns + fsl] = pressure * m.normal[nf + ff];
            ++cursor;
            continue;
        }
        const int start = cursor;
        while (cursor < stop) {
            const int sl = slots[cursor], f = b.slot_face[sl], c = m.owner[f];
            const double hh = q[c];
            if (hh <= dry || hh + z[c] - b.ext_bed[sl] <= dry) break;
            ++cursor;
        }
        const int end = cursor;
        int wet = 0;
        double lo = 1e300, hi = -1e300, area = 0., rate = 0.;
        for (int k = start; k < end; ++k) {
            const int sl = slots[k], f = b.slot_face[sl], c = m.owner[f];
            const double h0 = q[c], hf = fmax(h0 + z[c] - b.ext_bed[sl], 0.);
            if (h0 <= dry || hf <= dry) continue;
            const double u = (q[nc + c] * m.normal[f] + q[2 * nc + c] * m.normal[nf + f]) / h0;
            if (u >= sqrt(g * hf)) continue;
            lo = fmin(lo, b.ext_bed[sl] + 2. * dry);
            hi = fmax(hi, z[c] + h0);
            ++wet;
        }
        double level = 0.;
        bool fallback = false;
        if (wet) {
            hi = fmax(hi, lo + 1.);
            double r = nout_residual(m, b, slots, start, end, lo, slope, g, dry, law, rough, q, z, area, rate);
            if (!isfinite(r)) return 1;
            if (r < 0.) fallback = true;           // supercritical normal flow: keep the outgoing trace
            else {
                double rh = nout_residual(m, b, slots, start, end, hi, slope, g, dry, law, rough, q, z, area, rate);
                for (int it = 0; it < 60 && rh > 0.; ++it) {
                    hi = lo + 2. * (hi - lo);
                    rh = nout_residual(m, b, slots, start, end, hi, slope, g, dry, law, rough, q, z, area, rate);
                }
                if (!isfinite(rh) || rh > 0.) return 2;
                for (int it = 0; it < 90; ++it) {
                    const double mid = .5 * (lo + hi);
                    if (mid == lo || mid == hi) break;
                    r = nout_residual(m, b, slots, start, end, mid, slope, g, dry, law, rough, q, z, area, rate);
                    if (r > 0.) lo = mid; else hi = mid;
                }
                level = .5 * (lo + hi);
                r = nout_residual(m, b, slots, start, end, level, slope, g, dry, law, rough, q, z, area, rate);
                if (!isfinite(r) || fabs(r) > 1e-10 * fmax(1., fabs(rate))) return 3;
            }
        }
        for (int k = start; k < end; ++k) {
            const int sl = slots[k], f = b.slot_face[sl], c = m.owner[f];
            const double bed = b.ext_bed[sl], h0 = q[c], geom = fmax(h0 + z[c] - bed, 0.);
            const double nx = m.normal[f], ny = m.normal[nf + f];
            double ux = 0., uy = 0.;
            if (h0 > dry) { ux = q[nc + c] / h0; uy = q[2 * nc + c] / h0; }
            double un = ux * nx + uy * ny, h = geom;
            const double tx = ux - un * nx, ty = uy - un * ny;
            if (h0 <= dry || geom <= dry) { h = 0.; un = 0.; }
            else if (fallback) { }
            else if (un >= sqrt(g * geom)) { }
            else {
                const double incoming = un;
                h = fmax(level - bed, 0.);
                const double invariant = fmax(incoming + 2. * sqrt(g * geom), 0.), sonic = invariant * invariant / (9. * g);
                if (h < sonic) { h = sonic; un = sqrt(g * sonic); }
                else un = h > dry ? rating_velocity(h, geom, incoming, g) : 0.;
                if (un <= 0.) {
                    double left = dry, right = fmax(geom, 1.);
                    for (int it = 0; it < 60 && rating_velocity(right, geom, incoming, g) > 0.; ++it) right *= 2.;
                    for (int it = 0; it < 80; ++it) {
                        const double mid = .5 * (left + right);
                        if (rating_velocity(mid, geom, incoming, g) > 0.) left = mid; else right = mid;
                    }
                    h = .5 * (left + right);
                    un = 0.;
                }
            }
            if (!isfinite(h) || !isfinite(un) || sqrt(un * un + tx * tx + ty * ty) > speed) { bad = true; continue; }
            double water = 0., fx = 0., fy = 0., t0 = 0., t1 = 0., t2 = 0.;
            if (h > dry) {
                t0 = h; t1 = h * (un * nx + tx); t2 = h * (un * ny + ty);
                water = h * un;
                fx = water * (un * nx + tx) + .5 * g * h * h * nx;
                fy = water * (un * ny + ty) + .5 * g * h * h * ny;
            }
            const double pressure = h0 > dry ? .5 * g * (h0 * h0 - geom * geom) : 0.;
            b.trace[sl] = t0; b.trace[ns + sl] = t1; b.trace[2 * ns + sl] = t2;
            b.flux[sl] = water; b.flux[ns + sl] = fx + pressure * nx; b.flux[2 * ns + sl] = fy + pressure * ny;
        }
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Section solves with 128 logical lanes (river_exterior_outlet.h): the whole
// boundary CTA works on one section; lane l (threads 0..127) sums entries
// l, l+128, ... of the section and thread 0 adds the lane sums in lane order,
// the order of the reference's OpenMP and CUDA forms. Every thread of the
// CTA calls these functions (they synchronise the block).
// ---------------------------------------------------------------------------
constexpr int SECTION_LANES = 128;

struct SectionWork {
    double part[6][SECTION_LANES];
    double lo, hi, eta, residual, area, width, rate;
    double velocity, gross, derivative, scale;
    int error, done, stagnant, changed, count;
};

__device__ __forceinline__ double weir_velocity(double h, double hi, double ui, double g)
{
    return h > hi ? ui - (h - hi) * sqrt(.5 * g * (1. / h + 1. / hi)) : ui + 2. * (sqrt(g * hi) - sqrt(g * h));
}

// river_exterior_outlet.h:207-227
__device__ void weir_residual(SectionWork &w, const MeshDev &m, const BoundaryDev &b, int k0, int k1, double eta,
                              double g, double dry, double crest, double factor, const double *q, const double *z)
{
    for (int lane = threadIdx.x; lane < SECTION_LANES; lane += blockDim.x) {
        double area = 0., width = 0., rate = 0.;
        for (int k = k0 + lane; k < k1; k += SECTION_LANES) {
            if (!b.branch[k]) continue;
            const int f = b.slot_face[k], c = m.owner[f];
            const double bed = b.ext_bed[k], h = fmax(eta - bed, 0.), hi = fmax(q[c] + z[c] - bed, 0.);
            if (h <= dry) continue;
            const double u = fmax(weir_velocity(h, hi, b.invariant[k], g), 0.);
            if (u > 0.) { area += h * m.length[f]; width += m.length[f]; rate += h * u * m.length[f]; }
        }
        w.part[0][lane] = area; w.part[1][lane] = width; w.part[2][lane] = rate;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        w.area = w.width = w.rate = 0.;
        for (int lane = 0; lane < SECTION_LANES; ++lane) {
            w.area += w.part[0][lane]; w.width += w.part[1][lane]; w.rate += w.part[2][lane];
        }
        const double head = fmax(eta - crest, 0.);
        w.residual = w.rate - factor * head * sqrt(head);
    }
    __syncthreads();
}

// Free weir on segment sg (river_exterior_outlet.h:229-360): the common
// subcritical stage at which the outgoing Lax-curve discharge equals
// coefficient x width x head^1.5. Returns 0 or the section failure (a trial
// rejection in the reference); `bad` gets the speed-limit face status.
__device__ int weir_section(SectionWork &w, const MeshDev &m, const BoundaryDev &b, int sg, double g, double dry,
                            double speed, const double *q, const double *z, bool &bad)
{
    const int nc = m.nc, nf = m.nf, nseg = b.nseg, k0 = b.seg_off[sg], k1 = b.seg_off[sg + 1];
    const size_t ns = b.nslot;
    const double tol = 128. * EPS, crest = b.weir[sg], factor = b.weir[nseg + sg] * b.weir[2 * nseg + sg];
    if (threadIdx.x == 0) { w.error = 0; w.done = 0; w.eta = 0.; w.area = w.width = w.rate = 0.; }
    for (int lane = threadIdx.x; lane < SECTION_LANES; lane += blockDim.x) {
        double width = 0.;
        for (int k = k0 + lane; k < k1; k += SECTION_LANES) {
            const int f = b.slot_face[k], c = m.owner[f];
            b.branch[k] = 0; b.invariant[k] = 0.;
            const double h0 = q[c], h = fmax(h0 + z[c] - b.ext_bed[k], 0.);
            if (h0 <= dry || h <= dry) continue;
            const double un = (q[nc + c] * m.normal[f] + q[2 * nc + c] * m.normal[nf + f]) / h0;
            b.branch[k] = 1; b.invariant[k] = un; width += m.length[f];
        }
        w.part[1][lane] = width;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double width = 0.;
        for (int lane = 0; lane < SECTION_LANES; ++lane) width += w.part[1][lane];
        if (width == 0.) w.done = 1;
    }
    __syncthreads();
    if (w.done) {
        for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) b.branch[k] = 0;
        __syncthreads();
    } else {
        for (int lane = threadIdx.x; lane < SECTION_LANES; lane += blockDim.x) {
            double lo = -INFINITY, hi = -INFINITY;
            for (int k = k0 + lane; k < k1; k += SECTION_LANES) {
                if (b.branch[k] != 1) continue;
                const int c = m.owner[b.slot_face[k]];
                const double h0 = fmax(q[c] + z[c] - b.ext_bed[k], 0.), u = b.invariant[k];
                double left = 0., right = fmax(h0, 1.);
                for (int it = 0; it < 60 && weir_velocity(right, h0, u, g) > sqrt(g * right); ++it) right *= 2.;
                for (int it = 0; it < 70; ++it) {
                    const double mid = .5 * (left + right);
                    if (weir_velocity(mid, h0, u, g) > sqrt(g * mid)) left = mid; else right = mid;
                }
                lo = fmax(lo, b.ext_bed[k] + right);
                hi = fmax(hi, q[c] + z[c]);
            }
            w.part[0][lane] = lo; w.part[1][lane] = hi;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            w.lo = -INFINITY; w.hi = -INFINITY;
            for (int lane = 0; lane < SECTION_LANES; ++lane) { w.lo = fmax(w.lo, w.part[0][lane]); w.hi = fmax(w.hi, w.part[1][lane]); }
            w.lo = fmax(w.lo, crest);
            w.hi = fmax(w.hi, w.lo + 1.);
        }
        __syncthreads();
        weir_residual(w, m, b, k0, k1, w.lo, g, dry, crest, factor, q, z);
        if (threadIdx.x == 0 && (w.residual < 0. || !isfinite(w.residual))) w.error = 1;
        __syncthreads();
        if (!w.error) {
            weir_residual(w, m, b, k0, k1, w.hi, g, dry, crest, factor, q, z);
            for (int j = 0; j < 60 && w.residual > 0.; ++j) {
                if (threadIdx.x == 0) w.hi = w.lo + 2. * (w.hi - w.lo);
                __syncthreads();
                weir_residual(w, m, b, k0, k1, w.hi, g, dry, crest, factor, q, z);
            }
            if (threadIdx.x == 0 && (w.residual > 0. || !isfinite(w.residual))) w.error = 1;
            __syncthreads();
        }
        if (!w.error) {
            for (int j = 0; j < 90; ++j) {
                if (threadIdx.x == 0) { w.eta = w.lo + .5 * (w.hi - w.lo); w.stagnant = w.eta == w.lo || w.eta == w.hi; }
                __syncthreads();
                if (w.stagnant) break;
                weir_residual(w, m, b, k0, k1, w.eta, g, dry, crest, factor, q, z);
                if (threadIdx.x == 0) { if (w.residual > 0.) w.lo = w.eta; else w.hi = w.eta; }
                __syncthreads();
            }
            if (threadIdx.x == 0) w.eta = w.lo + .5 * (w.hi - w.lo);
            __syncthreads();
            weir_residual(w, m, b, k0, k1, w.eta, g, dry, crest, factor, q, z);
            if (threadIdx.x == 0) {
                const double head = fmax(w.eta - crest, 0.), requested = factor * head * sqrt(head);
                if (!isfinite(w.residual) || fabs(w.residual) > 1e-10 * fmax(requested, 1.)) w.error = 2;
            }
            __syncthreads();
            for (int lane = threadIdx.x; lane < SECTION_LANES; lane += blockDim.x) {
                double count = 0.;
                for (int k = k0 + lane; k < k1; k += SECTION_LANES) {
                    if (b.branch[k] != 1) continue;
                    const int c = m.owner[b.slot_face[k]];
                    const double bed = b.ext_bed[k], hi = fmax(q[c] + z[c] - bed, 0.), h = fmax(w.eta - bed, 0.);
                    const double u = weir_velocity(h, hi, b.invariant[k], g);
                    if (h <= dry || u <= 0.) { b.branch[k] = 0; continue; }
                    // a downstream-only shock may not enter the domain
                    if (h > hi && b.invariant[k] - h * sqrt(.5 * g * (1. / h + 1. / hi)) > tol) count += 1.;
                }
                w.part[0][lane] = count;
            }
            __syncthreads();
            if (threadIdx.x == 0)
                for (int lane = 0; lane < SECTION_LANES; ++lane) if (w.part[0][lane] > 0.) w.error = 5;
            __syncthreads();
        }
    }
    const int error = w.error;
    __syncthreads();
    if (error) return error;
    for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
        const int f = b.slot_face[k], c = m.owner[f];
        const double bed = b.ext_bed[k], h0 = q[c], geom = fmax(h0 + z[c] - bed, 0.);
        const double nx = m.normal[f], ny = m.normal[nf + f];
        double h = geom, ux = 0., uy = 0.;
        if (h0 > dry) { ux = q[nc + c] / h0; uy = q[2 * nc + c] / h0; } else h = 0.;
        double un = ux * nx + uy * ny;
        const double tx = ux - un * nx, ty = uy - un * ny;
        if (b.branch[k] == 0) {
            // a blocked stream reflects with its stagnation / shock depth
            if (geom > dry && h0 > dry && un != 0.) {
                double lo = 0., hi = fmax(geom, 1.);
                for (int it = 0; it < 60 && weir_velocity(hi, geom, un, g) > 0.; ++it) hi *= 2.;
                for (int it = 0; it < 80; ++it) {
                    const double mid = .5 * (lo + hi);
                    if (weir_velocity(mid, geom, un, g) > 0.) lo = mid; else hi = mid;
                }
                h = .5 * (lo + hi);
            }
            un = 0.;
        } else {
            h = fmax(w.eta - bed, 0.);
            un = weir_velocity(h, geom, b.invariant[k], g);
        }
        if (!isfinite(h) || !isfinite(un) || sqrt(un * un + tx * tx + ty * ty) > speed) { bad = true; continue; }
        double water = 0., fx = 0., fy = 0., t0 = 0., t1 = 0., t2 = 0.;
        if (h > dry) {
            t0 = h; t1 = h * (un * nx + tx); t2 = h * (un * ny + ty);
            water = t1 * nx + t2 * ny;
            fx = water * t1 / h + .5 * g * h * h * nx;
            fy = water * t2 / h + .5 * g * h * h * ny;
        }
        const double pressure = h0 > dry ? .5 * g * (h0 * h0 - geom * geom) : 0.;
        b.trace[k] = t0; b.trace[ns + k] = t1; b.trace[2 * ns + k] = t2;
        b.flux[k] = water; b.flux[ns + k] = fx + pressure * nx; b.flux[2 * ns + k] = fy + pressure * ny;
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Critical outlet (mode 4): on the controlled faces of an opening the
// outgoing characteristic discharge equals sqrt(g A^3 / B); faces turning
// inward or dry leave the control and the root is recomputed
// (river_exterior_outlet.h:29-175). Slot lists: `slots` null means the
// segment's own slots k0, k0+1, ...
// ---------------------------------------------------------------------------
__device__ __forceinline__ double resolved_bed(const MeshDev &m, const BoundaryDev &b, int k, const double *q,
                                               const double *z)
{
    const int c = m.owner[b.slot_face[k]];
    const double h = fmax(q[c], 0.), bed = b.ext_bed[k];
    if (h >= 1.e-3) return bed;
    const double bounded = fmax(bed, z[c] - h);
    double blend = fmin(1., fmax(0., (h - 1.e-4) / 9.e-4));
    blend = blend * blend * (3. - 2. * blend);
    return bed + (bounded - bed) * (1. - blend);
}

__device__ void crit_residual(SectionWork &w, const MeshDev &m, const BoundaryDev &b, const int *slots, int k0,
                              int n, double eta, double g, double dry, const double *q, const double *z)
{
    for (int lane = threadIdx.x; lane < SECTION_LANES; lane += blockDim.x) {
        double a = 0., width = 0., rate = 0.;
        for (int i = lane; i < n; i += SECTION_LANES) {
            const int k = slots ? slots[i] : k0 + i;
            if (b.branch[k] != 1) continue;
            const double h = fmax(eta - resolved_bed(m, b, k, q, z), 0.);
            if (h <= dry) continue;
            const double len = m.length[b.slot_face[k]];
            a += h * len; width += len; rate += h * (b.invariant[k] - 2. * sqrt(g * h)) * len;
        }
        w.part[0][lane] = a; w.part[1][lane] = width; w.part[2][lane] = rate;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0., width = 0., rate = 0.;
        for (int lane = 0; lane < SECTION_LANES; ++lane) { a += w.part[0][lane]; width += w.part[1][lane]; rate += w.part[2][lane]; }
        w.area = a; w.width = width; w.rate = rate;
        w.residual = rate - (width > 0. ? sqrt(g * a * a * a / width) : 0.);
    }
    __syncthreads();
}

__device__ int crit_group(SectionWork &w, const MeshDev &m, const BoundaryDev &b, const int *slots, int k0, int n,
                          double g, double dry, double speed, const double *q, const double *z, bool &bad)
{
    const int nc = m.nc, nf = m.nf;
    const size_t ns = b.nslot;
    const double tol = 128. * EPS;
    if (threadIdx.x == 0) { w.error = 0; w.done = 0; w.eta = 0.; w.area = w.width = w.rate = 0.; }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int k = slots ? slots[i] : k0 + i, f = b.slot_face[k], c = m.owner[f];
        b.branch[k] = 0; b.invariant[k] = 0.;
        const double h0 = q[c], h = fmax(h0 + z[c] - resolved_bed(m, b, k, q, z), 0.);
        if (h0 <= dry || h <= dry) continue;
        const double un = (q[nc + c] * m.normal[f] + q[2 * nc + c] * m.normal[nf + f]) / h0, wave = sqrt(g * h);
        if (un < -tol * fmax(1., fabs(un))) continue;
        if (un > wave * (1. + 1e-10)) { b.branch[k] = 2; continue; }
        b.branch[k] = 1; b.invariant[k] = un + 2. * wave;
    }
    __syncthreads();
    for (int active = 0; active <= n; ++active) {
        for (int lane = threadIdx.x; lane < SECTION_LANES; lane += blockDim.x) {
            double lo = INFINITY, hi = -INFINITY, count = 0.;
            for (int i = lane; i < n; i += SECTION_LANES) {
                const int k = slots ? slots[i] : k0 + i;
                if (b.branch[k] != 1) continue;
                const int c = m.owner[b.slot_face[k]];
                lo = fmin(lo, resolved_bed(m, b, k, q, z)); hi = fmax(hi, q[c] + z[c]); count += 1.;
            }
            w.part[0][lane] = lo; w.part[1][lane] = hi; w.part[2][lane] = count;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            w.lo = INFINITY; w.hi = -INFINITY; w.count = 0;
            for (int lane = 0; lane < SECTION_LANES; ++lane) {
                w.lo = fmin(w.lo, w.part[0][lane]); w.hi = fmax(w.hi, w.part[1][lane]); w.count += int(w.part[2][lane]);
            }
            if (w.count) w.lo += fmax(2. * dry, tol * fmax(1., fabs(w.lo)));
            else { w.done = 1; w.area = w.width = w.rate = 0.; }
        }
        __syncthreads();
        if (w.done) break;
        crit_residual(w, m, b, slots, k0, n, w.lo, g, dry, q, z);
        if (w.residual < 0.) {                     // unresolved controlled depth: the opening closes
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const int k = slots ? slots[i] : k0 + i;
                if (b.branch[k] == 1) b.branch[k] = 0;
            }
            if (threadIdx.x == 0) { w.done = 1; w.area = w.width = w.rate = 0.; w.eta = w.lo; }
            __syncthreads();
            break;
        }
        crit_residual(w, m, b, slots, k0, n, w.hi, g, dry, q, z);
        for (int j = 0; j < 60 && w.residual > 0.; ++j) {
            if (threadIdx.x == 0) w.hi = w.lo + 2. * (w.hi - w.lo);
            __syncthreads();
            crit_residual(w, m, b, slots, k0, n, w.hi, g, dry, q, z);
        }
        if (w.residual > 0. || !isfinite(w.residual)) {
            if (threadIdx.x == 0) w.error = 1;
            __syncthreads();
            break;
        }
        for (int j = 0; j < 90; ++j) {
            if (threadIdx.x == 0) { w.eta = w.lo + .5 * (w.hi - w.lo); w.stagnant = w.eta == w.lo || w.eta == w.hi; }
            __syncthreads();
            if (w.stagnant) break;
            crit_residual(w, m, b, slots, k0, n, w.eta, g, dry, q, z);
            if (threadIdx.x == 0) { if (w.residual > 0.) w.lo = w.eta; else w.hi = w.eta; }
            __syncthreads();
        }
        if (threadIdx.x == 0) w.eta = w.lo + .5 * (w.hi - w.lo);
        __syncthreads();
        for (int lane = threadIdx.x; lane < SECTION_LANES; lane += blockDim.x) {
            double changed = 0.;
            for (int i = lane; i < n; i += SECTION_LANES) {
                const int k = slots ? slots[i] : k0 + i;
                if (b.branch[k] != 1) continue;
                const double h = fmax(w.eta - resolved_bed(m, b, k, q, z), 0.), un = b.invariant[k] - 2. * sqrt(g * h);
                if (h <= dry || un < -tol) { b.branch[k] = 0; changed += 1.; }
            }
            w.part[0][lane] = changed;
        }
        __syncthreads();
        if (threadIdx.x == 0) { w.changed = 0; for (int lane = 0; lane < SECTION_LANES; ++lane) w.changed += int(w.part[0][lane]); }
        __syncthreads();
        if (w.changed) continue;
        crit_residual(w, m, b, slots, k0, n, w.eta, g, dry, q, z);
        if (threadIdx.x == 0) {
            const double qc = w.width > 0. ? sqrt(g * w.area * w.area * w.area / w.width) : 0.;
            if (w.area <= 0. || w.width <= 0. || !isfinite(w.residual) || fabs(w.residual) > 1e-10 * fmax(qc, 1.)) w.error = 2;
            w.done = 1;
        }
        __syncthreads();
        break;
    }
    if (threadIdx.x == 0 && !w.done && !w.error) w.error = 3;
    __syncthreads();
    const int error = w.error;
    __syncthreads();
    if (error) return error;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int k = slots ? slots[i] : k0 + i, f = b.slot_face[k], c = m.owner[f];
        const double rbed = resolved_bed(m, b, k, q, z), h0 = q[c], geom = fmax(h0 + z[c] - rbed, 0.);
        const double nx = m.normal[f], ny = m.normal[nf + f];
        double h = geom, ux = 0., uy = 0.;
        if (h0 > dry) { ux = q[nc + c] / h0; uy = q[2 * nc + c] / h0; } else h = 0.;
        double un = ux * nx + uy * ny;
        const double tx = ux - un * nx, ty = uy - un * ny;
        if (b.branch[k] == 0) un = 0.;
        else if (b.branch[k] == 1) { h = fmax(w.eta - rbed, 0.); un = b.invariant[k] - 2. * sqrt(g * h); }
        if (!isfinite(h) || !isfinite(un) || sqrt(un * un + tx * tx + ty * ty) > speed) { bad = true; continue; }
        double water = 0., fx = 0., fy = 0., t0 = 0., t1 = 0., t2 = 0.;
        if (h > dry) {
            t0 = h; t1 = h * (un * nx + tx); t2 = h * (un * ny + ty);
            water = t1 * nx + t2 * ny;
            fx = water * t1 / h + .5 * g * h * h * nx;
            fy = water * t2 / h + .5 * g * h * h * ny;
        }
        const double pressure = h0 > dry ? .5 * g * (h0 * h0 - geom * geom) : 0.;
        b.trace[k] = t0; b.trace[ns + k] = t1; b.trace[2 * ns + k] = t2;
        b.flux[k] = water; b.flux[ns + k] = fx + pressure * nx; b.flux[2 * ns + k] = fy + pressure * ny;
    }
    return 0;
}

// The critical owner of segment sg: the whole opening, then, when dry faces
// split its chains into several wet groups, each group alone with the dry
// faces closed at their owners' pressure (river_exterior_outlet.py:37-72).
__device__ int crit_section(SectionWork &w, const MeshDev &m, const BoundaryDev &b, int sg, double g, double dry,
                            double speed, const double *q, const double *z, bool &bad)
{
    const int nf = m.nf, k0 = b.seg_off[sg], n = b.seg_off[sg + 1] - k0;
    const size_t ns = b.nslot;
    bool bad_whole = false;
    const int err = crit_group(w, m, b, nullptr, k0, n, g, dry, speed, q, z, bad_whole);
    if (!b.crit_seg_chain) { bad = bad || bad_whole; return err; }
    __shared__ int ngroup;
    if (threadIdx.x == 0) {          // wet runs along each chain, as slot lists in the segment's scratch
        int groups = 0, flat = 0;
        for (int ch = b.crit_seg_chain[sg]; ch < b.crit_seg_chain[sg + 1]; ++ch) {
            bool open = false;
            for (int e = b.crit_chain_off[ch]; e < b.crit_chain_off[ch + 1]; ++e) {
                const int k = b.crit_chain_slot[e], c = m.owner[b.slot_face[k]];
                const double h = q[c], geom = h + z[c] - b.ext_bed[k];
                if ((h > dry) && (geom > dry)) { b.gslot[k0 + flat++] = k; open = true; }
                else if (open) { b.gend[k0 + groups++] = flat; open = false; }
            }
            if (open) b.gend[k0 + groups++] = flat;
        }
        ngroup = groups;
    }
    __syncthreads();
    const int groups = ngroup;
    __syncthreads();
    if (groups <= 1) { bad = bad || bad_whole; return err; }
    int worst = 0, start = 0;
    bool bad_groups = bad_whole;      // a face the groups do not rewrite keeps its earlier status
    for (int gi = 0; gi < groups; ++gi) {
        const int end = b.gend[k0 + gi];
        bool gb = false;
        const int e = crit_group(w, m, b, b.gslot + k0 + start, 0, end - start, g, dry, speed, q, z, gb);
        worst = max(worst, e);
        bad_groups = bad_groups || gb;
        start = end;
    }
    // dry chain faces close at their owners' pressure; their status clears
    bool any_dry_bad = false;
    for (int ch = b.crit_seg_chain[sg]; ch < b.crit_seg_chain[sg + 1]; ++ch)
        for (int e = b.crit_chain_off[ch] + threadIdx.x; e < b.crit_chain_off[ch + 1]; e += blockDim.x) {
            const int k = b.crit_chain_slot[e], f = b.slot_face[k], c = m.owner[f];
            const double h = q[c], geom = h + z[c] - b.ext_bed[k];
            if ((h > dry) && (geom > dry)) continue;
            const double height = fmax(q[c], 0.), pressure = .5 * g * height * height;
            b.trace[k] = 0.; b.trace[ns + k] = 0.; b.trace[2 * ns + k] = 0.;
            b.flux[k] = 0.; b.flux[ns + k] = pressure * m.normal[f]; b.flux[2 * ns + k] = pressure * m.normal[nf + f];
        }
    (void)any_dry_bad;
    __syncthreads();
    bad = bad || bad_groups;
    return worst;
}

// ---------------------------------------------------------------------------
// Exact-discharge inlet (mode 9, river_exterior_inlet.h): the exact 1-D SWE
// Riemann solution between a virtual reservoir at the requested water line
// and each face's interior state; the reservoir's common normal velocity is
// solved (bracket, then safeguarded Newton with the analytical derivative)
// so that the net section discharge equals the request.
// ---------------------------------------------------------------------------
struct InletRiemann {
    double h, u, derivative;
    int iterations, error;
};

__device__ __forceinline__ void inlet_wave(double h, double hk, double g, double &f, double &df)
{
    if (h > hk) {
        const double a = sqrt(.5 * g * (1. / h + 1. / hk));
        f = (h - hk) * a;
        df = a - .25 * g * (h - hk) / (a * h * h);
    } else {
        const double c = sqrt(g * h);
        f = 2. * (c - sqrt(g * hk));
        df = sqrt(g / h);
    }
}

// river_exterior_inlet.h:32-69: left = reservoir, right = interior (normal into the domain)
__device__ InletRiemann inlet_exact(double hl, double ul, double hr, double ur, double g)
{
    InletRiemann r = {0., 0., 0., 0, 0};
    const double cl = sqrt(g * hl), cr = sqrt(g * hr);
    if (hl == 0. && hr == 0.) return r;
    if (hr == 0. || hl == 0. || ur - ul >= 2. * (cl + cr)) {
        if (hl > 0. && ul - cl >= 0.) { r.h = hl; r.u = ul; r.derivative = hl; }
        else if (hl > 0. && ul + 2. * cl > 0.) { r.u = (ul + 2. * cl) / 3.; r.h = r.u * r.u / g; r.derivative = r.h; }
        else if (hr > 0. && ur + cr <= 0.) { r.h = hr; r.u = ur; }
        else if (hr > 0. && ur - 2. * cr < 0.) { r.u = (ur - 2. * cr) / 3.; r.h = r.u * r.u / g; }
        return r;
    }
    double guess = .5 * (cl + cr) - .25 * (ur - ul);
    guess = guess * guess / g;
    double lo = 0., hi = fmax(fmax(hl, hr), guess), fl, fr, dl, dr;
    inlet_wave(hi, hl, g, fl, dl);
    inlet_wave(hi, hr, g, fr, dr);
    for (int j = 0; j < 60 && fl + fr + ur - ul < 0.; ++j) {
        hi *= 2.;
        inlet_wave(hi, hl, g, fl, dl);
        inlet_wave(hi, hr, g, fr, dr);
    }
    if (!isfinite(hi) || fl + fr + ur - ul < 0.) { r.error = 1; return r; }
    const double scale = fmax(1., cl + cr + fabs(ul) + fabs(ur));
    double h = fmax(fmin(guess, hi), 1e-30), residual = 0.;
    for (int j = 0; j < 70; ++j) {
        inlet_wave(h, hl, g, fl, dl);
        inlet_wave(h, hr, g, fr, dr);
        residual = fl + fr + ur - ul;
        r.iterations = j + 1;
        if (fabs(residual) <= 4e-14 * scale) break;
        if (residual < 0.) lo = h; else hi = h;
        double next = h - residual / (dl + dr);
        if (!(next > lo && next < hi)) next = lo + .5 * (hi - lo);
        h = next;
    }
    inlet_wave(h, hl, g, fl, dl);
    inlet_wave(h, hr, g, fr, dr);
    residual = fl + fr + ur - ul;
    if (!isfinite(h) || fabs(residual) > 2e-11 * scale) { r.error = 2; return r; }
    const double u = .5 * (ul + ur + fr - fl), c = sqrt(g * h);
    r.h = h; r.u = u; r.derivative = fmax(0., (u + h * dr) / (dl + dr));
    if (u >= 0.) {
        if (h > hl) {
            if (ul - sqrt(.5 * g * h * (h + hl) / hl) >= 0.) { r.h = hl; r.u = ul; r.derivative = hl; }
        } else if (ul - cl >= 0.) { r.h = hl; r.u = ul; r.derivative = hl; }
        else if (u - c > 0.) { r.u = (ul + 2. * cl) / 3.; r.h = r.u * r.u / g; r.derivative = r.h; }
    } else {
        if (h > hr) {
            if (ur + sqrt(.5 * g * h * (h + hr) / hr) <= 0.) { r.h = hr; r.u = ur; r.derivative = 0.; }
        } else if (ur + cr <= 0.) { r.h = hr; r.u = ur; r.derivative = 0.; }
        else if (u + c < 0.) { r.u = (ur - 2. * cr) / 3.; r.h = r.u * r.u / g; r.derivative = 0.; }
    }
    return r;
}

// Interior depth above the face's exterior bed and inward normal speed of slot k.
__device__ __forceinline__ void inlet_interior(const MeshDev &m, const BoundaryDev &b, int k, double dry,
                                               const double *q, const double *z, double &hi, double &ui)
{
    const int nc = m.nc, f = b.slot_face[k], c = m.owner[f];
    const double h0 = q[c];
    hi = h0 > dry ? fmax(h0 + z[c] - b.ext_bed[k], 0.) : 0.;
    if (hi <= dry) hi = 0.;
    ui = h0 > dry ? -(q[nc + c] * m.normal[f] + q[2 * nc + c] * m.normal[m.nf + f]) / h0 : 0.;
}

// river_exterior_inlet.h:71-95: section discharge, its derivative and the
// gross throughflow at the common velocity w.velocity (lane sums, lane order).
__device__ void inlet_rate(SectionWork &w, const MeshDev &m, const BoundaryDev &b, int k0, int k1, double requested,
                           double g, double dry, const double *q, const double *z)
{
    for (int lane = threadIdx.x; lane < SECTION_LANES; lane += blockDim.x) {
        double rate = 0., derivative = 0., gross = 0.;
        int error = 0;
        for (int k = k0 + lane; k < k1; k += SECTION_LANES) {
            double hi, ui;
            inlet_interior(m, b, k, dry, q, z, hi, ui);
            double hr = fmax(requested - b.ext_bed[k], 0.);
            if (hr <= dry) hr = 0.;
            const InletRiemann r = inlet_exact(hr, w.velocity, hi, ui, g);
            const double len = m.length[b.slot_face[k]];
            rate += r.h * r.u * len; derivative += r.derivative * len;
            gross += fabs(r.h * r.u * len);
            error = max(error, r.error);
        }
        w.part[0][lane] = rate; w.part[1][lane] = derivative; w.part[4][lane] = error; w.part[5][lane] = gross;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        w.rate = w.derivative = w.gross = 0.;
        for (int lane = 0; lane < SECTION_LANES; ++lane) {
            w.rate += w.part[0][lane]; w.derivative += w.part[1][lane]; w.gross += w.part[5][lane];
            if (w.part[4][lane] != 0.) w.error = 5;
        }
    }
    __syncthreads();
}

// river_exterior_inlet.h:97-186: the inlet of segment sg. Returns 0 or the
// section failure (a trial rejection in the reference); `bad` gets the faces
// whose Riemann solution failed or exceeds the speed limit (face status 3).
__device__ int inlet_section(SectionWork &w, const MeshDev &m, const BoundaryDev &b, int sg, double g, double dry,
                             double speed, const double *q, const double *z, bool &bad)
{
    const int nc = m.nc, nf = m.nf, nseg = b.nseg, k0 = b.seg_off[sg], k1 = b.seg_off[sg + 1];
    const size_t ns = b.nslot;
    const double Q = b.forcing[sg], requested = b.forcing[nseg + sg];
    if (threadIdx.x == 0) w.error = 0;
    for (int lane = threadIdx.x; lane < SECTION_LANES; lane += blockDim.x) {
        double area = 0., scale = 1.;
        for (int k = k0 + lane; k < k1; k += SECTION_LANES) {
            double hi, ui;
            inlet_interior(m, b, k, dry, q, z, hi, ui);
            const double hr = fmax(requested - b.ext_bed[k], 0.);
            if (hr > dry) area += hr * m.length[b.slot_face[k]];
            scale = fmax(scale, fabs(ui) + 2. * sqrt(g * hi) + 2. * sqrt(g * hr));
        }
        w.part[0][lane] = area; w.part[1][lane] = scale;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        w.area = 0.; w.scale = 1.;
        for (int lane = 0; lane < SECTION_LANES; ++lane) { w.area += w.part[0][lane]; w.scale = fmax(w.scale, w.part[1][lane]); }
        if (!isfinite(Q) || Q < 0. || !isfinite(requested) || (Q > 0. && w.area <= 0.)) w.error = 1;
        w.velocity = w.area > 0. ? Q / w.area : 0.;
        w.scale = fmax(w.scale, 1. + fabs(w.velocity));
    }
    __syncthreads();
    if (Q > 0. && !w.error) {
        if (threadIdx.x == 0) { w.lo = w.velocity - w.scale; w.hi = w.velocity + w.scale; w.velocity = w.lo; }
        __syncthreads();
        inlet_rate(w, m, b, k0, k1, requested, g, dry, q, z);
        for (int j = 0; j < 60 && w.rate > Q && !w.error; ++j) {
            if (threadIdx.x == 0) { w.lo -= w.scale; w.scale *= 2.; w.velocity = w.lo; }
            __syncthreads();
            inlet_rate(w, m, b, k0, k1, requested, g, dry, q, z);
        }
        const bool low_bad = w.rate > Q;
        __syncthreads();
        if (threadIdx.x == 0) { if (low_bad) w.error = 2; w.velocity = w.hi; }
        __syncthreads();
        inlet_rate(w, m, b, k0, k1, requested, g, dry, q, z);
        for (int j = 0; j < 60 && w.rate < Q && !w.error; ++j) {
            if (threadIdx.x == 0) { w.hi += w.scale; w.scale *= 2.; w.velocity = w.hi; }
            __syncthreads();
            inlet_rate(w, m, b, k0, k1, requested, g, dry, q, z);
        }
        const bool high_bad = w.rate < Q;
        __syncthreads();
        if (threadIdx.x == 0) { if (high_bad) w.error = 2; w.velocity = fmin(w.hi, fmax(w.lo, Q / w.area)); }
        __syncthreads();
        for (int j = 0; j < 80 && !w.error; ++j) {
            inlet_rate(w, m, b, k0, k1, requested, g, dry, q, z);
            // net Q may be far below the signed face throughflow: relative
            // tolerance plus a double-precision budget on the gross flow
            if (fabs(w.rate - Q) <= 3e-13 * Q + 256. * EPS * w.gross) break;
            __syncthreads();
            if (threadIdx.x == 0) {
                if (w.rate < Q) w.lo = w.velocity; else w.hi = w.velocity;
                double next = w.derivative > 0. ? w.velocity + (Q - w.rate) / w.derivative : w.lo + .5 * (w.hi - w.lo);
                if (!(next > w.lo && next < w.hi)) next = w.lo + .5 * (w.hi - w.lo);
                w.velocity = next;
            }
            __syncthreads();
        }
        inlet_rate(w, m, b, k0, k1, requested, g, dry, q, z);
        const bool final_bad = !isfinite(w.rate) || fabs(w.rate - Q) > 1e-10 * Q + 1024. * EPS * w.gross;
        __syncthreads();
        if (threadIdx.x == 0 && final_bad) w.error = 3;
        __syncthreads();
    }
    const int error = w.error;
    const double velocity = w.velocity;
    __syncthreads();
    if (error) return error;
    for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
        const int f = b.slot_face[k], c = m.owner[f];
        const double nx = m.normal[f], ny = m.normal[nf + f], h0 = q[c];
        double hi, ui;
        inlet_interior(m, b, k, dry, q, z, hi, ui);
        const double vt = h0 > dry ? (-q[nc + c] * ny + q[2 * nc + c] * nx) / h0 : 0.;
        double hr = fmax(requested - b.ext_bed[k], 0.);
        if (hr <= dry) hr = 0.;
        InletRiemann r = Q == 0. ? inlet_exact(h0, -ui, h0, ui, g) : inlet_exact(hr, velocity, hi, ui, g);
        if (Q == 0.) r.u = 0.;
        if (r.error || !isfinite(r.h) || !isfinite(r.u) || fabs(r.u) > speed) { bad = true; continue; }
        const double water = -r.h * r.u, tangent = r.u < 0. ? vt : 0.;
        b.trace[k] = r.h; b.trace[ns + k] = water * nx - r.h * tangent * ny; b.trace[2 * ns + k] = water * ny + r.h * tangent * nx;
        const double pressure = Q == 0. ? 0. : .5 * g * (h0 * h0 - hi * hi);
        const double momentum = r.h * r.u * r.u + .5 * g * r.h * r.h + pressure;
        b.flux[k] = water;
        b.flux[ns + k] = momentum * nx - water * tangent * ny;
        b.flux[2 * ns + k] = momentum * ny + water * tangent * nx;
    }
    __syncthreads();
    return 0;
}

// ---------------------------------------------------------------------------
// Reference water lines of the exact-discharge inlets, written into the
// forcing stage before the exterior flux: 1 critical depth
// (river_exterior_section.h:17-74), 2 normal depth
// (river_exterior_normal.h:18-104). Every distinct bed level of the section
// starts one constant-wet-width branch (a candidate); 128 lanes take the
// candidates and thread 0 reduces the lanes to the lexicographic minimum of
// (rank, stage), which does not depend on the order. A solved line is kept
// per segment with its discharge and reused while the discharge is equal
// (the inputs besides it are fixed; the host clears the cache when it
// changes them), as the reference's SectionCache.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void line_pick(double rank, double cand, double &best, double &stage)
{
    if (rank < best || (rank == best && cand < stage)) { best = rank; stage = cand; }
}

__device__ void line_critical_candidate(const MeshDev &m, const BoundaryDev &b, int i, int k0, int k1, double Q,
                                        double g, double dry, double &rank, double &cand)
{
    const double level = b.ext_bed[i];
    double minimum = level, next = INFINITY, width = 0., excess = 0.;
    for (int k = k0; k < k1; ++k) {
        const double zb = b.ext_bed[k], len = m.length[b.slot_face[k]];
        minimum = fmin(minimum, zb);
        if (zb > level) next = fmin(next, zb);
        else { width += len; excess += (level - zb) * len; }
    }
    rank = INFINITY; cand = 0.;
    if (Q == 0.) { cand = minimum; rank = 0.; return; }
    const double area = cbrt(Q * Q * width / g), eta = level + (area - excess) / width;
    if (!(isfinite(area) && area > 0. && isfinite(eta) && eta > level + dry) || eta > next + dry) return;
    double actual = 0., wet_width = 0.;
    for (int k = k0; k < k1; ++k) {
        const double h = eta - b.ext_bed[k], len = m.length[b.slot_face[k]];
        if (h > dry) { actual += h * len; wet_width += len; }
    }
    if (wet_width != width || !(actual > 0.)) return;
    const double residual = fabs(Q * Q * wet_width / (g * actual * actual * actual) - 1.);
    const double tolerance = 1e-10 + 64. * EPS * fmax(1., fabs(eta)) * width / actual;
    if (residual > tolerance) return;
    cand = eta;
    rank = eta - minimum + Q * Q / (2. * g * actual * actual);
}

// wetted perimeter of slot k: its length plus the wetted steps to its neighbours
__device__ __forceinline__ double line_perimeter(const MeshDev &m, const BoundaryDev &b, int k, double eta, double dry)
{
    const double h = eta - b.ext_bed[k];
    if (h <= dry) return 0.;
    const int l = b.line_left[k], r = b.line_right[k];
    double hl = l < 0 ? 0. : fmax(eta - b.ext_bed[l], 0.), hr = r < 0 ? 0. : fmax(eta - b.ext_bed[r], 0.);
    if (hl <= dry) hl = 0.;
    if (hr <= dry) hr = 0.;
    return m.length[b.slot_face[k]] + fmax(h - hl, 0.) + fmax(h - hr, 0.);
}

__device__ double line_rate(const MeshDev &m, const BoundaryDev &b, int k0, int k1, double eta, double slope,
                            double g, double dry, int law, double rough)
{
    double area = 0., perimeter = 0., drag = 0.;
    for (int k = k0; k < k1; ++k) {
        const double h = eta - b.ext_bed[k];
        if (h > dry) { area += h * m.length[b.slot_face[k]]; perimeter += line_perimeter(m, b, k, eta, dry); }
    }
    if (!(area > 0. && perimeter > 0.)) return 0.;
    const double c = nout_chezy(law, fmax(area / perimeter, dry), rough, g);
    for (int k = k0; k < k1; ++k)
        if (eta - b.ext_bed[k] > dry) drag += line_perimeter(m, b, k, eta, dry) / (c * c);
    return drag > 0. ? area * sqrt(area * slope / drag) : 0.;
}

__device__ void line_normal_candidate(const MeshDev &m, const BoundaryDev &b, int i, int k0, int k1, double Q,
                                      double slope, double g, double dry, int law, double rough, double &rank,
                                      double &cand)
{
    rank = INFINITY; cand = 0.;
    const double level = b.ext_bed[i];
    const int fi = b.slot_face[i];
    double minimum = level, next = INFINITY;
    for (int k = k0; k < k1; ++k) {
        const double zb = b.ext_bed[k];
        minimum = fmin(minimum, zb);
        if (zb > level) next = fmin(next, zb);
        if (zb == level && b.slot_face[k] < fi) return;          // one candidate per distinct level
    }
    if (Q == 0.) { cand = rank = minimum; return; }
    const double epsilon = 8. * EPS * fmax(1., fabs(level));
    double lo = level + dry + epsilon, hi = isfinite(next) ? next + dry : level + fmax(1., 64. * dry);
    if (!(hi > lo)) return;
    double rlo = line_rate(m, b, k0, k1, lo, slope, g, dry, law, rough) - Q;
    double rhi = line_rate(m, b, k0, k1, hi, slope, g, dry, law, rough) - Q;
    if (!isfinite(next))
        for (int k = 0; k < 60 && rhi < 0.; ++k) {
            hi = level + 2. * (hi - level);
            rhi = line_rate(m, b, k0, k1, hi, slope, g, dry, law, rough) - Q;
        }
    if (!isfinite(rlo) || !isfinite(rhi)) return;
    const double start = lo, end = hi;
    double previous = rlo;
    bool found = false;
    for (int j = 1; j <= 32; ++j) {          // sub-brackets: the lowest sign change of the branch
        const double at = start + (end - start) * (double(j) / 32.);
        const double value = j == 32 ? rhi : line_rate(m, b, k0, k1, at, slope, g, dry, law, rough) - Q;
        if (isfinite(value) && ((previous <= 0. && value >= 0.) || (previous >= 0. && value <= 0.))) {
            hi = at; rhi = value; rlo = previous; found = true;
            break;
        }
        lo = at; previous = value;
    }
    if (!found) return;
    for (int j = 0; j < 80; ++j) {
        const double mid = lo + .5 * (hi - lo);
        if (mid == lo || mid == hi) break;
        const double value = line_rate(m, b, k0, k1, mid, slope, g, dry, law, rough) - Q;
        if ((rlo <= 0. && value >= 0.) || (rlo >= 0. && value <= 0.)) { hi = mid; rhi = value; }
        else { lo = mid; rlo = value; }
    }
    const double eta = fabs(rlo) < fabs(rhi) ? lo : hi;
    const double rate = line_rate(m, b, k0, k1, eta, slope, g, dry, law, rough);
    const double tolerance = 1e-10 + 128. * EPS * fmax(1., fabs(eta)) / fmax(eta - minimum, dry);
    if (isfinite(rate) && fabs(rate / Q - 1.) <= tolerance) { cand = eta; rank = eta; }
}

// The line of segment sg (block-cooperative); false when the section has no
// resolved root (the reference rejects the trial).
__device__ bool line_section(SectionWork &w, const MeshDev &m, const BoundaryDev &b, int sg, double g, double dry,
                             int law, double rough)
{
    const int k0 = b.seg_off[sg], k1 = b.seg_off[sg + 1], kind = b.line_kind[sg];
    const double Q = b.forcing[sg];
    const bool cached = b.line_q[sg] == Q;
    __syncthreads();
    if (cached) {
        if (threadIdx.x == 0) b.forcing[b.nseg + sg] = b.line_stage[sg];
        __syncthreads();
        return true;
    }
    for (int lane = threadIdx.x; lane < SECTION_LANES; lane += blockDim.x) {
        double best = INFINITY, stage = 0.;
        for (int i = k0 + lane; i < k1; i += SECTION_LANES) {
            double rank, cand;
            if (kind == 1) line_critical_candidate(m, b, i, k0, k1, Q, g, dry, rank, cand);
            else line_normal_candidate(m, b, i, k0, k1, Q, b.line_slope[sg], g, dry, law, rough, rank, cand);
            line_pick(rank, cand, best, stage);
        }
        w.part[0][lane] = best; w.part[1][lane] = stage;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double best = INFINITY, stage = 0.;
        for (int lane = 0; lane < SECTION_LANES; ++lane) line_pick(w.part[0][lane], w.part[1][lane], best, stage);
        w.error = !isfinite(best);
        if (!w.error) {
            b.forcing[b.nseg + sg] = stage;
            b.line_q[sg] = Q;
            b.line_stage[sg] = stage;
        }
    }
    __syncthreads();
    const bool ok = !w.error;
    __syncthreads();
    return ok;
}

// Exact-discharge inlet allocation of one scenario (boundary CTA, after the outlet cap).
__device__ void inlet_allocation(const MeshDev &m, const BoundaryDev &b, const Ctrl &ct, const double *base, int s0,
                                 int s1, int u0, int u1)
{
    // exact-discharge inlet allocation (inlet_feasibility.py:34-57): each
    // owner's outward inlet debit capped by its stock after its other
    // boundary debits (owner factor kept per slot in terms), then per inlet
    // segment the removed outflow taken from its incoming faces; sums in
    // boundary order, as the reference's bincounts
    __syncthreads();
    const size_t ns = b.nslot;
    for (int u = u0 + threadIdx.x; u < u1; u += blockDim.x) {
        const int c = b.own_cell[u];
        double total = 0., reserved = 0.;
        for (int j = b.own_off[u]; j < b.own_off[u + 1]; ++j) {
            const int k = b.own_slot[j], f = b.slot_face[k];
            const double rate = fmax(b.flux[k], 0.) * m.length[f];
            if (b.seg_mode[m.bid[f]] == 9) total += rate; else reserved += rate;
        }
        const double available = fmax(0., base[c] * m.area[c] / ct.trial - reserved);
        const double ratio = fmin(1., available / fmax(total, 1e-300)) * (1. - 32. * EPS);
        const double factor = total > available ? ratio : 1.;
        for (int j = b.own_off[u]; j < b.own_off[u + 1]; ++j) b.terms[b.own_slot[j]] = factor;
    }
    __syncthreads();
    for (int sg = s0 + threadIdx.x; sg < s1; sg += blockDim.x) {
        if (b.seg_mode[sg] != 9) continue;
        double removed = 0., incoming = 0.;
        for (int k = b.seg_off[sg]; k < b.seg_off[sg + 1]; ++k) {
            const double water = b.flux[k], len = m.length[b.slot_face[k]];
            removed += water > 0. ? fmax(water, 0.) * len * (1. - b.terms[k]) : 0.;
            incoming += fmax(-water, 0.) * len;
        }
        const bool feasible = removed <= incoming;
        const double in_scale = incoming > 0. ? 1. - removed / fmax(incoming, 1e-300) : 1.;
        for (int k = b.seg_off[sg]; k < b.seg_off[sg + 1]; ++k) {
            const double water = b.flux[k];
            const double scale = (feasible && water > 0.) ? b.terms[k] : ((feasible && water < 0.) ? in_scale : 1.);
            const double depth = b.trace[k], denom = fmax(depth, 1e-300);
            const double ux = depth > 0. ? b.trace[ns + k] / denom : 0.;
            const double uy = depth > 0. ? b.trace[2 * ns + k] / denom : 0.;
            b.flux[ns + k] += (scale * scale - 1.) * water * ux;
            b.flux[2 * ns + k] += (scale * scale - 1.) * water * uy;
            b.flux[k] = water * scale;
            b.trace[ns + k] *= scale;
            b.trace[2 * ns + k] *= scale;
        }
    }
}

// The scenario's sum over its open faces of (outward water flux x length),
// with each face's water as the update consumes it (the mixed form carries
// it in FP32: F(flux)); per-thread strided sums, a butterfly within each
// warp, then thread 0 adds the warp sums in warp order (a fixed order: the
// same value on every run). The controller turns the stage sums into the
// boundary ledger.
constexpr int BOUNDARY_WARPS = 32;
template <class F>
__device__ void boundary_water(const MeshDev &m, const BoundaryDev &b, Ctrl &ct, int stage, int k0, int k1)
{
    __shared__ double part[BOUNDARY_WARPS], apart[BOUNDARY_WARPS];
    __syncthreads();
    double acc = 0., aacc = 0.;
    for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
        const double v = double(F(b.flux[k])) * m.length[b.slot_face[k]];
        acc += v;
        aacc += fabs(v);
    }
    for (int o = 16; o > 0; o >>= 1) {
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
        aacc += __shfl_xor_sync(0xffffffffu, aacc, o);
    }
    if ((threadIdx.x & 31) == 0) { part[threadIdx.x >> 5] = acc; apart[threadIdx.x >> 5] = aacc; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double total = 0., gross = 0.;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { total += part[i]; gross += apart[i]; }
        ct.bflux[stage - 1] = total;
        ct.bgross[stage - 1] = gross;
    }
}

// stage 1 / 2: the SSPRK stages (state work / q1, its own stock, clock t or
// t + dt); STAGE_HANCOCK: the HLLC predicted state q1 at t + dt/2, outlet
// stock of the substep's start state work (hllc.py:91-97), status of stage 1.
constexpr int STAGE_HANCOCK = 3;

template <class F>
__global__ void k_boundary(MeshDev m, StateDev s, BoundaryDev b, Ctrl *ctrl, int stage_in)
{
    __shared__ double tile_buf[BOUNDARY_TILES];
    const int sid = blockIdx.x;
    Ctrl &ct = ctrl[sid];
    const bool hancock = stage_in == STAGE_HANCOCK;
    const int stage = hancock ? 1 : stage_in;
    if (skip_stage(ct, stage)) return;
    const int s0 = b.scen_seg[sid], s1 = b.scen_seg[sid + 1];
    if (s0 == s1) return;
    const int nc = m.nc;
    const double *q = stage == 1 && !hancock ? s.work : s.q1;
    const double *base = hancock ? s.work : q;    // stock of the stage start (the substep start for Hancock)
    const double *z = s.z;
    const double dry = ct.dry, grav = ct.grav;
    const double t = ct.time0 + ct.elapsed + (stage == 2 ? ct.trial : hancock ? .5 * ct.trial : 0.0);
    // forcing at the stage clock (piecewise linear tables, else constant)
    if (b.table_len > 0)
        for (int sg = s0 + threadIdx.x; sg < s1; sg += blockDim.x)
            for (int row = 0; row < 2; ++row) {
                const int L = b.table_len;
                const double *y = b.table_value + ((size_t)row * b.nseg + sg) * L;
                double val;
                if (t <= b.table_time[0]) val = y[0];
                else if (t >= b.table_time[L - 1]) val = y[L - 1];
                else {
                    // last knot at or before t, capped at L - 2; (1 - w) y_i + w y_{i+1}
                    // (RiverHydraulicSchedule.sample, river_hydraulic_schedule.py:57-65)
                    int i = 0;
                    while (i < L - 2 && b.table_time[i + 1] <= t) ++i;
                    const double w = (t - b.table_time[i]) / (b.table_time[i + 1] - b.table_time[i]);
                    val = (1. - w) * y[i] + w * y[i + 1];
                }
                b.forcing[(size_t)row * b.nseg + sg] = val;
            }
    // critical, then normal reference lines of the exact-discharge inlets
    // (river_exterior_bed.py:199-200); a section without a root rejects the trial
    __shared__ SectionWork section;
    bool line_failed = false;
    if (b.line_kind) {
        for (int pass = 1; pass <= 2; ++pass)
            for (int sg = s0; sg < s1; ++sg)          // block-uniform
                if (b.seg_mode[sg] == 9 && b.line_kind[sg] == pass &&
                    !line_section(section, m, b, sg, grav, dry, ct.roughness_mode, ct.roughness_value))
                    line_failed = true;
        __syncthreads();
    }
    const int k0 = b.seg_off[s0], k1 = b.seg_off[s1];
    for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
        const int f = b.slot_face[k], c = m.owner[f];
        const double w = q[c] > dry ? m.length[f] : 0.;
        b.terms[k] = (z[c] + q[c]) * w;
        b.terms[(size_t)b.nslot + k] = w;
    }
    __syncthreads();
    segment_sums(b, s0, s1, 0, 0, tile_buf);
    segment_sums(b, s0, s1, 1, 1, tile_buf);
    const int rmode = ct.roughness_mode < 3 ? ct.roughness_mode : 3;
    const int waqua = ct.roughness_mode == 4;
    const int nseg = b.nseg;
    for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
        const int f = b.slot_face[k], c = m.owner[f], sg = m.bid[f];
        double w = 0.;
        const double bed = b.ext_bed[k];
        const int mode = b.seg_mode[sg];
        if (mode == 6 && b.seg_sums[nseg + sg] > 0.) {
            const double h = fmax(q[c] + z[c] - bed, 0.);
            const double section = fmax(b.seg_sums[sg] / b.seg_sums[nseg + sg] - bed, 0.);
            if (h > dry && section > 0.)
                w = double(pow(F(section), F(1.5)) *
                           exterior_chezy<F>(rmode, F(h), F(ct.roughness_value), F(dry), F(grav), waqua)) * m.length[f];
        }
        b.terms[2 * (size_t)b.nslot + k] = w;
    }
    __syncthreads();
    segment_sums(b, s0, s1, 2, 2, tile_buf);
    unsigned bad = 0;
    for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
        const int f = b.slot_face[k], c = m.owner[f], sg = m.bid[f], mode = b.seg_mode[sg];
        double tr0 = 0., tr1 = 0., tr2 = 0., fl0 = 0., fl1 = 0., fl2 = 0.;
        const double h0 = q[c], nx = m.normal[f], ny = m.normal[m.nf + f], bed = b.ext_bed[k];
        const double total = b.seg_sums[2 * (size_t)nseg + sg];
        const double Q = b.forcing[sg], stagev = b.forcing[nseg + sg];
        int st = 0;
        if (!(mode == 4 || mode == 5 || mode == 9 || mode == 10 || mode == 11)) {
            double h = fmax(h0 + z[c] - bed, 0.), geometric = h, ux = 0., uy = 0.;
            if (h0 > dry) { ux = q[nc + c] / h0; uy = q[2 * nc + c] / h0; }
            double un = ux * nx + uy * ny, tx = ux - un * nx, ty = uy - un * ny, normal_speed = 0.;
            if (mode == 6) {
                if (Q > 0. && total <= 0.) st = 1;
                else if (h > dry && Q > 0.) normal_speed = -Q * b.terms[2 * (size_t)b.nslot + k] / (total * h * m.length[f]);
            } else if (mode == 3) {
                if (h0 <= dry) h = 0.;
                else if (h > dry) {
                    if (un < sqrt(grav * h)) st = 6;
                    else normal_speed = un;
                }
            } else if (mode == 2) {
                const double prescribed = fmax(stagev - bed, 0.);
                const int policy = b.stage_policy[sg];
                if (policy && (h0 <= dry || h <= dry) && prescribed > dry) st = 4;
                else {
                    if (h0 <= dry) h = 0.;
                    if (h > dry) {
                        const double wave = sqrt(grav * h);
                        if (un <= -wave) {
                            if (policy) st = 5;
                            else { normal_speed = 0.; tx = ty = 0.; }
                        } else {
                            const double target = fmax(stagev - bed, 0.);
                            double hb, ub;
                            stage_wave(h, un, target, grav, hb, ub);
                            if (ub < 0. && policy) {
                                if (ub <= -sqrt(grav * hb)) st = 5;
                                else { h = hb; normal_speed = ub; tx = ty = 0.; }
                            } else if (ub < 0.) { normal_speed = 0.; tx = ty = 0.; }
                            else { h = hb; normal_speed = ub; }
                        }
                    }
                }
            } else st = 2;
            if (!st && (!isfinite(h) || !isfinite(normal_speed) || h < 0. ||
                        sqrt(normal_speed * normal_speed + tx * tx + ty * ty) > ct.speed_limit)) st = 3;
            if (!st) {
                double water = 0., fx = 0., fy = 0.;
                if (h > dry) {
                    tr0 = h;
                    tr1 = h * (normal_speed * nx + tx);
                    tr2 = h * (normal_speed * ny + ty);
                    water = tr1 * nx + tr2 * ny;
                    fx = water * tr1 / h + .5 * grav * h * h * nx;
                    fy = water * tr2 / h + .5 * grav * h * h * ny;
                }
                double pressure = h0 > dry ? .5 * grav * (h0 * h0 - geometric * geometric) : 0.;
                fl0 = water; fl1 = fx + pressure * nx; fl2 = fy + pressure * ny;
            }
        }
        if (st) bad = 1;
        b.trace[k] = tr0; b.trace[(size_t)b.nslot + k] = tr1; b.trace[2 * (size_t)b.nslot + k] = tr2;
        b.flux[k] = fl0; b.flux[(size_t)b.nslot + k] = fl1; b.flux[2 * (size_t)b.nslot + k] = fl2;
    }
    __syncthreads();
    // section owners of the remaining outlet modes, after the face loop, in
    // the reference's order (river_exterior_bed.py:213-217): a normal-depth
    // chain without a root rejects the trial before the rating owner runs; a
    // rating section without a solution fails the scenario
    __shared__ int section_reject;
    if (threadIdx.x == 0) section_reject = line_failed;
    __syncthreads();
    if (b.inlet && !section_reject) {
        bool inlet_failed = false;
        for (int sg = s0; sg < s1; ++sg)              // block-uniform: the CTA solves one section at a time
            if (b.seg_mode[sg] == 9) {
                bool sbad = false;
                if (inlet_section(section, m, b, sg, grav, dry, ct.speed_limit, q, z, sbad)) inlet_failed = true;
                if (sbad) bad = 1;
            }
        if (threadIdx.x == 0 && inlet_failed) section_reject = 1;
        __syncthreads();
    }
    if (b.branch && !section_reject) {
        bool crit_failed = false;
        for (int sg = s0; sg < s1; ++sg)              // block-uniform: the CTA solves one section at a time
            if (b.seg_mode[sg] == 4) {
                bool sbad = false;
                if (crit_section(section, m, b, sg, grav, dry, ct.speed_limit, q, z, sbad)) crit_failed = true;
                if (sbad) bad = 1;
            }
        if (threadIdx.x == 0 && crit_failed) section_reject = 1;
        __syncthreads();
    }
    if (b.weir && !section_reject) {
        for (int sg = s0; sg < s1; ++sg)              // block-uniform: the CTA solves one section at a time
            if (b.seg_mode[sg] == 5) {
                bool sbad = false;
                const int e = weir_section(section, m, b, sg, grav, dry, ct.speed_limit, q, z, sbad);
                if (threadIdx.x == 0 && e) section_reject = 1;
                if (sbad) bad = 1;
            }
        __syncthreads();
    }
    if (b.scen_chain && !section_reject) {
        const int law = ct.roughness_mode;
        for (int ch = b.scen_chain[sid] + threadIdx.x; ch < b.scen_chain[sid + 1]; ch += blockDim.x) {
            bool sbad = false;
            if (normal_chain(m, b, ch, grav, dry, ct.speed_limit, law, ct.roughness_value, q, z, sbad))
                atomicOr(&section_reject, 1);
            if (sbad) bad = 1;
        }
    }
    __syncthreads();
    if (!section_reject)
        for (int sg = s0 + threadIdx.x; sg < s1; sg += blockDim.x)
            if (b.seg_mode[sg] == 11) {
                bool sbad = false;
                if (rating_section(m, b, sg, grav, dry, ct.speed_limit, q, z, sbad)) raise_status(ct, stage, ST_FATAL);
                if (sbad) bad = 1;
            }
    if (section_reject) bad = 1;
    if (bad) raise_status(ct, stage, ST_SPATIAL);
    __syncthreads();
    // outlet stock cap, one thread per unique owner, its faces in boundary order
    const int u0 = b.scen_own[sid], u1 = b.scen_own[sid + 1];
    for (int u = u0 + threadIdx.x; u < u1; u += blockDim.x) {
        const int c = b.own_cell[u];
        double total = 0., reserved = 0.;
        for (int j = b.own_off[u]; j < b.own_off[u + 1]; ++j) {
            const int k = b.own_slot[j], f = b.slot_face[k];
            const double debit = fmax(b.flux[k], 0.) * m.length[f];
            if (is_outlet(b.seg_mode[m.bid[f]])) total += debit; else reserved += debit;
        }
        const double available = fmax(0., base[c] * m.area[c] / ct.trial - reserved);
        const double ratio = fmin(1., available / fmax(total, 1e-300)) * (1. - 32. * EPS);
        const double factor = total > available ? ratio : 1.;
        for (int j = b.own_off[u]; j < b.own_off[u + 1]; ++j) {
            const int k = b.own_slot[j], f = b.slot_face[k];
            const double water = b.flux[k];
            const double scale = (is_outlet(b.seg_mode[m.bid[f]]) && water > 0.) ? factor : 1.;
            const double depth = b.trace[k], denom = fmax(depth, 1e-300);
            const double ux = depth > 0. ? b.trace[(size_t)b.nslot + k] / denom : 0.;
            const double uy = depth > 0. ? b.trace[2 * (size_t)b.nslot + k] / denom : 0.;
            b.flux[(size_t)b.nslot + k] += (scale * scale - 1.) * water * ux;
            b.flux[2 * (size_t)b.nslot + k] += (scale * scale - 1.) * water * uy;
            b.flux[k] = water * scale;
            b.trace[(size_t)b.nslot + k] *= scale;
            b.trace[2 * (size_t)b.nslot + k] *= scale;
        }
    }
    if (b.inlet) inlet_allocation(m, b, ct, base, s0, s1, u0, u1);
    boundary_water<F>(m, b, ct, stage, k0, k1);
}

// ---------------------------------------------------------------------------
// Cells: primitive values, limited least-squares gradients, flattening flag.
// Depth, surface and bed stay FP64 (the stage reconstruction); gradients,
// limiter factors and the projection run in F.
// ---------------------------------------------------------------------------
// Roundoff scale of the arithmetic type: the reference's FP64 thresholds
// (64 eps, 2e-14) are kept verbatim for F = double; in FP32 the same tests
// are widened to FP32 rounding so that a projection vertex lying on its own
// constraints is not rejected by rounding noise.
template <class F> struct Eps { static constexpr double value = 2.2204460492503131e-16; };
template <> struct Eps<float> { static constexpr double value = 1.1920928955078125e-07; };

template <class F>
__device__ __forceinline__ bool feasible(F x, F y, int count, const F *ax, const F *ay, const F *bb)
{
    for (int i = 0; i < count; ++i) {
        F tol = F(2.e-14);
        if (sizeof(F) != 8) tol += F(16. * Eps<F>::value) * (fabs(ax[i] * x) + fabs(ay[i] * y) + fabs(bb[i]));
        if (ax[i] * x + ay[i] * y > bb[i] + tol) return false;
    }
    return true;
}

template <class F>
__device__ __noinline__ void project_pair(F &x, F &y, int count, const F *ax, const F *ay, const F *bb)
{
    const F rx = x, ry = y;
    if (feasible<F>(rx, ry, count, ax, ay, bb)) return;
    F bx = F(0.), by = F(0.), best = rx * rx + ry * ry;
    for (int i = 0; i < count; ++i) {
        const F dot = ax[i] * rx + ay[i] * ry - bb[i];
        F cx = rx - dot * ax[i], cy = ry - dot * ay[i];
        F d = (cx - rx) * (cx - rx) + (cy - ry) * (cy - ry);
        if (d < best && feasible<F>(cx, cy, count, ax, ay, bb)) { bx = cx; by = cy; best = d; }
        for (int j = 0; j < i; ++j) {
            const F det = ax[i] * ay[j] - ay[i] * ax[j];
            if (fabs(det) < F(1.e-12)) continue;
            cx = (bb[i] * ay[j] - ay[i] * bb[j]) / det;
            cy = (ax[i] * bb[j] - bb[i] * ax[j]) / det;
            d = (cx - rx) * (cx - rx) + (cy - ry) * (cy - ry);
            if (d < best && feasible<F>(cx, cy, count, ax, ay, bb)) { bx = cx; by = cy; best = d; }
        }
    }
    x = bx; y = by;
}

// MAXF bounds the faces of one cell (4 for triangle/quad meshes, 32 in general).
template <class F, int MAXF>
__global__ void __launch_bounds__(128) k_cells(MeshDev m, StateDev s, Ctrl *ctrl, Work w, int stage)
{
    const int nc = m.nc, nf = m.nf, nadj = m.nadj;
    FOR_ACTIVE_CELLS(m.act, c) {
        Ctrl &ct = ctrl[m.cell_sid[c]];
        if (skip_stage(ct, stage)) continue;
        const double *q = stage == 1 ? s.work : s.q1;
        const double *z = s.z;
        const double dry = ct.dry, grav = ct.grav;
        const double h = q[c], hu = q[nc + c], hv = q[2 * nc + c], zc = z[c];
        if (h < 0.0 || !isfinite(h) || !isfinite(zc) || !isfinite(hu) || !isfinite(hv))
            raise_status(ct, stage, ST_SPATIAL);
        double centre[4] = {h + zc, 0., 0., zc};
        if (h > dry) { centre[1] = double(F(hu) / F(h)); centre[2] = double(F(hv) / F(h)); }
        double lo[4], hi[4];
        F gx[4] = {F(0.), F(0.), F(0.), F(0.)}, gy[4] = {F(0.), F(0.), F(0.), F(0.)};
#pragma unroll
        for (int p = 0; p < 4; ++p) { lo[p] = centre[p]; hi[p] = centre[p]; }
        const int k0 = m.offset[c], k1 = m.offset[c + 1];
        // active: wet, or touching an open face or a wet neighbour
        bool active = h > dry;
        F bx[4] = {F(0.), F(0.), F(0.), F(0.)}, by[4] = {F(0.), F(0.), F(0.), F(0.)};
        for (int k = k0; k < k1; ++k) {
            const int f = m.faces[k];
            const int n = m.signs[k] < 0 ? m.owner[f] : m.neighbour[f];
            if (n < 0) { if (m.bid[f] >= 0) active = true; continue; }
            const double hn = q[n], zn = z[n];
            if (hn > dry) active = true;
            double vn[4] = {hn + zn, 0., 0., zn};
            if (hn > dry) { vn[1] = double(F(q[nc + n]) / F(hn)); vn[2] = double(F(q[2 * nc + n]) / F(hn)); }
            const F rx = F(m.ls_delta[k]), ry = F(m.ls_delta[nadj + k]), wt = F(m.ls_weight[k]);
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                double adj = vn[p];
                if (p == 0 && centre[0] - centre[3] > dry && vn[0] - vn[3] <= dry && vn[3] >= centre[0]) adj = centre[0];
                const F d = F(adj - centre[p]);
                bx[p] += wt * rx * d;
                by[p] += wt * ry * d;
                lo[p] = fmin(lo[p], adj); hi[p] = fmax(hi[p], adj);
            }
        }
        if (active) {
            const F a11 = F(m.ls_matrix[c]), a12 = F(m.ls_matrix[nc + c]), a22 = F(m.ls_matrix[2 * nc + c]),
                    det = F(m.ls_matrix[3 * nc + c]);
            if (a11 + a22 > F(0.0)) {
                if (h > dry)
                    for (int k = k0; k < k1; ++k) {
                        const int f = m.faces[k];
                        if (m.neighbour[f] >= 0 || m.bid[f] >= 0) continue;
                        const double nx = m.normal[f], ny = m.normal[nf + f];
                        const double un = centre[1] * nx + centre[2] * ny;
                        const double mx = centre[1] - 2. * un * nx, my = centre[2] - 2. * un * ny;
                        lo[1] = fmin(lo[1], mx); hi[1] = fmax(hi[1], mx);
                        lo[2] = fmin(lo[2], my); hi[2] = fmax(hi[2], my);
                    }
                const bool full = det > F(1.e-12) * ((a11 + a22) * (a11 + a22));
#pragma unroll
                for (int p = 0; p < 4; ++p) {
                    if (full) {
                        gx[p] = (a22 * bx[p] - a12 * by[p]) / det;
                        gy[p] = (a11 * by[p] - a12 * bx[p]) / det;
                    } else {
                        gx[p] = (a11 * bx[p] + a12 * by[p]) / ((a11 + a22) * (a11 + a22));
                        gy[p] = (a12 * bx[p] + a22 * by[p]) / ((a11 + a22) * (a11 + a22));
                    }
                }
                const double hh = centre[0] - centre[3];
                const F sq = hh > dry ? sqrt(F(grav) * F(hh)) : F(0.);
                const F bedtol = F(64.0 * Eps<F>::value) * fmax(F(1.0), F(fabs(centre[3])));
                F theta1 = F(1.), theta2 = F(1.);
                F ax0[2 * MAXF], ay0[2 * MAXF], b0[2 * MAXF];
                F ax3[2 * MAXF], ay3[2 * MAXF], b3[2 * MAXF];
                int n0 = 0, n3 = 0;
                for (int k = k0; k < k1; ++k) {
                    const int f = m.faces[k];
                    const int side = m.signs[k] < 0;
                    const F rx = F(m.disp[side * nf + f]), ry = F(m.disp[(2 + side) * nf + f]);
                    // an open stage outlet with a subcritical wet owner keeps its bed slope
                    if (m.bmode[f] == 2 && m.neighbour[f] < 0 && hh > dry &&
                        fabs(F(centre[1]) * F(m.normal[f]) + F(centre[2]) * F(m.normal[nf + f])) < sq &&
                        fabs(gx[3] * rx + gy[3] * ry) > bedtol) continue;
#pragma unroll
                    for (int p = 1; p < 3; ++p) {
                        const F d = gx[p] * rx + gy[p] * ry;
                        if (fabs(d) <= F(64.0 * Eps<F>::value) * fmax(F(1.0), F(fmax(fabs(centre[p]), fmax(fabs(lo[p]), fabs(hi[p]))))))
                            continue;
                        F &th = p == 1 ? theta1 : theta2;
                        if (d > F(0.)) th = fmin(th, F(hi[p] - centre[p]) / d);
                        if (d < F(0.)) th = fmin(th, F(lo[p] - centre[p]) / d);
                    }
                    const F len = F(m.disp_len[side * nf + f]);
                    if (len <= F(0.)) continue;
                    const F ux = F(m.disp_unit[side * nf + f]), uy = F(m.disp_unit[(2 + side) * nf + f]);
                    ax0[n0] = ux; ay0[n0] = uy; b0[n0++] = fmax(F(0.), F(hi[0] - centre[0])) / len;
                    ax0[n0] = -ux; ay0[n0] = -uy; b0[n0++] = fmax(F(0.), F(centre[0] - lo[0])) / len;
                    if (m.neighbour[f] < 0 && m.bid[f] < 0) continue;   // walls do not bound the bed
                    ax3[n3] = ux; ay3[n3] = uy; b3[n3++] = fmax(F(0.), F(hi[3] - centre[3])) / len;
                    ax3[n3] = -ux; ay3[n3] = -uy; b3[n3++] = fmax(F(0.), F(centre[3] - lo[3])) / len;
                }
                F px0 = gx[0], py0 = gy[0], px3 = gx[3], py3 = gy[3];
                project_pair<F>(px0, py0, n0, ax0, ay0, b0);
                project_pair<F>(px3, py3, n3, ax3, ay3, b3);
                gx[1] *= fmax(F(0.), theta1); gy[1] *= fmax(F(0.), theta1);
                gx[2] *= fmax(F(0.), theta2); gy[2] *= fmax(F(0.), theta2);
                gx[0] = px0; gy[0] = py0; gx[3] = px3; gy[3] = py3;
            }
        }
        bool flatten = h <= dry;
        if (!flatten)
            for (int k = k0; k < k1; ++k) {
                const int f = m.faces[k];
                const int side = (c == m.owner[f]) ? 0 : 1;
                const F rx = F(m.disp[side * nf + f]), ry = F(m.disp[(2 + side) * nf + f]);
                const double eta = (centre[0] + double(gx[0] * rx)) + double(gy[0] * ry);
                const double zb = (centre[3] + double(gx[3] * rx)) + double(gy[3] * ry);
                if (eta - zb <= dry || fabs(zb - centre[3]) >= h) { flatten = true; break; }
            }
        CellRec r;
        r.h = h; r.eta = centre[0]; r.u = centre[1]; r.v = centre[2]; r.b = centre[3];
#pragma unroll
        for (int p = 0; p < 4; ++p) { r.gx[p] = double(gx[p]); r.gy[p] = double(gy[p]); }
        r.flags = (flatten ? 1 : 0) | (active ? 2 : 0);
        r.pad = 0; r.pad2 = 0.;
        w.rec[c] = r;
    }
}

// ---------------------------------------------------------------------------
// Faces: traces, hydrostatic reconstruction, f-wave, flux assembly.
// Traces, the common-bed stage, pressures and the bed source are FP64; the
// Riemann solve and the advective fluxes run in F.
// ---------------------------------------------------------------------------
struct Side { double h, hu, hv, b, raw; };

template <class F>
__device__ __forceinline__ Side face_side(const CellRec &r, double rx_, double ry_, double dry, bool dryface,
                                          unsigned &bad)
{
    const F rx = F(rx_), ry = F(ry_);
    double val[4] = {(r.eta + double(F(r.gx[0]) * rx)) + double(F(r.gy[0]) * ry),
                     double((F(r.u) + F(r.gx[1]) * rx) + F(r.gy[1]) * ry),
                     double((F(r.v) + F(r.gx[2]) * rx) + F(r.gy[2]) * ry),
                     (r.b + double(F(r.gx[3]) * rx)) + double(F(r.gy[3]) * ry)};
    const bool constant = r.flags & 1;
    if (constant) {
        val[0] = r.eta; val[1] = r.u; val[2] = r.v;
        if (r.eta - r.b <= dry) val[3] = r.b;
    }
    if (!isfinite(val[0]) || !isfinite(val[1]) || !isfinite(val[2]) || !isfinite(val[3])) bad = 1;
    Side o = {0., 0., 0., 0., 0.};
    if (dryface) return o;
    double depth = fmax(val[0] - val[3], 0.);
    o.raw = depth;
    if (r.h <= dry || (constant && depth <= dry)) depth = 0.;
    o.h = depth; o.hu = depth * val[1]; o.hv = depth * val[2]; o.b = val[3];
    return o;
}

template <class F>
// Four resident blocks of 128 threads (at most 128 registers): a single
// 75k-face scenario then fits the 152 SMs in one wave of 16 warps each; with
// the unconstrained 168 registers it took 1.3 waves at 12 warps per SM and
// the FP64 pipe sat idle in the tail.
#ifndef BRX_FP64_FACES_MIN_BLOCKS
#define BRX_FP64_FACES_MIN_BLOCKS 4
#endif
__global__ void __launch_bounds__(128, BRX_FP64_FACES_MIN_BLOCKS) k_faces(MeshDev m, StateDev s, BoundaryDev b, Ctrl *ctrl, Work w, int stage,
                                               double *trace, const int *hkt)
{
    const int nf = m.nf, nc = m.nc;
    FOR_ACTIVE_FACES(m.act, f) {
        Ctrl &ct = ctrl[m.face_sid[f]];
        if (skip_stage(ct, stage)) continue;
        const double dry = ct.dry, grav = ct.grav;
        const int c = m.owner[f], n = m.neighbour[f];
        const double nx = m.normal[f], ny = m.normal[nf + f];
        const CellRec rc = w.rec[c];
        const double pc = .5 * grav * rc.h * rc.h;
        const int slot = m.bslot[f];
        if (slot >= 0) {
            // open face: the exterior owner's flux, owner/exterior CFL speed
            const double *q = stage == 1 ? s.work : s.q1;
            const double fl0 = b.flux[slot], fl1 = b.flux[(size_t)b.nslot + slot], fl2 = b.flux[2 * (size_t)b.nslot + slot];
            const double hb = b.trace[slot];
            const double hq = q[c];
            const double a = hq > dry ? fabs((q[nc + c] * nx + q[2 * nc + c] * ny) / hq) + sqrt(grav * hq) : 0.;
            const double bb = hb > dry ? fabs((b.trace[(size_t)b.nslot + slot] * nx + b.trace[2 * (size_t)b.nslot + slot] * ny) / hb) +
                                             sqrt(grav * hb) : 0.;
            w.ws[f] = make_double2(fl0, fmax(a, bb));
            w.gf[f] = make_double4_32a(fl1 - pc * nx, fl2 - pc * ny, 0., 0.);
            continue;
        }
        CellRec rn;
        if (n >= 0) rn = w.rec[n];
        int kind = n >= 0 ? 1 : 2;
        if (rc.h <= dry && (n < 0 || rn.h <= dry)) kind = 0;
        unsigned bad = 0;
        const Side L = face_side<F>(rc, m.disp[f], m.disp[2 * nf + f], dry, kind == 0, bad);
        Side R = {0., 0., 0., 0., 0.};
        if (n >= 0) R = face_side<F>(rn, m.disp[nf + f], m.disp[3 * nf + f], dry, kind == 0, bad);
        double water = 0., speed = 0., l1 = 0., l2 = 0., r1 = 0., r2 = 0.;
        if (kind != 0) {
            double hL = L.h, xL = L.hu, yL = L.hv, bL = L.b;
            double hR = R.h, xR = R.hu, yR = R.hv, bR = R.b;
            double rawR = R.raw;
            if (kind == 2) {
                hR = hL; xR = xL; yR = yL; bR = bL; rawR = L.raw;   // mirrored trace
            }
            // rotation to the face frame (prepare)
            double xRr = xR, yRr = yR;
            if (kind == 2) {
                const double dot = xL * nx + yL * ny;
                xRr = xL - 2.0 * dot * nx; yRr = yL - 2.0 * dot * ny;
            }
            const double unL = xL * nx + yL * ny, utL = xL * (-ny) + yL * nx;
            const double unR = xRr * nx + yRr * ny, utR = xRr * (-ny) + yRr * nx;
            double loc[8] = {hL, unL, utL, bL, hR, unR, utR, bR};
            if (kind == 1) {
                const double top = fmax(bL, bR);
                const double tol = 16. * EPS * fmax(dry, fmax(fabs(top), fmax(fabs(hL + bL), fabs(hR + bR))));
                double hl = fmax(0., hL + bL - top), hr = fmax(0., hR + bR - top);
                if (hl <= dry + tol) hl = 0.;
                if (hr <= dry + tol) hr = 0.;
                loc[0] = hl; loc[3] = top; loc[4] = hr; loc[7] = top;
                loc[1] = hL > dry ? unL * (hl / hL) : 0.;
                loc[2] = hL > dry ? utL * (hl / hL) : 0.;
                loc[5] = hR > dry ? unR * (hr / hR) : 0.;
                loc[6] = hR > dry ? utR * (hr / hR) : 0.;
            }
            if (trace && n >= 0 && hkt[m.face_sid[f]]) put_trace(trace, nf, f, loc, rc.flags & 1, rn.flags & 1);
            bool closed = false;
            if (kind == 1 && !(fmin(rc.h, rn.h) > dry)) {
                const double dc = m.distance[f], dn = m.distance[nf + f];
                double shared;
                if (dc + dn > DBL_MIN_)
                    shared = (dn * (rc.b + rc.h) + dc * (rn.b + rn.h)) / (dc + dn) - fmax(rc.b, rn.b);
                else
                    shared = 0.5 * ((rc.b + rc.h) + (rn.b + rn.h)) - fmax(rc.b, rn.b);
                closed = shared <= dry;
                if (closed) {
                    bool opens = false;
                    if (hL > dry && hR <= dry && unL / hL > 0.0) {
                        const RType<F> t = riemann_type<F>(F(hL), F(hL), F(unL / hL), F(-unL / hL), F(dry), F(grav));
                        opens = t.hm > hL + dry && t.hm + bL > bR + dry;
                    } else if (hR > dry && hL <= dry && -unR / hR > 0.0) {
                        const RType<F> t = riemann_type<F>(F(hR), F(hR), F(-unR / hR), F(unR / hR), F(dry), F(grav));
                        opens = t.hm > hR + dry && t.hm + bR > bL + dry;
                    }
                    closed = !opens;
                }
            }
            double l[3] = {0., 0., 0.}, r[3] = {0., 0., 0.};
            FWaveOut<F> fwo;
            F locf[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) locf[j] = F(loc[j]);
            const int fst = fwave<F>(locf, F(grav), F(dry), fwo);
            if (fst) bad = 1;
            if (closed) {
                l[1] = 0.5 * grav * (hL * hL) * nx; l[2] = 0.5 * grav * (hL * hL) * ny;
                r[1] = 0.5 * grav * (hR * hR) * nx; r[2] = 0.5 * grav * (hR * hR) * ny;
                if (hL > dry) speed = fmax(speed, fabs(loc[1] / hL) + sqrt(grav * hL));
                if (hR > dry) speed = fmax(speed, fabs(loc[5] / hR) + sqrt(grav * hR));
            } else {
                const double starL = loc[0], starR = loc[4];
                double pl[3] = {0., 0., 0.}, pr[3] = {0., 0., 0.};
                if (starL > dry) {
                    const double hu = loc[1], hv = loc[2];
                    pl[0] = hu; pl[1] = double(F(hu) * F(hu) / F(starL)) + 0.5 * grav * (starL * starL);
                    pl[2] = double(F(hu) * F(hv) / F(starL));
                }
                if (starR > dry) {
                    const double hu = loc[5], hv = loc[6];
                    pr[0] = hu; pr[1] = double(F(hu) * F(hu) / F(starR)) + 0.5 * grav * (starR * starR);
                    pr[2] = double(F(hu) * F(hv) / F(starR));
                }
#pragma unroll
                for (int j = 0; j < 3; ++j) { pl[j] += double(fwo.amdq[j]); pr[j] -= double(fwo.apdq[j]); }
                l[0] = pl[0]; l[1] = pl[1] * nx + pl[2] * (-ny); l[2] = pl[1] * ny + pl[2] * nx;
                r[0] = pr[0]; r[1] = pr[1] * nx + pr[2] * (-ny); r[2] = pr[1] * ny + pr[2] * nx;
                // left/right mass fluxes agree to the Riemann solve's precision (1e-10 in FP64)
                const double consistency = sizeof(F) == 8 ? 1.e-10 : 2.e-5;
                if (fabs(l[0] - r[0]) > consistency * fmax(1.0, fmax(fabs(l[0]), fabs(r[0])))) bad = 1;
                l[0] = 0.5 * (l[0] + r[0]); r[0] = l[0];
                speed = double(fmax(fabs(fwo.s[0]), fmax(fabs(fwo.s[1]), fabs(fwo.s[2]))));
                if (kind == 1) {
                    const double cl = .5 * grav * (hL * hL - starL * starL), cr = .5 * grav * (hR * hR - starR * starR);
                    l[1] += cl * nx; l[2] += cl * ny; r[1] += cr * nx; r[2] += cr * ny;
                }
                if (kind == 2) {
                    l[0] = 0.0;
                    const double pressure = wall_pressure<double>(hL, loc[1], grav, dry);
                    l[1] = pressure * nx; l[2] = pressure * ny;
                    r[0] = l[0]; r[1] = l[1]; r[2] = l[2];
                }
            }
            if (rc.h > dry) {
                const double corr = (rc.flags & 1) ? 0.5 * grav * (rc.h * rc.h - hL * hL)
                                                   : 0.5 * grav * (rc.h + L.raw) * (bL - rc.b);
                l[1] += corr * nx; l[2] += corr * ny;
            }
            if (n >= 0) {
                if (rn.h > dry) {
                    const double corr = (rn.flags & 1) ? 0.5 * grav * (rn.h * rn.h - hR * hR)
                                                       : 0.5 * grav * (rn.h + rawR) * (bR - rn.b);
                    r[1] += corr * nx; r[2] += corr * ny;
                }
            } else { r[0] = l[0]; r[1] = l[1]; r[2] = l[2]; }
            if (!isfinite(l[0]) || !isfinite(l[1]) || !isfinite(l[2]) || !isfinite(r[0]) || !isfinite(r[1]) ||
                !isfinite(r[2])) bad = 1;
            water = l[0]; l1 = l[1]; l2 = l[2]; r1 = r[1]; r2 = r[2];
        }
        if (kind == 0 && trace && n >= 0 && hkt[m.face_sid[f]]) {
            const double zero[8] = {0., 0., 0., 0., 0., 0., 0., 0.};
            put_trace(trace, nf, f, zero, rc.flags & 1, rn.flags & 1);
        }
        if (bad) raise_status(ct, stage, ST_SPATIAL);
        w.ws[f] = make_double2(water, speed);
        const double pn = n >= 0 ? .5 * grav * rn.h * rn.h : 0.;
        w.gf[f] = make_double4_32a(l1 - pc * nx, l2 - pc * ny, r1 - pn * nx, r2 - pn * ny);
    }
}

// ---------------------------------------------------------------------------
// Gather: rate, donor inventory / boundary reservation, CFL frequency.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_gather(MeshDev m, StateDev s, Ctrl *ctrl, Work w, int stage)
{
    const int nc = m.nc;
    const int stride = gridDim.x * blockDim.x;
    // warp-uniform trip count: every lane reaches the warp reduction below
    const int na = m.act.count[1];
    for (int first = blockIdx.x * blockDim.x; first < na; first += stride) {   // warp-uniform trip count
        const int c = first + (int)threadIdx.x < na ? active_cell(m.act, first + threadIdx.x) : nc;
        bool have = false;
        double fr = 0.;
        int sid = 0;
        if (c < nc) {
            sid = m.cell_sid[c];
            Ctrl &ct = ctrl[sid];
            if (!skip_stage(ct, stage)) {
                const double *base = stage == 1 ? s.work : s.q1;
                const double dt = ct.trial, area = m.area[c];
                const bool active = w.rec[c].flags & 2;
                double sum0 = 0., sum1 = 0., sum2 = 0., out = 0., freq = 0., ext = 0., interior = 0.;
                const bool owns_open = m.cflags[c] & 1;
                for (int k = m.offset[c]; k < m.offset[c + 1]; ++k) {
                    const int f = m.faces[k];
                    const double len = m.length[f];
                    const double wt = len / area;
                    const double2 ws = w.ws[f];
                    const double4_32a gf = w.gf[f];
                    if (m.signs[k] > 0) { sum0 += wt * ws.x; sum1 += wt * gf.x; sum2 += wt * gf.y; }
                    else { sum0 -= wt * ws.x; sum1 -= wt * gf.z; sum2 -= wt * gf.w; }
                    const double debit = fmax(m.signs[k] * ws.x, 0.) * len;
                    out += debit;
                    if (owns_open) { if (m.bslot[f] >= 0) ext += debit; else interior += debit; }
                    freq += len * ws.y;
                }
                double r0 = 0., r1 = 0., r2 = 0.;
                if (active) { r0 = -sum0; r1 = -sum1; r2 = -sum2; }
                w.rate[c] = r0; w.rate[nc + c] = r1; w.rate[2 * nc + c] = r2;
                double theta = 1.;
                if (out > 0. && dt * out >= base[c] * area)
                    theta = fmin(1., base[c] * area / (dt * out)) * (1. - 32. * 2.2204460492503131e-16);
                if (owns_open) {
                    const double available = base[c] * area / dt;
                    if (ext > available) raise_status(ct, stage, ST_BUDGET);
                    const double factor = fmin(1., (available - ext) / fmax(interior, 1e-300)) * (1. - 32. * EPS);
                    theta = (interior > 0. && interior >= available - ext) ? factor : 1.;
                }
                w.theta[c] = theta;
                fr = freq / area;
                if (isnan(fr)) raise_status(ct, stage, ST_FREQ);
                else have = true;
            }
        }
        unsigned long long *peak0 = stage == 1 ? &ctrl[0].peak1 : &ctrl[0].peak2;
        warp_max_peak(peak0, sizeof(Ctrl), sid, have, fr);
    }
}

// midpoint_faces: limit donor outflow, carry the removed advective momentum.
__global__ void __launch_bounds__(256) k_limit(MeshDev m, StateDev s, Ctrl *ctrl, Work w, int stage)
{
    const int nf = m.nf, nc = m.nc;
    FOR_ACTIVE_FACES(m.act, f) {
        const Ctrl &ct = ctrl[m.face_sid[f]];
        if (skip_stage(ct, stage)) continue;
        const double *q = stage == 1 ? s.work : s.q1;
        double water = w.ws[f].x, cx = 0., cy = 0.;
        if (water != 0. && m.bslot[f] < 0) {
            const int donor = water < 0. ? m.neighbour[f] : m.owner[f];
            if (donor >= 0) {
                const double th = w.theta[donor];
                if (th != 1.) {
                    const double delta = (th - 1.) * water;
                    water *= th;
                    const double hd = q[donor];
                    if (hd > ct.dry) { cx = delta * q[nc + donor] / hd; cy = delta * q[2 * nc + donor] / hd; }
                }
            }
        }
        w.lim[f] = make_double4_32a(water, cx, cy, 0.);
    }
}

// ---------------------------------------------------------------------------
// Conservative wet-bank viscosity (shoreline_viscosity.py:57-72): velocity
// gradients of the safe state by the flow engines' least squares
// (bend_methods_v1_kernels.h:23-39, rows u and v; dry columns read as depth
// 0.001001 without momentum, secondary_vector_ops.py:39-48), then the
// shared-face stress of wet columns (shoreline_viscosity.h:14-33); the
// updates gather it as sum(s len stress) / area after the rotor terms.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_visc_grad(MeshDev m, Work w, const double *q, Ctrl *ctrl, int stage)
{
    const int n = m.nc, na = m.nadj;
    const ViscDev v = w.visc;
    FOR_ACTIVE_CELLS(m.act, i) {
        const int sid = m.cell_sid[i];
        if (!(v.nu[sid] > 0.) || skip_stage(ctrl[sid], stage)) continue;
        const double dry = ctrl[sid].dry;
        const bool wi = q[i] > dry;
        const double hi = wi ? q[i] : .001001;
        const double x0 = (wi ? q[n + i] : 0.) / hi, x1 = (wi ? q[2 * n + i] : 0.) / hi;
        double bx0 = 0., bx1 = 0., by0 = 0., by1 = 0.;
        for (int k = m.offset[i]; k < m.offset[i + 1]; ++k) {
            const int f = m.faces[k], j = m.owner[f] == i ? m.neighbour[f] : m.owner[f];
            if (j < 0) continue;
            const double dx = v.dxdy[k], dy = v.dxdy[na + k], wt = 1. / (dx * dx + dy * dy);
            const bool wj = q[j] > dry;
            const double hj = wj ? q[j] : .001001;
            const double y0 = (wj ? q[n + j] : 0.) / hj, y1 = (wj ? q[2 * n + j] : 0.) / hj;
            bx0 += wt * dx * (y0 - x0); by0 += wt * dy * (y0 - x0);
            bx1 += wt * dx * (y1 - x1); by1 += wt * dy * (y1 - x1);
        }
        v.grad[i] = v.inverse[i] * bx0 + v.inverse[n + i] * by0;
        v.grad[n + i] = v.inverse[n + i] * bx0 + v.inverse[2 * n + i] * by0;
        v.grad[2 * n + i] = v.inverse[i] * bx1 + v.inverse[n + i] * by1;
        v.grad[3 * n + i] = v.inverse[n + i] * bx1 + v.inverse[2 * n + i] * by1;
    }
}

__global__ void __launch_bounds__(256) k_visc_faces(MeshDev m, Work w, const double *q, const double *z, Ctrl *ctrl,
                                                    int stage)
{
    const int n = m.nc, nf = m.nf;
    const ViscDev v = w.visc;
    FOR_ACTIVE_FACES(m.act, i) {
        const int sid = m.face_sid[i];
        const double nu = v.nu[sid];
        if (!(nu > 0.) || skip_stage(ctrl[sid], stage)) continue;
        const double dry = ctrl[sid].dry;
        double sx = 0., sy = 0.;
        const int o = m.owner[i], j = m.neighbour[i];
        if (j >= 0 && q[o] > dry && q[j] > dry) {
            double h = fmin(q[o], q[j]);
            h = fmin(h, fmax(0., .5 * (q[o] + z[o] + q[j] + z[j]) - fmax(z[o], z[j])));
            const double d = m.distance[i] + m.distance[nf + i], wo = m.distance[nf + i] / d, wj = m.distance[i] / d;
            const double nx = m.normal[i], ny = m.normal[nf + i], dx = v.xy[j] - v.xy[o], dy = v.xy[n + j] - v.xy[n + o];
            const double dn = dx * nx + dy * ny;
            const double tx = dx - dn * nx, ty = dy - dn * ny;
            const double du = q[n + j] / q[j] - q[n + o] / q[o], dv = q[2 * n + j] / q[j] - q[2 * n + o] / q[o];
            const double ux = wo * v.grad[o] + wj * v.grad[j], uy = wo * v.grad[n + o] + wj * v.grad[n + j];
            const double vx = wo * v.grad[2 * n + o] + wj * v.grad[2 * n + j];
            const double vy = wo * v.grad[3 * n + o] + wj * v.grad[3 * n + j];
            sx = nu * h * (du - ux * tx - uy * ty) / dn;
            sy = nu * h * (dv - vx * tx - vy * ty) / dn;
        }
        v.face[i] = sx;
        v.face[nf + i] = sy;
    }
}

// The wet-bank viscosity's momentum rate of one cell: sum(s len stress) / area
// with unit weights (flow2dh_fixed_bed_kernels.h:54-60).
__device__ __forceinline__ void add_viscosity(const MeshDev &m, const ViscDev &v, int c, double area, double &r1,
                                              double &r2)
{
    const int nf = m.nf;
    double x = 0., y = 0.;
    for (int k = m.offset[c]; k < m.offset[c + 1]; ++k) {
        const int f = m.faces[k];
        x += m.signs[k] * m.length[f] * v.face[f];
        y += m.signs[k] * m.length[f] * v.face[nf + f];
    }
    r1 += 1. * x / area;
    r2 += 1. * y / area;
}

// midpoint_gather + stage combination (+ closing drag on the second stage).
// With rate_out set, the final rate is stored there and no state is written.
// Owner computes: each cell forms the donor-limited flux of its faces itself
// (midpoint_faces, river_midpoint.h:30-41), with the same operations as
// k_limit, so both cells of a face use the same value and no limited-flux
// buffer goes through memory (k_limit still fills one for the water output
// of a single residual).
template <class F>
__global__ void __launch_bounds__(256) k_update(MeshDev m, StateDev s, Ctrl *ctrl, Work w, int stage,
                                                double *rate_out, TurbDev t, int turb)
{
    const int nc = m.nc;
    const double *q = stage == 1 ? s.work : s.q1;
    FOR_ACTIVE_CELLS(m.act, c) {
        const int sid = m.cell_sid[c];
        Ctrl &ct = ctrl[sid];
        if (skip_stage(ct, stage)) continue;
        const double area = m.area[c];
        double mass = 0., mx = 0., my = 0.;
        for (int k = m.offset[c]; k < m.offset[c + 1]; ++k) {
            const int f = m.faces[k];
            const double wt = m.signs[k] * m.length[f] / area;
            double water = w.ws[f].x;
            if (water != 0. && m.bslot[f] < 0) {
                const int donor = water < 0. ? m.neighbour[f] : m.owner[f];
                if (donor >= 0) {
                    const double th = w.theta[donor];
                    if (th != 1.) {
                        const double delta = (th - 1.) * water;
                        water *= th;
                        const double hd = q[donor];
                        if (hd > ct.dry) {
                            mx -= wt * (delta * q[nc + donor] / hd);
                            my -= wt * (delta * q[2 * nc + donor] / hd);
                        }
                    }
                }
            }
            mass -= wt * water;
        }
        const double r0 = mass;
        double r1 = w.rate[nc + c] + mx, r2 = w.rate[2 * nc + c] + my;
        if (turb && t.hkt[sid]) add_rotor_momentum(m, t, sid, c, area, r1, r2);
        if (w.visc.nu && w.visc.nu[sid] > 0.) add_viscosity(m, w.visc, c, area, r1, r2);
        if (!isfinite(r0) || !isfinite(r1) || !isfinite(r2)) raise_status(ct, stage, ST_RATE);
        if (rate_out) { rate_out[c] = r0; rate_out[nc + c] = r1; rate_out[2 * nc + c] = r2; continue; }
        const double dt = ct.trial, dry = ct.dry;
        if (stage == 1) {
            const double h = s.work[c] + dt * r0;
            double hu = s.work[nc + c] + dt * r1, hv = s.work[2 * nc + c] + dt * r2;
            if (h < 0) raise_status(ct, 1, ST_ENDPOINT);
            if (h <= dry) { hu = 0.; hv = 0.; }
            s.q1[c] = h; s.q1[nc + c] = hu; s.q1[2 * nc + c] = hv;
        } else {
            double h = .5 * s.work[c] + .5 * (s.q1[c] + dt * r0);
            double hu = .5 * s.work[nc + c] + .5 * (s.q1[nc + c] + dt * r1);
            double hv = .5 * s.work[2 * nc + c] + .5 * (s.q1[2 * nc + c] + dt * r2);
            if (!isfinite(h) || !isfinite(hu) || !isfinite(hv) || h < 0) raise_status(ct, 2, ST_ENDPOINT);
            if (h <= dry) { hu = 0.; hv = 0.; }
            drag_cell<F>(ct, .5 * dt, h, hu, hv);
            double *qn = ct.cur ? s.q[0] : s.q[1];
            qn[c] = h; qn[nc + c] = hu; qn[2 * nc + c] = hv;
        }
    }
}

// ---------------------------------------------------------------------------
// Control: accept/reject the trial and set the next one (RiverExplicit.advance).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void set_trial(Ctrl &c)
{
    c.trial = fmin(c.hint, c.dt_outer - c.elapsed);
    c.truncated = c.trial < c.hint * (1 - 1e-12);
    c.status1 = 0; c.status2 = 0; c.peak1 = 0ull; c.peak2 = 0ull;
    c.gravf = float(c.grav); c.dryf = float(c.dry); c.trialf = float(c.trial);
    c.roughf = float(c.roughness_value); c.cfl1 = 0;
}

// The active set of the next trial from the control blocks, as runs of
// consecutive active scenarios: warp 0 scans the scenarios 32 at a time
// (ballots for run starts, shuffle scans for the cell and face prefixes).
__device__ void active_rebuild(const Ctrl *ctrl, int nscen, const ActiveDev &a)
{
    if (threadIdx.x >= 32) return;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x;
    int nrun = 0, ncell = 0, nface = 0;
    bool carry = false;                       // the previous chunk's last scenario was active
    for (int base = 0; base < nscen; base += 32) {
        const int i = base + lane;
        const bool on = i < nscen && ctrl[i].active && !ctrl[i].done;
        bool prev = __shfl_up_sync(full, on, 1);
        if (lane == 0) prev = carry;
        const bool first = on && !prev;
        const int cells = on ? a.cell_off[i + 1] - a.cell_off[i] : 0;
        const int faces = on ? a.face_off[i + 1] - a.face_off[i] : 0;
        const unsigned starts = __ballot_sync(full, first);
        int cs = cells, fs = faces;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int x = __shfl_up_sync(full, cs, d), y = __shfl_up_sync(full, fs, d);
            if (lane >= d) { cs += x; fs += y; }
        }
        if (first) {
            const int r = nrun + __popc(starts & ((1u << lane) - 1u));
            const int c0 = ncell + cs - cells, f0 = nface + fs - faces;
            a.cstart[r] = c0; a.cdelta[r] = a.cell_off[i] - c0;
            a.fstart[r] = f0; a.fdelta[r] = a.face_off[i] - f0;
        }
        nrun += __popc(starts);
        ncell += __shfl_sync(full, cs, 31);
        nface += __shfl_sync(full, fs, 31);
        carry = __shfl_sync(full, on, 31);
    }
    if (lane == 0) {
        a.cstart[nrun] = ncell; a.fstart[nrun] = nface;
        a.count[0] = nrun; a.count[1] = ncell; a.count[2] = nface;
    }
}

// Active set of the first trial of an interval (after the host's control upload).
__global__ void k_active_init(const Ctrl *ctrl, int nscen, ActiveDev a) { active_rebuild(ctrl, nscen, a); }

__device__ void control_one(Ctrl &c);

// Substep control of every scenario (one block), then the next trial's active set.
__global__ void k_control(Ctrl *ctrl, int nscen, ActiveDev a)
{
    for (int i = threadIdx.x; i < nscen; i += blockDim.x) control_one(ctrl[i]);
    __syncthreads();
    active_rebuild(ctrl, nscen, a);
}

// A chained scenario has completed an interval: record it and begin the
// next one as the host begins an interval (begin_interval_each), with the
// start time advanced by one interval and the controller's hint carried
// over, so the chain reproduces consecutive intervals bit for bit. The
// accepted state stays in the buffer it is in (the kernels read q[cur]).
__device__ __forceinline__ void chain_next(Ctrl &c)
{
    IvStat &r = c.hist[c.chain_pos];
    r.substeps = c.substeps; r.rejections = c.rejections; r.failed = 0; r.pad = 0;
    r.min_dt = c.min_dt; r.max_dt = c.max_dt; r.cfl_max = c.cfl_max; r.hint = c.hint;
    r.ledger = c.ledger; r.gross = c.gross;
    c.time0 += c.dt_outer;
    c.elapsed = 0.0;
    c.substeps = c.rejections = 0;
    c.min_dt = c.max_dt = c.cfl_max = 0.0;
    c.bflux[0] = c.bflux[1] = c.ledger = 0.0;
    c.bgross[0] = c.bgross[1] = c.gross = 0.0;
    --c.chain_left;
    ++c.chain_pos;
}

__device__ void control_one(Ctrl &c)
{
    if (!c.active || c.done) return;
    // a rotor outside its model's domain ends the scenario (the reference raises)
    if ((c.status1 | c.status2) & ST_TURBINE) { c.failed = 4; c.done = 1; return; }
    if ((c.status1 | c.status2) & ST_FATAL) { c.failed = 5; c.done = 1; return; }
    const double f1 = bits_to_double(c.peak1), f2 = bits_to_double(c.peak2);
    // the reference's frequency peak only sees stages that reached the CFL evaluation
    double peak = 0.;
    bool reject = false;
    if (c.status1 & ST_PRE) reject = true;
    else {
        peak = f1;
        if (c.trial * f1 > c.cfl * (1 + 1e-12) || (c.status1 & ST_ENDPOINT)) reject = true;
        else if (c.status2 & ST_PRE) reject = true;
        else {
            peak = fmax(peak, f2);
            if (c.trial * f2 > c.cfl * (1 + 1e-12) || (c.status2 & ST_ENDPOINT)) reject = true;
        }
    }
    if (reject) {
        c.rejections++;
        c.hint = peak > 0 ? fmin(.5 * c.trial, .98 * c.cfl / peak) : .5 * c.trial;
        if (c.hint < c.floor_ || c.rejections > 100) { c.failed = 1; c.done = 1; return; }
    } else {
        c.cur ^= 1;
        c.elapsed += c.trial;
        c.ledger -= c.trial * (c.one_stage ? c.bflux[0] : .5 * (c.bflux[0] + c.bflux[1]));
        c.gross += c.trial * (c.one_stage ? c.bgross[0] : .5 * (c.bgross[0] + c.bgross[1]));
        c.substeps++;
        if (c.substeps == 1 || c.trial < c.min_dt) c.min_dt = c.trial;
        if (c.trial > c.max_dt) c.max_dt = c.trial;
        if (c.trial * peak > c.cfl_max) c.cfl_max = c.trial * peak;
        const double growth = c.truncated ? c.hint : 2 * c.trial;
        c.hint = peak > 0 ? fmin(growth, .98 * c.cfl / peak) : growth;
        if (c.substeps > c.max_substeps) { c.failed = 2; c.done = 1; return; }
        if (!(c.elapsed < c.dt_outer - 1e-13 * fmax(1., c.dt_outer))) {
            if (c.chain_left <= 0) { c.done = 1; return; }
            chain_next(c);
        }
    }
    set_trial(c);
}

// Limited water flux of the last stage into a caller buffer.
__global__ void k_water_out(MeshDev m, Work w, double *water)
{
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < m.nf; f += gridDim.x * blockDim.x) water[f] = w.lim[f].x;
}

// Make the caller-bound buffer q[0] hold every scenario's accepted state.
// Compensated per-scenario totals of a state: water volume sum(A h) and
// mechanical energy per unit density sum(A (|hu|^2 / (2h) + g h^2 / 2 + g h z))
// (kinetic only where h > dry). Neumaier summation: each thread a strided
// slice, then thread 0 combines the 256 partial pairs in thread order, so the
// result is the same on every run.
__device__ __forceinline__ void neumaier_add(double &sum, double &comp, double v)
{
    const double t = sum + v;
    if (fabs(sum) >= fabs(v)) comp += (sum - t) + v;
    else comp += (v - t) + sum;
    sum = t;
}

__global__ void __launch_bounds__(256) k_totals(MeshDev m, const double *q, const double *z, const double *gd,
                                                double *out)
{
    __shared__ double part[256][4];
    const int sid = blockIdx.x, nc = m.nc;
    const int c0 = m.act.cell_off[sid], c1 = m.act.cell_off[sid + 1];
    const double g = gd[2 * sid], dry = gd[2 * sid + 1];     // the scenario's gravity and dry depth
    double ms = 0., mc = 0., es = 0., ec = 0.;
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        const double h = q[c], a = m.area[c];
        neumaier_add(ms, mc, a * h);
        double e = .5 * g * h * h + g * h * z[c];
        if (h > dry) e += .5 * (q[nc + c] * q[nc + c] + q[2 * nc + c] * q[2 * nc + c]) / h;
        neumaier_add(es, ec, a * e);
    }
    part[threadIdx.x][0] = ms; part[threadIdx.x][1] = mc;
    part[threadIdx.x][2] = es; part[threadIdx.x][3] = ec;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s0 = 0., c0s = 0., s1 = 0., c1s = 0.;
        for (int t = 0; t < (int)blockDim.x; ++t) {
            neumaier_add(s0, c0s, part[t][0]); c0s += part[t][1];
            neumaier_add(s1, c1s, part[t][2]); c1s += part[t][3];
        }
        out[2 * sid] = s0 + c0s;
        out[2 * sid + 1] = s1 + c1s;
    }
}

__global__ void k_commit(MeshDev m, StateDev s, Ctrl *ctrl)
{
    const int nc = m.nc;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        if (!ctrl[m.cell_sid[c]].cur) continue;
        s.q[0][c] = s.q[1][c];
        s.q[0][nc + c] = s.q[1][nc + c];
        s.q[0][2 * nc + c] = s.q[1][2 * nc + c];
    }
}

}  // namespace BRX_NS
