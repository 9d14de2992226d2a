// HLLC / MUSCL-Hancock option of the river step (FP64, reference operation order).
//
// One substep = drag(dt/2) -> cells (limited MUSCL gradients + half-step
// predictor) -> [rotor source on the start state -> predictor source] ->
// exterior boundary on the predicted state at t + dt/2 -> faces (HLLC / HLLE
// with hydrostatic reconstruction, rotor acoustic correction fused) ->
// budget (donor factors, CFL frequency) -> [rotor source on the predicted
// state] -> update (donor limiter fused, rotor source, drag(dt/2)) ->
// control. The same Ctrl clock as the f-wave step, one stage per substep.
//
// Restated from (file:line in the reference):
//   cells      src/braids_core/hydraulics/hllc.h:15-50 (hllc_reconstruct)
//   predictor  hllc.h:74-77 (hllc_predict_source)
//   flux       hllc.h:52-72 (hllc_flux)
//   faces      hllc.h:80-114 (hllc_faces), hllc_turbines.h:13-31
//   budget     hllc.h:116-132 (hllc_budget)
//   update     hllc.h:134-155 (hllc_limit, hllc_update)
//   step       src/braids_core/hydraulics/hllc.py:76-118 (_spatial_step)
//   controller hllc.py:131-149 (advance)
#pragma once
#include "brx_common.cuh"

namespace brx {

// Per CSR entry of the HLLC incidence (each cell's faces in ascending face
// number, hllc.py:29-34): face (bitwise NOT when the cell is the face's
// neighbour), the other cell or a code, and the stencil geometry.
enum : int { HE_WALL = -1, HE_OPEN = -2 };

struct HllcDev {
    const int2 *ent;             // (nadj) x: face or ~face (neighbour side); y: other cell, HE_WALL, HE_OPEN
    const double4_32a *geo;      // (nadj) offset to the neighbour / wall mirror (x, y); face midpoint - centroid (z, w)
    const double *inverse;       // (3, nc) least-squares inverse (i11, i12, i22)
};

// Predicted primitives and limited gradients of one cell (96 bytes):
// p = (eta, u, v, b) at t + dt/2; g = (d/dx, d/dy) of eta, u, v, b.
struct __align__(32) HCell {
    double p[4];
    double g[8];
};
static_assert(sizeof(HCell) == 96, "HLLC cell record is three 32-byte sectors");

__device__ __forceinline__ int hent_face(int x) { return x >= 0 ? x : ~x; }

// hllc.h:52-72: HLLC flux of one rotated face; HLLE where a side is dry or
// the contact state is inadmissible.
__device__ __forceinline__ void hllc_riemann(double hl, double ul, double vl, double hr, double ur, double vr,
                                             double g, double dry, double out[3], double &speed)
{
    const double cl = sqrt(g * hl), cr = sqrt(g * hr);
    double sl = fmin(ul - cl, ur - cr), sr = fmax(ul + cl, ur + cr);
    if (hl <= dry) sl = ur - 2. * cr;
    if (hr <= dry) sr = ul + 2. * cl;
    speed = fmax(fabs(sl), fabs(sr));
    const double fl0 = hl * ul, fl1 = hl * ul * ul + .5 * g * hl * hl, fl2 = hl * ul * vl;
    const double fr0 = hr * ur, fr1 = hr * ur * ur + .5 * g * hr * hr, fr2 = hr * ur * vr;
    if (hl <= dry && hr <= dry) { out[0] = out[1] = out[2] = 0.; speed = 0.; return; }
    if (sl >= 0.) { out[0] = fl0; out[1] = fl1; out[2] = fl2; return; }
    if (sr <= 0.) { out[0] = fr0; out[1] = fr1; out[2] = fr2; return; }
    const double a = hl * (sl - ul), b = hr * (sr - ur), den = a - b;
    const double sm = fabs(den) > 1e-30 ? (.5 * g * (hr * hr - hl * hl) + a * ul - b * ur) / den : 0.;
    if (hl > dry && hr > dry && sl < sm && sm < sr) {
        const double hs = sm >= 0. ? a / (sl - sm) : b / (sr - sm);
        if (hs >= 0. && isfinite(hs)) {
            if (sm >= 0.) {
                out[0] = fl0 + sl * (hs - hl); out[1] = fl1 + sl * (hs * sm - hl * ul);
                out[2] = fl2 + sl * (hs * vl - hl * vl);
            } else {
                out[0] = fr0 + sr * (hs - hr); out[1] = fr1 + sr * (hs * sm - hr * ur);
                out[2] = fr2 + sr * (hs * vr - hr * vr);
            }
            return;
        }
    }
    const double w = sr - sl, ss = sl * sr;
    out[0] = (sr * fl0 - sl * fr0 + ss * (hr - hl)) / w;
    out[1] = (sr * fl1 - sl * fr1 + ss * (hr * ur - hl * ul)) / w;
    out[2] = (sr * fl2 - sl * fr2 + ss * (hr * vr - hl * vl)) / w;
}

// ---------------------------------------------------------------------------
// Cells: limited MUSCL gradients of (eta, u, v, b) over the neighbours and
// mirrored walls (open faces take no part), then the half-step predictor.
// A nonfinite prediction makes the scenario's CFL frequency infinite, as
// the reference's budget does for a flagged cell.
// ---------------------------------------------------------------------------
template <int MAXF>
__global__ void __launch_bounds__(128) k_hllc_cells(MeshDev m, StateDev s, HllcDev h, HCell *rec, Ctrl *ctrl)
{
    const int nc = m.nc, nf = m.nf;
    FOR_ACTIVE_CELLS(m.act, c) {
        const int sid = m.cell_sid[c];
        Ctrl &ct = ctrl[sid];
        if (!ct.active || ct.done) continue;
        const double *q = s.work, *z = s.z;
        const double dry = ct.dry, g = ct.grav, dt = ct.trial;
        const double h0 = q[c];
        double cv[4] = {h0 + z[c], h0 > dry ? q[nc + c] / h0 : 0., h0 > dry ? q[2 * nc + c] / h0 : 0., z[c]};
        double bx[4] = {0., 0., 0., 0.}, by[4] = {0., 0., 0., 0.}, lo[4], hi[4];
        double mx[MAXF], my[MAXF];
#pragma unroll
        for (int k = 0; k < 4; ++k) lo[k] = hi[k] = cv[k];
        const int k0 = m.offset[c], deg = m.offset[c + 1] - k0;
#pragma unroll
        for (int e = 0; e < MAXF; ++e) {
            if (e >= deg) continue;
            const int2 en = h.ent[k0 + e];
            const double4_32a gm = h.geo[k0 + e];
            mx[e] = gm.z; my[e] = gm.w;
            if (en.y == HE_OPEN) continue;
            double o[4];
            if (en.y >= 0) {
                const int j = en.y;
                const double hj = q[j];
                o[0] = hj + z[j]; o[1] = hj > dry ? q[nc + j] / hj : 0.; o[2] = hj > dry ? q[2 * nc + j] / hj : 0.;
                o[3] = z[j];
                if (o[0] - o[3] <= dry && o[3] >= cv[0]) o[0] = cv[0];
            } else {
                const int f = hent_face(en.x);
                const double nx = m.normal[f], ny = m.normal[nf + f];
#pragma unroll
                for (int k = 0; k < 4; ++k) o[k] = cv[k];
                const double un = cv[1] * nx + cv[2] * ny;
                o[1] -= 2. * un * nx; o[2] -= 2. * un * ny;
            }
            const double dx = gm.x, dy = gm.y, d2 = dx * dx + dy * dy;
            if (d2 <= 0.) continue;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const double d = o[k] - cv[k];
                bx[k] += d * dx / d2; by[k] += d * dy / d2;
                lo[k] = fmin(lo[k], o[k]); hi[k] = fmax(hi[k], o[k]);
            }
        }
        const double i0 = h.inverse[c], i1 = h.inverse[nc + c], i2 = h.inverse[2 * nc + c];
        HCell r;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const double gx = i0 * bx[k] + i1 * by[k], gy = i1 * bx[k] + i2 * by[k];
            double lim = 1.;
#pragma unroll
            for (int e = 0; e < MAXF; ++e) {
                if (e >= deg) continue;
                const double d = gx * mx[e] + gy * my[e];
                if (d > 0.) lim = fmin(lim, (hi[k] - cv[k]) / d);
                else if (d < 0.) lim = fmin(lim, (lo[k] - cv[k]) / d);
            }
            r.g[2 * k] = lim * gx; r.g[2 * k + 1] = lim * gy;
        }
        const double hc = cv[0] - cv[3];
        if (hc <= dry)
#pragma unroll
            for (int k = 0; k < 6; ++k) r.g[k] = 0.;
        const double u = cv[1], w = cv[2];
        double eta = cv[0] - .5 * dt * (u * (r.g[0] - r.g[6]) + w * (r.g[1] - r.g[7]) + hc * (r.g[2] + r.g[5]));
        double uh = u - .5 * dt * (u * r.g[2] + w * r.g[3] + g * r.g[0]);
        double wh = w - .5 * dt * (u * r.g[4] + w * r.g[5] + g * r.g[1]);
        if (eta < cv[3]) { eta = cv[0]; uh = u; wh = w; }
        if (hc <= dry) { eta = cv[0]; uh = 0.; wh = 0.; }
        r.p[0] = eta; r.p[1] = uh; r.p[2] = wh; r.p[3] = cv[3];
        rec[c] = r;
        const double hh = fmax(0., eta - cv[3]);
        s.q1[c] = hh; s.q1[nc + c] = hh * uh; s.q1[2 * nc + c] = hh * wh;
        if (!isfinite(eta) || !isfinite(uh) || !isfinite(wh)) atomic_max_nonneg(&ct.peak1, INFINITY);
    }
}

// Half-step rotor source on the predicted state of scenarios with rotors
// (hllc.h:74-77); the rate is the HLLC owner's rotor momentum at the start
// state (ambient stress, actuator sink).
__global__ void __launch_bounds__(256) k_hllc_predict(MeshDev m, StateDev s, TurbDev t, HCell *rec, Ctrl *ctrl)
{
    const int nc = m.nc;
    FOR_ACTIVE_CELLS(m.act, c) {
        const int sid = m.cell_sid[c];
        if (!t.hkt[sid]) continue;
        const Ctrl &ct = ctrl[sid];
        if (!ct.active || ct.done) continue;
        double r1 = 0., r2 = 0.;
        add_rotor_momentum(m, t, sid, c, m.area[c], r1, r2, false);
        const double hh = s.q1[c];
        const double mu = s.q1[nc + c] + .5 * ct.trial * r1, mv = s.q1[2 * nc + c] + .5 * ct.trial * r2;
        s.q1[nc + c] = mu; s.q1[2 * nc + c] = mv;
        rec[c].p[1] = hh > ct.dry ? mu / hh : 0.;
        rec[c].p[2] = hh > ct.dry ? mv / hh : 0.;
    }
}

// Face value of predicted primitive k of a cell at a face (centroid offset dx, dy).
__device__ __forceinline__ double hllc_face_value(const HCell &r, int k, double dx, double dy)
{
    return r.p[k] + r.g[2 * k] * dx + r.g[2 * k + 1] * dy;
}

// ---------------------------------------------------------------------------
// Faces: exterior flux on open faces (less the cell-reference pressure),
// HLLC with hydrostatic reconstruction elsewhere, the rotor acoustic
// correction on fully wet interior faces of rotor scenarios. Writes
// (water, speed) and (owner-side momentum x, y, neighbour-side x, y).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_hllc_faces(MeshDev m, BoundaryDev b, const HCell *rec, Work w, TurbDev t,
                                                    int turb, Ctrl *ctrl)
{
    const int nf = m.nf;
    FOR_ACTIVE_FACES(m.act, f) {
        const int sid = m.face_sid[f];
        const Ctrl &ct = ctrl[sid];
        if (!ct.active || ct.done || (ct.status1 & ST_PRE)) continue;
        const double g = ct.grav, dry = ct.dry;
        const int l = m.owner[f], r = m.neighbour[f];
        const double nx = m.normal[f], ny = m.normal[nf + f];
        const HCell rl = rec[l];
        const int slot = m.bslot[f];
        if (slot >= 0) {
            const size_t ns = b.nslot;
            const double h = fmax(0., rl.p[0] - rl.p[3]);
            const double e0 = b.flux[slot], e1 = b.flux[ns + slot], e2 = b.flux[2 * ns + slot];
            const double m1 = e1 - .5 * g * h * h * nx, m2 = e2 - .5 * g * h * h * ny;
            const double hb = b.trace[slot];
            const double ub = hb > dry ? (b.trace[ns + slot] * nx + b.trace[2 * ns + slot] * ny) / hb : 0.;
            const double speed = fmax(fabs(rl.p[1] * nx + rl.p[2] * ny) + sqrt(g * h), fabs(ub) + sqrt(g * fmax(hb, 0.)));
            w.ws[f] = make_double2(e0, speed);
            w.gf[f] = make_double4_32a(m1, m2, m1, m2);
            continue;
        }
        const double dxl = m.disp[f], dyl = m.disp[2 * (size_t)nf + f];
        double L[4], R[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) L[k] = hllc_face_value(rl, k, dxl, dyl);
        HCell rr;
        if (r >= 0) {
            rr = rec[r];
            const double dxr = m.disp[nf + f], dyr = m.disp[3 * (size_t)nf + f];
#pragma unroll
            for (int k = 0; k < 4; ++k) R[k] = hllc_face_value(rr, k, dxr, dyr);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) R[k] = L[k];
        }
        const bool ldry = rl.p[0] - rl.p[3] <= dry, rdry = r >= 0 && rr.p[0] - rr.p[3] <= dry;
        // rotor acoustic correction inputs: the unmodified fully wet face states
        const bool acoustic = turb && t.hkt[sid] && r >= 0 && !ldry && !rdry;
        double corr = 0.;
        bool apply = false;
        if (acoustic) {
            const double bed = fmax(L[3], R[3]), hl = L[0] - bed, hr = R[0] - bed, hm = .5 * (hl + hr);
            if (!(fmin(hl, hr) <= dry || fabs(hr - hl) > .005 * hm)) {
                const double c = sqrt(g * hm), th = fmin(1., fmax(hypot(L[1], L[2]), hypot(R[1], R[2])) / c);
                const double du = (R[1] - L[1]) * nx + (R[2] - L[2]) * ny;
                corr = .5 * (1. - th) * c * (2. * hl * hr / (hl + hr)) * du;
                apply = true;
            }
        }
        if (ldry || rdry) { L[3] = rl.p[3]; R[3] = r < 0 ? L[3] : rr.p[3]; }
        if (ldry) { L[0] = L[3]; L[1] = L[2] = 0.; }
        if (rdry) { R[0] = R[3]; R[1] = R[2] = 0.; }
        if (r < 0) { const double un = R[1] * nx + R[2] * ny; R[1] -= 2. * un * nx; R[2] -= 2. * un * ny; }
        const double top = fmax(L[3], R[3]), hl = fmax(0., L[0] - L[3]), hr = fmax(0., R[0] - R[3]);
        const double hls = fmax(0., L[0] - top), hrs = fmax(0., R[0] - top);
        double out[3], speed;
        hllc_riemann(hls, L[1] * nx + L[2] * ny, -L[1] * ny + L[2] * nx, hrs, R[1] * nx + R[2] * ny,
                     -R[1] * ny + R[2] * nx, g, dry, out, speed);
        const double el = fmax(0., rl.p[0] - L[3]), er = r < 0 ? el : fmax(0., rr.p[0] - R[3]);
        const double pl = .5 * g * (hl * hl - hls * hls - el * el), pr = .5 * g * (hr * hr - hrs * hrs - er * er);
        double l1 = (out[1] + pl) * nx - out[2] * ny, l2 = (out[1] + pl) * ny + out[2] * nx;
        double r1 = (out[1] + pr) * nx - out[2] * ny, r2 = (out[1] + pr) * ny + out[2] * nx;
        if (apply) { l1 += corr * nx; r1 += corr * nx; l2 += corr * ny; r2 += corr * ny; }
        w.ws[f] = make_double2(r < 0 ? 0. : out[0], speed);
        w.gf[f] = make_double4_32a(l1, l2, r1, r2);
    }
}

// ---------------------------------------------------------------------------
// Budget: donor factor (prescribed exterior debits reserved first; -1 marks
// an unfunded one) and the CFL frequency sum(len * speed) / area.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_hllc_budget(MeshDev m, StateDev s, HllcDev h, Work w, Ctrl *ctrl)
{
    const int nc = m.nc;
    const int stride = gridDim.x * blockDim.x;
    const int na = m.act.count[1];
    for (int first = blockIdx.x * blockDim.x; first < na; first += stride) {   // warp-uniform trip count
        const int c = first + (int)threadIdx.x < na ? active_cell(m.act, first + threadIdx.x) : nc;
        bool have = false;
        double fr = 0.;
        int sid = 0;
        if (c < nc) {
            sid = m.cell_sid[c];
            Ctrl &ct = ctrl[sid];
            if (ct.active && !ct.done && !(ct.status1 & ST_PRE)) {
                double outgoing = 0., prescribed = 0., sum = 0.;
                for (int k = m.offset[c]; k < m.offset[c + 1]; ++k) {
                    const int2 en = h.ent[k];
                    const int f = hent_face(en.x), sign = en.x >= 0 ? 1 : -1;
                    const double2 ws = w.ws[f];
                    const double len = m.length[f];
                    const double debit = fmax(0., sign * ws.x) * len;
                    if (en.y == HE_OPEN) prescribed += debit; else outgoing += debit;
                    sum += ws.y * len;
                }
                const double area = m.area[c];
                fr = sum / area;
                double theta = 1.;
                const double available = s.work[c] * area / ct.trial;
                if (prescribed > available) theta = -1.;
                else if (outgoing > 0. && outgoing >= available - prescribed)
                    theta = fmin(1., (available - prescribed) / outgoing) * (1. - 32. * EPS);
                w.theta[c] = theta;
                if (isnan(fr)) raise_status(ct, 1, ST_FREQ);
                else have = true;
            }
        }
        warp_max_peak(&ctrl[0].peak1, sizeof(Ctrl), sid, have, fr);
    }
}

// ---------------------------------------------------------------------------
// Update: each face's donor-limited flux (formed identically by both of its
// cells), the conservative update, the rotor source at the predicted state,
// drag(dt/2); the result goes to the inactive state buffer.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_hllc_update(MeshDev m, StateDev s, HllcDev h, Work w, TurbDev t, int turb,
                                                     Ctrl *ctrl)
{
    const int nc = m.nc;
    FOR_ACTIVE_CELLS(m.act, c) {
        const int sid = m.cell_sid[c];
        Ctrl &ct = ctrl[sid];
        if (!ct.active || ct.done || stage1_failed(ct)) continue;
        const double *q = s.work;
        const double dt = ct.trial, dry = ct.dry, area = m.area[c];
        double v0 = q[c], v1 = q[nc + c], v2 = q[2 * nc + c];
        bool bad = false;
        for (int k = m.offset[c]; k < m.offset[c + 1]; ++k) {
            const int2 en = h.ent[k];
            const int f = hent_face(en.x), sign = en.x >= 0 ? 1 : -1;
            const double2 ws = w.ws[f];
            const double4_32a gf = w.gf[f];
            double water = ws.x, l1 = gf.x, l2 = gf.y, r1 = gf.z, r2 = gf.w;
            if (water != 0.) {
                const int donor = water < 0. ? m.neighbour[f] : m.owner[f];
                if (donor >= 0) {
                    const double th = w.theta[donor];
                    if (en.y == HE_OPEN) bad = bad || th < 0.;
                    else if (!(th >= 1.)) {
                        const double factor = fmax(0., th), delta = (factor - 1.) * water;
                        water = water * factor;
                        const double hd = q[donor];
                        if (hd > dry) {
                            const double d1 = delta * q[nc + donor] / hd, d2 = delta * q[2 * nc + donor] / hd;
                            l1 += d1; r1 += d1; l2 += d2; r2 += d2;
                        }
                    }
                }
            }
            const double a = dt * sign * m.length[f] / area;
            v0 -= a * water;
            v1 -= a * (sign > 0 ? l1 : r1);
            v2 -= a * (sign > 0 ? l2 : r2);
        }
        if (v0 <= dry) { v1 = 0.; v2 = 0.; }
        bad = bad || !isfinite(v0) || !isfinite(v1) || !isfinite(v2) || v0 < 0.;
        if (turb && t.hkt[sid]) {
            double r1 = 0., r2 = 0.;
            add_rotor_momentum(m, t, sid, c, area, r1, r2, false);
            v1 += dt * r1; v2 += dt * r2;
            bad = bad || !isfinite(v1) || !isfinite(v2);
        }
        if (bad) { raise_status(ct, 1, ST_ENDPOINT); continue; }
        drag_cell<double>(ct, .5 * dt, v0, v1, v2);
        double *out = ct.cur ? s.q[0] : s.q[1];
        out[c] = v0; out[nc + c] = v1; out[2 * nc + c] = v2;
    }
}

}  // namespace brx
