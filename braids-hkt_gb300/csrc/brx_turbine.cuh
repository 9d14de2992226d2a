// Rotor arrays: Thetis actuator-disk sink, coverage gate, diagnostics and the
// balanced-pressure / ambient-stress face terms. FP64 in both arithmetic
// forms (turbine power is integrated in FP64); compiled in the FP64 unit
// without FMA contraction so the operation order follows the reference:
//
//   wet gradients       src/braids_core/sediment/river_turbine_flow.h:13-37
//   rotor sample        river_turbine_thetis.py:263-297 (ThetisRotor.sample)
//   coverage gate       river_turbine_flow.py:82-120 (CoveredRotor._operating_state)
//   cut-in              river_turbine_thetis.py:219-241 (stop_below_cut_in)
//   cell terms          river_turbine_thetis.py:175-216 (cell_terms, lookup)
//   sink                river_turbine_thetis.py:356-362 (ThetisArray.apply)
//   balanced pressure   river_turbine_flow.h:54-82
//   ambient stress      river_hydrokinetic_stress.h:13-35
//
// One CTA per rotor reduces its support and rotor-plane samples (a handful of
// cells), decides the operating state and writes the per-cell sink
// coefficients; the sink itself is formed per support cell, summing the
// rotors that cover the cell in rotor order.
#pragma once
#include "brx_common.cuh"

namespace brx {

enum { TD_ACTIVE = 0, TD_REASON, TD_MARGIN, TD_CLEARANCE, TD_U1, TD_U0, TD_DEPTH, TD_CT, TD_CP, TD_FORCE,
       TD_POWER, TD_REMOVED, TD_LOW, TD_HIGH, TD_ERROR, TD_N = 16 };
enum { TP_D = 0, TP_HUB, TP_BEDCLEAR, TP_SURFCLEAR, TP_TOL, TP_MODE, TP_CT, TP_CP, TP_N };
enum { TM_CONSTANT = 0, TM_SPEED_TABLE = 1, TM_INCIDENT_TABLE = 2, TM_INCIDENT_CURVES = 3 };
enum { TR_COVERED = 0, TR_DEPTH, TR_BED, TR_SURFCLEAR, TR_BEDCLEAR, TR_DRY, TR_REVERSE, TR_NOFLOW, TR_CUTIN };
constexpr double PI_D = 3.14159265358979323846;
constexpr int TURB_THREADS = 128;

// Wet-only least-squares gradients of u, v, eta (fully wet pairs) and of the
// bed (all neighbours, unweighted metric) of one cell:
// g = u_x u_y v_x v_y eta_x eta_y b_x b_y.
__device__ __forceinline__ void hkt_cell_gradient(const MeshDev &m, const TurbDev &t, const double *q,
                                                  const double *z, double dry, int i, double g[8])
{
    const int n = m.nc, na = m.nadj;
    {
        double xx = 0., xy = 0., yy = 0., bx[3] = {0., 0., 0.}, by[3] = {0., 0., 0.}, bz[2] = {0., 0.};
        const bool wet = q[i] > dry;
        for (int s = m.offset[i]; s < m.offset[i + 1]; ++s) {
            const int f = m.faces[s];
            const int j = m.signs[s] < 0 ? m.owner[f] : m.neighbour[f];
            if (j < 0) continue;
            const double dx = t.dxdy[s], dy = t.dxdy[na + s], w = 1. / (dx * dx + dy * dy), dz = z[j] - z[i];
            bz[0] += w * dx * dz; bz[1] += w * dy * dz;
            if (!wet || q[j] <= dry) continue;
            xx += w * dx * dx; xy += w * dx * dy; yy += w * dy * dy;
            const double d[3] = {q[n + j] / q[j] - q[n + i] / q[i], q[2 * n + j] / q[j] - q[2 * n + i] / q[i],
                                 (q[j] + z[j]) - (q[i] + z[i])};
#pragma unroll
            for (int k = 0; k < 3; ++k) { bx[k] += w * dx * d[k]; by[k] += w * dy * d[k]; }
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) g[k] = 0.;
        g[6] = t.inverse[i] * bz[0] + t.inverse[n + i] * bz[1];
        g[7] = t.inverse[n + i] * bz[0] + t.inverse[2 * n + i] * bz[1];
        const double det = xx * yy - xy * xy;
        if (det > 1e-12 * fmax(1., xx * yy))
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                g[2 * k] = (yy * bx[k] - xy * by[k]) / det;
                g[2 * k + 1] = (xx * by[k] - xy * bx[k]) / det;
            }
    }
}

__global__ void __launch_bounds__(256) k_hkt_gradients(MeshDev m, TurbDev t, const double *q, const double *z,
                                                       Ctrl *ctrl, int stage)
{
    const int n = m.nc;
    FOR_ACTIVE_CELLS(m.act, i) {
        const int sid = m.cell_sid[i];
        if (!t.hkt[sid]) continue;
        const Ctrl &ct = ctrl[sid];
        if (stage && skip_stage(ct, stage)) continue;
        double g[8];
        hkt_cell_gradient(m, t, q, z, ct.dry, i, g);
#pragma unroll
        for (int k = 0; k < 8; ++k) t.grad[k * n + i] = g[k];
    }
}

// numpy.interp on one table, zero outside [x0, xlast); the knot slopes
// (y[k+1]-y[k])/(x[k+1]-x[k]) are precomputed with the same division
__device__ __forceinline__ double table_lookup(const double *x, const double *y, const double *slope, int count,
                                               double v)
{
    if (!(v >= x[0]) || v >= x[count - 1]) return 0.;
    int lo = 0, hi = count - 1;           // x[lo] <= v < x[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (x[mid] <= v) lo = mid; else hi = mid;
    }
    if (v == x[lo]) return y[lo];
    return slope[lo] * (v - x[lo]) + y[lo];
}

// Thetis terms of one cell: K, P, incident speed U, Ct, Cp. Returns 0 or an error code.
__device__ int rotor_cell_terms(const TurbDev &t, int r, double depth, double u, double v, double out[5])
{
    const double *p = t.param + (size_t)r * TP_N;
    const double D = p[TP_D];
    const int mode = (int)p[TP_MODE];
    const int *cv = t.curve + 4 * r;
    const double *tx = t.curve_x + cv[0], *ty = t.curve_y + cv[0], *ts = t.curve_slope + cv[0];
    const double *px = t.curve_x + cv[2], *py = t.curve_y + cv[2], *ps = t.curve_slope + cv[2];
    const double speed = hypot(u, v);
    const double area = PI_D * (D * D) / 4;
    if (mode == TM_INCIDENT_TABLE || mode == TM_INCIDENT_CURVES) {
        if (depth < D * (1 - 1e-10)) return 2;
        const double c = PI_D * D / (4 * depth);
        double low = tx[0], high = tx[cv[1] - 1];
        const double smin = low * .5 * (1 + sqrt(1 - c * ty[0]));
        const double smax = high * .5 * (1 + sqrt(1 - c * ty[cv[1] - 1]));
        const bool active = speed >= smin && speed < smax;
        // induction-corrected operating point: bisection on the incident speed
        if (t.flat_thrust[r]) {
            // constant Ct: every lookup inside the table returns ty[0] (slope 0),
            // and 0 at or above the last knot; the square root is hoisted
            const double in_table = .5 * (1 + sqrt(1 - c * ty[0])), beyond = .5 * (1 + sqrt(1 - c * 0.));
            for (int it = 0; it < 44; ++it) {
                const double mid = .5 * (low + high);
                const double local = mid * ((mid >= tx[0] && mid < tx[cv[1] - 1]) ? in_table : beyond);
                if (local < speed) low = mid; else high = mid;
            }
        } else {
            for (int it = 0; it < 44; ++it) {
                const double mid = .5 * (low + high);
                const double ct = table_lookup(tx, ty, ts, cv[1], mid);
                const double local = mid * .5 * (1 + sqrt(1 - c * ct));
                if (local < speed) low = mid; else high = mid;
            }
        }
        const double incident = active ? .5 * (low + high) : speed;
        const double ct = active ? table_lookup(tx, ty, ts, cv[1], incident) : 0.;
        const double cp = active ? table_lookup(px, py, ps, cv[3], incident) : 0.;
        const double alpha = .5 * (1 + sqrt(1 - c * ct));
        out[0] = area * ct / (2 * (alpha * alpha));
        out[1] = .5 * area * cp * (incident * incident * incident);
        out[2] = incident; out[3] = ct; out[4] = cp;
        return 0;
    }
    const double ct = mode == TM_CONSTANT ? p[TP_CT] : table_lookup(tx, ty, ts, cv[1], speed);
    const double radicand = 1 - area * ct / (D * depth);
    if (radicand < 0) return 1;
    const double alpha = .5 * (1 + sqrt(radicand));
    const double incident = speed / alpha;
    const double cp = mode == TM_CONSTANT ? p[TP_CP] : table_lookup(px, py, ps, cv[3], incident);
    out[0] = area * ct / (2 * (alpha * alpha));
    out[1] = .5 * area * cp * (incident * incident * incident);
    out[2] = incident; out[3] = ct; out[4] = cp;
    return 0;
}

template <int N>
__device__ __forceinline__ void block_sum(double (&s)[N][TURB_THREADS], double (&v)[N])
{
    const int tid = threadIdx.x;
#pragma unroll
    for (int k = 0; k < N; ++k) s[k][tid] = v[k];
    __syncthreads();
    for (int w = TURB_THREADS / 2; w > 0; w >>= 1) {
        if (tid < w)
#pragma unroll
            for (int k = 0; k < N; ++k) s[k][tid] += s[k][tid + w];
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = s[k][0];
    __syncthreads();
}

// One rotor per CTA: plane and support samples, the operating state, the sink
// coefficients and the rotor's diagnostics. stage 0 samples a state outside a
// trial (no skip, no status).
__global__ void __launch_bounds__(TURB_THREADS) k_turbine_sample(MeshDev m, TurbDev t, const double *q,
                                                                 const double *z, Ctrl *ctrl, int stage, double *diag)
{
    __shared__ double red[6][TURB_THREADS];
    __shared__ int flags[3];
    const int r = blockIdx.x, tid = threadIdx.x;
    const int sid = t.rotor_sid[r];
    Ctrl &ct = ctrl[sid];
    if (stage && skip_stage(ct, stage)) return;      // uniform over the CTA
    const int n = m.nc, np_ = t.np;
    const double dry = ct.dry;
    const double *p = t.param + (size_t)r * TP_N;
    const double D = p[TP_D], tol = p[TP_TOL];
    const double top = p[TP_HUB] + D / 2, bottom = p[TP_HUB] - D / 2;
    const int mode = (int)p[TP_MODE];
    const int *cv = t.curve + 4 * r;
    if (tid < 3) flags[tid] = 0;
    // rotor plane: lowest surface, highest bed
    double low = INFINITY, high = -INFINITY;
    for (int j = t.plane_offset[r] + tid; j < t.plane_offset[r + 1]; j += TURB_THREADS) {
        const int c = t.plane_cell[j];
        double g[8];
        hkt_cell_gradient(m, t, q, z, dry, c, g);          // the plane cell's own gradients, FP64
        const double eta = q[c] + z[c];
        const double surface = eta + g[4] * t.plane_delta[j] + g[5] * t.plane_delta[np_ + j];
        const double bed = z[c] + g[6] * t.plane_delta[j] + g[7] * t.plane_delta[np_ + j];
        low = fmin(low, fmin(surface, eta)); high = fmax(high, fmax(bed, z[c]));
    }
    red[0][tid] = low; red[1][tid] = high;
    __syncthreads();
    for (int w = TURB_THREADS / 2; w > 0; w >>= 1) {
        if (tid < w) {
            red[0][tid] = fmin(red[0][tid], red[0][tid + w]);
            red[1][tid] = fmax(red[1][tid], red[1][tid + w]);
        }
        __syncthreads();
    }
    low = red[0][0]; high = red[1][0];
    __syncthreads();
    // support: dry cells, weighted speed and depth, cut-in
    double sums[2] = {0., 0.};
    bool support_dry = false, below = false;
    for (int e = t.support_offset[r] + tid; e < t.support_offset[r + 1]; e += TURB_THREADS) {
        const int c = t.support_cell[e];
        const double h = q[c], u = q[n + c] / fmax(h, dry), v = q[2 * n + c] / fmax(h, dry);
        const double speed = hypot(u, v), w = t.support_weight[e];
        if (h <= dry) support_dry = true;
        sums[0] += w * speed; sums[1] += w * h;
        t.kcell[e] = 0.;
        if (mode != TM_CONSTANT) {
            double minimum = t.curve_x[cv[0]];
            if (mode != TM_SPEED_TABLE) minimum = minimum * .5 * (1 + sqrt(1 - PI_D * D * t.curve_y[cv[0]] / (4 * h)));
            if (speed < minimum) below = true;
        }
    }
    if (support_dry) atomicOr(&flags[0], 1);
    if (below) atomicOr(&flags[1], 1);
    block_sum<2>(*reinterpret_cast<double (*)[2][TURB_THREADS]>(red), sums);
    const double u1 = sums[0], depth = sums[1];
    const double margin = low - top, clearance = bottom - high;
    int reason = TR_COVERED;
    if (margin < tol) reason = TR_DEPTH;
    else if (clearance < tol) reason = TR_BED;
    else if (margin + tol < p[TP_SURFCLEAR]) reason = TR_SURFCLEAR;
    else if (clearance + tol < p[TP_BEDCLEAR]) reason = TR_BEDCLEAR;
    else if (flags[0]) reason = TR_DRY;
    bool active = reason == TR_COVERED;
    if (active && u1 <= 1e-10) { active = false; reason = u1 < 0 ? TR_REVERSE : TR_NOFLOW; }
    if (active && mode != TM_CONSTANT && flags[1]) { active = false; reason = TR_CUTIN; }
    double out[6] = {0., 0., 0., 0., 0., 0.};   // F, removed, P, incoming, Ct, Cp
    if (active) {
        int err = 0;
        for (int e = t.support_offset[r] + tid; e < t.support_offset[r + 1]; e += TURB_THREADS) {
            const int c = t.support_cell[e];
            const double h = q[c], u = q[n + c] / fmax(h, dry), v = q[2 * n + c] / fmax(h, dry);
            const double speed = hypot(u, v), w = t.support_weight[e], density = t.support_density[e];
            double k[5];
            const int e2 = rotor_cell_terms(t, r, h, u, v, k);
            if (e2) { err = e2; continue; }
            t.kcell[e] = k[0] * density / m.area[c];
            out[0] += k[0] * density * (speed * speed);
            out[1] += k[0] * density * (speed * speed * speed);
            out[2] += k[1] * density;
            out[3] += w * k[2]; out[4] += w * k[3]; out[5] += w * k[4];
        }
        if (err) atomicMax(&flags[2], err);
        block_sum<6>(red, out);
    }
    if (tid == 0) {
        double *d = diag + (size_t)r * TD_N;
        for (int k = 0; k < TD_N; ++k) d[k] = 0.;
        d[TD_ACTIVE] = active; d[TD_REASON] = reason; d[TD_MARGIN] = margin; d[TD_CLEARANCE] = clearance;
        d[TD_U1] = u1; d[TD_U0] = active ? out[3] : u1; d[TD_DEPTH] = depth; d[TD_LOW] = low; d[TD_HIGH] = high;
        if (active) {
            d[TD_FORCE] = out[0]; d[TD_REMOVED] = out[1]; d[TD_POWER] = out[2];
            d[TD_CT] = out[4]; d[TD_CP] = out[5];
        }
        d[TD_ERROR] = flags[2];
        if (flags[2] && stage) raise_status(ct, stage, ST_TURBINE);
    }
    // actuator sink of the support cells no other rotor's support holds:
    // 0 - k |u| u from this rotor alone (k_turbine_raw's sum with one term);
    // each thread reads the coefficients it wrote itself
    if (stage)
        for (int e = t.support_offset[r] + tid; e < t.support_offset[r + 1]; e += TURB_THREADS) {
            if (!t.single[e]) continue;
            const int c = t.support_cell[e];
            const double h = q[c], u = q[n + c] / fmax(h, dry), v = q[2 * n + c] / fmax(h, dry);
            const double speed = hypot(u, v);
            const double kc = t.kcell[e];
            double rx = 0., ry = 0.;
            rx -= kc * speed * u;
            ry -= kc * speed * v;
            t.raw[c] = rx; t.raw[n + c] = ry;
        }
}

// Actuator sink per support cell: 0 - sum over its rotors of k |u| u.
__global__ void __launch_bounds__(256) k_turbine_raw(MeshDev m, TurbDev t, const double *q, Ctrl *ctrl, int stage)
{
    const int n = m.nc;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < t.nucell; i += gridDim.x * blockDim.x) {
        const int c = t.ucell[i];
        const Ctrl &ct = ctrl[m.cell_sid[c]];
        if (stage && skip_stage(ct, stage)) continue;
        const double h = q[c], u = q[n + c] / fmax(h, ct.dry), v = q[2 * n + c] / fmax(h, ct.dry);
        const double speed = hypot(u, v);
        double rx = 0., ry = 0.;
        for (int k = t.uoff[i]; k < t.uoff[i + 1]; ++k) {
            const double kc = t.kcell[t.uent[k]];
            rx -= kc * speed * u;
            ry -= kc * speed * v;
        }
        t.raw[c] = rx; t.raw[n + c] = ry;
    }
}

// Face terms of scenarios with rotors: symmetric-strain ambient stress and the
// balanced pressure correction.
__global__ void __launch_bounds__(128) k_hkt_faces(MeshDev m, TurbDev t, const double *q, const double *z,
                                                   Ctrl *ctrl, int stage)
{
    const int nf = m.nf, n = m.nc;
    FOR_ACTIVE_FACES(m.act, i) {
        const int sid = m.face_sid[i];
        if (!t.hkt[sid]) continue;
        const Ctrl &ct = ctrl[sid];
        if (stage && skip_stage(ct, stage)) continue;
        const double gravity = ct.grav, dry = ct.dry;
        const int a = m.owner[i], b = m.neighbour[i];
        const double nx = m.normal[i], ny = m.normal[nf + i];
        const double da = m.distance[i], db = b >= 0 ? m.distance[nf + i] : 0.;
        if (t.stress[sid]) {
            double ox = 0., oy = 0.;
            if (b >= 0 && q[a] > dry && q[b] > dry) {
                double h = fmin(q[a], q[b]);
                h = fmin(h, fmax(0., .5 * (q[a] + z[a] + q[b] + z[b]) - fmax(z[a], z[b])));
                const double d = da + db, wo = db / d, wj = da / d;
                const double visc = wo * t.nu[a] + wj * t.nu[b];
                const double dx = t.xy[b] - t.xy[a], dy = t.xy[n + b] - t.xy[n + a];
                const double dn = dx * nx + dy * ny;
                const double du = q[n + b] / q[b] - q[n + a] / q[a], dv = q[2 * n + b] / q[b] - q[2 * n + a] / q[a];
                double ux = wo * t.grad[a] + wj * t.grad[b], uy = wo * t.grad[n + a] + wj * t.grad[n + b];
                double vx = wo * t.grad[2 * n + a] + wj * t.grad[2 * n + b], vy = wo * t.grad[3 * n + a] + wj * t.grad[3 * n + b];
                const double cu = (du - ux * dx - uy * dy) / dn, cvv = (dv - vx * dx - vy * dy) / dn;
                ux += cu * nx; uy += cu * ny; vx += cvv * nx; vy += cvv * ny;
                ox = visc * h * (2. * ux * nx + (uy + vx) * ny);
                oy = visc * h * ((uy + vx) * nx + 2. * vy * ny);
            }
            t.sface[i] = ox; t.sface[nf + i] = oy;
        }
        if (!t.balanced) continue;
        double px = 0., py = 0.;
        if (b >= 0 && q[a] > dry && q[b] > dry) {
            const double *tr = t.trace;
            const double bed = fmax(fmax(z[a], z[b]), fmax(tr[6 * nf + i], tr[7 * nf + i]));
            const double ha = fmax(0., q[a] + z[a] - bed), hb = fmax(0., q[b] + z[b] - bed);
            const double hl = fmax(0., tr[i] - bed), hr = fmax(0., tr[nf + i] - bed);
            const double h = .5 * (hl + hr);
            const double old = .25 * gravity * (hl * hl + hr * hr);
            double po = old, pn = old;
            if (tr[8 * nf + i] != 0.) po += .5 * gravity * (ha * ha - hl * hl);
            if (tr[9 * nf + i] != 0.) pn += .5 * gravity * (hb * hb - hr * hr);
            // zero outside the fully wet, small-surface-jump, consistent-pressure scope
            if (!(fmin(fmin(ha, hb), fmin(hl, hr)) <= dry) && !(fabs(hr - hl) > .005 * h) &&
                !(fabs(po - pn) > 128. * EPS * fmax(1., fmax(fabs(po), fabs(pn))))) {
                const double d = da + db, wa = db / d, wb = da / d;
                const double sx = wa * t.mdisp[i] + wb * t.mdisp[2 * nf + i];
                const double sy = wa * t.mdisp[nf + i] + wb * t.mdisp[3 * nf + i];
                double pressure = .5 * gravity * (wa * ha * ha + wb * hb * hb);
                pressure += gravity * sx * (wa * ha * t.grad[4 * n + a] + wb * hb * t.grad[4 * n + b]);
                pressure += gravity * sy * (wa * ha * t.grad[5 * n + a] + wb * hb * t.grad[5 * n + b]);
                pressure += da * db / d * ((t.raw[a] - t.raw[b]) * nx + (t.raw[n + a] - t.raw[n + b]) * ny);
                double delta = .5 * (po + pn) - pressure;
                const double speed = sqrt(gravity * h), theta = fmin(1., fmax(tr[4 * nf + i], tr[5 * nf + i]) / speed);
                delta -= .5 * (1. - theta) * speed * (2. * hl * hr / (hl + hr)) * (tr[3 * nf + i] - tr[2 * nf + i]);
                px = delta * nx; py = delta * ny;
            }
        }
        t.pface[i] = px; t.pface[nf + i] = py;
    }
}

}  // namespace brx
