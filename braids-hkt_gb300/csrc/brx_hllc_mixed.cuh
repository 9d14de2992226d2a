// Mixed-precision form of the HLLC / MUSCL-Hancock method (included by
// brx_mixed.cu inside namespace brx_mx; FP32 arithmetic with FMA contraction
// and fast division / square root).
//
// Same algorithm as the FP64 kernels of brx_hllc.cuh (the reference's
// hllc.h:15-155, hllc_turbines.h:13-31, hllc.py:76-118), rearranged as the
// mixed f-wave form is:
//   * cell values enter as the FP32 primitive records of the opening drag
//     (depth, velocities, wet bit, FP64 stage as an FP32 pair); differences
//     of stages are formed from the pairs, bed differences come from tables
//     rebuilt from the FP64 bed (hcdb), so every reconstructed face value is
//     an FP32 quantity on the depth scale, relative to the owner's bed;
//   * the predicted cell record keeps the predicted stage as an increment
//     over the cell's stage, the predicted conserved state for the exterior
//     owner is formed in FP64 from the FP64 depth;
//   * the momentum flux minus the gathering cell's reference pressure is
//     evaluated as 1/2 g (h - e)(h + e) - (1/2 g h*) h*, with the HLLC flux's
//     hydrostatic term (1/2 g h*) h* rounded identically, and the star-state
//     increments h* - h of the contact solution as h (s_m - u) / (s - s_m):
//     a surface at rest gives exactly zero water and momentum fluxes;
//   * depth and mass stay FP64 (FP64 signed weights; the donor factor
//     carries the FP32 outflow margin of the f-wave form); momentum sums,
//     the rotor acoustic correction and drag run in FP32.
// The rotor arrays of the HLLC owner (actuator sink, acoustic correction)
// are supported; its ambient stress is not (the method switch refuses it).

// Predicted record of one cell (48 bytes).
struct __align__(16) HCellF {
    float de;          // predicted stage - stage of the opening state
    float u, v;        // predicted velocities
    float g[8];        // limited gradients of eta, u, v, b (x, y)
    float pad;
};
static_assert(sizeof(HCellF) == 48, "mixed HLLC record is 48 bytes");

// codes of the other side of an HLLC incidence entry (as brx_hllc.cuh)
constexpr int HX_WALL = -1, HX_OPEN = -2;
__device__ __forceinline__ int hx_face(int x) { return x >= 0 ? x : ~x; }

// hllc.h:52-72 in FP32: HLLC flux of one rotated face, HLLE where a side is
// dry or the contact state is inadmissible. pl, pr: the hydrostatic flux
// terms (1/2 g hl) hl and (1/2 g hr) hr, rounded separately, which the
// caller subtracts again from the gathering cells' pressure.
__device__ __forceinline__ void hllc_riemann_f(float hl, float ul, float vl, float hr, float ur, float vr, float g,
                                               float dry, float pl, float pr, float out[3], float &speed)
{
    const float cl = sqrtf(g * hl), cr = sqrtf(g * hr);
    float sl = fminf(ul - cl, ur - cr), sr = fmaxf(ul + cl, ur + cr);
    if (hl <= dry) sl = ur - 2.f * cr;
    if (hr <= dry) sr = ul + 2.f * cl;
    speed = fmaxf(fabsf(sl), fabsf(sr));
    const float fl0 = hl * ul, fl1 = __fadd_rn(__fmul_rn(__fmul_rn(hl, ul), ul), pl), fl2 = hl * ul * vl;
    const float fr0 = hr * ur, fr1 = __fadd_rn(__fmul_rn(__fmul_rn(hr, ur), ur), pr), fr2 = hr * ur * vr;
    if (hl <= dry && hr <= dry) { out[0] = out[1] = out[2] = 0.f; speed = 0.f; return; }
    if (sl >= 0.f) { out[0] = fl0; out[1] = fl1; out[2] = fl2; return; }
    if (sr <= 0.f) { out[0] = fr0; out[1] = fr1; out[2] = fr2; return; }
    const float a = hl * (sl - ul), b = hr * (sr - ur), den = a - b;
    // (hr - hl)(hr + hl), not hr^2 - hl^2: a contracted hr * hr - hl * hl
    // leaves the rounding residual of hl^2 for equal depths, a spurious
    // contact speed and water flux on a surface at rest
    const float sm = fabsf(den) > 1e-30f ? __fdividef(.5f * g * ((hr - hl) * (hr + hl)) + a * ul - b * ur, den) : 0.f;
    if (hl > dry && hr > dry && sl < sm && sm < sr) {
        // star depth minus side depth, h (s_m - u) / (s - s_m): zero for a state at rest
        const float dl = __fdividef(hl * (sm - ul), sl - sm), dr = __fdividef(hr * (sm - ur), sr - sm);
        const float hs = sm >= 0.f ? hl + dl : hr + dr;
        if (hs >= 0.f && isfinite(hs)) {
            if (sm >= 0.f) {
                out[0] = fl0 + sl * dl;
                out[1] = __fadd_rn(fl1, __fmul_rn(sl, hs * sm - hl * ul));
                out[2] = fl2 + sl * (dl * vl);
            } else {
                out[0] = fr0 + sr * dr;
                out[1] = __fadd_rn(fr1, __fmul_rn(sr, hs * sm - hr * ur));
                out[2] = fr2 + sr * (dr * vr);
            }
            return;
        }
    }
    const float w = sr - sl, ss = sl * sr;
    out[0] = __fdividef(sr * fl0 - sl * fr0 + ss * (hr - hl), w);
    out[1] = __fdividef(sr * fl1 - sl * fr1 + ss * (hr * ur - hl * ul), w);
    out[2] = __fdividef(sr * fl2 - sl * fr2 + ss * (hr * vr - hl * vl), w);
}

// ---------------------------------------------------------------------------
// Cells: limited MUSCL gradients over the neighbours and mirrored walls (open
// faces take no part), the half-step predictor; the predicted conserved
// state in q1 (FP64) for the exterior owner at t + dt/2.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) km_hllc_cells(MeshDev m, StateDev s, Ctrl *ctrl, MixedGeo g, HCellF *rec)
{
    const int nc = m.nc;
    const MxPrim *P = reinterpret_cast<const MxPrim *>(g.prim[0]);
    FOR_ACTIVE_CELLS(m.act, c) {
        Ctrl &ct = ctrl[m.cell_sid[c]];
        if (!ct.active || ct.done) continue;
        const MxPrim pc = P[c];
        const bool wet = pc.wet != 0;
        const float grav = ct.gravf, dt = ct.trialf;
        // values relative to the cell: stage and bed differences, velocities absolute
        const float cv[4] = {0.f, pc.u, pc.v, 0.f};
        float bx[4] = {0.f, 0.f, 0.f, 0.f}, by[4] = {0.f, 0.f, 0.f, 0.f}, lo[4], hi[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) lo[k] = hi[k] = cv[k];
        const int k0 = m.offset[c], deg = m.offset[c + 1] - k0;
        for (int e = 0; e < deg; ++e) {
            const int2 en = g.hent[k0 + e];
            if (en.y == HX_OPEN) continue;
            const float4 gm = g.hgeo[k0 + e];
            float o[4];
            if (en.y >= 0) {
                const MxPrim pj = P[en.y];
                o[0] = (pj.ehi - pc.ehi) + (pj.elo - pc.elo);
                o[1] = pj.u; o[2] = pj.v;
                o[3] = g.hcdb[k0 + e];
                // a dry neighbour whose bed rises above the surface contributes the surface
                if (!pj.wet && o[3] >= pc.h) o[0] = 0.f;
            } else {
                const float2 nn = g.fnorm[hx_face(en.x)];
                const float un = pc.u * nn.x + pc.v * nn.y;
                o[0] = 0.f; o[3] = 0.f;
                o[1] = pc.u - 2.f * un * nn.x; o[2] = pc.v - 2.f * un * nn.y;
            }
            if (gm.x == 0.f && gm.y == 0.f) continue;        // coincident centres
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float d = o[k] - cv[k];
                bx[k] += d * gm.x; by[k] += d * gm.y;
                lo[k] = fminf(lo[k], o[k]); hi[k] = fmaxf(hi[k], o[k]);
            }
        }
        const float4 inv = g.hinv[c];
        HCellF r;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float gx = inv.x * bx[k] + inv.y * by[k], gy = inv.y * bx[k] + inv.z * by[k];
            float lim = 1.f;
            for (int e = 0; e < deg; ++e) {
                const float4 gm = g.hgeo[k0 + e];
                const float d = gx * gm.z + gy * gm.w;
                if (d > 0.f) lim = fminf(lim, __fdividef(hi[k] - cv[k], d));
                else if (d < 0.f) lim = fminf(lim, __fdividef(lo[k] - cv[k], d));
            }
            r.g[2 * k] = lim * gx; r.g[2 * k + 1] = lim * gy;
        }
        if (!wet)
#pragma unroll
            for (int k = 0; k < 6; ++k) r.g[k] = 0.f;
        const float hc = pc.h, u = pc.u, w = pc.v;
        float de = -.5f * dt * (u * (r.g[0] - r.g[6]) + w * (r.g[1] - r.g[7]) + hc * (r.g[2] + r.g[5]));
        float uh = u - .5f * dt * (u * r.g[2] + w * r.g[3] + grav * r.g[0]);
        float wh = w - .5f * dt * (u * r.g[4] + w * r.g[5] + grav * r.g[1]);
        if (hc + de < 0.f) { de = 0.f; uh = u; wh = w; }
        if (!wet) { de = 0.f; uh = 0.f; wh = 0.f; }
        r.de = de; r.u = uh; r.v = wh; r.pad = 0.f;
        rec[c] = r;
        const double hh = fmax(0., s.work[c] + f2d(de));
        s.q1[c] = hh; s.q1[nc + c] = hh * f2d(uh); s.q1[2 * nc + c] = hh * f2d(wh);
        if (!isfinite(de) || !isfinite(uh) || !isfinite(wh)) atomic_max_nonneg(&ct.peak1, INFINITY);
    }
}

// Half-step rotor source on the predicted state (hllc.h:74-77): the HLLC
// owner's rotor momentum (the actuator sink) at the start state.
__global__ void __launch_bounds__(256) km_hllc_predict(MeshDev m, StateDev s, TurbDev t, Ctrl *ctrl, HCellF *rec)
{
    const int nc = m.nc;
    FOR_ACTIVE_CELLS(m.act, c) {
        const int sid = m.cell_sid[c];
        if (!t.hkt[sid]) continue;
        const Ctrl &ct = ctrl[sid];
        if (!ct.active || ct.done || !t.foot[c]) continue;
        const double hh = s.q1[c];
        const double mu = s.q1[nc + c] + .5 * ct.trial * t.raw[c], mv = s.q1[2 * nc + c] + .5 * ct.trial * t.raw[nc + c];
        s.q1[nc + c] = mu; s.q1[2 * nc + c] = mv;
        const bool wet = !le_threshold(hh, ct.dry);
        const float hf = d2f(hh);
        rec[c].u = wet ? d2f(mu) / hf : 0.f;
        rec[c].v = wet ? d2f(mv) / hf : 0.f;
    }
}

// ---------------------------------------------------------------------------
// Faces: exterior flux on open faces (less the cell-reference pressure),
// HLLC with hydrostatic reconstruction elsewhere, the rotor acoustic
// correction on fully wet interior faces of rotor scenarios.
// Writes (water, speed) and (owner-side momentum x, y, neighbour-side x, y).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) km_hllc_faces(MeshDev m, StateDev s, BoundaryDev b, Ctrl *ctrl, Work w,
                                                     MixedGeo g, TurbDev t, int turb, const HCellF *rec)
{
    const MxPrim *P = reinterpret_cast<const MxPrim *>(g.prim[0]);
    float2 *ws = reinterpret_cast<float2 *>(w.ws);
    float4 *gf = reinterpret_cast<float4 *>(w.gf);
    FOR_ACTIVE_FACES(m.act, f) {
        const int sid = m.face_sid[f];
        const Ctrl &ct = ctrl[sid];
        if (!ct.active || ct.done || (ct.status1 & ST_PRE)) continue;
        const float grav = ct.gravf, dry = ct.dryf, half_g = .5f * grav;
        const int l = m.owner[f], r = m.neighbour[f];
        const float2 nn = g.fnorm[f];
        const float nx = nn.x, ny = nn.y;
        const HCellF rl = rec[l];
        const int slot = m.bslot[f];
        if (slot >= 0) {
            // the exterior owner's flux and speed at the predicted state (FP64, few faces)
            const size_t ns = b.nslot;
            const double gd = ct.grav, h = s.q1[l];
            const double e0 = b.flux[slot], e1 = b.flux[ns + slot], e2 = b.flux[2 * ns + slot];
            const double m1 = e1 - .5 * gd * h * h * m.normal[f], m2 = e2 - .5 * gd * h * h * m.normal[m.nf + f];
            const double hb = b.trace[slot];
            const double ub = hb > ct.dry ? (b.trace[ns + slot] * m.normal[f] + b.trace[2 * ns + slot] * m.normal[m.nf + f]) / hb
                                          : 0.;
            const double speed = fmax(fabs(double(rl.u) * m.normal[f] + double(rl.v) * m.normal[m.nf + f]) + sqrt(gd * h),
                                      fabs(ub) + sqrt(gd * fmax(hb, 0.)));
            ws[f] = make_float2(float(e0), float(speed));
            gf[f] = make_float4(float(m1), float(m2), float(m1), float(m2));
            continue;
        }
        const MxPrim pl = P[l];
        const float4 dsp = g.fdisp[f];
        // face values above the owner's bed: stage (depth-scale), velocities, bed
        float L[4], R[4];
        const float incl = rl.de + rl.g[0] * dsp.x + rl.g[1] * dsp.y;
        L[0] = pl.h + incl;
        L[1] = rl.u + rl.g[2] * dsp.x + rl.g[3] * dsp.y;
        L[2] = rl.v + rl.g[4] * dsp.x + rl.g[5] * dsp.y;
        L[3] = rl.g[6] * dsp.x + rl.g[7] * dsp.y;
        const float pel = pl.h + rl.de;          // predicted stage of the owner above its bed
        HCellF rr;
        float per = pel, rbase = pl.h, rbed = 0.f;
        if (r >= 0) {
            rr = rec[r];
            const MxPrim pr = P[r];
            rbase = pl.h + ((pr.ehi - pl.ehi) + (pr.elo - pl.elo));     // neighbour stage above the owner's bed
            rbed = g.fdb[f];
            R[0] = rbase + (rr.de + rr.g[0] * dsp.z + rr.g[1] * dsp.w);
            R[1] = rr.u + rr.g[2] * dsp.z + rr.g[3] * dsp.w;
            R[2] = rr.v + rr.g[4] * dsp.z + rr.g[5] * dsp.w;
            R[3] = rbed + (rr.g[6] * dsp.z + rr.g[7] * dsp.w);
            per = rbase + rr.de;
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) R[k] = L[k];
        }
        const bool ldry = pel - 0.f <= dry, rdry = r >= 0 && per - rbed <= dry;
        const bool acoustic = turb && t.hkt[sid] && r >= 0 && !ldry && !rdry;
        float corr = 0.f;
        bool apply = false;
        if (acoustic) {
            const float bed = fmaxf(L[3], R[3]), hl = L[0] - bed, hr = R[0] - bed, hm = .5f * (hl + hr);
            if (!(fminf(hl, hr) <= dry || fabsf(hr - hl) > .005f * hm)) {
                const float c = sqrtf(grav * hm);
                const float th = fminf(1.f, __fdividef(fmaxf(hypotf(L[1], L[2]), hypotf(R[1], R[2])), c));
                const float du = (R[1] - L[1]) * nx + (R[2] - L[2]) * ny;
                corr = .5f * (1.f - th) * c * __fdividef(2.f * hl * hr, hl + hr) * du;
                apply = true;
            }
        }
        if (ldry || rdry) { L[3] = 0.f; R[3] = r < 0 ? L[3] : rbed; }
        if (ldry) { L[0] = L[3]; L[1] = L[2] = 0.f; }
        if (rdry) { R[0] = R[3]; R[1] = R[2] = 0.f; }
        if (r < 0) { const float un = R[1] * nx + R[2] * ny; R[1] -= 2.f * un * nx; R[2] -= 2.f * un * ny; }
        const float top = fmaxf(L[3], R[3]), hl = fmaxf(0.f, L[0] - L[3]), hr = fmaxf(0.f, R[0] - R[3]);
        const float hls = fmaxf(0.f, L[0] - top), hrs = fmaxf(0.f, R[0] - top);
        // hydrostatic flux terms of the reconstructed states, rounded once and used twice
        const float ps_l = __fmul_rn(__fmul_rn(half_g, hls), hls), ps_r = __fmul_rn(__fmul_rn(half_g, hrs), hrs);
        float out[3], speed;
        hllc_riemann_f(hls, L[1] * nx + L[2] * ny, -L[1] * ny + L[2] * nx, hrs, R[1] * nx + R[2] * ny,
                       -R[1] * ny + R[2] * nx, grav, dry, ps_l, ps_r, out, speed);
        const float el = fmaxf(0.f, pel - L[3]), er = r < 0 ? el : fmaxf(0.f, per - R[3]);
        // 1/2 g (h^2 - h*^2 - e^2) of each gathering cell: the pressure of its
        // face state above its reference, less the hydrostatic flux term
        const float p_l = __fsub_rn(__fmul_rn(half_g, __fmul_rn(hl - el, hl + el)), ps_l);
        const float p_r = __fsub_rn(__fmul_rn(half_g, __fmul_rn(hr - er, hr + er)), ps_r);
        const float fl = __fadd_rn(out[1], p_l), fr = __fadd_rn(out[1], p_r);
        float l1 = fl * nx - out[2] * ny, l2 = fl * ny + out[2] * nx;
        float r1 = fr * nx - out[2] * ny, r2 = fr * ny + out[2] * nx;
        if (apply) { l1 += corr * nx; r1 += corr * nx; l2 += corr * ny; r2 += corr * ny; }
        ws[f] = make_float2(r < 0 ? 0.f : out[0], speed);
        gf[f] = make_float4(l1, l2, r1, r2);
    }
}

// ---------------------------------------------------------------------------
// Budget: donor factor (prescribed exterior debits reserved first, -1 marks
// an unfunded one; FP32 sums, FP64 factor with the f-wave form's margin) and
// the CFL frequency sum(len * speed) / area.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) km_hllc_budget(MeshDev m, StateDev s, Ctrl *ctrl, Work w, MixedGeo g)
{
    const int nc = m.nc;
    const float2 *ws = reinterpret_cast<const float2 *>(w.ws);
    float *theta32 = reinterpret_cast<float *>(w.theta);
    const int stride = gridDim.x * blockDim.x;
    const int na = m.act.count[1];
    for (int first = blockIdx.x * blockDim.x; first < na; first += stride) {   // warp-uniform trip count
        const int c = first + (int)threadIdx.x < na ? active_cell(m.act, first + threadIdx.x) : nc;
        bool have = false;
        float fr = 0.f;
        int sid = 0;
        if (c < nc) {
            sid = m.cell_sid[c];
            Ctrl &ct = ctrl[sid];
            if (ct.active && !ct.done && !(ct.status1 & ST_PRE)) {
                float outgoing = 0.f, prescribed = 0.f, sum = 0.f;
                for (int k = m.offset[c]; k < m.offset[c + 1]; ++k) {
                    const int2 en = g.hent[k];
                    const float wk = g.hw4[k];                 // signed length / area
                    const float2 v = ws[hx_face(en.x)];
                    const float debit = fmaxf(0.f, wk * v.x);
                    if (en.y == HX_OPEN) prescribed += debit; else outgoing += debit;
                    sum += v.y * fabsf(wk);
                }
                fr = sum;
                float theta = 1.f;
                if (ct.trialf * (outgoing + prescribed) >= 0.999f * d2f(s.work[c])) {
                    const double available = s.work[c] / ct.trial;
                    const double pres = double(prescribed), pres_hi = pres * (1. + DONOR_MARGIN);
                    const double out_hi = double(outgoing) * (1. + DONOR_MARGIN);
                    if (pres > available) theta = -1.f;
                    else if (outgoing > 0.f && out_hi >= available - pres_hi)
                        theta = float(fmax(0., fmin(1., (available - pres_hi) / out_hi) * (1. - 32. * EPS)));
                }
                theta32[c] = theta;
                if (isnan(fr)) raise_status(ct, 1, ST_FREQ);
                else have = true;
            }
        }
        warp_max_peak_f(&ctrl[0].peak1, sizeof(Ctrl), sid, have, fr);
    }
}

// ---------------------------------------------------------------------------
// Update: each face's donor-limited flux (formed identically by both of its
// cells), the conservative update (FP64 mass with FP64 weights, FP32
// momentum sums), the rotor sink at the predicted state, drag(dt/2); the
// result goes to the inactive state buffer.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) km_hllc_update(MeshDev m, StateDev s, Ctrl *ctrl, Work w, MixedGeo g,
                                                      TurbDev t, int turb)
{
    const int nc = m.nc;
    const float2 *ws = reinterpret_cast<const float2 *>(w.ws);
    const float4 *gf = reinterpret_cast<const float4 *>(w.gf);
    const float *theta32 = reinterpret_cast<const float *>(w.theta);
    const MxPrim *P = reinterpret_cast<const MxPrim *>(g.prim[0]);
    FOR_ACTIVE_CELLS(m.act, c) {
        const int sid = m.cell_sid[c];
        Ctrl &ct = ctrl[sid];
        if (!ct.active || ct.done || stage1_failed(ct)) continue;
        double mass = 0.;
        float m1 = 0.f, m2 = 0.f;
        bool bad = false;
        for (int k = m.offset[c]; k < m.offset[c + 1]; ++k) {
            const int2 en = g.hent[k];
            const int f = hx_face(en.x);
            const bool own = en.x >= 0;
            const float wk = g.hw4[k];
            const float2 v = ws[f];
            const float4 fm = gf[f];
            const float wf = v.x;
            double water = f2d(wf);
            float l1 = own ? fm.x : fm.z, l2 = own ? fm.y : fm.w;
            if (wf != 0.f) {
                // the donor is the owner for outward (positive) water, else the neighbour
                const int donor = (wf > 0.f) == own ? c : en.y;
                if (en.y == HX_OPEN) {
                    if (donor == c && theta32[c] < 0.f) bad = true;
                } else if (donor >= 0) {
                    const float th = theta32[donor];
                    if (!(th >= 1.f)) {
                        const float factor = fmaxf(0.f, th), delta = (factor - 1.f) * wf;
                        water = f2d(wf) * f2d(factor);            // exact product
                        const MxPrim pd = P[donor];
                        if (pd.wet) { l1 += delta * pd.u; l2 += delta * pd.v; }
                    }
                }
            }
            mass -= g.hw8[k] * water;
            m1 -= wk * l1;
            m2 -= wk * l2;
        }
        const double dt = ct.trial;
        double v0 = s.work[c] + dt * mass;
        double v1 = s.work[nc + c] + dt * f2d(m1), v2 = s.work[2 * nc + c] + dt * f2d(m2);
        if (le_threshold(v0, ct.dry)) { v1 = 0.; v2 = 0.; }
        bad = bad || !finite64(v0) || !finite64(v1) || !finite64(v2) || lt_zero(v0);
        if (turb && t.hkt[sid] && t.foot[c]) {
            v1 += dt * t.raw[c]; v2 += dt * t.raw[nc + c];
            bad = bad || !finite64(v1) || !finite64(v2);
        }
        if (bad) { raise_status(ct, 1, ST_ENDPOINT); continue; }
        drag_f(ct, .5f * ct.trialf, v0, v1, v2);
        double *out = ct.cur ? s.q[0] : s.q[1];
        out[c] = v0; out[nc + c] = v1; out[2 * nc + c] = v2;
    }
}
