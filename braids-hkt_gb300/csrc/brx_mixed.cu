// Mixed-precision form of the river step.
//
// Same algorithm as the FP64 form (the reference's reconstruction, hydrostatic
// reconstruction at the common face bed, augmented f-wave, flux assembly,
// donor limiter and SSPRK(2,2) update), rearranged so that the face and cell
// sweeps run in FP32:
//
//   * the cell record keeps depth h and bed b in FP64 and everything else
//     (velocities, limited gradients) in FP32, 64 bytes;
//   * every reconstructed face value is an FP32 increment relative to its
//     cell (surface d_eta, bed d_b, velocity); only differences of the FP64
//     cell depths and beds are formed in FP64, once per neighbour;
//   * the hydrostatic part of the momentum flux minus the gathering cell's
//     own pressure is evaluated in perturbation form,
//        1/2 g [ (hL - h)(hL + h) + (h + raw) d_b ],
//     which cancels exactly for a surface at rest in FP32 arithmetic, so the
//     lake-at-rest balance does not rest on FP64;
//   * the Riemann solve, limiter, projection and drag run in FP32;
//   * mass bookkeeping (limited water flux, donor factors, the depth update)
//     uses FP64 signed weights s*len/area, so mass telescopes exactly.
//
// This unit is compiled with FMA contraction and fast FP32 division / sqrt.
#include "brx_launch.h"
#include "brx_fwave.cuh"

namespace brx_mx {
using namespace brx;

constexpr float FEPS = 1.1920928955078125e-07f;

// 64-byte cell record of the mixed form.
struct __align__(16) MxRec {
    double h, b;
    float u, v;
    float gx[4], gy[4];          // eta, u, v, b
    int flags;                   // bit0 flatten, bit1 active
    float pad;
};
static_assert(sizeof(MxRec) == 64, "mixed record is half a line");

struct __align__(16) MxLim {
    double water;                // limited mass flux (FP64: both cells use this value)
    float cx, cy;                // momentum correction
};

__device__ __forceinline__ bool feasible_f(float x, float y, int count, const float *ax, const float *ay,
                                           const float *bb)
{
    for (int i = 0; i < count; ++i) {
        const float tol = 2.e-14f + 16.f * FEPS * (fabsf(ax[i] * x) + fabsf(ay[i] * y) + fabsf(bb[i]));
        if (ax[i] * x + ay[i] * y > bb[i] + tol) return false;
    }
    return true;
}

// Nearest feasible point of the bound polygon, as the directional projection
// limiter: the best feasible candidate among single-constraint projections and
// pairwise vertices. The polygon contains the origin (all bounds are >= 0) and
// is convex, so its nearest point is unique and lies on a constraint the
// unlimited gradient violates: only violated constraints seed candidates.
__device__ __noinline__ void project_f(float &x, float &y, int count, const float *ax, const float *ay,
                                       const float *bb)
{
    const float rx = x, ry = y;
    if (feasible_f(rx, ry, count, ax, ay, bb)) return;
    float bx = 0.f, by = 0.f, best = rx * rx + ry * ry;
    for (int i = 0; i < count; ++i) {
        const float dot = ax[i] * rx + ay[i] * ry - bb[i];
        if (dot <= 0.f) continue;                 // satisfied: cannot be the only active constraint
        float cx = rx - dot * ax[i], cy = ry - dot * ay[i];
        float d = (cx - rx) * (cx - rx) + (cy - ry) * (cy - ry);
        if (d < best && feasible_f(cx, cy, count, ax, ay, bb)) { bx = cx; by = cy; best = d; }
        for (int j = 0; j < count; ++j) {
            if (j == i) continue;
            const float det = ax[i] * ay[j] - ay[i] * ax[j];
            if (fabsf(det) < 1.e-12f) continue;
            cx = (bb[i] * ay[j] - ay[i] * bb[j]) / det;
            cy = (ax[i] * bb[j] - bb[i] * ax[j]) / det;
            d = (cx - rx) * (cx - rx) + (cy - ry) * (cy - ry);
            if (d < best && feasible_f(cx, cy, count, ax, ay, bb)) { bx = cx; by = cy; best = d; }
        }
    }
    x = bx; y = by;
}

// ---------------------------------------------------------------------------
// Cells
// ---------------------------------------------------------------------------
template <int MAXF>
__global__ void __launch_bounds__(128) km_cells(MeshDev m, StateDev s, Ctrl *ctrl, Work w, MixedGeo g, int stage)
{
    const int nc = m.nc;
    MxRec *rec = reinterpret_cast<MxRec *>(w.rec);
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        Ctrl &ct = ctrl[m.cell_sid[c]];
        if (skip_stage(ct, stage)) continue;
        const double *q = stage == 1 ? s.work : s.q1;
        const double dry = ct.dry;
        const float grav = float(ct.grav);
        const double h = q[c], hu = q[nc + c], hv = q[2 * nc + c], zc = s.z[c];
        if (h < 0.0 || !isfinite(h) || !isfinite(zc) || !isfinite(hu) || !isfinite(hv))
            raise_status(ct, stage, ST_SPATIAL);
        const bool wet = h > dry;
        const float u = wet ? float(hu) / float(h) : 0.f, v = wet ? float(hv) / float(h) : 0.f;
        // bounds of eta and b relative to the cell (centre = 0), of u and v absolute
        float lo[4] = {0.f, u, v, 0.f}, hi[4] = {0.f, u, v, 0.f};
        float bx[4] = {0.f, 0.f, 0.f, 0.f}, by[4] = {0.f, 0.f, 0.f, 0.f};
        const int k0 = m.offset[c], k1 = m.offset[c + 1];
        bool active = wet;
        for (int k = k0; k < k1; ++k) {
            const int2 id = g.cidx[k];
            const int n = id.x;
            if (n < 0) { if (id.y & 1) active = true; continue; }
            const double hn = q[n], zn = s.z[n];
            const bool wetn = hn > dry;
            if (wetn) active = true;
            const double ddb = zn - zc;
            float d[4];
            d[0] = float((hn - h) + ddb);
            d[1] = (wetn ? float(q[nc + n]) / float(hn) : 0.f) - u;
            d[2] = (wetn ? float(q[2 * nc + n]) / float(hn) : 0.f) - v;
            d[3] = float(ddb);
            // a dry neighbour whose bed rises above the wet surface contributes the surface
            if (wet && !wetn && ddb >= h) d[0] = 0.f;
            const float4 ge = g.cent[k];
            const float wt = g.cwt[k];
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                bx[p] += wt * ge.x * d[p];
                by[p] += wt * ge.y * d[p];
                const float val = (p == 1 || p == 2) ? d[p] + (p == 1 ? u : v) : d[p];
                lo[p] = fminf(lo[p], val); hi[p] = fmaxf(hi[p], val);
            }
        }
        float gx[4] = {0.f, 0.f, 0.f, 0.f}, gy[4] = {0.f, 0.f, 0.f, 0.f};
        const float4 inv = g.cinv[c];
        if (active && (inv.x != 0.f || inv.y != 0.f || inv.z != 0.f)) {
            if (wet)
                for (int k = k0; k < k1; ++k) {
                    if (!(g.cidx[k].y & 4)) continue;
                    const float2 nn = g.fnorm[m.faces[k]];
                    const float un = u * nn.x + v * nn.y;
                    const float mx = u - 2.f * un * nn.x, my = v - 2.f * un * nn.y;
                    lo[1] = fminf(lo[1], mx); hi[1] = fmaxf(hi[1], mx);
                    lo[2] = fminf(lo[2], my); hi[2] = fmaxf(hi[2], my);
                }
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                gx[p] = inv.x * bx[p] + inv.y * by[p];
                gy[p] = inv.y * bx[p] + inv.z * by[p];
            }
            const float hf = float(h);
            const float sq = wet ? sqrtf(grav * hf) : 0.f;
            const float bedtol = 64.f * FEPS * fmaxf(1.f, fabsf(float(zc)));
            float theta1 = 1.f, theta2 = 1.f;
            // pass 1: Barth factors of u, v and feasibility of the eta / bed gradients
            bool feas0 = true, feas3 = true;
            for (int k = k0; k < k1; ++k) {
                const int2 id = g.cidx[k];
                const float4 ge = g.cent[k];
                const float rx = ge.z, ry = ge.w;
                if ((id.y & 2) && wet) {
                    // an open stage outlet with a subcritical wet owner keeps its bed slope
                    const float2 nn = g.fnorm[m.faces[k]];
                    if (fabsf(u * nn.x + v * nn.y) < sq && fabsf(gx[3] * rx + gy[3] * ry) > bedtol) continue;
                }
#pragma unroll
                for (int p = 1; p < 3; ++p) {
                    const float dd = gx[p] * rx + gy[p] * ry;
                    const float ctr = p == 1 ? u : v;
                    if (fabsf(dd) <= 64.f * FEPS * fmaxf(1.f, fmaxf(fabsf(ctr), fmaxf(fabsf(lo[p]), fabsf(hi[p])))))
                        continue;
                    float &th = p == 1 ? theta1 : theta2;
                    if (dd > 0.f) th = fminf(th, (hi[p] - ctr) / dd);
                    if (dd < 0.f) th = fminf(th, (lo[p] - ctr) / dd);
                }
                const float len = sqrtf(rx * rx + ry * ry);
                if (len <= 0.f) continue;
                const float inv_len = 1.f / len, ux = rx * inv_len, uy = ry * inv_len;
                const float e0 = ux * gx[0] + uy * gy[0];
                const float t0 = 2.e-14f + 16.f * FEPS * (fabsf(ux * gx[0]) + fabsf(uy * gy[0]));
                if (e0 > fmaxf(0.f, hi[0]) * inv_len + t0 + 16.f * FEPS * fmaxf(0.f, hi[0]) * inv_len ||
                    -e0 > fmaxf(0.f, -lo[0]) * inv_len + t0 + 16.f * FEPS * fmaxf(0.f, -lo[0]) * inv_len) feas0 = false;
                if (id.y & 4) continue;
                const float e3 = ux * gx[3] + uy * gy[3];
                const float t3 = 2.e-14f + 16.f * FEPS * (fabsf(ux * gx[3]) + fabsf(uy * gy[3]));
                if (e3 > fmaxf(0.f, hi[3]) * inv_len + t3 + 16.f * FEPS * fmaxf(0.f, hi[3]) * inv_len ||
                    -e3 > fmaxf(0.f, -lo[3]) * inv_len + t3 + 16.f * FEPS * fmaxf(0.f, -lo[3]) * inv_len) feas3 = false;
            }
            float px0 = gx[0], py0 = gy[0], px3 = gx[3], py3 = gy[3];
            if (!feas0 || !feas3) {
                // pass 2: the bound polygons, only for a gradient that leaves them
                float ax0[2 * MAXF], ay0[2 * MAXF], b0[2 * MAXF];
                float ax3[2 * MAXF], ay3[2 * MAXF], b3[2 * MAXF];
                int n0 = 0, n3 = 0;
                for (int k = k0; k < k1; ++k) {
                    const int2 id = g.cidx[k];
                    const float4 ge = g.cent[k];
                    const float rx = ge.z, ry = ge.w;
                    if ((id.y & 2) && wet) {
                        const float2 nn = g.fnorm[m.faces[k]];
                        if (fabsf(u * nn.x + v * nn.y) < sq && fabsf(gx[3] * rx + gy[3] * ry) > bedtol) continue;
                    }
                    const float len = sqrtf(rx * rx + ry * ry);
                    if (len <= 0.f) continue;
                    const float inv_len = 1.f / len, ux = rx * inv_len, uy = ry * inv_len;
                    ax0[n0] = ux; ay0[n0] = uy; b0[n0++] = fmaxf(0.f, hi[0]) * inv_len;
                    ax0[n0] = -ux; ay0[n0] = -uy; b0[n0++] = fmaxf(0.f, -lo[0]) * inv_len;
                    if (id.y & 4) continue;   // walls do not bound the bed
                    ax3[n3] = ux; ay3[n3] = uy; b3[n3++] = fmaxf(0.f, hi[3]) * inv_len;
                    ax3[n3] = -ux; ay3[n3] = -uy; b3[n3++] = fmaxf(0.f, -lo[3]) * inv_len;
                }
                if (!feas0) project_f(px0, py0, n0, ax0, ay0, b0);
                if (!feas3) project_f(px3, py3, n3, ax3, ay3, b3);
            }
            gx[1] *= fmaxf(0.f, theta1); gy[1] *= fmaxf(0.f, theta1);
            gx[2] *= fmaxf(0.f, theta2); gy[2] *= fmaxf(0.f, theta2);
            gx[0] = px0; gy[0] = py0; gx[3] = px3; gy[3] = py3;
        }
        bool flatten = !wet;
        if (!flatten) {
            const float hf = float(h);
            for (int k = k0; k < k1; ++k) {
                const float4 ge = g.cent[k];
                const float de = gx[0] * ge.z + gy[0] * ge.w, db = gx[3] * ge.z + gy[3] * ge.w;
                if (hf + (de - db) <= float(dry) || fabsf(db) >= hf) { flatten = true; break; }
            }
        }
        MxRec r;
        r.h = h; r.b = zc; r.u = u; r.v = v;
#pragma unroll
        for (int p = 0; p < 4; ++p) { r.gx[p] = gx[p]; r.gy[p] = gy[p]; }
        r.flags = (flatten ? 1 : 0) | (active ? 2 : 0);
        r.pad = 0.f;
        rec[c] = r;
    }
}

// ---------------------------------------------------------------------------
// Faces
// ---------------------------------------------------------------------------
struct MxSide {
    float h, hu, hv;   // trace depth and momenta
    float raw;         // raw reconstructed depth (>= 0)
    float db;          // face bed - cell bed
    float dh;          // trace depth - cell depth
    float de;          // face surface - cell surface
};

__device__ __forceinline__ MxSide mx_side(const MxRec &r, float rx, float ry, float dry, bool dryface, unsigned &bad)
{
    float de = r.gx[0] * rx + r.gy[0] * ry;
    float uu = r.u + (r.gx[1] * rx + r.gy[1] * ry);
    float vv = r.v + (r.gx[2] * rx + r.gy[2] * ry);
    float db = r.gx[3] * rx + r.gy[3] * ry;
    const float hf = float(r.h);
    const bool constant = r.flags & 1;
    if (constant) {
        de = 0.f; uu = r.u; vv = r.v;
        if (hf <= dry) db = 0.f;
    }
    if (!isfinite(de) || !isfinite(uu) || !isfinite(vv) || !isfinite(db)) bad = 1;
    MxSide o = {0.f, 0.f, 0.f, 0.f, db, -hf, de};
    if (dryface) return o;
    const float rel = de - db;
    const float raw = fmaxf(hf + rel, 0.f);
    o.raw = raw;
    float depth = raw;
    if (r.h <= double(dry) || (constant && raw <= dry)) depth = 0.f;
    o.h = depth; o.hu = depth * uu; o.hv = depth * vv;
    o.dh = (depth == hf + rel) ? rel : depth - hf;
    return o;
}

// (hL - h)(hL + h) + (h + raw) d_b with both products rounded separately:
// for a surface at rest dh = -d_b and raw = hL, so the two products are
// exact negatives of each other and the sum is exactly zero. An FMA would
// round only one of them and leave a residual.
__device__ __forceinline__ float hydro_perturbation(float dh, float hL, float h, float raw, float db)
{
    return __fadd_rn(__fmul_rn(dh, hL + h), __fmul_rn(h + raw, db));
}

__global__ void __launch_bounds__(128) km_faces(MeshDev m, StateDev s, BoundaryDev b, Ctrl *ctrl, Work w,
                                                MixedGeo g, int stage)
{
    const int nf = m.nf, nc = m.nc;
    const MxRec *rec = reinterpret_cast<const MxRec *>(w.rec);
    float2 *ws = reinterpret_cast<float2 *>(w.ws);
    float4 *gf = reinterpret_cast<float4 *>(w.gf);
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
        Ctrl &ct = ctrl[m.face_sid[f]];
        if (skip_stage(ct, stage)) continue;
        const float dry = float(ct.dry), grav = float(ct.grav);
        const float half_g = 0.5f * grav;
        const int c = m.owner[f], n = m.neighbour[f];
        const float2 nn = g.fnorm[f];
        const float nx = nn.x, ny = nn.y;
        const MxRec rc = rec[c];
        const float hc = float(rc.h);
        const int slot = m.bslot[f];
        if (slot >= 0) {
            // open face: the exterior owner's flux and the owner/exterior CFL speed (FP64, few faces)
            const double *q = stage == 1 ? s.work : s.q1;
            const double dn = m.normal[f], dm = m.normal[nf + f], gd = ct.grav, dd = ct.dry;
            const double fl0 = b.flux[slot], fl1 = b.flux[(size_t)b.nslot + slot], fl2 = b.flux[2 * (size_t)b.nslot + slot];
            const double hb = b.trace[slot], hq = q[c];
            const double pc = .5 * gd * hq * hq;
            const double a = hq > dd ? fabs((q[nc + c] * dn + q[2 * nc + c] * dm) / hq) + sqrt(gd * hq) : 0.;
            const double bb = hb > dd ? fabs((b.trace[(size_t)b.nslot + slot] * dn + b.trace[2 * (size_t)b.nslot + slot] * dm) / hb) +
                                            sqrt(gd * hb) : 0.;
            ws[f] = make_float2(float(fl0), float(fmax(a, bb)));
            gf[f] = make_float4(float(fl1 - pc * dn), float(fl2 - pc * dm), 0.f, 0.f);
            continue;
        }
        MxRec rn;
        if (n >= 0) rn = rec[n];
        int kind = n >= 0 ? 1 : 2;
        if (rc.h <= double(dry) && (n < 0 || rn.h <= double(dry))) kind = 0;
        unsigned bad = 0;
        const float4 dsp = g.fdisp[f];
        const MxSide L = mx_side(rc, dsp.x, dsp.y, dry, kind == 0, bad);
        MxSide R = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const float hn = n >= 0 ? float(rn.h) : 0.f;
        if (n >= 0) R = mx_side(rn, dsp.z, dsp.w, dry, kind == 0, bad);
        float water = 0.f, speed = 0.f;
        float gl1 = 0.f, gl2 = 0.f, gr1 = 0.f, gr2 = 0.f;
        if (kind != 0) {
            float hL = L.h, xL = L.hu, yL = L.hv;
            float hR = R.h, xR = R.hu, yR = R.hv;
            // beds relative to the owner's bed
            // surfaces and beds relative to the owner's surface / bed; both sides
            // share the owner's FP32 depth as base, so a surface at rest gives
            // bit-identical hydrostatic depths on the two sides
            const float bLr = L.db;
            float bRr = n >= 0 ? float(rn.b - rc.b) + R.db : L.db;
            const float sL = hc + L.de;
            float sR = n >= 0 ? hc + (float((rn.h + rn.b) - (rc.h + rc.b)) + R.de) : sL;
            if (kind == 2) { hR = hL; xR = xL; yR = yL; bRr = bLr; sR = sL; }
            float xRr = xR, yRr = yR;
            if (kind == 2) {
                const float dot = xL * nx + yL * ny;
                xRr = xL - 2.f * dot * nx; yRr = yL - 2.f * dot * ny;
            }
            const float unL = xL * nx + yL * ny, utL = xL * (-ny) + yL * nx;
            const float unR = xRr * nx + yRr * ny, utR = xRr * (-ny) + yRr * nx;
            float loc[8] = {hL, unL, utL, 0.f, hR, unR, utR, 0.f};
            if (kind == 1) {
                const float top = fmaxf(bLr, bRr);
                const float bc = float(rc.b);
                const float tol = 16.f * FEPS * fmaxf(dry, fmaxf(fabsf(bc + top), fmaxf(fabsf(bc + hL + bLr), fabsf(bc + hR + bRr))));
                float hl = hL > 0.f ? fmaxf(0.f, sL - top) : 0.f, hr = hR > 0.f ? fmaxf(0.f, sR - top) : 0.f;
                if (hl <= dry + tol) hl = 0.f;
                if (hr <= dry + tol) hr = 0.f;
                loc[0] = hl; loc[4] = hr;
                loc[1] = hL > dry ? unL * (hl / hL) : 0.f;
                loc[2] = hL > dry ? utL * (hl / hL) : 0.f;
                loc[5] = hR > dry ? unR * (hr / hR) : 0.f;
                loc[6] = hR > dry ? utR * (hr / hR) : 0.f;
            }
            bool closed = false;
            if (kind == 1 && !(fminf(hc, hn) > dry)) {
                // wet/dry face: the shared surface from distance-weighted cell stages (FP64, rare)
                const float2 di = g.fdist[f];
                const double dc = di.x, dn = di.y;
                double shared;
                if (dc + dn > 0.0)
                    shared = (dn * (rc.b + rc.h) + dc * (rn.b + rn.h)) / (dc + dn) - fmax(rc.b, rn.b);
                else
                    shared = 0.5 * ((rc.b + rc.h) + (rn.b + rn.h)) - fmax(rc.b, rn.b);
                closed = shared <= double(dry);
                if (closed) {
                    bool opens = false;
                    if (hL > dry && hR <= dry && unL / hL > 0.f) {
                        const RType<float> t = riemann_type<float>(hL, hL, unL / hL, -unL / hL, dry, grav);
                        opens = t.hm > hL + dry && t.hm + bLr > bRr + dry;
                    } else if (hR > dry && hL <= dry && -unR / hR > 0.f) {
                        const RType<float> t = riemann_type<float>(hR, hR, -unR / hR, unR / hR, dry, grav);
                        opens = t.hm > hR + dry && t.hm + bRr > bLr + dry;
                    }
                    closed = !opens;
                }
            }
            FWaveOut<float> fwo;
            const int fst = fwave<float>(loc, grav, dry, fwo);
            if (fst) bad = 1;
            // dynamic (non-hydrostatic) part of the left/right fluxes in the face frame
            float dl0 = 0.f, dl1 = 0.f, dl2 = 0.f, dr0 = 0.f, dr1 = 0.f, dr2 = 0.f;
            // hydrostatic part beyond 1/2 g hL^2 (wall reflection)
            float wallx = 0.f;
            if (closed) {
                if (hL > dry) speed = fmaxf(speed, fabsf(loc[1] / hL) + sqrtf(grav * hL));
                if (hR > dry) speed = fmaxf(speed, fabsf(loc[5] / hR) + sqrtf(grav * hR));
            } else {
                const float starL = loc[0], starR = loc[4];
                if (starL > dry) { dl0 = loc[1]; dl1 = loc[1] * loc[1] / starL; dl2 = loc[1] * loc[2] / starL; }
                if (starR > dry) { dr0 = loc[5]; dr1 = loc[5] * loc[5] / starR; dr2 = loc[5] * loc[6] / starR; }
                dl0 += fwo.amdq[0]; dl1 += fwo.amdq[1]; dl2 += fwo.amdq[2];
                dr0 -= fwo.apdq[0]; dr1 -= fwo.apdq[1]; dr2 -= fwo.apdq[2];
                // the HR pressures 1/2 g star^2 and their side corrections 1/2 g (h^2 - star^2) add up to 1/2 g h^2
                if (fabsf(dl0 - dr0) > 2.e-5f * fmaxf(1.f, fmaxf(fabsf(dl0), fabsf(dr0)))) bad = 1;
                dl0 = 0.5f * (dl0 + dr0); dr0 = dl0;
                speed = fmaxf(fabsf(fwo.s[0]), fmaxf(fabsf(fwo.s[1]), fabsf(fwo.s[2])));
                if (kind == 2) {
                    // exact reflecting-wall pressure replaces the whole wall momentum flux
                    const float p = wall_pressure<float>(hL, loc[1], grav, dry);
                    dl0 = 0.f; dl1 = 0.f; dl2 = 0.f;
                    // rounded separately: a wall at rest has p == (half_g hL) hL
                    // bit for bit, so the difference is exactly zero (an FMA
                    // would leave the rounding residual of p)
                    wallx = __fsub_rn(p, __fmul_rn(__fmul_rn(half_g, hL), hL));
                    dr0 = dl0; dr1 = dl1; dr2 = dl2;
                }
            }
            // rotate the dynamic parts back; add the hydrostatic perturbation relative to each cell
            const float lx = dl1 * nx - dl2 * ny + wallx * nx, ly = dl1 * ny + dl2 * nx + wallx * ny;
            float hsL;
            if (hc > dry) hsL = (rc.flags & 1) ? 0.f : half_g * hydro_perturbation(L.dh, hL, hc, L.raw, L.db);
            else hsL = half_g * (hL - hc) * (hL + hc);
            gl1 = lx + hsL * nx; gl2 = ly + hsL * ny;
            if (n >= 0) {
                const float rx_ = dr1 * nx - dr2 * ny, ry_ = dr1 * ny + dr2 * nx;
                float hsR;
                if (hn > dry) hsR = (rn.flags & 1) ? 0.f : half_g * hydro_perturbation(R.dh, hR, hn, R.raw, R.db);
                else hsR = half_g * (hR - hn) * (hR + hn);
                gr1 = rx_ + hsR * nx; gr2 = ry_ + hsR * ny;
            }
            water = dl0;
            if (!isfinite(water) || !isfinite(gl1) || !isfinite(gl2) || !isfinite(gr1) || !isfinite(gr2)) bad = 1;
        } else {
            // dry face: zero flux, the cells' own pressure still enters the gather
            gl1 = -half_g * hc * hc * nx; gl2 = -half_g * hc * hc * ny;
            gr1 = -half_g * hn * hn * nx; gr2 = -half_g * hn * hn * ny;
        }
        if (bad) raise_status(ct, stage, ST_SPATIAL);
        ws[f] = make_float2(water, speed);
        gf[f] = make_float4(gl1, gl2, gr1, gr2);
    }
}

// ---------------------------------------------------------------------------
// Gather: rate, donor factor, CFL frequency (rate form, FP64 mass)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) km_gather(MeshDev m, StateDev s, Ctrl *ctrl, Work w, MixedGeo g, int stage)
{
    const int nc = m.nc;
    const float2 *ws = reinterpret_cast<const float2 *>(w.ws);
    const float4 *gf = reinterpret_cast<const float4 *>(w.gf);
    const MxRec *rec = reinterpret_cast<const MxRec *>(w.rec);
    const int stride = gridDim.x * blockDim.x;
    for (int first = blockIdx.x * blockDim.x; first < nc; first += stride) {
        const int c = first + threadIdx.x;
        bool have = false;
        double fr = 0.;
        int sid = 0;
        if (c < nc) {
            sid = m.cell_sid[c];
            Ctrl &ct = ctrl[sid];
            if (!skip_stage(ct, stage)) {
                const double *base = stage == 1 ? s.work : s.q1;
                const double dt = ct.trial;
                const bool active = rec[c].flags & 2;
                const bool owns_open = m.cflags[c] & 1;
                double sum0 = 0., out = 0., ext = 0., interior = 0.;
                float sum1 = 0.f, sum2 = 0.f, freq = 0.f;
                for (int k = m.offset[c]; k < m.offset[c + 1]; ++k) {
                    const int f = m.faces[k];
                    const double wk = g.cw8[k];            // s * len / area
                    const float2 wsf = ws[f];
                    const float4 gff = gf[f];
                    const double flow = wk * double(wsf.x);   // outward water rate of this cell
                    sum0 += flow;
                    if (wk > 0.) { sum1 += float(wk) * gff.x; sum2 += float(wk) * gff.y; }
                    else { sum1 += float(wk) * gff.z; sum2 += float(wk) * gff.w; }
                    const double debit = fmax(flow, 0.);
                    out += debit;
                    if (owns_open) { if (m.bslot[f] >= 0) ext += debit; else interior += debit; }
                    freq += fabsf(float(wk)) * wsf.y;
                }
                double r0 = 0.;
                float r1 = 0.f, r2 = 0.f;
                if (active) { r0 = -sum0; r1 = -sum1; r2 = -sum2; }
                w.rate[c] = r0; w.rate[nc + c] = r1; w.rate[2 * nc + c] = r2;
                const double hb = base[c];
                double theta = 1.;
                if (out > 0. && dt * out >= hb) theta = fmin(1., hb / (dt * out)) * (1. - 32. * EPS);
                if (owns_open) {
                    const double available = hb / dt;
                    if (ext > available) raise_status(ct, stage, ST_BUDGET);
                    const double factor = fmin(1., (available - ext) / fmax(interior, 1e-300)) * (1. - 32. * EPS);
                    theta = (interior > 0. && interior >= available - ext) ? factor : 1.;
                }
                w.theta[c] = theta;
                fr = double(freq);
                if (isnan(fr)) raise_status(ct, stage, ST_FREQ);
                else have = true;
            }
        }
        unsigned long long *peak0 = stage == 1 ? &ctrl[0].peak1 : &ctrl[0].peak2;
        warp_max_peak(peak0, sizeof(Ctrl), sid, have, fr);
    }
}

// Donor-limited water flux (FP64) and the momentum it carries.
__global__ void __launch_bounds__(256) km_limit(MeshDev m, StateDev s, Ctrl *ctrl, Work w, int stage)
{
    const int nf = m.nf, nc = m.nc;
    const float2 *ws = reinterpret_cast<const float2 *>(w.ws);
    MxLim *lim = reinterpret_cast<MxLim *>(w.lim);
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
        const Ctrl &ct = ctrl[m.face_sid[f]];
        if (skip_stage(ct, stage)) continue;
        const double *q = stage == 1 ? s.work : s.q1;
        double water = double(ws[f].x);
        float cx = 0.f, cy = 0.f;
        if (water != 0. && m.bslot[f] < 0) {
            const int donor = water < 0. ? m.neighbour[f] : m.owner[f];
            if (donor >= 0) {
                const double th = w.theta[donor];
                if (th != 1.) {
                    const double delta = (th - 1.) * water;
                    water *= th;
                    const double hd = q[donor];
                    if (hd > ct.dry) {
                        const float inv = 1.f / float(hd);
                        cx = float(delta) * float(q[nc + donor]) * inv;
                        cy = float(delta) * float(q[2 * nc + donor]) * inv;
                    }
                }
            }
        }
        MxLim l;
        l.water = water; l.cx = cx; l.cy = cy;
        lim[f] = l;
    }
}

__device__ __forceinline__ void drag_f(const Ctrl &ct, double dt, double &h, double &hu, double &hv)
{
    if (h <= ct.dry) { hu = 0.; hv = 0.; return; }
    const float hf = float(h), uf = float(hu), vf = float(hv);
    float c;
    const float val = float(ct.roughness_value);
    if (ct.roughness_mode == 1) c = val;
    else if (ct.roughness_mode == 2) c = powf(hf, 1.f / 6.f) / val;
    else if (ct.roughness_mode == 3) c = sqrtf(9.81f) / .41f * log1pf(30.f * hf / (2.718281828459045f * val));
    else c = 18.f * log10f(12.f * fmaxf(.5f, hf / val));
    const float speed = sqrtf(uf * uf + vf * vf) / hf;
    const float factor = 1.f / (1.f + float(dt) * float(ct.grav) * speed / (c * c * hf));
    hu *= factor;
    hv *= factor;
}

__global__ void __launch_bounds__(256) km_update(MeshDev m, StateDev s, Ctrl *ctrl, Work w, MixedGeo g, int stage,
                                                 double *rate_out)
{
    const int nc = m.nc;
    const MxLim *lim = reinterpret_cast<const MxLim *>(w.lim);
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        Ctrl &ct = ctrl[m.cell_sid[c]];
        if (skip_stage(ct, stage)) continue;
        double mass = 0.;
        float mx = 0.f, my = 0.f;
        for (int k = m.offset[c]; k < m.offset[c + 1]; ++k) {
            const MxLim L = lim[m.faces[k]];
            const double wk = g.cw8[k];
            mass -= wk * L.water;
            mx -= float(wk) * L.cx;
            my -= float(wk) * L.cy;
        }
        const double r0 = mass, r1 = w.rate[nc + c] + double(mx), r2 = w.rate[2 * nc + c] + double(my);
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
            drag_f(ct, .5 * dt, h, hu, hv);
            double *qn = ct.cur ? s.q[0] : s.q[1];
            qn[c] = h; qn[nc + c] = hu; qn[2 * nc + c] = hv;
        }
    }
}

__global__ void km_open_drag(MeshDev m, StateDev s, Ctrl *ctrl)
{
    const int nc = m.nc;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const Ctrl &ct = ctrl[m.cell_sid[c]];
        if (!ct.active || ct.done) continue;
        const double *q = ct.cur ? s.q[1] : s.q[0];
        double h = q[c], hu = q[nc + c], hv = q[2 * nc + c];
        drag_f(ct, .5 * ct.trial, h, hu, hv);
        s.work[c] = h; s.work[nc + c] = hu; s.work[2 * nc + c] = hv;
    }
}

}  // namespace brx_mx

// The boundary CTA of the mixed form is the FP64 kernel (few faces, FP64 sums).
#define BRX_NS brx_mixb
#include "brx_kernels.cuh"

namespace brx {

int mixed_kernel(const Launch &L, int kind, int stage, double *rate_out)
{
    cudaStream_t st = L.stream;
    switch (kind) {
    case K_DRAG:
        brx_mx::km_open_drag<<<L.grid_c256, 256, 0, st>>>(L.mesh, L.state, L.ctrl);
        return 1;
    case K_BOUNDARY:
        if (!L.nslot) return 0;
        brx_mixb::k_boundary<float><<<L.nscen, 256, 0, st>>>(L.mesh, L.state, L.bnd, L.ctrl, stage);
        return 1;
    case K_CELLS:
        if (L.maxdeg <= 4)
            brx_mx::km_cells<4><<<L.grid_c, 128, 0, st>>>(L.mesh, L.state, L.ctrl, L.work, L.mx, stage);
        else
            brx_mx::km_cells<MAX_CELL_FACES><<<L.grid_c, 128, 0, st>>>(L.mesh, L.state, L.ctrl, L.work, L.mx, stage);
        return 1;
    case K_FACES:
        brx_mx::km_faces<<<L.grid_f, 128, 0, st>>>(L.mesh, L.state, L.bnd, L.ctrl, L.work, L.mx, stage);
        return 1;
    case K_GATHER:
        brx_mx::km_gather<<<L.grid_c256, 256, 0, st>>>(L.mesh, L.state, L.ctrl, L.work, L.mx, stage);
        return 1;
    case K_LIMIT:
        brx_mx::km_limit<<<L.grid_f256, 256, 0, st>>>(L.mesh, L.state, L.ctrl, L.work, stage);
        return 1;
    case K_UPDATE:
        brx_mx::km_update<<<L.grid_c256, 256, 0, st>>>(L.mesh, L.state, L.ctrl, L.work, L.mx, stage, rate_out);
        return 1;
    }
    return 0;
}

}  // namespace brx
