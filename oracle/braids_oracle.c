/*
 * CPU oracle of the BRAIDS-HKT augmented f-wave river step.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker that the CUDA path is
 * compared against; nothing in the product links, loads or calls it. It is
 * used by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline
 * leg.
 *
 * It restates, in plain C with FMA contraction disabled (-ffp-contract=off),
 * the FP64 arithmetic the reference generates for this path after its own
 * source transforms, and the Python orchestration around it:
 *
 *   spatial residual  src/braids_core/sediment/river_midpoint.py:100-176
 *   SSPRK(2,2) stage  src/braids_core/sediment/river_explicit.py:63-119
 *   substep control   src/braids_core/sediment/river_explicit.py:121-154
 *   reconstruction    src/braids_support/gpu_fwave/reconstruction.cu:24-212
 *                     + wall_bed_hydraulics.cuda_source transforms
 *                       (src/braids_core/sediment/wall_bed_hydraulics.py:32-36)
 *   face preparation  src/braids_support/gpu_fwave/resident_update.cu:11-55
 *                     + hydrostatic reconstruction transform
 *                       (src/braids_support/sediment/river_morphodynamics/hydrostatic_step_probe.py:37-57,
 *                        face_activity.py:30-37)
 *   augmented f-wave  src/braids_support/gpu_fwave/augmented_fwave.cu:28-334
 *   flux assembly     src/braids_support/gpu_fwave/resident_update.cu:57-148
 *                     + reflecting wall (src/braids_core/sediment/reflecting_wall.py:10-31,76-79)
 *   CSR gather        src/braids_gpu/implicit_midpoint_fwave.cu:65-90
 *   positivity        src/braids_core/sediment/river_midpoint.h:13-41
 *   boundary budget   src/braids_core/sediment/river_explicit_boundary_budget.py:37-54
 *   outlet stock      src/braids_core/hydraulics/outlet_feasibility.py:25-38
 *   exterior traces   src/braids_core/sediment/river_exterior_bed.h:29-174,
 *                     river_exterior_bed.py:183-233
 *   CFL frequency     src/braids_core/sediment/river_explicit.h:13-26
 *   Manning drag      src/braids_core/sediment/river_hydraulic_drag.h:3-16,
 *                     river_roughness.py:42-47
 *   Exner / MPM       src/braids_core/sediment/shoreline_solver.py:209-240 (finish, bed_faces),
 *                     flow2dh_mobile_bed.py:101-109, river_mpm.h:12-46 (mixture, mpm),
 *                     flow2dh_mobile_kernels.h:13-53, bend_methods_v1_kernels.h:23-39,389-405,
 *                     src/braids_gpu/flow_bed_slope_runtime.cu:13-144 (Koch-Flokstra, mode 3)
 *   turbines          src/braids_core/sediment/river_turbine_flow.py:230-239 (momentum order),
 *                     river_turbine_flow.h:13-82 (wet gradients, surface pack, pressure),
 *                     river_hydrokinetic_stress.h:13-35 (ambient stress),
 *                     river_turbine_thetis.py:182-216,263-297 (cell terms, sample),
 *                     river_turbine_flow.py:82-120 (coverage gate),
 *                     flow2dh_fixed_bed_kernels.h:54-60 (face momentum gather)
 *
 * Scope: meshes without WENO stencils or virtual-wall triangles (the
 * generated Delaunay meshes), outlet_extension = 0, cells with at most 32
 * faces (so the projection limiter always runs). Under those conditions the
 * dead branches of the reference kernels are omitted here; the surviving
 * arithmetic is kept operation for operation.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OM_EPS 2.2204460492503131e-16
#define OM_PI 3.14159265358979323846
#define OM_DBL_MIN 2.2250738585072014e-308

/* Rejection kinds, mirroring the reference's BendTrialRejected reasons. */
enum { OM_OK = 0, OM_REJECT_SPATIAL = 1, OM_REJECT_CFL = 2, OM_REJECT_BUDGET = 3, OM_FAIL = 4 };

typedef struct {
    int nc, nf, nadj, nb;
    const int *owner, *neighbour, *bid, *bmode, *offset, *faces, *signs;
    const double *normal, *length, *area;          /* (2,nf) (nf) (nc) */
    const double *ls_matrix, *ls_weight, *ls_delta; /* (4,nc) (nadj) (2,nadj) */
    const double *disp, *disp_len, *distance;       /* (2,2,nf) (2,nf) (2,nf) */
    const int *boundary_offset, *boundary_faces;    /* (nb+1) (sum) */
    /* controls */
    double grav, dry, cfl, speed_limit;
    int roughness_mode;                            /* 1 chezy, 2 manning, 3/4 white-colebrook */
    double roughness_value;
    /* open boundaries */
    const int *seg_mode;                           /* (nb) hydraulic mode per segment */
    const int *stage_policy;                       /* (nb) */
    const double *exterior_bed;                    /* (nf) exterior bed elevation on open faces */
    double *forcing;                               /* (2,nb) row 0 discharge Q, row 1 stage */
    /* forcing tables (optional): per segment piecewise-linear Q(t) and stage(t) */
    int table_len;                                 /* 0 = constant forcing */
    const double *table_time;                      /* (table_len) */
    const double *table_value;                     /* (2, nb, table_len) */
    int threads;
    const struct om_turbines *turb;                /* rotors (NULL: none) */
    /* Q-H rating curves of mode-11 outlets: segment b's knots are
     * rating_offset[b] .. rating_offset[b+1]-1 (elevation increasing) */
    const int *rating_offset;                      /* (nb+1) or NULL */
    const double *rating_q, *rating_eta;
    /* normal-depth outlets (mode 10): connected face chains of their
     * segments, in segment order, each with its bed slope */
    int nchain;
    const int *chain_offset, *chain_face;          /* (nchain+1), faces */
    const double *chain_slope;                     /* (nchain) */
    /* free-weir outlets (mode 5): per segment crest [m], coefficient
     * [m^0.5/s], effective width [m] (3, nb) */
    const double *weir;
    /* critical outlets (mode 4): the connected face chains of their
     * segments (critical_offset (nb+1) over chains, chain faces) */
    const int *crit_seg_chain;                     /* (nb+1) chain range per segment, or NULL */
    const int *crit_chain_offset, *crit_chain_face;
    /* reference water lines of the mode-9 inlets: 0 the forcing stage,
     * 1 critical depth, 2 normal depth (energy slope per segment, the
     * physical neighbour faces along the section, -1 at a gap or an end) */
    const int *inlet_line;                         /* (nb) or NULL */
    const double *inlet_slope;                     /* (nb) */
    const int *line_left, *line_right;             /* (nf) */
    /* conservative wet-bank viscosity (shoreline_viscosity.py:46-72): its
     * coefficient [m2/s] (0: not installed), the flow engines' unweighted
     * least-squares metric (bend_methods_v1.py:100-128: centre offsets per
     * CSR entry, pseudo-inverse per cell), cell centres, and scratch for the
     * velocity gradients (4, nc) and face stresses (2, nf) */
    double visc;
    const double *vdxdy, *vinv, *xy;
    double *vgrad, *vface;
} om_ctx;

/* ------------------------------------------------------------------ */
/* Small helpers                                                       */
/* ------------------------------------------------------------------ */
static inline int om_other(const om_ctx *m, int k)
{
    const int f = m->faces[k];
    return m->signs[k] < 0 ? m->owner[f] : m->neighbour[f];
}

static inline int om_open(const om_ctx *m, int f)
{
    return m->neighbour[f] < 0 && m->bid[f] >= 0;
}

/* Mode-9 segments exist: the exact-discharge inlet owner and its stock-aware
 * allocation run (river_exterior_bed.py:103-105, river_explicit_boundary_budget.py:12). */
static inline int om_has_inlet(const om_ctx *m)
{
    for (int b = 0; b < m->nb; ++b)
        if (m->seg_mode[b] == 9) return 1;
    return 0;
}

/* ------------------------------------------------------------------ */
/* GeoClaw Riemann type (riemanntype, maxiter = 1)                     */
/* augmented_fwave.cu:33-105                                            */
/* ------------------------------------------------------------------ */
typedef struct { double hm, s1m, s2m; } om_rtype;

static om_rtype om_riemann_type(double hL, double hR, double uL, double uR, double drytol, double g)
{
    om_rtype o;
    const double hmin = fmin(hR, hL), hmax = fmax(hR, hL), delu = uR - uL;
    if (hmin <= drytol) {
        o.hm = 0.0;
        o.s1m = uR + uL - 2.0 * sqrt(g * hR) + 2.0 * sqrt(g * hL);
        o.s2m = o.s1m;
        return o;
    }
    const double fmin_ = delu + 2.0 * (sqrt(g * hmin) - sqrt(g * hmax));
    const double fmax_ = delu + (hmax - hmin) * sqrt(0.5 * g * (hmax + hmin) / (hmax * hmin));
    if (fmin_ > 0.0) {                       /* two rarefactions */
        const double root = fmax(0.0, -delu + 2.0 * (sqrt(g * hL) + sqrt(g * hR)));
        o.hm = (1.0 / (16.0 * g)) * (root * root);
        o.s1m = uL + 2.0 * sqrt(g * hL) - 3.0 * sqrt(g * o.hm);
        o.s2m = uR - 2.0 * sqrt(g * hR) + 3.0 * sqrt(g * o.hm);
    } else if (fmax_ <= 0.0) {               /* two shocks: one Newton step on sqrt(h) */
        double h0 = hmax;
        const double gL = sqrt(0.5 * g * (1.0 / h0 + 1.0 / hL));
        const double gR = sqrt(0.5 * g * (1.0 / h0 + 1.0 / hR));
        const double F0 = delu + (h0 - hL) * gL + (h0 - hR) * gR;
        const double dfdh = gL - g * (h0 - hL) / (4.0 * (h0 * h0) * gL) +
                            gR - g * (h0 - hR) / (4.0 * (h0 * h0) * gR);
        const double slope = 2.0 * sqrt(h0) * dfdh;
        const double root = sqrt(h0) - F0 / slope;
        h0 = root * root;
        o.hm = h0;
        const double u1m = uL - (o.hm - hL) * sqrt((0.5 * g) * (1.0 / o.hm + 1.0 / hL));
        const double u2m = uR + (o.hm - hR) * sqrt((0.5 * g) * (1.0 / o.hm + 1.0 / hR));
        o.s1m = u1m - sqrt(g * o.hm);
        o.s2m = u2m + sqrt(g * o.hm);
    } else {                                 /* shock + rarefaction: one secant step */
        double h0 = hmin;
        const double F0 = delu + 2.0 * (sqrt(g * h0) - sqrt(g * hmax)) +
                          (h0 - hmin) * sqrt(0.5 * g * (1.0 / h0 + 1.0 / hmin));
        const double slope = (fmax_ - F0) / (hmax - hmin);
        h0 = h0 - F0 / slope;
        o.hm = h0;
        if (hL > hR) {
            o.s1m = uL + 2.0 * sqrt(g * hL) - 3.0 * sqrt(g * o.hm);
            o.s2m = uL + 2.0 * sqrt(g * hL) - sqrt(g * o.hm);
        } else {
            o.s2m = uR - 2.0 * sqrt(g * hR) + 3.0 * sqrt(g * o.hm);
            o.s1m = uR - 2.0 * sqrt(g * hR) + sqrt(g * o.hm);
        }
    }
    return o;
}

static inline double om_det3(const double a[3][3])
{
    const double d1 = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]);
    const double d2 = a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]);
    const double d3 = a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
    return d1 - d2 + d3;
}

/* ------------------------------------------------------------------ */
/* Augmented f-wave on one face, local normal/tangent frame.           */
/* augmented_fwave.cu:115-262 (riemann_aug_JCP, maxiter 1, no rare     */
/* corrector) and :264-334 (the rpn2 wrapper with dry-wall reflection). */
/* out: [0:3] amdq, [3:6] apdq, [6:9] speeds, [9+3w+c] fwave(c, w).    */
/* Returns the status word (0 ok, bit0 clamp, bit1 nonfinite, -1 bad). */
/* ------------------------------------------------------------------ */
int om_fwave_face(const double in[8], double grav, double drytol, double out[18])
{
    int status = 0;
    for (int r = 0; r < 18; ++r) out[r] = 0.0;
    int finite = isfinite(grav) && isfinite(drytol) && grav > 0.0 && drytol >= 0.0;
    for (int r = 0; r < 8; ++r) finite = finite && isfinite(in[r]);
    if (!finite) return -1;
    double hL = in[0], huL = in[1], hvL = in[2], bL = in[3];
    double hR = in[4], huR = in[5], hvR = in[6], bR = in[7];
    if (hL < 0.0) { hL = 0.0; huL = 0.0; hvL = 0.0; status |= 1; }
    if (hR < 0.0) { hR = 0.0; huR = 0.0; hvR = 0.0; status |= 1; }
    if (hL <= drytol && hR <= drytol) return status;

    double uL, uR, vL, vR, phiL, phiR;
    if (hR > drytol) {
        uR = huR / hR; vR = hvR / hR;
        phiR = 0.5 * grav * (hR * hR) + (huR * huR) / hR;
    } else { hR = 0.0; huR = 0.0; hvR = 0.0; uR = 0.0; vR = 0.0; phiR = 0.0; }
    if (hL > drytol) {
        uL = huL / hL; vL = hvL / hL;
        phiL = 0.5 * grav * (hL * hL) + (huL * huL) / hL;
    } else { hL = 0.0; huL = 0.0; hvL = 0.0; uL = 0.0; vL = 0.0; phiL = 0.0; }
    double wall[3] = {1.0, 1.0, 1.0};
    if (hR <= drytol) {
        const om_rtype t = om_riemann_type(hL, hL, uL, -uL, drytol, grav);
        const double hstar = fmax(hL, t.hm);
        if (hstar + bL < bR) {
            wall[1] = 0.0; wall[2] = 0.0;
            hR = hL; huR = -huL; bR = bL; phiR = phiL; uR = -uL; vR = vL;
        } else if (hL + bL < bR) bR = hL + bL;
    } else if (hL <= drytol) {
        const om_rtype t = om_riemann_type(hR, hR, -uR, uR, drytol, grav);
        const double hstar = fmax(hR, t.hm);
        if (hstar + bR < bL) {
            wall[0] = 0.0; wall[1] = 0.0;
            hL = hR; huL = -huR; bL = bR; phiL = phiR; uL = -uR; vL = vR;
        } else if (hR + bR < bL) bL = hR + bR;
    }
    const double sL = uL - sqrt(grav * hL), sR = uR + sqrt(grav * hR);
    const double uhat = (sqrt(grav * hL) * uL + sqrt(grav * hR) * uR) /
                        (sqrt(grav * hR) + sqrt(grav * hL));
    const double chat = sqrt(grav * 0.5 * (hR + hL));
    double sE1 = fmin(sL, uhat - chat), sE2 = fmax(sR, uhat + chat);

    /* riemann_aug_JCP */
    const double g = grav;
    double r[3][3], lambda[3], delta[3], beta[3], fw[3][3];
    const double delh = hR - hL, delhu = huR - huL, delphi = phiR - phiL, delb = bR - bL;
    const om_rtype t = om_riemann_type(hL, hR, uL, uR, drytol, g);
    const double s1m = t.s1m, s2m = t.s2m;
    lambda[0] = fmin(sE1, s2m);
    lambda[2] = fmax(sE2, s1m);
    sE1 = lambda[0];
    sE2 = lambda[2];
    const double hstarHLL = fmax((huL - huR + sE2 * hR - sE1 * hL) / (sE2 - sE1), 0.0);
    for (int w = 0; w < 3; ++w) { r[0][w] = 1.0; r[1][w] = lambda[w]; r[2][w] = lambda[w] * lambda[w]; }
    lambda[1] = 0.5 * (lambda[0] + lambda[2]);
    r[0][1] = 0.0; r[1][1] = 0.0; r[2][1] = 1.0;

    const double crit = fmax(drytol * g, 1.0e-6);
    const double crit2 = sqrt(crit);
    const double hbar = fmax(0.5 * (hL + hR), 0.0);
    const double usum = uL + uR;
    const double s1s2bar = 0.25 * (usum * usum) - g * hbar;
    const double s1s2tilde = fmax(0.0, uL * uR) - g * hbar;
    int sonic = 0;
    if (fabs(s1s2bar) <= crit) sonic = 1;
    else if (s1s2bar * s1s2tilde <= crit * crit) sonic = 1;
    else if (s1s2bar * sE1 * sE2 <= crit * crit) sonic = 1;
    else if (fmin(fabs(sE1), fabs(sE2)) < crit2) sonic = 1;
    else if (sE1 < crit2 && s1m > -crit2) sonic = 1;
    else if (sE2 > -crit2 && s2m < crit2) sonic = 1;
    else if ((uL + sqrt(g * hL)) * (uR + sqrt(g * hR)) < 0.0) sonic = 1;
    else if ((uL - sqrt(g * hL)) * (uR - sqrt(g * hR)) < 0.0) sonic = 1;

    double deldelh = sonic ? -delb : delb * g * hbar / s1s2bar;
    if (sE1 < -crit && sE2 > crit) {
        deldelh = fmin(deldelh, hstarHLL * (sE2 - sE1) / sE2);
        deldelh = fmax(deldelh, hstarHLL * (sE2 - sE1) / sE1);
    } else if (sE1 >= crit) {
        deldelh = fmin(deldelh, hstarHLL * (sE2 - sE1) / sE1);
        deldelh = fmax(deldelh, -hL);
    } else if (sE2 <= -crit) {
        deldelh = fmin(deldelh, hR);
        deldelh = fmax(deldelh, hstarHLL * (sE2 - sE1) / sE2);
    }
    double deldelphi = sonic ? -g * hbar * delb : -delb * g * hbar * s1s2tilde / s1s2bar;
    deldelphi = fmin(deldelphi, g * fmax(-hL * delb, -hR * delb));
    deldelphi = fmax(deldelphi, g * fmin(-hL * delb, -hR * delb));
    delta[0] = delh - deldelh;
    delta[1] = delhu;
    delta[2] = delphi - deldelphi;
    const double det = om_det3(r);
    for (int k = 0; k < 3; ++k) {
        double a[3][3];
        for (int w = 0; w < 3; ++w)
            for (int c = 0; c < 3; ++c) a[c][w] = r[c][w];
        a[0][k] = delta[0]; a[1][k] = delta[1]; a[2][k] = delta[2];
        beta[k] = om_det3(a) / det;
    }
    for (int w = 0; w < 3; ++w) {
        fw[w][0] = beta[w] * r[1][w];
        fw[w][1] = beta[w] * r[2][w];
        fw[w][2] = beta[w] * r[1][w];
    }
    fw[0][2] = fw[0][2] * vL;
    fw[2][2] = fw[2][2] * vR;
    fw[1][2] = 0.0;
    const double hustar = huL + fw[0][0];
    if (hustar <= 0.0)
        fw[0][2] = fw[0][2] + (hR * uR * vR - hL * uL * vL - fw[0][2] - fw[2][2]);
    else
        fw[2][2] = fw[2][2] + (hR * uR * vR - hL * uL * vL - fw[0][2] - fw[2][2]);

    double am[3] = {0.0, 0.0, 0.0}, ap[3] = {0.0, 0.0, 0.0};
    for (int w = 0; w < 3; ++w) {
        const double s = lambda[w] * wall[w];
        out[6 + w] = s;
        for (int c = 0; c < 3; ++c) {
            const double v = fw[w][c] * wall[w];
            out[9 + 3 * w + c] = v;
            if (s < -1.0e-14) am[c] = am[c] + v;
            else if (s > 1.0e-14) ap[c] = ap[c] + v;
            else { am[c] = am[c] + 0.5 * v; ap[c] = ap[c] + 0.5 * v; }
        }
    }
    for (int c = 0; c < 3; ++c) { out[c] = am[c]; out[3 + c] = ap[c]; }
    for (int r2 = 0; r2 < 18; ++r2) if (!isfinite(out[r2])) status |= 2;
    return status;
}

/* Exact reflecting-wall pressure (reflecting_wall.py:10-31). */
static double om_wall_pressure(double h, double momentum, double g, double dry)
{
    if (h <= dry) return 0.0;
    const double c = sqrt(g * h), v = momentum / h / c;
    double ratio;
    if (v <= 0.0) { const double a = fmax(0.0, 1.0 + 0.5 * v); ratio = a * a; }
    else {
        double lo = 1.0, hi = 1.0 + sqrt(2.0) * v, rr = 1.0 + v;
        for (int k = 0; k < 32; ++k) {
            const double s = sqrt(0.5 * (1.0 + 1.0 / rr));
            const double f = (rr - 1.0) * s - v;
            if (fabs(f) <= 2.e-15 * fmax(1.0, v)) break;
            if (f > 0.0) hi = rr; else lo = rr;
            const double df = s - (rr - 1.0) / (4.0 * s * rr * rr);
            const double trial = rr - f / df;
            rr = (trial > lo && trial < hi) ? trial : 0.5 * (lo + hi);
        }
        ratio = rr;
    }
    const double star = h * ratio;
    return 0.5 * g * star * star;
}

/* ------------------------------------------------------------------ */
/* Reconstruction                                                       */
/* ------------------------------------------------------------------ */

/* Primitive variables (eta, u, v, b), the active mask and the input
 * status (reconstruction.cu:24-39). */
void om_primitive(const om_ctx *m, const double *q, const double *z,
                  double *v, int *active, int *status)
{
    const int nc = m->nc;
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nc; ++c) {
        const double h = q[c];
        v[c] = h + z[c]; v[nc + c] = 0.0; v[2 * nc + c] = 0.0; v[3 * nc + c] = z[c];
        if (h > m->dry) { v[nc + c] = q[nc + c] / h; v[2 * nc + c] = q[2 * nc + c] / h; }
        int act = h > m->dry;
        if (!act)
            for (int k = m->offset[c]; k < m->offset[c + 1]; ++k) {
                const int f = m->faces[k], n = om_other(m, k);
                if (m->bid[f] >= 0 || (n >= 0 && q[n] > m->dry)) { act = 1; break; }
            }
        active[c] = act;
        status[c] = (h < 0.0 || !isfinite(h) || !isfinite(z[c]) || !isfinite(q[nc + c]) ||
                     !isfinite(q[2 * nc + c])) ? 1 : 0;
    }
}

static int om_feasible(double x, double y, int count, const double *ax, const double *ay, const double *b)
{
    for (int i = 0; i < count; ++i)
        if (ax[i] * x + ay[i] * y > b[i] + 2.e-14) return 0;
    return 1;
}

/* Nearest point of the bound polygon to the unlimited gradient: candidates
 * are single-constraint projections and pairwise vertices
 * (braids_project_pair in the directional hydraulic limiter transform). */
static void om_project(double *x, double *y, int count, const double *ax, const double *ay, const double *b)
{
    const double rx = *x, ry = *y;
    if (om_feasible(rx, ry, count, ax, ay, b)) return;
    double bx = 0.0, by = 0.0, best = rx * rx + ry * ry;
    for (int i = 0; i < count; ++i) {
        const double dot = ax[i] * rx + ay[i] * ry - b[i];
        double cx = rx - dot * ax[i], cy = ry - dot * ay[i];
        double d = (cx - rx) * (cx - rx) + (cy - ry) * (cy - ry);
        if (d < best && om_feasible(cx, cy, count, ax, ay, b)) { bx = cx; by = cy; best = d; }
        for (int j = 0; j < i; ++j) {
            const double det = ax[i] * ay[j] - ay[i] * ax[j];
            if (fabs(det) < 1.e-12) continue;
            cx = (b[i] * ay[j] - ay[i] * b[j]) / det;
            cy = (ax[i] * b[j] - b[i] * ax[j]) / det;
            d = (cx - rx) * (cx - rx) + (cy - ry) * (cy - ry);
            if (d < best && om_feasible(cx, cy, count, ax, ay, b)) { bx = cx; by = cy; best = d; }
        }
    }
    *x = bx; *y = by;
}

/* Limited least-squares gradients and the flattening flag of every cell
 * (transformed reconstruction_cells). grad is (4,2,nc): row 2m = d/dx, 2m+1 = d/dy. */
void om_cells(const om_ctx *m, const double *q, const double *v, const int *active,
              double *grad, int *constant)
{
    const int nc = m->nc, nf = m->nf, nadj = m->nadj;
    const double dry = m->dry, grav = m->grav;
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nc; ++c) {
        double centre[4], lo[4], hi[4], gx[4] = {0, 0, 0, 0}, gy[4] = {0, 0, 0, 0};
        for (int k = 0; k < 4; ++k) { centre[k] = v[k * nc + c]; lo[k] = centre[k]; hi[k] = centre[k]; }
        const int k0 = m->offset[c], k1 = m->offset[c + 1];
        if (active[c]) {
            double bx[4] = {0, 0, 0, 0}, by[4] = {0, 0, 0, 0};
            const double a11 = m->ls_matrix[c], a12 = m->ls_matrix[nc + c],
                         a22 = m->ls_matrix[2 * nc + c], det = m->ls_matrix[3 * nc + c];
            for (int k = k0; k < k1; ++k) {
                const int n = om_other(m, k);
                if (n < 0) continue;
                const double rx = m->ls_delta[k], ry = m->ls_delta[nadj + k], w = m->ls_weight[k];
                for (int p = 0; p < 4; ++p) {
                    double adj = v[p * nc + n];
                    /* a dry neighbour whose bed rises above the wet surface contributes the surface */
                    if (p == 0 && centre[0] - centre[3] > dry && v[n] - v[3 * nc + n] <= dry &&
                        v[3 * nc + n] >= centre[0]) adj = centre[0];
                    bx[p] += w * rx * (adj - centre[p]);
                    by[p] += w * ry * (adj - centre[p]);
                    lo[p] = fmin(lo[p], adj); hi[p] = fmax(hi[p], adj);
                }
            }
            if (a11 + a22 > 0.0) {
                /* Wall-mirrored velocity bounds (wall_velocity_bounds transform). */
                if (q[c] > dry)
                    for (int k = k0; k < k1; ++k) {
                        const int f = m->faces[k];
                        if (m->neighbour[f] >= 0 || m->bid[f] >= 0) continue;
                        const double nx = m->normal[f], ny = m->normal[nf + f];
                        const double un = centre[1] * nx + centre[2] * ny;
                        const double mx = centre[1] - 2. * un * nx, my = centre[2] - 2. * un * ny;
                        lo[1] = fmin(lo[1], mx); hi[1] = fmax(hi[1], mx);
                        lo[2] = fmin(lo[2], my); hi[2] = fmax(hi[2], my);
                    }
                for (int p = 0; p < 4; ++p) {
                    if (det > 1.e-12 * ((a11 + a22) * (a11 + a22))) {
                        gx[p] = (a22 * bx[p] - a12 * by[p]) / det;
                        gy[p] = (a11 * by[p] - a12 * bx[p]) / det;
                    } else {
                        gx[p] = (a11 * bx[p] + a12 * by[p]) / ((a11 + a22) * (a11 + a22));
                        gy[p] = (a12 * bx[p] + a22 * by[p]) / ((a11 + a22) * (a11 + a22));
                    }
                }
                const double h = centre[0] - centre[3];
                /* Barth-type factor for the velocities; eta and bed go through the projection below. */
                double theta[4] = {1., 1., 1., 1.};
                for (int k = k0; k < k1; ++k) {
                    const int f = m->faces[k];
                    const int side = m->signs[k] < 0;
                    const double rx = m->disp[side * nf + f], ry = m->disp[(2 + side) * nf + f];
                    if (om_open(m, f) && m->bmode[f] == 2 && h > dry &&
                        fabs(centre[1] * m->normal[f] + centre[2] * m->normal[nf + f]) < sqrt(grav * h) &&
                        fabs(gx[3] * rx + gy[3] * ry) > 64.0 * OM_EPS * fmax(1.0, fabs(centre[3]))) continue;
                    for (int p = 1; p < 3; ++p) {
                        const double d = gx[p] * rx + gy[p] * ry;
                        if (fabs(d) <= 64.0 * OM_EPS * fmax(1.0, fmax(fabs(centre[p]), fmax(fabs(lo[p]), fabs(hi[p])))))
                            continue;
                        if (d > 0.) theta[p] = fmin(theta[p], (hi[p] - centre[p]) / d);
                        if (d < 0.) theta[p] = fmin(theta[p], (lo[p] - centre[p]) / d);
                    }
                }
                double px[2] = {gx[0], gx[3]}, py[2] = {gy[0], gy[3]};
                for (int a = 0; a < 2; ++a) {
                    const int p = a ? 3 : 0;
                    double ax[64], ay[64], b[64];
                    int count = 0;
                    for (int k = k0; k < k1; ++k) {
                        const int f = m->faces[k];
                        const int side = m->signs[k] < 0;
                        const double rx = m->disp[side * nf + f], ry = m->disp[(2 + side) * nf + f];
                        const double len = m->disp_len[side * nf + f];
                        if (om_open(m, f) && m->bmode[f] == 2 && h > dry &&
                            fabs(centre[1] * m->normal[f] + centre[2] * m->normal[nf + f]) < sqrt(grav * h) &&
                            fabs(gx[3] * rx + gy[3] * ry) > 64.0 * OM_EPS * fmax(1.0, fabs(centre[3]))) continue;
                        if (len <= 0. || (p == 3 && m->neighbour[f] < 0 && m->bid[f] < 0)) continue;
                        ax[count] = rx / len; ay[count] = ry / len; b[count++] = fmax(0., hi[p] - centre[p]) / len;
                        ax[count] = -rx / len; ay[count] = -ry / len; b[count++] = fmax(0., centre[p] - lo[p]) / len;
                    }
                    om_project(&px[a], &py[a], count, ax, ay, b);
                }
                for (int p = 1; p < 3; ++p) { gx[p] *= fmax(0., theta[p]); gy[p] *= fmax(0., theta[p]); }
                gx[0] = px[0]; gy[0] = py[0]; gx[3] = px[1]; gy[3] = py[1];
            }
        }
        /* Wet/dry flattening: a reconstructed face depth at or below dry, or a
         * face bed departing from the cell bed by at least the depth. */
        int flatten = q[c] <= dry;
        if (!flatten)
            for (int k = k0; k < k1; ++k) {
                const int f = m->faces[k];
                const int side = (c == m->owner[f]) ? 0 : 1;
                const double rx = m->disp[side * nf + f], ry = m->disp[(2 + side) * nf + f];
                const double eta = (centre[0] + gx[0] * rx) + gy[0] * ry;
                const double zb = (centre[3] + gx[3] * rx) + gy[3] * ry;
                if (eta - zb <= dry || fabs(zb - centre[3]) >= q[c]) { flatten = 1; break; }
            }
        constant[c] = flatten;
        for (int p = 0; p < 4; ++p) { grad[(2 * p) * nc + c] = gx[p]; grad[(2 * p + 1) * nc + c] = gy[p]; }
    }
}

/* Face traces (10,nf) and kinds (reconstruction.cu:170-212): rows 0-3 left
 * h,hu,hv,b; 4-7 right; 8-9 raw depths. Kind 0 dry, 1 interior, 2 wall, 3 open. */
void om_faces(const om_ctx *m, const double *q, const double *v, const double *grad,
              const int *constant, double *trace, int *kind, int *status)
{
    const int nc = m->nc, nf = m->nf;
    const double dry = m->dry;
#pragma omp parallel for schedule(static)
    for (int f = 0; f < nf; ++f) {
        status[f] = 0;
        for (int j = 0; j < 10; ++j) trace[j * nf + f] = 0.0;
        const int c = m->owner[f], n = m->neighbour[f];
        int type = n >= 0 ? 1 : (m->bid[f] < 0 ? 2 : 3);
        if (m->bid[f] < 0 && q[c] <= dry && (n < 0 || q[n] <= dry)) type = 0;
        kind[f] = type;
        for (int side = 0; side < 2; ++side) {
            const int cell = side == 0 ? c : n;
            if (cell < 0) continue;
            double val[4];
            const double rx = m->disp[side * nf + f], ry = m->disp[(2 + side) * nf + f];
            for (int p = 0; p < 4; ++p)
                val[p] = (v[p * nc + cell] + grad[(2 * p) * nc + cell] * rx) + grad[(2 * p + 1) * nc + cell] * ry;
            if (constant[cell]) {
                for (int p = 0; p < 3; ++p) val[p] = v[p * nc + cell];
                if (v[cell] - v[3 * nc + cell] <= dry) val[3] = v[3 * nc + cell];
            }
            for (int p = 0; p < 4; ++p) if (!isfinite(val[p])) status[f] |= 1;
            if (type == 0) continue;
            double depth = fmax(val[0] - val[3], 0.);
            trace[(8 + side) * nf + f] = depth;
            if (q[cell] <= dry || (constant[cell] && depth <= dry)) depth = 0.;
            trace[(4 * side) * nf + f] = depth;
            trace[(4 * side + 1) * nf + f] = depth * val[1];
            trace[(4 * side + 2) * nf + f] = depth * val[2];
            trace[(4 * side + 3) * nf + f] = val[3];
        }
        if (type == 2) {
            for (int j = 0; j < 4; ++j) trace[(4 + j) * nf + f] = trace[j * nf + f];
            trace[9 * nf + f] = trace[8 * nf + f];
        }
    }
}

/* ------------------------------------------------------------------ */
/* Face flux                                                            */
/* ------------------------------------------------------------------ */

/* Rotation, hydrostatic reconstruction at the common face bed and the
 * closed-face test (transformed resident_prepare_faces). */
void om_prepare(const om_ctx *m, const double *trace, const double *q, const double *z,
                const int *kind, double *local, int *closed)
{
    const int nf = m->nf;
    const double dry = m->dry, grav = m->grav;
#pragma omp parallel for schedule(static)
    for (int f = 0; f < nf; ++f) {
        for (int j = 0; j < 8; ++j) local[j * nf + f] = 0.0;
        closed[f] = 0;
        if (kind[f] == 0 || kind[f] == 3) continue;
        const int c = m->owner[f], n = m->neighbour[f];
        const double nx = m->normal[f], ny = m->normal[nf + f];
        double hL = trace[f], xL = trace[nf + f], yL = trace[2 * nf + f], bL = trace[3 * nf + f];
        double hR = trace[4 * nf + f], xR = trace[5 * nf + f], yR = trace[6 * nf + f], bR = trace[7 * nf + f];
        if (kind[f] == 2) {
            hR = hL; bR = bL;
            const double dot = xL * nx + yL * ny;
            xR = xL - 2.0 * dot * nx; yR = yL - 2.0 * dot * ny;
        }
        const double unL = xL * nx + yL * ny, utL = xL * (-ny) + yL * nx;
        const double unR = xR * nx + yR * ny, utR = xR * (-ny) + yR * nx;
        local[f] = hL; local[nf + f] = unL; local[2 * nf + f] = utL; local[3 * nf + f] = bL;
        local[4 * nf + f] = hR; local[5 * nf + f] = unR; local[6 * nf + f] = utR; local[7 * nf + f] = bR;
        if (kind[f] == 1) {
            const double top = fmax(bL, bR);
            const double tol = 16. * OM_EPS * fmax(dry, fmax(fabs(top), fmax(fabs(hL + bL), fabs(hR + bR))));
            double hl = fmax(0., hL + bL - top), hr = fmax(0., hR + bR - top);
            if (hl <= dry + tol) hl = 0.;
            if (hr <= dry + tol) hr = 0.;
            local[f] = hl; local[3 * nf + f] = top; local[4 * nf + f] = hr; local[7 * nf + f] = top;
            local[nf + f] = hL > dry ? unL * (hl / hL) : 0.;
            local[2 * nf + f] = hL > dry ? utL * (hl / hL) : 0.;
            local[5 * nf + f] = hR > dry ? unR * (hr / hR) : 0.;
            local[6 * nf + f] = hR > dry ? utR * (hr / hR) : 0.;
        }
        if (kind[f] != 1 || fmin(q[c], q[n]) > dry) continue;
        const double dc = m->distance[f], dn = m->distance[nf + f];
        double shared;
        if (dc + dn > OM_DBL_MIN)
            shared = (dn * (z[c] + q[c]) + dc * (z[n] + q[n])) / (dc + dn) - fmax(z[c], z[n]);
        else
            shared = 0.5 * ((z[c] + q[c]) + (z[n] + q[n])) - fmax(z[c], z[n]);
        int blocked = shared <= dry;
        if (blocked) {
            int opens = 0;
            if (hL > dry && hR <= dry && unL / hL > 0.0) {
                const om_rtype t = om_riemann_type(hL, hL, unL / hL, -unL / hL, dry, grav);
                opens = t.hm > hL + dry && t.hm + bL > bR + dry;
            } else if (hR > dry && hL <= dry && -unR / hR > 0.0) {
                const om_rtype t = om_riemann_type(hR, hR, -unR / hR, unR / hR, dry, grav);
                opens = t.hm > hR + dry && t.hm + bR > bL + dry;
            }
            blocked = !opens;
        }
        closed[f] = blocked;
    }
}

void om_fwave(const om_ctx *m, const double *local, double *riemann, int *status)
{
    const int nf = m->nf;
#pragma omp parallel for schedule(static)
    for (int f = 0; f < nf; ++f) {
        double in[8], out[18];
        for (int j = 0; j < 8; ++j) in[j] = local[j * nf + f];
        status[f] = om_fwave_face(in, m->grav, m->dry, out);
        for (int j = 0; j < 18; ++j) riemann[j * nf + f] = out[j];
    }
}

/* Left/right physical fluxes with the within-cell hydrostatic bed source
 * (transformed resident_assemble_flux). Open faces (kind 3) are left to the
 * exterior owner, which replaces them wholesale. */
void om_assemble(const om_ctx *m, const double *trace, const double *local, const double *riemann,
                 const double *q, const double *z, const int *kind, const int *hydro_constant,
                 const int *closed, double *fl, double *fr, double *speed, int *face_status)
{
    const int nf = m->nf;
    const double dry = m->dry, grav = m->grav;
#pragma omp parallel for schedule(static)
    for (int f = 0; f < nf; ++f) {
        face_status[f] = 0; speed[f] = 0.0;
        for (int j = 0; j < 3; ++j) { fl[j * nf + f] = 0.0; fr[j * nf + f] = 0.0; }
        if (kind[f] == 0 || kind[f] == 3) continue;
        const int c = m->owner[f], n = m->neighbour[f];
        const double nx = m->normal[f], ny = m->normal[nf + f], hL = trace[f];
        const double hR = kind[f] == 2 ? hL : trace[4 * nf + f];
        double l[3] = {0, 0, 0}, r[3] = {0, 0, 0}, s = 0.0;
        if (closed[f]) {
            l[1] = 0.5 * grav * (hL * hL) * nx; l[2] = 0.5 * grav * (hL * hL) * ny;
            r[1] = 0.5 * grav * (hR * hR) * nx; r[2] = 0.5 * grav * (hR * hR) * ny;
            if (hL > dry) s = fmax(s, fabs(local[nf + f] / hL) + sqrt(grav * hL));
            if (hR > dry) s = fmax(s, fabs(local[5 * nf + f] / hR) + sqrt(grav * hR));
        } else {
            const double starL = local[f], starR = local[4 * nf + f];
            double pl[3] = {0, 0, 0}, pr[3] = {0, 0, 0};
            if (starL > dry) {
                const double hu = local[nf + f], hv = local[2 * nf + f];
                pl[0] = hu; pl[1] = (hu * hu) / starL + 0.5 * grav * (starL * starL); pl[2] = hu * hv / starL;
            }
            if (starR > dry) {
                const double hu = local[5 * nf + f], hv = local[6 * nf + f];
                pr[0] = hu; pr[1] = (hu * hu) / starR + 0.5 * grav * (starR * starR); pr[2] = hu * hv / starR;
            }
            for (int j = 0; j < 3; ++j) { pl[j] += riemann[j * nf + f]; pr[j] -= riemann[(3 + j) * nf + f]; }
            l[0] = pl[0]; l[1] = pl[1] * nx + pl[2] * (-ny); l[2] = pl[1] * ny + pl[2] * nx;
            r[0] = pr[0]; r[1] = pr[1] * nx + pr[2] * (-ny); r[2] = pr[1] * ny + pr[2] * nx;
            if (fabs(l[0] - r[0]) > 1.e-10 * fmax(1.0, fmax(fabs(l[0]), fabs(r[0])))) face_status[f] = 1;
            l[0] = 0.5 * (l[0] + r[0]); r[0] = l[0];
            s = fmax(fabs(riemann[6 * nf + f]), fmax(fabs(riemann[7 * nf + f]), fabs(riemann[8 * nf + f])));
            if (kind[f] == 1) {
                const double cl = .5 * grav * (hL * hL - starL * starL), cr = .5 * grav * (hR * hR - starR * starR);
                l[1] += cl * nx; l[2] += cl * ny; r[1] += cr * nx; r[2] += cr * ny;
            }
            if (kind[f] == 2) {
                l[0] = 0.0;
                const double pressure = om_wall_pressure(hL, local[nf + f], grav, dry);
                l[1] = pressure * nx; l[2] = pressure * ny;
                for (int j = 0; j < 3; ++j) r[j] = l[j];
            }
        }
        if (q[c] > dry) {
            const double corr = hydro_constant[c] ? 0.5 * grav * (q[c] * q[c] - hL * hL)
                                                  : 0.5 * grav * (q[c] + trace[8 * nf + f]) * (trace[3 * nf + f] - z[c]);
            l[1] += corr * nx; l[2] += corr * ny;
        }
        if (n >= 0) {
            if (q[n] > dry) {
                const double corr = hydro_constant[n] ? 0.5 * grav * (q[n] * q[n] - hR * hR)
                                                      : 0.5 * grav * (q[n] + trace[9 * nf + f]) * (trace[7 * nf + f] - z[n]);
                r[1] += corr * nx; r[2] += corr * ny;
            }
        } else for (int j = 0; j < 3; ++j) r[j] = l[j];
        speed[f] = s;
        for (int j = 0; j < 3; ++j) {
            fl[j * nf + f] = l[j]; fr[j * nf + f] = r[j];
            if (!isfinite(l[j]) || !isfinite(r[j])) face_status[f] |= 4;
        }
    }
}

/* rate = -sum_k s_k len/A (f - g h^2/2 n) over active cells (implicit_full_rate_from_faces). */
void om_gather(const om_ctx *m, const double *q, const double *fl, const double *fr,
               const int *active, double *rate)
{
    const int nc = m->nc, nf = m->nf;
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nc; ++c) {
        for (int j = 0; j < 3; ++j) rate[j * nc + c] = 0.0;
        if (!active[c]) continue;
        double sum[3] = {0, 0, 0};
        const double pressure = .5 * m->grav * q[c] * q[c];
        for (int k = m->offset[c]; k < m->offset[c + 1]; ++k) {
            const int f = m->faces[k];
            const double w = m->length[f] / m->area[c];
            if (m->signs[k] > 0) {
                sum[0] += w * fl[f];
                sum[1] += w * (fl[nf + f] - pressure * m->normal[f]);
                sum[2] += w * (fl[2 * nf + f] - pressure * m->normal[nf + f]);
            } else {
                sum[0] -= w * fr[f];
                sum[1] -= w * (fr[nf + f] - pressure * m->normal[f]);
                sum[2] -= w * (fr[2 * nf + f] - pressure * m->normal[nf + f]);
            }
        }
        for (int j = 0; j < 3; ++j) rate[j * nc + c] = -sum[j];
    }
}

/* ------------------------------------------------------------------ */
/* Open boundaries (exterior owner)                                     */
/* ------------------------------------------------------------------ */

static double om_exterior_chezy(int mode, double h, double parameter, double floor_, double gravity, int waqua)
{
    const double d = fmax(h, floor_);
    if (mode == 1) return parameter;
    if (mode == 2) return pow(d, 1. / 6.) / parameter;
    return waqua ? 18. * log10(12. * fmax(.5, d / parameter))
                 : sqrt(gravity) / .41 * log1p(30. * d / (exp(1.) * parameter));
}

/* Outward 1-wave half-Riemann state with a prescribed exterior depth. */
static int om_stage_wave(double h, double un, double target, double gravity, double *depth, double *velocity)
{
    const double c = sqrt(gravity * h);
    *depth = h; *velocity = un;
    if (target > h) {
        const double k = sqrt(.5 * gravity * (1. / target + 1. / h));
        const double shock = un - target * k;
        if (shock >= 0.) return 0;
        *depth = target; *velocity = un - (target - h) * k;
        return 1;
    }
    if (un - c >= 0.) return 0;
    const double cb = sqrt(gravity * target), ub = un + 2. * (c - cb);
    if (ub - cb > 0. || target == 0.) {
        *velocity = (un + 2. * c) / 3.; *depth = (*velocity) * (*velocity) / gravity;
        return 2;
    }
    *depth = target; *velocity = ub;
    return 1;
}

/* Per-segment sums in tiles of 64 faces, then over tiles: the fixed
 * reduction tree of exterior_partial / exterior_totals. */
static void om_segment_sums(const om_ctx *m, const double *input, int fields, double *result)
{
    const int nb = m->nb, nf = m->nf;
    int longest = 0;
    for (int b = 0; b < nb; ++b) {
        const int len = m->boundary_offset[b + 1] - m->boundary_offset[b];
        if (len > longest) longest = len;
    }
    int tiles = (longest + 63) / 64;
    if (tiles < 1) tiles = 1;
    for (int field = 0; field < fields; ++field)
        for (int b = 0; b < nb; ++b) {
            double total = 0.0;
            const int end = m->boundary_offset[b + 1];
            for (int tile = 0; tile < tiles; ++tile) {
                double sum = 0.0;
                for (int k = m->boundary_offset[b] + 64 * tile; k < end && k < m->boundary_offset[b] + 64 * (tile + 1); ++k)
                    sum += input[field * nf + m->boundary_faces[k]];
                total += sum;
            }
            result[field * nb + b] = total;
        }
}

/* Sample piecewise-linear forcing tables at time t into forcing (2,nb). */
void om_sample_forcing(om_ctx *m, double t)
{
    if (m->table_len <= 0) return;
    const int L = m->table_len, nb = m->nb;
    for (int row = 0; row < 2; ++row)
        for (int b = 0; b < nb; ++b) {
            const double *y = m->table_value + ((size_t)row * nb + b) * L;
            double val;
            if (t <= m->table_time[0]) val = y[0];
            else if (t >= m->table_time[L - 1]) val = y[L - 1];
            else {
                /* river_hydraulic_schedule.py:57-65 (inside the table) */
                int i = 0;
                while (i < L - 2 && m->table_time[i + 1] <= t) ++i;
                const double w = (t - m->table_time[i]) / (m->table_time[i + 1] - m->table_time[i]);
                val = (1. - w) * y[i] + w * y[i + 1];
            }
            m->forcing[row * nb + b] = val;
        }
}

/* Exterior traces and fluxes on open faces (ExteriorBed.evaluate).
 * work needs 3*nf doubles; stage_out (2,nb), total_out (nb). Returns 0 or
 * the first nonzero face status. */
/* ------------------------------------------------------------------ */
/* Q-H rating outlet (mode 11): one common water elevation across the   */
/* opening at which the outgoing characteristic discharge equals the    */
/* rating curve (src/braids_core/sediment/river_rating_outlet.h:15-102). */
/* ------------------------------------------------------------------ */
enum { OM_EXTERIOR_FATAL = 100 };

static double om_rating_velocity(double h, double hi, double u, double g)
{
    return h > hi ? u - (h - hi) * sqrt(.5 * g * (1. / h + 1. / hi)) : u + 2. * (sqrt(g * hi) - sqrt(g * h));
}

static double om_rating_q(const om_ctx *m, int b, double eta)
{
    const int a = m->rating_offset[b], end = m->rating_offset[b + 1];
    const double *tq = m->rating_q, *te = m->rating_eta;
    if (eta <= te[a]) return tq[a];
    if (eta >= te[end - 1]) return tq[end - 1];
    int lo = a, hi = end - 1;
    while (hi - lo > 1) { const int mid = (lo + hi) / 2; if (te[mid] <= eta) lo = mid; else hi = mid; }
    const double w = (eta - te[lo]) / (te[hi] - te[lo]);
    return (1. - w) * tq[lo] + w * tq[hi];
}

static double om_rating_residual(const om_ctx *m, int b, double eta, const double *q, const double *z, double *actual)
{
    const int nc = m->nc, nf = m->nf;
    const double g = m->grav, dry = m->dry;
    double Q = 0.;
    for (int k = m->boundary_offset[b]; k < m->boundary_offset[b + 1]; ++k) {
        const int f = m->boundary_faces[k], c = m->owner[f];
        const double bed = m->exterior_bed[f], hc = q[c], hi = fmax(hc + z[c] - bed, 0.);
        if (hc <= dry || hi <= dry) continue;
        const double u = (q[nc + c] * m->normal[f] + q[2 * nc + c] * m->normal[nf + f]) / hc;
        if (u >= sqrt(g * hi)) { Q += hi * u * m->length[f]; continue; }
        const double h = fmax(eta - bed, 0.);
        if (h > dry) Q += h * fmax(om_rating_velocity(h, hi, u, g), 0.) * m->length[f];
    }
    *actual = Q;
    return Q - om_rating_q(m, b, eta);
}

/* Returns 0, or the section's failure (1 no bracket, 2 residual, 3 a
 * fictitious zero-flow root), on which the reference raises ValueError. */
static int om_rating_outlet(const om_ctx *m, int b, const double *q, const double *z, double *trace, double *flux,
                            int *status)
{
    const int nc = m->nc, nf = m->nf;
    const double g = m->grav, dry = m->dry, speed = m->speed_limit;
    const int first = m->rating_offset[b], last = m->rating_offset[b + 1] - 1;
    double lo = m->rating_eta[first], hi = m->rating_eta[last];
    int wet = 0;
    for (int k = m->boundary_offset[b]; k < m->boundary_offset[b + 1]; ++k) {
        const int f = m->boundary_faces[k], c = m->owner[f];
        const double h0 = q[c], h = fmax(h0 + z[c] - m->exterior_bed[f], 0.);
        if (h0 <= dry || h <= dry) continue;
        const double u = (q[nc + c] * m->normal[f] + q[2 * nc + c] * m->normal[nf + f]) / h0;
        if (u >= sqrt(g * h)) continue;
        /* the subcritical branch: the lowest admissible level of this face */
        double left = dry, right = fmax(h, 1.);
        for (int it = 0; it < 60 && om_rating_velocity(right, h, u, g) > sqrt(g * right); ++it) right *= 2.;
        for (int it = 0; it < 60; ++it) {
            const double mid = .5 * (left + right);
            if (om_rating_velocity(mid, h, u, g) > sqrt(g * mid)) left = mid; else right = mid;
        }
        lo = fmax(lo, m->exterior_bed[f] + right);
        ++wet;
    }
    double level = 0., actual = 0.;
    if (wet) {
        if (!(lo <= hi)) return 1;
        const double rlo = om_rating_residual(m, b, lo, q, z, &actual);
        const double rhi = om_rating_residual(m, b, hi, q, z, &actual);
        if (!isfinite(rlo) || !isfinite(rhi) || rlo < 0. || rhi > 0.) return 1;
        for (int it = 0; it < 90; ++it) {
            const double mid = .5 * (lo + hi);
            if (mid == lo || mid == hi) break;
            if (om_rating_residual(m, b, mid, q, z, &actual) > 0.) lo = mid; else hi = mid;
        }
        level = .5 * (lo + hi);
        const double r = om_rating_residual(m, b, level, q, z, &actual);
        if (!isfinite(r) || fabs(r) > 1e-10 * fmax(1., fabs(actual))) return 2;
        if (actual <= 1e-14)
            for (int k = m->boundary_offset[b]; k < m->boundary_offset[b + 1]; ++k) {
                const int f = m->boundary_faces[k], c = m->owner[f];
                const double hc = q[c], hh = fmax(hc + z[c] - m->exterior_bed[f], 0.);
                if (hc <= dry || hh <= dry) continue;
                const double ui = (q[nc + c] * m->normal[f] + q[2 * nc + c] * m->normal[nf + f]) / hc;
                const double h = fmax(level - m->exterior_bed[f], 0.);
                if (h > dry && ui < sqrt(g * hh) && om_rating_velocity(h, hh, ui, g) < -1e-12) return 3;
            }
    }
    for (int k = m->boundary_offset[b]; k < m->boundary_offset[b + 1]; ++k) {
        const int f = m->boundary_faces[k], c = m->owner[f];
        const double bed = m->exterior_bed[f], h0 = q[c], geom = fmax(h0 + z[c] - bed, 0.);
        const double nx = m->normal[f], ny = m->normal[nf + f];
        double ux = 0., uy = 0.;
        if (h0 > dry) { ux = q[nc + c] / h0; uy = q[2 * nc + c] / h0; }
        double un = ux * nx + uy * ny, h = geom;
        const double tx = ux - un * nx, ty = uy - un * ny;
        if (h0 <= dry || geom <= dry) { h = 0.; un = 0.; }
        else if (un >= sqrt(g * geom)) { /* supercritical outflow: no downstream control */ }
        else {
            const double incoming = un;
            h = fmax(level - bed, 0.);
            un = h > dry ? om_rating_velocity(h, geom, incoming, g) : 0.;
            if (un <= 0.) {             /* reflected: the stagnation depth of the incoming stream */
                double left = dry, right = fmax(geom, 1.);
                for (int it = 0; it < 60 && om_rating_velocity(right, geom, incoming, g) > 0.; ++it) right *= 2.;
                for (int it = 0; it < 80; ++it) {
                    const double mid = .5 * (left + right);
                    if (om_rating_velocity(mid, geom, incoming, g) > 0.) left = mid; else right = mid;
                }
                h = .5 * (left + right);
                un = 0.;
            }
        }
        if (!isfinite(h) || !isfinite(un) || sqrt(un * un + tx * tx + ty * ty) > speed) { status[f] = 3; continue; }
        double water = 0., fx = 0., fy = 0.;
        if (h > dry) {
            trace[f] = h; trace[nf + f] = h * (un * nx + tx); trace[2 * nf + f] = h * (un * ny + ty);
            water = h * un;
            fx = water * (un * nx + tx) + .5 * g * h * h * nx;
            fy = water * (un * ny + ty) + .5 * g * h * h * ny;
        } else trace[f] = trace[nf + f] = trace[2 * nf + f] = 0.;
        const double pressure = h0 > dry ? .5 * g * (h0 * h0 - geom * geom) : 0.;
        flux[f] = water; flux[nf + f] = fx + pressure * nx; flux[2 * nf + f] = fy + pressure * ny;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Normal-depth outlet (mode 10): per connected face chain, the section  */
/* level at which the outgoing characteristic discharge equals the       */
/* uniform-flow conveyance at the chain's bed slope                      */
/* (src/braids_core/sediment/river_normal_outlet.h:17-134).              */
/* ------------------------------------------------------------------ */
static double om_nout_chezy(int law, double r, double value, double g)
{
    if (law == 1) return value;
    if (law == 2) return pow(r, 1. / 6.) / value;
    if (law == 3) return sqrt(g) / .41 * log1p(30. * r / (exp(1.) * value));
    return 18. * log10(12. * fmax(.5, r / value));
}

static double om_nout_residual(const om_ctx *m, const int *faces, int start, int end, double eta, double slope,
                               const double *q, const double *z, double *area_out, double *q_out)
{
    const int nc = m->nc, nf = m->nf, law = m->roughness_mode;
    const double g = m->grav, dry = m->dry, *bed = m->exterior_bed;
    double area = 0., perimeter = 0., rate = 0., drag = 0., prev = 0.;
    for (int k = start; k < end; ++k) {
        const int f = faces[k];
        const double h = fmax(eta - bed[f], 0.);
        area += h * m->length[f];
        perimeter += h > dry ? m->length[f] : 0.;
        if (k == start) perimeter += h; else perimeter += fabs(h - prev);
        prev = h;
    }
    perimeter += prev;
    if (area <= 0. || perimeter <= 0.) { *area_out = 0.; *q_out = 0.; return 0.; }
    const double radius = area / perimeter;
    const double manning_radius = law == 2 ? pow(radius, 1. / 6.) : 0.;
    for (int k = start; k < end; ++k) {
        const int f = faces[k], c = m->owner[f];
        const double h0 = q[c], hi = fmax(h0 + z[c] - bed[f], 0.), h = fmax(eta - bed[f], 0.);
        double face_rate = 0.;
        if (h0 > dry && hi > dry) {
            const double ui = (q[nc + c] * m->normal[f] + q[2 * nc + c] * m->normal[nf + f]) / h0;
            if (ui >= sqrt(g * hi)) face_rate = ui * hi;
            else {
                const double invariant = fmax(ui + 2. * sqrt(g * hi), 0.), sonic = invariant * invariant / (9. * g);
                if (h < sonic) face_rate = sonic * sqrt(g * sonic);
                else if (h > dry) face_rate = h * fmax(om_rating_velocity(h, hi, ui, g), 0.);
            }
        }
        rate += face_rate * m->length[f];
        if (h <= dry) continue;
        const double left = k == start ? 0. : fmax(eta - bed[faces[k - 1]], 0.);
        const double right = k + 1 == end ? 0. : fmax(eta - bed[faces[k + 1]], 0.);
        const double p = m->length[f] + fmax(h - left, 0.) + fmax(h - right, 0.);
        const double C = law == 2 ? manning_radius / m->roughness_value
                                  : om_nout_chezy(law, radius, m->roughness_value, g);
        drag += p / (C * C);
    }
    *area_out = area; *q_out = rate;
    return rate - (drag > 0. ? area * sqrt(area * slope / drag) : 0.);
}

/* One chain; 0 or the section failure (a trial rejection in the reference). */
static int om_normal_chain(const om_ctx *m, int ch, const double *q, const double *z, double *trace, double *flux,
                           int *status)
{
    const int nc = m->nc, nf = m->nf;
    const double g = m->grav, dry = m->dry, speed = m->speed_limit, *bed = m->exterior_bed;
    const int *faces = m->chain_face;
    const double slope = m->chain_slope[ch];
    int cursor = m->chain_offset[ch];
    const int stop = m->chain_offset[ch + 1];
    while (cursor < stop) {
        const int ff = faces[cursor], fc = m->owner[ff];
        const double fh = q[fc], fgeom = fmax(fh + z[fc] - bed[ff], 0.);
        if (fh <= dry || fgeom <= dry) {          /* a dry face closes with its owner's pressure */
            trace[ff] = trace[nf + ff] = trace[2 * nf + ff] = 0.;
            flux[ff] = 0.;
            const double pressure = fh > dry ? .5 * g * fh * fh : 0.;
            flux[nf + ff] = pressure * m->normal[ff]; flux[2 * nf + ff] = pressure * m->normal[nf + ff];
            ++cursor;
            continue;
        }
        const int start = cursor;
        while (cursor < stop) {
            const int f = faces[cursor], c = m->owner[f];
            const double hh = q[c];
            if (hh <= dry || hh + z[c] - bed[f] <= dry) break;
            ++cursor;
        }
        const int end = cursor;
        int wet = 0;
        double lo = 1e300, hi = -1e300, area = 0., rate = 0.;
        for (int k = start; k < end; ++k) {
            const int f = faces[k], c = m->owner[f];
            const double h0 = q[c], hf = fmax(h0 + z[c] - bed[f], 0.);
            if (h0 <= dry || hf <= dry) continue;
            const double u = (q[nc + c] * m->normal[f] + q[2 * nc + c] * m->normal[nf + f]) / h0;
            if (u >= sqrt(g * hf)) continue;
            lo = fmin(lo, bed[f] + 2. * dry);
            hi = fmax(hi, z[c] + h0);
            ++wet;
        }
        double level = 0.;
        int fallback = 0;
        if (wet) {
            hi = fmax(hi, lo + 1.);
            double r = om_nout_residual(m, faces, start, end, lo, slope, q, z, &area, &rate);
            if (!isfinite(r)) return 1;
            if (r < 0.) fallback = 1;             /* supercritical normal flow: keep the outgoing trace */
            else {
                double rh = om_nout_residual(m, faces, start, end, hi, slope, q, z, &area, &rate);
                for (int it = 0; it < 60 && rh > 0.; ++it) {
                    hi = lo + 2. * (hi - lo);
                    rh = om_nout_residual(m, faces, start, end, hi, slope, q, z, &area, &rate);
                }
                if (!isfinite(rh) || rh > 0.) return 2;
                for (int it = 0; it < 90; ++it) {
                    const double mid = .5 * (lo + hi);
                    if (mid == lo || mid == hi) break;
                    r = om_nout_residual(m, faces, start, end, mid, slope, q, z, &area, &rate);
                    if (r > 0.) lo = mid; else hi = mid;
                }
                level = .5 * (lo + hi);
                r = om_nout_residual(m, faces, start, end, level, slope, q, z, &area, &rate);
                if (!isfinite(r) || fabs(r) > 1e-10 * fmax(1., fabs(rate))) return 3;
            }
        }
        for (int k = start; k < end; ++k) {
            const int f = faces[k], c = m->owner[f];
            const double h0 = q[c], geom = fmax(h0 + z[c] - bed[f], 0.);
            const double nx = m->normal[f], ny = m->normal[nf + f];
            double ux = 0., uy = 0.;
            if (h0 > dry) { ux = q[nc + c] / h0; uy = q[2 * nc + c] / h0; }
            double un = ux * nx + uy * ny, h = geom;
            const double tx = ux - un * nx, ty = uy - un * ny;
            if (h0 <= dry || geom <= dry) { h = 0.; un = 0.; }
            else if (fallback) { }
            else if (un >= sqrt(g * geom)) { }
            else {
                const double incoming = un;
                h = fmax(level - bed[f], 0.);
                const double invariant = fmax(incoming + 2. * sqrt(g * geom), 0.), sonic = invariant * invariant / (9. * g);
                if (h < sonic) { h = sonic; un = sqrt(g * sonic); }
                else un = h > dry ? om_rating_velocity(h, geom, incoming, g) : 0.;
                if (un <= 0.) {
                    double left = dry, right = fmax(geom, 1.);
                    for (int it = 0; it < 60 && om_rating_velocity(right, geom, incoming, g) > 0.; ++it) right *= 2.;
                    for (int it = 0; it < 80; ++it) {
                        const double mid = .5 * (left + right);
                        if (om_rating_velocity(mid, geom, incoming, g) > 0.) left = mid; else right = mid;
                    }
                    h = .5 * (left + right);
                    un = 0.;
                }
            }
            if (!isfinite(h) || !isfinite(un) || sqrt(un * un + tx * tx + ty * ty) > speed) { status[f] = 3; continue; }
            double water = 0., fx = 0., fy = 0.;
            if (h > dry) {
                trace[f] = h; trace[nf + f] = h * (un * nx + tx); trace[2 * nf + f] = h * (un * ny + ty);
                water = h * un;
                fx = water * (un * nx + tx) + .5 * g * h * h * nx;
                fy = water * (un * ny + ty) + .5 * g * h * h * ny;
            } else trace[f] = trace[nf + f] = trace[2 * nf + f] = 0.;
            const double pressure = h0 > dry ? .5 * g * (h0 * h0 - geom * geom) : 0.;
            flux[f] = water; flux[nf + f] = fx + pressure * nx; flux[2 * nf + f] = fy + pressure * ny;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Section solves with 128 logical lanes (river_exterior_outlet.h): lane  */
/* l sums the section's entries l, l+128, ...; lane sums then add up in   */
/* lane order, which is what makes the reference's OpenMP and CUDA sums   */
/* identical. Restated here sequentially.                                 */
/* ------------------------------------------------------------------ */
#define OM_LANES 128

static double om_weir_velocity(double h, double hi, double ui, double g)
{
    return h > hi ? ui - (h - hi) * sqrt(.5 * g * (1. / h + 1. / hi)) : ui + 2. * (sqrt(g * hi) - sqrt(g * h));
}

typedef struct { double area, width, rate, residual; } om_section_sum;

/* river_exterior_outlet.h:207-227 */
static om_section_sum om_weir_residual(const om_ctx *m, const int *faces, int n, double eta, double crest,
                                       double factor, const int *branch, const double *invariant, const double *q,
                                       const double *z)
{
    const double g = m->grav, dry = m->dry;
    double part[3][OM_LANES];
    for (int lane = 0; lane < OM_LANES; ++lane) {
        double area = 0., width = 0., rate = 0.;
        for (int k = lane; k < n; k += OM_LANES) {
            const int f = faces[k], c = m->owner[f];
            if (!branch[f]) continue;
            const double bed = m->exterior_bed[f], h = fmax(eta - bed, 0.), hi = fmax(q[c] + z[c] - bed, 0.);
            if (h <= dry) continue;
            const double u = fmax(om_weir_velocity(h, hi, invariant[f], g), 0.);
            if (u > 0.) { area += h * m->length[f]; width += m->length[f]; rate += h * u * m->length[f]; }
        }
        part[0][lane] = area; part[1][lane] = width; part[2][lane] = rate;
    }
    om_section_sum r = {0., 0., 0., 0.};
    for (int lane = 0; lane < OM_LANES; ++lane) { r.area += part[0][lane]; r.width += part[1][lane]; r.rate += part[2][lane]; }
    const double head = fmax(eta - crest, 0.);
    r.residual = r.rate - factor * head * sqrt(head);
    return r;
}

/* Free weir on one segment (river_exterior_outlet.h:229-360); 0 or the
 * section failure (a trial rejection in the reference). branch / invariant
 * are per-face scratch. */
static int om_weir_section(const om_ctx *m, int b, const double *q, const double *z, double *trace, double *flux,
                           int *status, int *branch, double *invariant)
{
    const int nc = m->nc, nf = m->nf, nb = m->nb;
    const double g = m->grav, dry = m->dry, speed = m->speed_limit;
    const double tol = 128. * OM_EPS, crest = m->weir[b], factor = m->weir[nb + b] * m->weir[2 * nb + b];
    const int *faces = m->boundary_faces + m->boundary_offset[b];
    const int n = m->boundary_offset[b + 1] - m->boundary_offset[b];
    int error = 0, done = 0;
    double eta = 0.;
    {
        double width = 0.;
        for (int lane = 0; lane < OM_LANES; ++lane) {
            double wl = 0.;
            for (int k = lane; k < n; k += OM_LANES) {
                const int f = faces[k], c = m->owner[f];
                branch[f] = 0; invariant[f] = 0.;
                const double h0 = q[c], h = fmax(h0 + z[c] - m->exterior_bed[f], 0.);
                if (h0 <= dry || h <= dry) continue;
                const double un = (q[nc + c] * m->normal[f] + q[2 * nc + c] * m->normal[nf + f]) / h0;
                branch[f] = 1; invariant[f] = un; wl += m->length[f];
            }
            width += wl;
        }
        if (width == 0.) done = 1;
    }
    if (done) for (int k = 0; k < n; ++k) branch[faces[k]] = 0;
    else {
        double lo = -INFINITY, hi = -INFINITY;
        for (int k = 0; k < n; ++k) {       /* lane maxima, then the maximum over lanes: order-free */
            const int f = faces[k];
            if (branch[f] != 1) continue;
            const int c = m->owner[f];
            const double h0 = fmax(q[c] + z[c] - m->exterior_bed[f], 0.), u = invariant[f];
            double left = 0., right = fmax(h0, 1.);
            for (int it = 0; it < 60 && om_weir_velocity(right, h0, u, g) > sqrt(g * right); ++it) right *= 2.;
            for (int it = 0; it < 70; ++it) {
                const double mid = .5 * (left + right);
                if (om_weir_velocity(mid, h0, u, g) > sqrt(g * mid)) left = mid; else right = mid;
            }
            lo = fmax(lo, m->exterior_bed[f] + right);
            hi = fmax(hi, q[c] + z[c]);
        }
        lo = fmax(lo, crest);
        hi = fmax(hi, lo + 1.);
        om_section_sum r = om_weir_residual(m, faces, n, lo, crest, factor, branch, invariant, q, z);
        if (r.residual < 0. || !isfinite(r.residual)) error = 1;
        if (!error) {
            r = om_weir_residual(m, faces, n, hi, crest, factor, branch, invariant, q, z);
            for (int j = 0; j < 60 && r.residual > 0.; ++j) {
                hi = lo + 2. * (hi - lo);
                r = om_weir_residual(m, faces, n, hi, crest, factor, branch, invariant, q, z);
            }
            if (r.residual > 0. || !isfinite(r.residual)) error = 1;
        }
        if (!error) {
            for (int j = 0; j < 90; ++j) {
                eta = lo + .5 * (hi - lo);
                if (eta == lo || eta == hi) break;
                r = om_weir_residual(m, faces, n, eta, crest, factor, branch, invariant, q, z);
                if (r.residual > 0.) lo = eta; else hi = eta;
            }
            eta = lo + .5 * (hi - lo);
            r = om_weir_residual(m, faces, n, eta, crest, factor, branch, invariant, q, z);
            const double head = fmax(eta - crest, 0.), requested = factor * head * sqrt(head);
            if (!isfinite(r.residual) || fabs(r.residual) > 1e-10 * fmax(requested, 1.)) error = 2;
            double bad = 0.;
            for (int k = 0; k < n; ++k) {
                const int f = faces[k];
                if (branch[f] != 1) continue;
                const int c = m->owner[f];
                const double bed = m->exterior_bed[f], hi2 = fmax(q[c] + z[c] - bed, 0.), h = fmax(eta - bed, 0.);
                const double u = om_weir_velocity(h, hi2, invariant[f], g);
                if (h <= dry || u <= 0.) { branch[f] = 0; continue; }
                if (h > hi2 && invariant[f] - h * sqrt(.5 * g * (1. / h + 1. / hi2)) > tol) bad += 1.;
            }
            if (bad > 0.) error = 5;
        }
    }
    if (error) return error;
    for (int k = 0; k < n; ++k) {
        const int f = faces[k], c = m->owner[f];
        const double bed = m->exterior_bed[f], h0 = q[c], geom = fmax(h0 + z[c] - bed, 0.);
        const double nx = m->normal[f], ny = m->normal[nf + f];
        double h = geom, ux = 0., uy = 0.;
        if (h0 > dry) { ux = q[nc + c] / h0; uy = q[2 * nc + c] / h0; } else h = 0.;
        double un = ux * nx + uy * ny;
        const double tx = ux - un * nx, ty = uy - un * ny;
        if (branch[f] == 0) {
            /* a blocked stream reflects with its stagnation / shock depth */
            if (geom > dry && h0 > dry && un != 0.) {
                double lo = 0., hi = fmax(geom, 1.);
                for (int it = 0; it < 60 && om_weir_velocity(hi, geom, un, g) > 0.; ++it) hi *= 2.;
                for (int it = 0; it < 80; ++it) {
                    const double mid = .5 * (lo + hi);
                    if (om_weir_velocity(mid, geom, un, g) > 0.) lo = mid; else hi = mid;
                }
                h = .5 * (lo + hi);
            }
            un = 0.;
        } else {
            h = fmax(eta - bed, 0.);
            un = om_weir_velocity(h, geom, invariant[f], g);
        }
        if (!isfinite(h) || !isfinite(un) || sqrt(un * un + tx * tx + ty * ty) > speed) { status[f] = 3; continue; }
        double water = 0., fx = 0., fy = 0.;
        if (h > dry) {
            trace[f] = h; trace[nf + f] = h * (un * nx + tx); trace[2 * nf + f] = h * (un * ny + ty);
            water = trace[nf + f] * nx + trace[2 * nf + f] * ny;
            fx = water * trace[nf + f] / h + .5 * g * h * h * nx;
            fy = water * trace[2 * nf + f] / h + .5 * g * h * h * ny;
        }
        const double pressure = h0 > dry ? .5 * g * (h0 * h0 - geom * geom) : 0.;
        flux[f] = water; flux[nf + f] = fx + pressure * nx; flux[2 * nf + f] = fy + pressure * ny;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Prescribed-discharge inlet with a reference water line (mode 9): the   */
/* exact one-dimensional SWE Riemann solution between a virtual reservoir */
/* at the requested line and each face's interior state, the reservoir's  */
/* common normal velocity solved for the exact net section discharge      */
/* (src/braids_core/sediment/river_exterior_inlet.h:20-205).              */
/* ------------------------------------------------------------------ */
typedef struct { double h, u, derivative; int iterations, error; } om_inlet_riemann;

static void om_inlet_wave(double h, double hk, double g, double *f, double *df)
{
    if (h > hk) {
        const double a = sqrt(.5 * g * (1. / h + 1. / hk));
        *f = (h - hk) * a;
        *df = a - .25 * g * (h - hk) / (a * h * h);
    } else {
        const double c = sqrt(g * h);
        *f = 2. * (c - sqrt(g * hk));
        *df = sqrt(g / h);
    }
}

static om_inlet_riemann om_inlet_exact(double hl, double ul, double hr, double ur, double g)
{
    om_inlet_riemann r = {0., 0., 0., 0, 0};
    const double cl = sqrt(g * hl), cr = sqrt(g * hr);
    if (hl == 0. && hr == 0.) return r;
    if (hr == 0. || hl == 0. || ur - ul >= 2. * (cl + cr)) {        /* a dry side or vacuum */
        if (hl > 0. && ul - cl >= 0.) { r.h = hl; r.u = ul; r.derivative = hl; }
        else if (hl > 0. && ul + 2. * cl > 0.) { r.u = (ul + 2. * cl) / 3.; r.h = r.u * r.u / g; r.derivative = r.h; }
        else if (hr > 0. && ur + cr <= 0.) { r.h = hr; r.u = ur; }
        else if (hr > 0. && ur - 2. * cr < 0.) { r.u = (ur - 2. * cr) / 3.; r.h = r.u * r.u / g; }
        return r;
    }
    /* the star depth: safeguarded Newton on the shock / rarefaction curves */
    double guess = .5 * (cl + cr) - .25 * (ur - ul);
    guess = guess * guess / g;
    double lo = 0., hi = fmax(fmax(hl, hr), guess), fl, fr, dl, dr;
    om_inlet_wave(hi, hl, g, &fl, &dl);
    om_inlet_wave(hi, hr, g, &fr, &dr);
    for (int j = 0; j < 60 && fl + fr + ur - ul < 0.; ++j) {
        hi *= 2.;
        om_inlet_wave(hi, hl, g, &fl, &dl);
        om_inlet_wave(hi, hr, g, &fr, &dr);
    }
    if (!isfinite(hi) || fl + fr + ur - ul < 0.) { r.error = 1; return r; }
    double h = fmax(fmin(guess, hi), 1e-30), residual = 0.;
    for (int j = 0; j < 70; ++j) {
        om_inlet_wave(h, hl, g, &fl, &dl);
        om_inlet_wave(h, hr, g, &fr, &dr);
        residual = fl + fr + ur - ul;
        r.iterations = j + 1;
        if (fabs(residual) <= 4e-14 * fmax(1., cl + cr + fabs(ul) + fabs(ur))) break;
        if (residual < 0.) lo = h; else hi = h;
        double next = h - residual / (dl + dr);
        if (!(next > lo && next < hi)) next = lo + .5 * (hi - lo);
        h = next;
    }
    om_inlet_wave(h, hl, g, &fl, &dl);
    om_inlet_wave(h, hr, g, &fr, &dr);
    residual = fl + fr + ur - ul;
    if (!isfinite(h) || fabs(residual) > 2e-11 * fmax(1., cl + cr + fabs(ul) + fabs(ur))) { r.error = 2; return r; }
    const double u = .5 * (ul + ur + fr - fl), c = sqrt(g * h);
    r.h = h; r.u = u; r.derivative = fmax(0., (u + h * dr) / (dl + dr));
    if (u >= 0.) {
        if (h > hl) {
            const double shock = ul - sqrt(.5 * g * h * (h + hl) / hl);
            if (shock >= 0.) { r.h = hl; r.u = ul; r.derivative = hl; }
        } else if (ul - cl >= 0.) { r.h = hl; r.u = ul; r.derivative = hl; }
        else if (u - c > 0.) { r.u = (ul + 2. * cl) / 3.; r.h = r.u * r.u / g; r.derivative = r.h; }
    } else {
        if (h > hr) {
            const double shock = ur + sqrt(.5 * g * h * (h + hr) / hr);
            if (shock <= 0.) { r.h = hr; r.u = ur; r.derivative = 0.; }
        } else if (ur + cr <= 0.) { r.h = hr; r.u = ur; r.derivative = 0.; }
        else if (u + c < 0.) { r.u = (ur - 2. * cr) / 3.; r.h = r.u * r.u / g; r.derivative = 0.; }
    }
    return r;
}

typedef struct { double rate, derivative, area, gross; int max_inner, error; } om_inlet_sum;

static om_inlet_sum om_inlet_rate(const om_ctx *m, const int *faces, int n, double velocity, double requested,
                                  const double *q, const double *z, int max_inner)
{
    const int nc = m->nc, nf = m->nf;
    const double g = m->grav, dry = m->dry;
    double part[6][OM_LANES];
    for (int lane = 0; lane < OM_LANES; ++lane) {
        double rate = 0., derivative = 0., area = 0., inner = 0., error = 0., gross = 0.;
        for (int k = lane; k < n; k += OM_LANES) {
            const int f = faces[k], o = m->owner[f];
            const double bed = m->exterior_bed[f], h0 = q[o];
            double hi = h0 > dry ? fmax(h0 + z[o] - bed, 0.) : 0.;
            if (hi <= dry) hi = 0.;
            const double ui = h0 > dry ? -(q[nc + o] * m->normal[f] + q[2 * nc + o] * m->normal[nf + f]) / h0 : 0.;
            double hr = fmax(requested - bed, 0.);
            if (hr <= dry) hr = 0.;
            const om_inlet_riemann r = om_inlet_exact(hr, velocity, hi, ui, g);
            rate += r.h * r.u * m->length[f]; derivative += r.derivative * m->length[f]; area += r.h * m->length[f];
            gross += fabs(r.h * r.u * m->length[f]);
            inner = fmax(inner, r.iterations); error = fmax(error, r.error);
        }
        part[0][lane] = rate; part[1][lane] = derivative; part[2][lane] = area; part[3][lane] = inner;
        part[4][lane] = error; part[5][lane] = gross;
    }
    om_inlet_sum s = {0., 0., 0., 0., max_inner, 0};
    for (int lane = 0; lane < OM_LANES; ++lane) {
        s.rate += part[0][lane]; s.derivative += part[1][lane]; s.area += part[2][lane]; s.gross += part[5][lane];
        s.max_inner = (int)fmax(s.max_inner, part[3][lane]);
        if (part[4][lane]) s.error = 5;
    }
    return s;
}

/* One mode-9 segment; 0 or its failure (a trial rejection in the reference). */
static int om_inlet_section(const om_ctx *m, int b, const double *q, const double *z, double *trace, double *flux,
                            int *status)
{
    const int nc = m->nc, nf = m->nf, nb = m->nb;
    const double g = m->grav, dry = m->dry, speed = m->speed_limit;
    const double Q = m->forcing[b], requested = m->forcing[nb + b];
    const int *faces = m->boundary_faces + m->boundary_offset[b];
    const int n = m->boundary_offset[b + 1] - m->boundary_offset[b];
    int error = 0, max_inner = 0;
    double reference_area = 0., scale = 1.;
    for (int lane = 0; lane < OM_LANES; ++lane) {
        double area = 0., sc = 1.;
        for (int k = lane; k < n; k += OM_LANES) {
            const int f = faces[k], o = m->owner[f];
            status[f] = 0;
            const double bed = m->exterior_bed[f], h0 = q[o];
            double hi = h0 > dry ? fmax(h0 + z[o] - bed, 0.) : 0.;
            if (hi <= dry) hi = 0.;
            const double ui = h0 > dry ? -(q[nc + o] * m->normal[f] + q[2 * nc + o] * m->normal[nf + f]) / h0 : 0.;
            const double hr = fmax(requested - bed, 0.);
            if (hr > dry) area += hr * m->length[f];
            sc = fmax(sc, fabs(ui) + 2. * sqrt(g * hi) + 2. * sqrt(g * hr));
        }
        reference_area += area;
        scale = fmax(scale, sc);
    }
    if (!isfinite(Q) || Q < 0. || !isfinite(requested) || (Q > 0. && reference_area <= 0.)) error = 1;
    double velocity = reference_area > 0. ? Q / reference_area : 0.;
    scale = fmax(scale, 1. + fabs(velocity));
    if (Q > 0. && !error) {
        double lo = velocity - scale, hi = velocity + scale;
        om_inlet_sum r = om_inlet_rate(m, faces, n, lo, requested, q, z, max_inner);
        max_inner = r.max_inner; if (r.error) error = r.error;
        for (int j = 0; j < 60 && r.rate > Q && !error; ++j) {
            lo -= scale; scale *= 2.;
            r = om_inlet_rate(m, faces, n, lo, requested, q, z, max_inner);
            max_inner = r.max_inner; if (r.error) error = r.error;
        }
        if (r.rate > Q) error = 2;
        r = om_inlet_rate(m, faces, n, hi, requested, q, z, max_inner);
        max_inner = r.max_inner; if (r.error) error = r.error;
        for (int j = 0; j < 60 && r.rate < Q && !error; ++j) {
            hi += scale; scale *= 2.;
            r = om_inlet_rate(m, faces, n, hi, requested, q, z, max_inner);
            max_inner = r.max_inner; if (r.error) error = r.error;
        }
        if (r.rate < Q) error = 2;
        velocity = fmin(hi, fmax(lo, Q / reference_area));
        for (int j = 0; j < 80 && !error; ++j) {
            r = om_inlet_rate(m, faces, n, velocity, requested, q, z, max_inner);
            max_inner = r.max_inner; if (r.error) error = r.error;
            if (fabs(r.rate - Q) <= 3e-13 * Q + 256. * OM_EPS * r.gross) break;
            if (r.rate < Q) lo = velocity; else hi = velocity;
            double next = r.derivative > 0. ? velocity + (Q - r.rate) / r.derivative : lo + .5 * (hi - lo);
            if (!(next > lo && next < hi)) next = lo + .5 * (hi - lo);
            velocity = next;
        }
        r = om_inlet_rate(m, faces, n, velocity, requested, q, z, max_inner);
        max_inner = r.max_inner; if (r.error) error = r.error;
        if (!isfinite(r.rate) || fabs(r.rate - Q) > 1e-10 * Q + 1024. * OM_EPS * r.gross) error = 3;
    }
    if (error) return error;
    for (int k = 0; k < n; ++k) {
        const int f = faces[k], o = m->owner[f];
        const double nx = m->normal[f], ny = m->normal[nf + f], bed = m->exterior_bed[f], h0 = q[o];
        double hi = h0 > dry ? fmax(h0 + z[o] - bed, 0.) : 0.;
        if (hi <= dry) hi = 0.;
        const double ui = h0 > dry ? -(q[nc + o] * nx + q[2 * nc + o] * ny) / h0 : 0.;
        const double vt = h0 > dry ? (-q[nc + o] * ny + q[2 * nc + o] * nx) / h0 : 0.;
        double hr = fmax(requested - bed, 0.);
        if (hr <= dry) hr = 0.;
        om_inlet_riemann r = Q == 0. ? om_inlet_exact(h0, -ui, h0, ui, g) : om_inlet_exact(hr, velocity, hi, ui, g);
        if (Q == 0.) r.u = 0.;
        if (r.error || !isfinite(r.h) || !isfinite(r.u) || fabs(r.u) > speed) { status[f] = 3; continue; }
        const double water = -r.h * r.u, tangent = r.u < 0. ? vt : 0.;
        trace[f] = r.h; trace[nf + f] = water * nx - r.h * tangent * ny; trace[2 * nf + f] = water * ny + r.h * tangent * nx;
        const double pressure = Q == 0. ? 0. : .5 * g * (h0 * h0 - hi * hi);
        const double momentum = r.h * r.u * r.u + .5 * g * r.h * r.h + pressure;
        flux[f] = water; flux[nf + f] = momentum * nx - water * tangent * ny; flux[2 * nf + f] = momentum * ny + water * tangent * nx;
    }
    return 0;
}

/* Reference water lines written into the forcing stage of mode-9 inlets
 * before the exterior flux (ExteriorBed.evaluate, river_exterior_bed.py:
 * 195-200). Each distinct bed level of the section starts one
 * constant-wet-width branch; the branches' candidates are reduced to the
 * lexicographic minimum of (rank, stage) (section_critical_partial / _total,
 * river_exterior_section.h:51-74, a running minimum whose result does not
 * depend on the tiling). */
static void om_line_pick(double rank, double cand, double *best, double *stage)
{
    if (rank < *best || (rank == *best && cand < *stage)) { *best = rank; *stage = cand; }
}

/* Critical-depth line (CriticalSection, river_exterior_section.h:17-49):
 * Q^2 W / (g A^3) = 1 on the branch, the minimum specific energy wins. */
static int om_line_critical(om_ctx *m, int b)
{
    const int nb = m->nb, k0 = m->boundary_offset[b], k1 = m->boundary_offset[b + 1];
    const int *faces = m->boundary_faces;
    const double *bed = m->exterior_bed, *length = m->length;
    const double Q = m->forcing[b], g = m->grav, dry = m->dry;
    double best = INFINITY, stage = 0.;
    for (int i = k0; i < k1; ++i) {
        const double level = bed[faces[i]];
        double minimum = level, next = INFINITY, width = 0., excess = 0.;
        for (int k = k0; k < k1; ++k) {
            const int f = faces[k];
            const double zb = bed[f];
            minimum = fmin(minimum, zb);
            if (zb > level) next = fmin(next, zb);
            else { width += length[f]; excess += (level - zb) * length[f]; }
        }
        double cand = 0., energy = INFINITY;
        if (Q == 0.) { cand = minimum; energy = 0.; }
        else {
            const double area = cbrt(Q * Q * width / g), eta = level + (area - excess) / width;
            if (isfinite(area) && area > 0. && isfinite(eta) && eta > level + dry && !(eta > next + dry)) {
                double actual = 0., wet_width = 0.;
                for (int k = k0; k < k1; ++k) {
                    const int f = faces[k];
                    const double h = eta - bed[f];
                    if (h > dry) { actual += h * length[f]; wet_width += length[f]; }
                }
                if (wet_width == width && actual > 0.) {
                    const double residual = fabs(Q * Q * wet_width / (g * actual * actual * actual) - 1.);
                    const double tolerance = 1e-10 + 64. * OM_EPS * fmax(1., fabs(eta)) * width / actual;
                    if (!(residual > tolerance)) { cand = eta; energy = eta - minimum + Q * Q / (2. * g * actual * actual); }
                }
            }
        }
        om_line_pick(energy, cand, &best, &stage);
    }
    if (!isfinite(best)) return 1;
    m->forcing[nb + b] = stage;
    return 0;
}

/* Wetted perimeter of face f at level eta: its length plus the wetted
 * vertical steps to its physical neighbours (river_exterior_normal.h:25-31). */
static double om_line_perimeter(const om_ctx *m, int f, double eta)
{
    const double *bed = m->exterior_bed, dry = m->dry;
    const double h = eta - bed[f];
    if (h <= dry) return 0.;
    const int l = m->line_left[f], r = m->line_right[f];
    double hl = l < 0 ? 0. : fmax(eta - bed[l], 0.), hr = r < 0 ? 0. : fmax(eta - bed[r], 0.);
    if (hl <= dry) hl = 0.;
    if (hr <= dry) hr = 0.;
    return m->length[f] + fmax(h - hl, 0.) + fmax(h - hr, 0.);
}

/* Uniform-flow discharge of the section at level eta (normal_rate,
 * river_exterior_normal.h:32-57, without bedform feedback). */
static double om_line_rate(const om_ctx *m, int b, double eta, double slope)
{
    const int k0 = m->boundary_offset[b], k1 = m->boundary_offset[b + 1];
    const int *faces = m->boundary_faces;
    const double *bed = m->exterior_bed, dry = m->dry;
    double area = 0., perimeter = 0., drag = 0.;
    for (int k = k0; k < k1; ++k) {
        const int f = faces[k];
        const double h = eta - bed[f];
        if (h > dry) { area += h * m->length[f]; perimeter += om_line_perimeter(m, f, eta); }
    }
    double rate = 0.;
    if (area > 0. && perimeter > 0.) {
        const double radius = area / perimeter;
        const double c = om_nout_chezy(m->roughness_mode, fmax(radius, dry), m->roughness_value, m->grav);
        for (int k = k0; k < k1; ++k) {
            const int f = faces[k];
            if (eta - bed[f] <= dry) continue;
            drag += om_line_perimeter(m, f, eta) / (c * c);
        }
        if (drag > 0.) rate = area * sqrt(area * slope / drag);
    }
    return rate;
}

/* Normal-depth line (NormalSection, river_exterior_normal.h:59-104): per
 * distinct bed level the lowest bracketed root of rate(eta) = Q (32
 * sub-brackets, 80 bisections, a final relative check); the lowest root wins. */
static int om_line_normal(om_ctx *m, int b)
{
    const int nb = m->nb, k0 = m->boundary_offset[b], k1 = m->boundary_offset[b + 1];
    const int *faces = m->boundary_faces;
    const double *bed = m->exterior_bed;
    const double Q = m->forcing[b], dry = m->dry, slope = m->inlet_slope[b];
    double best = INFINITY, stage = 0.;
    for (int i = k0; i < k1; ++i) {
        const int fi = faces[i];
        const double level = bed[fi];
        double minimum = level, next = INFINITY;
        int duplicate = 0;
        for (int k = k0; k < k1; ++k) {
            const int f = faces[k];
            const double zb = bed[f];
            minimum = fmin(minimum, zb);
            if (zb > level) next = fmin(next, zb);
            if (zb == level && f < fi) duplicate = 1;
        }
        if (duplicate) continue;
        if (Q == 0.) { om_line_pick(minimum, minimum, &best, &stage); continue; }
        const double epsilon = 8. * OM_EPS * fmax(1., fabs(level));
        double lo = level + dry + epsilon, hi = isfinite(next) ? next + dry : level + fmax(1., 64. * dry);
        if (!(hi > lo)) continue;
        double rlo = om_line_rate(m, b, lo, slope) - Q, rhi = om_line_rate(m, b, hi, slope) - Q;
        if (!isfinite(next))
            for (int k = 0; k < 60 && rhi < 0.; ++k) {
                hi = level + 2. * (hi - level);
                rhi = om_line_rate(m, b, hi, slope) - Q;
            }
        if (!isfinite(rlo) || !isfinite(rhi)) continue;
        const double start = lo, end = hi;
        double previous = rlo;
        int found = 0;
        for (int j = 1; j <= 32; ++j) {
            const double at = start + (end - start) * ((double)j / 32.);
            const double value = j == 32 ? rhi : om_line_rate(m, b, at, slope) - Q;
            if (isfinite(value) && ((previous <= 0. && value >= 0.) || (previous >= 0. && value <= 0.))) {
                hi = at; rhi = value; rlo = previous; found = 1;
                break;
            }
            lo = at; previous = value;
        }
        if (!found) continue;
        for (int j = 0; j < 80; ++j) {
            const double mid = lo + .5 * (hi - lo);
            if (mid == lo || mid == hi) break;
            const double value = om_line_rate(m, b, mid, slope) - Q;
            if ((rlo <= 0. && value >= 0.) || (rlo >= 0. && value <= 0.)) { hi = mid; rhi = value; }
            else { lo = mid; rlo = value; }
        }
        const double eta = fabs(rlo) < fabs(rhi) ? lo : hi;
        const double rate = om_line_rate(m, b, eta, slope);
        const double tolerance = 1e-10 + 128. * OM_EPS * fmax(1., fabs(eta)) / fmax(eta - minimum, dry);
        if (isfinite(rate) && fabs(rate / Q - 1.) <= tolerance) om_line_pick(eta, eta, &best, &stage);
    }
    if (!isfinite(best)) return 1;
    m->forcing[nb + b] = stage;
    return 0;
}

/* Critical lines, then normal lines (river_exterior_bed.py:199-200); 0 or a
 * trial rejection. */
static int om_inlet_lines(om_ctx *m)
{
    if (!m->inlet_line) return 0;
    for (int b = 0; b < m->nb; ++b)
        if (m->seg_mode[b] == 9 && m->inlet_line[b] == 1 && om_line_critical(m, b)) return OM_REJECT_SPATIAL;
    for (int b = 0; b < m->nb; ++b)
        if (m->seg_mode[b] == 9 && m->inlet_line[b] == 2 && om_line_normal(m, b)) return OM_REJECT_SPATIAL;
    return 0;
}

/* Stock-aware allocation of the mode-9 inlets (InletFeasibility.__call__,
 * src/braids_core/hydraulics/inlet_feasibility.py:35-57): outward inlet
 * debit capped by each owner's stock after other boundary debits, the
 * removed outflow taken from the section's incoming faces. Sums follow the
 * boundary face order. work needs 3*nc + 2*nb doubles. */
void om_inlet_feasibility(const om_ctx *m, const double *base, double dt, double *flux, double *trace, double *work)
{
    const int nc = m->nc, nf = m->nf, nb = m->nb;
    const int nbf = m->boundary_offset[nb];
    double *total = work, *reserved = work + nc, *scale_c = work + 2 * (size_t)nc;
    double *removed_b = work + 3 * (size_t)nc, *incoming_b = removed_b + nb;
    for (int k = 0; k < nbf; ++k) { const int c = m->owner[m->boundary_faces[k]]; total[c] = 0.; reserved[c] = 0.; }
    for (int b = 0; b < nb; ++b) { removed_b[b] = 0.; incoming_b[b] = 0.; }
    for (int k = 0; k < nbf; ++k) {
        const int f = m->boundary_faces[k], c = m->owner[f];
        const double rate = fmax(flux[f], 0.) * m->length[f];
        if (m->seg_mode[m->bid[f]] == 9) total[c] += rate; else reserved[c] += rate;
    }
    for (int k = 0; k < nbf; ++k) {
        const int c = m->owner[m->boundary_faces[k]];
        const double available = fmax(0., base[c] * m->area[c] / dt - reserved[c]);
        const double ratio = fmin(1., available / fmax(total[c], 1e-300)) * (1. - 32. * OM_EPS);
        scale_c[c] = total[c] > available ? ratio : 1.;
    }
    for (int k = 0; k < nbf; ++k) {
        const int f = m->boundary_faces[k], c = m->owner[f], b = m->bid[f];
        if (m->seg_mode[b] != 9) continue;
        const double water = flux[f], debit = fmax(water, 0.) * m->length[f];
        removed_b[b] += water > 0. ? debit * (1. - scale_c[c]) : 0.;
        incoming_b[b] += fmax(-water, 0.) * m->length[f];
    }
    for (int k = 0; k < nbf; ++k) {
        const int f = m->boundary_faces[k], c = m->owner[f], b = m->bid[f];
        if (m->seg_mode[b] != 9) continue;
        const double water = flux[f];
        const int feasible = removed_b[b] <= incoming_b[b];
        const double in_scale = incoming_b[b] > 0. ? 1. - removed_b[b] / fmax(incoming_b[b], 1e-300) : 1.;
        const double sc = (feasible && water > 0.) ? scale_c[c] : ((feasible && water < 0.) ? in_scale : 1.);
        const double depth = trace[f], denom = fmax(depth, 1e-300);
        const double ux = depth > 0. ? trace[nf + f] / denom : 0., uy = depth > 0. ? trace[2 * nf + f] / denom : 0.;
        flux[nf + f] += (sc * sc - 1.) * water * ux;
        flux[2 * nf + f] += (sc * sc - 1.) * water * uy;
        flux[f] = water * sc;
        trace[nf + f] *= sc;
        trace[2 * nf + f] *= sc;
    }
}

/* ------------------------------------------------------------------ */
/* Critical outlet (mode 4): outgoing characteristic discharge equal to  */
/* sqrt(g A^3 / B) on the controlled faces of the opening, faces that     */
/* turn inward or dry removed and the root recomputed                     */
/* (river_exterior_outlet.h:29-175), per wet group of each chain when a   */
/* dry bar splits the opening (river_exterior_outlet.py:37-72).           */
/* ------------------------------------------------------------------ */
static double om_resolved_bed(const om_ctx *m, int f, const double *q, const double *z)
{
    const int c = m->owner[f];
    const double h = fmax(q[c], 0.), bed = m->exterior_bed[f];
    if (h >= 1.e-3) return bed;
    const double bounded = fmax(bed, z[c] - h);
    double blend = fmin(1., fmax(0., (h - 1.e-4) / 9.e-4));
    blend = blend * blend * (3. - 2. * blend);
    return bed + (bounded - bed) * (1. - blend);
}

static om_section_sum om_crit_residual(const om_ctx *m, const int *faces, int n, double eta, const int *branch,
                                       const double *invariant, const double *q, const double *z)
{
    const double g = m->grav, dry = m->dry;
    double part[3][OM_LANES];
    for (int lane = 0; lane < OM_LANES; ++lane) {
        double a = 0., width = 0., rate = 0.;
        for (int k = lane; k < n; k += OM_LANES) {
            const int f = faces[k];
            if (branch[f] != 1) continue;
            const double h = fmax(eta - om_resolved_bed(m, f, q, z), 0.);
            if (h <= dry) continue;
            a += h * m->length[f]; width += m->length[f]; rate += h * (invariant[f] - 2. * sqrt(g * h)) * m->length[f];
        }
        part[0][lane] = a; part[1][lane] = width; part[2][lane] = rate;
    }
    om_section_sum r = {0., 0., 0., 0.};
    for (int lane = 0; lane < OM_LANES; ++lane) { r.area += part[0][lane]; r.width += part[1][lane]; r.rate += part[2][lane]; }
    r.residual = r.rate - (r.width > 0. ? sqrt(g * r.area * r.area * r.area / r.width) : 0.);
    return r;
}

/* One critical section over faces[0..n); 0 or its failure (a trial rejection). */
static int om_crit_group(const om_ctx *m, const int *faces, int n, const double *q, const double *z, double *trace,
                         double *flux, int *status, int *branch, double *invariant)
{
    const int nc = m->nc, nf = m->nf;
    const double g = m->grav, dry = m->dry, speed = m->speed_limit, tol = 128. * OM_EPS;
    int error = 0, done = 0;
    double eta = 0.;
    for (int k = 0; k < n; ++k) {
        const int f = faces[k], c = m->owner[f];
        branch[f] = 0; invariant[f] = 0.;
        const double h0 = q[c], h = fmax(h0 + z[c] - om_resolved_bed(m, f, q, z), 0.);
        if (h0 <= dry || h <= dry) continue;
        const double un = (q[nc + c] * m->normal[f] + q[2 * nc + c] * m->normal[nf + f]) / h0, wave = sqrt(g * h);
        if (un < -tol * fmax(1., fabs(un))) continue;
        if (un > wave * (1. + 1e-10)) { branch[f] = 2; continue; }
        branch[f] = 1; invariant[f] = un + 2. * wave;
    }
    for (int active = 0; active <= n; ++active) {
        double lo = INFINITY, hi = -INFINITY;
        int count = 0;
        for (int k = 0; k < n; ++k) {         /* lane min / max / counts: order-free */
            const int f = faces[k];
            if (branch[f] != 1) continue;
            lo = fmin(lo, om_resolved_bed(m, f, q, z));
            hi = fmax(hi, q[m->owner[f]] + z[m->owner[f]]);
            ++count;
        }
        if (count) lo += fmax(2. * dry, tol * fmax(1., fabs(lo)));
        else { done = 1; break; }
        om_section_sum r = om_crit_residual(m, faces, n, lo, branch, invariant, q, z);
        if (r.residual < 0.) {                /* unresolved controlled depth: the opening closes */
            for (int k = 0; k < n; ++k) if (branch[faces[k]] == 1) branch[faces[k]] = 0;
            done = 1; eta = lo;
            break;
        }
        r = om_crit_residual(m, faces, n, hi, branch, invariant, q, z);
        for (int j = 0; j < 60 && r.residual > 0.; ++j) {
            hi = lo + 2. * (hi - lo);
            r = om_crit_residual(m, faces, n, hi, branch, invariant, q, z);
        }
        if (r.residual > 0. || !isfinite(r.residual)) { error = 1; break; }
        for (int j = 0; j < 90; ++j) {
            eta = lo + .5 * (hi - lo);
            if (eta == lo || eta == hi) break;
            r = om_crit_residual(m, faces, n, eta, branch, invariant, q, z);
            if (r.residual > 0.) lo = eta; else hi = eta;
        }
        eta = lo + .5 * (hi - lo);
        int changed = 0;
        for (int k = 0; k < n; ++k) {
            const int f = faces[k];
            if (branch[f] != 1) continue;
            const double h = fmax(eta - om_resolved_bed(m, f, q, z), 0.), un = invariant[f] - 2. * sqrt(g * h);
            if (h <= dry || un < -tol) { branch[f] = 0; ++changed; }
        }
        if (changed) continue;
        r = om_crit_residual(m, faces, n, eta, branch, invariant, q, z);
        const double qc = r.width > 0. ? sqrt(g * r.area * r.area * r.area / r.width) : 0.;
        if (r.area <= 0. || r.width <= 0. || !isfinite(r.residual) || fabs(r.residual) > 1e-10 * fmax(qc, 1.)) error = 2;
        done = 1;
        break;
    }
    if (!done && !error) error = 3;
    if (error) return error;
    for (int k = 0; k < n; ++k) {
        const int f = faces[k], c = m->owner[f];
        const double rbed = om_resolved_bed(m, f, q, z), h0 = q[c], geom = fmax(h0 + z[c] - rbed, 0.);
        const double nx = m->normal[f], ny = m->normal[nf + f];
        double h = geom, ux = 0., uy = 0.;
        if (h0 > dry) { ux = q[nc + c] / h0; uy = q[2 * nc + c] / h0; } else h = 0.;
        double un = ux * nx + uy * ny;
        const double tx = ux - un * nx, ty = uy - un * ny;
        if (branch[f] == 0) un = 0.;
        else if (branch[f] == 1) { h = fmax(eta - rbed, 0.); un = invariant[f] - 2. * sqrt(g * h); }
        if (!isfinite(h) || !isfinite(un) || sqrt(un * un + tx * tx + ty * ty) > speed) { status[f] = 3; continue; }
        double water = 0., fx = 0., fy = 0.;
        if (h > dry) {
            trace[f] = h; trace[nf + f] = h * (un * nx + tx); trace[2 * nf + f] = h * (un * ny + ty);
            water = trace[nf + f] * nx + trace[2 * nf + f] * ny;
            fx = water * trace[nf + f] / h + .5 * g * h * h * nx;
            fy = water * trace[2 * nf + f] / h + .5 * g * h * h * ny;
        }
        const double pressure = h0 > dry ? .5 * g * (h0 * h0 - geom * geom) : 0.;
        flux[f] = water; flux[nf + f] = fx + pressure * nx; flux[2 * nf + f] = fy + pressure * ny;
    }
    return 0;
}

/* The critical owner of segment b: the whole opening, then, when dry faces
 * split its chains into several wet groups, each group on its own with the
 * dry faces closed at their owners' pressure. 0 or a failure. */
static int om_crit_section(const om_ctx *m, int b, const double *q, const double *z, double *trace, double *flux,
                           int *status, int *branch, double *invariant, int *scratch)
{
    const int nf = m->nf;
    const double g = m->grav, dry = m->dry;
    const int *faces = m->boundary_faces + m->boundary_offset[b];
    const int n = m->boundary_offset[b + 1] - m->boundary_offset[b];
    int err = om_crit_group(m, faces, n, q, z, trace, flux, status, branch, invariant);
    if (!m->crit_seg_chain) return err;
    /* wet groups: runs of wet faces along each chain */
    int ngroup = 0, nflat = 0, *gfaces = scratch, *gend = scratch + n;
    for (int ch = m->crit_seg_chain[b]; ch < m->crit_seg_chain[b + 1]; ++ch) {
        int open = 0;
        for (int k = m->crit_chain_offset[ch]; k < m->crit_chain_offset[ch + 1]; ++k) {
            const int f = m->crit_chain_face[k], c = m->owner[f];
            const double h = q[c], geom = h + z[c] - m->exterior_bed[f];
            const int wet = (h > dry) && (geom > dry);
            if (wet) { gfaces[nflat++] = f; open = 1; }
            else if (open) { gend[ngroup++] = nflat; open = 0; }
        }
        if (open) gend[ngroup++] = nflat;
    }
    if (ngroup <= 1) return err;
    int worst = 0, start = 0;
    for (int gi = 0; gi < ngroup; ++gi) {
        const int e = om_crit_group(m, gfaces + start, gend[gi] - start, q, z, trace, flux, status, branch, invariant);
        if (e > worst) worst = e;
        start = gend[gi];
    }
    for (int ch = m->crit_seg_chain[b]; ch < m->crit_seg_chain[b + 1]; ++ch)
        for (int k = m->crit_chain_offset[ch]; k < m->crit_chain_offset[ch + 1]; ++k) {
            const int f = m->crit_chain_face[k], c = m->owner[f];
            const double h = q[c], geom = h + z[c] - m->exterior_bed[f];
            if ((h > dry) && (geom > dry)) continue;
            const double height = fmax(q[c], 0.), pressure = .5 * g * height * height;
            trace[f] = trace[nf + f] = trace[2 * nf + f] = 0.;
            flux[f] = 0.; flux[nf + f] = pressure * m->normal[f]; flux[2 * nf + f] = pressure * m->normal[nf + f];
            status[f] = 0;
        }
    return worst;
}

int om_exterior(om_ctx *m, const double *q, const double *z, double time,
                double *trace, double *flux, int *status, double *work,
                double *stage_out, double *total_out)
{
    const int nc = m->nc, nf = m->nf, nb = m->nb;
    const double dry = m->dry, gravity = m->grav;
    om_sample_forcing(m, time);
    {
        const int line = om_inlet_lines(m);
        if (line) return line;
    }
    const double *forcing = m->forcing;
    double *terms = work, *weights = work + 2 * (size_t)nf;
    for (int f = 0; f < nf; ++f) {
        const int c = m->owner[f];
        const double w = om_open(m, f) && q[c] > dry ? m->length[f] : 0.;
        terms[f] = (z[c] + q[c]) * w;
        terms[nf + f] = w;
    }
    om_segment_sums(m, terms, 2, stage_out);
    const int rmode = m->roughness_mode < 3 ? m->roughness_mode : 3;
    const int waqua = m->roughness_mode == 4;
    for (int f = 0; f < nf; ++f) {
        weights[f] = 0.;
        if (!om_open(m, f)) continue;
        const int b = m->bid[f], c = m->owner[f];
        const double *bed = m->exterior_bed;
        if (m->seg_mode[b] == 9) {
            const double h = fmax(forcing[nb + b] - bed[f], 0.);
            if (h > dry) weights[f] = h * m->length[f];
            continue;
        }
        if (m->seg_mode[b] != 6 || stage_out[nb + b] <= 0.) continue;
        const double h = fmax(q[c] + z[c] - bed[f], 0.);
        const double section = fmax(stage_out[b] / stage_out[nb + b] - bed[f], 0.);
        if (h > dry && section > 0.)
            weights[f] = pow(section, 1.5) * om_exterior_chezy(rmode, h, m->roughness_value, dry, gravity, waqua) * m->length[f];
    }
    om_segment_sums(m, weights, 1, total_out);
    int first = 0;
    for (int i = 0; i < nf; ++i) {
        status[i] = 0;
        for (int k = 0; k < 3; ++k) { trace[k * nf + i] = 0.; flux[k * nf + i] = 0.; }
        if (!om_open(m, i)) continue;
        const int b = m->bid[i], c = m->owner[i], mode = m->seg_mode[b];
        const double h0 = q[c], nx = m->normal[i], ny = m->normal[nf + i], bed = m->exterior_bed[i];
        if (mode == 4 || mode == 5 || mode == 9 || mode == 10 || mode == 11) continue;
        double h = fmax(h0 + z[c] - bed, 0.), geometric = h, ux = 0., uy = 0.;
        if (h0 > dry) { ux = q[nc + c] / h0; uy = q[2 * nc + c] / h0; }
        double un = ux * nx + uy * ny, tx = ux - un * nx, ty = uy - un * ny, normal_speed = 0.;
        int st = 0;
        if (mode == 6) {
            const double Q = forcing[b];
            if (Q > 0. && total_out[b] <= 0.) st = 1;
            else if (h > dry && Q > 0.) normal_speed = -Q * weights[i] / (total_out[b] * h * m->length[i]);
        } else if (mode == 3) {
            if (h0 <= dry) h = 0.;
            else if (h > dry) {
                if (un < sqrt(gravity * h)) st = 6;
                else normal_speed = un;
            }
        } else if (mode == 2) {
            const double prescribed = fmax(forcing[nb + b] - bed, 0.);
            if (m->stage_policy[b] && (h0 <= dry || h <= dry) && prescribed > dry) st = 4;
            else {
                if (h0 <= dry) h = 0.;
                if (h > dry) {
                    const double wave = sqrt(gravity * h);
                    if (un <= -wave) {
                        if (m->stage_policy[b]) st = 5;
                        else { normal_speed = 0.; tx = ty = 0.; }
                    } else {
                        const double target = fmax(forcing[nb + b] - bed, 0.);
                        double hb, ub;
                        om_stage_wave(h, un, target, gravity, &hb, &ub);
                        if (ub < 0. && m->stage_policy[b]) {
                            if (ub <= -sqrt(gravity * hb)) st = 5;
                            else { h = hb; normal_speed = ub; tx = ty = 0.; }
                        } else if (ub < 0.) { normal_speed = 0.; tx = ty = 0.; }
                        else { h = hb; normal_speed = ub; }
                    }
                }
            }
        } else st = 2;
        if (!st && (!isfinite(h) || !isfinite(normal_speed) || h < 0. ||
                    sqrt(normal_speed * normal_speed + tx * tx + ty * ty) > m->speed_limit)) st = 3;
        if (st) { status[i] = st; if (!first) first = st; continue; }
        double water = 0., fx = 0., fy = 0.;
        if (h > dry) {
            trace[i] = h;
            trace[nf + i] = h * (normal_speed * nx + tx);
            trace[2 * nf + i] = h * (normal_speed * ny + ty);
            water = trace[nf + i] * nx + trace[2 * nf + i] * ny;
            fx = water * trace[nf + i] / h + .5 * gravity * h * h * nx;
            fy = water * trace[2 * nf + i] / h + .5 * gravity * h * h * ny;
        }
        double pressure = h0 > dry ? .5 * gravity * (h0 * h0 - geometric * geometric) : 0.;
        flux[i] = water; flux[nf + i] = fx + pressure * nx; flux[2 * nf + i] = fy + pressure * ny;
    }
    /* section owners of the remaining outlet modes, in the reference's order
     * (river_exterior_bed.py:213-217): a normal-depth failure rejects the
     * trial before the rating owner runs; a rating failure is fatal */
    if (om_has_inlet(m)) {
        int inlet_failed = 0;
        for (int b = 0; b < nb; ++b)
            if (m->seg_mode[b] == 9 && om_inlet_section(m, b, q, z, trace, flux, status)) inlet_failed = 1;
        if (inlet_failed) return OM_REJECT_SPATIAL;
    }
    {
        int any = 0;
        for (int b = 0; b < nb; ++b) any = any || m->seg_mode[b] == 4;
        if (any) {
            int *branch = (int *)calloc((size_t)nf, sizeof(int));
            double *invariant = (double *)calloc((size_t)nf, sizeof(double));
            int *scratch = (int *)calloc(2 * (size_t)nf + 2, sizeof(int));
            int crit_failed = 0;
            for (int b = 0; b < nb; ++b)
                if (m->seg_mode[b] == 4 && om_crit_section(m, b, q, z, trace, flux, status, branch, invariant, scratch))
                    crit_failed = 1;
            free(branch); free(invariant); free(scratch);
            if (crit_failed) return OM_REJECT_SPATIAL;
        }
    }
    if (m->weir) {
        int *branch = (int *)calloc((size_t)nf, sizeof(int));
        double *invariant = (double *)calloc((size_t)nf, sizeof(double));
        int weir_failed = 0;
        for (int b = 0; b < nb; ++b)
            if (m->seg_mode[b] == 5 && om_weir_section(m, b, q, z, trace, flux, status, branch, invariant)) {
                weir_failed = 1;
                break;
            }
        free(branch); free(invariant);
        if (weir_failed) return OM_REJECT_SPATIAL;
    }
    int normal_failed = 0;
    for (int ch = 0; ch < m->nchain; ++ch)
        if (om_normal_chain(m, ch, q, z, trace, flux, status)) normal_failed = 1;
    if (normal_failed) return OM_REJECT_SPATIAL;
    for (int b = 0; b < nb; ++b)
        if (m->seg_mode[b] == 11 && om_rating_outlet(m, b, q, z, trace, flux, status)) return OM_EXTERIOR_FATAL;
    if (!first)
        for (int i = 0; i < nf; ++i)
            if (status[i]) { first = status[i]; break; }
    return first;
}

static int om_is_outlet(int mode)
{
    return mode == 2 || mode == 3 || mode == 4 || mode == 5 || mode == 10 || mode == 11;
}

/* Cap outward outlet flux by the owner's start-of-stage stock
 * (OutletFeasibility.__call__). Sums follow the boundary face order.
 * work needs 3*nc doubles (only boundary owners are touched). */
void om_outlet_feasibility(const om_ctx *m, const double *base, double dt, double *flux, double *trace,
                           double *work)
{
    const int nc = m->nc, nf = m->nf, nb = m->nb;
    const int nbf = m->boundary_offset[nb];
    double *total = work, *reserved = work + nc, *factor = work + 2 * (size_t)nc;
    for (int k = 0; k < nbf; ++k) { const int c = m->owner[m->boundary_faces[k]]; total[c] = 0.0; reserved[c] = 0.0; }
    for (int k = 0; k < nbf; ++k) {
        const int f = m->boundary_faces[k], c = m->owner[f];
        const int out = om_is_outlet(m->seg_mode[m->bid[f]]);
        const double debit = fmax(flux[f], 0.) * m->length[f];
        if (out) total[c] += debit; else reserved[c] += debit;
    }
    for (int k = 0; k < nbf; ++k) {
        const int c = m->owner[m->boundary_faces[k]];
        const double available = fmax(0., base[c] * m->area[c] / dt - reserved[c]);
        const double ratio = fmin(1., available / fmax(total[c], 1e-300)) * (1. - 32. * OM_EPS);
        factor[c] = total[c] > available ? ratio : 1.;
    }
    for (int k = 0; k < nbf; ++k) {
        const int f = m->boundary_faces[k], c = m->owner[f];
        const int out = om_is_outlet(m->seg_mode[m->bid[f]]);
        const double water = flux[f];
        const double scale = (out && water > 0.) ? factor[c] : 1.;
        const double depth = trace[f], denom = fmax(depth, 1e-300);
        const double ux = depth > 0. ? trace[nf + f] / denom : 0.;
        const double uy = depth > 0. ? trace[2 * nf + f] / denom : 0.;
        flux[nf + f] += (scale * scale - 1.) * water * ux;
        flux[2 * nf + f] += (scale * scale - 1.) * water * uy;
        flux[f] = water * scale;
        trace[nf + f] *= scale;
        trace[2 * nf + f] *= scale;
    }
}

/* ------------------------------------------------------------------ */
/* Positivity: donor inventory, boundary reservation, face limiting     */
/* ------------------------------------------------------------------ */

void om_inventory(const om_ctx *m, double dt, const double *base, const double *water, double *theta)
{
    const int nc = m->nc;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nc; ++i) {
        double out = 0.;
        for (int k = m->offset[i]; k < m->offset[i + 1]; ++k) {
            const int f = m->faces[k];
            out += fmax(m->signs[k] * water[f], 0.) * m->length[f];
        }
        theta[i] = 1.;
        if (out > 0. && dt * out >= base[i] * m->area[i])
            theta[i] = fmin(1., base[i] * m->area[i] / (dt * out)) * (1. - 32. * 2.2204460492503131e-16);
    }
}

/* Reserve prescribed boundary debits before limiting interior donors
 * (ExplicitBoundaryBudget.reserve). Returns OM_REJECT_BUDGET when an open
 * boundary alone would take more than the owner holds. */
int om_reserve(const om_ctx *m, double dt, const double *base, const double *water, double *theta)
{
    const int nb = m->nb, nbf = m->boundary_offset[nb];
    int reject = 0;
    for (int kk = 0; kk < nbf; ++kk) {
        const int c = m->owner[m->boundary_faces[kk]];
        /* visit each boundary owner once: the first boundary face it owns */
        int seen = 0;
        for (int j = 0; j < kk; ++j) if (m->owner[m->boundary_faces[j]] == c) { seen = 1; break; }
        if (seen) continue;
        double ext = 0., interior = 0.;
        for (int k = m->offset[c]; k < m->offset[c + 1]; ++k) {
            const int f = m->faces[k];
            const double debit = fmax(m->signs[k] * water[f], 0.) * m->length[f];
            if (om_open(m, f)) ext += debit; else interior += debit;
        }
        const double available = base[c] * m->area[c] / dt;
        if (ext > available) reject = 1;
        const double factor = fmin(1., (available - ext) / fmax(interior, 1e-300)) * (1. - 32. * OM_EPS);
        theta[c] = (interior > 0. && interior >= available - ext) ? factor : 1.;
    }
    return reject ? OM_REJECT_BUDGET : OM_OK;
}

/* Limit each donor's outgoing water by theta and move the removed
 * advective momentum with it (midpoint_faces). Open faces keep their
 * budgeted flux (they are restored by the boundary budget). */
void om_limit_faces(const om_ctx *m, const double *q, const double *theta, double *water, double *correction)
{
    const int nc = m->nc, nf = m->nf;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nf; ++i) {
        correction[i] = 0.; correction[nf + i] = 0.;
        if (water[i] == 0.) continue;
        if (om_open(m, i)) continue;
        const int donor = water[i] < 0. ? m->neighbour[i] : m->owner[i];
        if (donor < 0 || theta[donor] == 1.) continue;
        const double delta = (theta[donor] - 1.) * water[i];
        water[i] *= theta[donor];
        if (q[donor] > m->dry) {
            correction[i] = delta * q[nc + donor] / q[donor];
            correction[nf + i] = delta * q[2 * nc + donor] / q[donor];
        }
    }
}

/* Replace the mass rate with the limited water divergence and add the
 * momentum corrections (midpoint_gather). */
void om_limit_gather(const om_ctx *m, const double *water, const double *correction, double *rate)
{
    const int n = m->nc, nf = m->nf;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double mass = 0., mx = 0., my = 0.;
        for (int k = m->offset[i]; k < m->offset[i + 1]; ++k) {
            const int f = m->faces[k];
            const double w = m->signs[k] * m->length[f] / m->area[i];
            mass -= w * water[f]; mx -= w * correction[f]; my -= w * correction[nf + f];
        }
        rate[i] = mass; rate[n + i] += mx; rate[2 * n + i] += my;
    }
}

/* Face-sum CFL frequency per cell; open faces use the larger of the owner
 * and exterior trace wave speeds (explicit_frequency). */
double om_frequency(const om_ctx *m, const double *q, const double *speed, const double *ext_trace, double *freq)
{
    const int n = m->nc, nf = m->nf;
    const double dry = m->dry, grav = m->grav;
    double peak = 0.0;
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(max:peak) reduction(|:bad)
    for (int i = 0; i < n; ++i) {
        double sum = 0.;
        for (int k = m->offset[i]; k < m->offset[i + 1]; ++k) {
            const int f = m->faces[k];
            double s = speed[f];
            if (om_open(m, f)) {
                const int o = m->owner[f];
                const double h = q[o], hb = ext_trace[f], nx = m->normal[f], ny = m->normal[nf + f];
                const double a = h > dry ? fabs((q[n + o] * nx + q[2 * n + o] * ny) / h) + sqrt(grav * h) : 0.;
                const double b = hb > dry ? fabs((ext_trace[nf + f] * nx + ext_trace[2 * nf + f] * ny) / hb) + sqrt(grav * hb) : 0.;
                s = fmax(a, b);
            }
            sum += m->length[f] * s;
        }
        freq[i] = sum / m->area[i];
        if (!isfinite(freq[i])) bad = 1;
        if (freq[i] > peak) peak = freq[i];
    }
    return bad ? NAN : peak;
}

/* ------------------------------------------------------------------ */
/* Manning / Chezy cell drag (river_cell_drag)                          */
/* ------------------------------------------------------------------ */
static double om_chezy(int method, double depth, double value)
{
    if (method == 1) return value;
    if (method == 2) return pow(depth, 1. / 6.) / value;
    if (method == 3) return sqrt(9.81) / .41 * log1p(30. * depth / (exp(1.) * value));
    return 18. * log10(12. * fmax(.5, depth / value));
}

void om_drag(const om_ctx *m, double dt, double *q)
{
    const int n = m->nc;
    const double g = m->grav, dry = m->dry;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const double h = q[i];
        if (h <= dry) { q[n + i] = q[2 * n + i] = 0.; continue; }
        const double c = om_chezy(m->roughness_mode, h, m->roughness_value);
        const double speed = sqrt(q[n + i] * q[n + i] + q[2 * n + i] * q[2 * n + i]) / h;
        const double factor = 1. / (1. + dt * g * speed / (c * c * h));
        q[n + i] *= factor; q[2 * n + i] *= factor;
    }
}

/* ------------------------------------------------------------------ */
/* Orchestration                                                        */
/* ------------------------------------------------------------------ */

/* Scratch for one spatial evaluation. */
/* ------------------------------------------------------------------ */
/* Turbines: Thetis actuator sink, coverage gate, balanced pressure    */
/* ------------------------------------------------------------------ */
enum { OM_TURB_FIELDS = 16 };
/* per-rotor parameter record (doubles): D, hub elevation, minimum bed and
 * surface clearances, tolerance, mode, Ct, Cp (constant mode, Cp resolved) */
enum { OM_TP_D = 0, OM_TP_HUB, OM_TP_BEDCLEAR, OM_TP_SURFCLEAR, OM_TP_TOL, OM_TP_MODE, OM_TP_CT, OM_TP_CP, OM_TP_N };
/* control modes */
enum { OM_CONSTANT = 0, OM_SPEED_TABLE = 1, OM_INCIDENT_TABLE = 2, OM_INCIDENT_CURVES = 3 };
/* diagnostic record fields */
enum { OM_TD_ACTIVE = 0, OM_TD_REASON, OM_TD_MARGIN, OM_TD_CLEARANCE, OM_TD_U1, OM_TD_U0, OM_TD_DEPTH,
       OM_TD_CT, OM_TD_CP, OM_TD_FORCE, OM_TD_POWER, OM_TD_REMOVED, OM_TD_LOW, OM_TD_HIGH, OM_TD_ERROR };
/* inactive reasons, in the order the gate tests them */
enum { OM_R_COVERED = 0, OM_R_DEPTH, OM_R_BED, OM_R_SURFCLEAR, OM_R_BEDCLEAR, OM_R_DRY, OM_R_REVERSE,
       OM_R_NOFLOW, OM_R_CUTIN };

typedef struct om_turbines {
    int nr;
    const int *support_offset, *support_cell;          /* (nr+1), (ns) */
    const double *support_weight, *support_density;    /* normalized bump weight, density integral */
    const int *plane_offset, *plane_cell;              /* (nr+1), (np) */
    const double *plane_delta;                         /* (2, np) */
    const double *param;                               /* (nr, OM_TP_N) */
    const int *curve;                                  /* (nr, 4): thrust first, count; power first, count */
    const double *curve_x, *curve_y;
    const double *nu;                                  /* (nc) ambient viscosity, NULL: none */
    int pressure;                                      /* balanced-pressure correction on */
    const double *dxdy, *inverse, *xy, *mdisp;         /* (2,nadj) (3,nc) (2,nc) (4,nf) */
    double *diag;                                      /* (nr, OM_TURB_FIELDS) last evaluation */
    double *grad, *raw, *face, *work, *trace, *kcell;  /* scratch (10,nc) (3,nc) (2,nf) (3,nc) (10,nf) (ns) */
    int *fstatus;                                      /* (nf) */
} om_turbines;

/* Wet-only least-squares gradients of u, v, eta and the bed (river_turbine_flow.h:13-37). */
void om_hkt_gradients(const om_ctx *m, const om_turbines *T, const double *q, const double *z, double *out)
{
    const int n = m->nc, na = m->nadj;
    const double dry = m->dry;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        for (int k = 0; k < 10; ++k) out[k * n + i] = 0.;
        double xx = 0., xy = 0., yy = 0., bx[3] = {0., 0., 0.}, by[3] = {0., 0., 0.}, bz[2] = {0., 0.};
        const int wet = q[i] > dry;
        for (int s = m->offset[i]; s < m->offset[i + 1]; ++s) {
            const int j = om_other(m, s);
            if (j < 0) continue;
            const double dx = T->dxdy[s], dy = T->dxdy[na + s], w = 1. / (dx * dx + dy * dy), dz = z[j] - z[i];
            bz[0] += w * dx * dz; bz[1] += w * dy * dz;
            if (!wet || q[j] <= dry) continue;
            xx += w * dx * dx; xy += w * dx * dy; yy += w * dy * dy;
            const double d[3] = {q[n + j] / q[j] - q[n + i] / q[i], q[2 * n + j] / q[j] - q[2 * n + i] / q[i],
                                 (q[j] + z[j]) - (q[i] + z[i])};
            for (int k = 0; k < 3; ++k) { bx[k] += w * dx * d[k]; by[k] += w * dy * d[k]; }
        }
        out[6 * n + i] = T->inverse[i] * bz[0] + T->inverse[n + i] * bz[1];
        out[7 * n + i] = T->inverse[n + i] * bz[0] + T->inverse[2 * n + i] * bz[1];
        const double det = xx * yy - xy * xy;
        if (det > 1e-12 * fmax(1., xx * yy))
            for (int k = 0; k < 3; ++k) {
                out[2 * k * n + i] = (yy * bx[k] - xy * by[k]) / det;
                out[(2 * k + 1) * n + i] = (xx * by[k] - xy * bx[k]) / det;
            }
    }
}

/* numpy.interp on one table, zero outside [x0, xlast) (river_turbine_thetis.py:158-172) */
static double om_lookup(const double *x, const double *y, int count, double v)
{
    if (!(v >= x[0]) || v >= x[count - 1]) return 0.;
    int j = 0;
    while (j + 1 < count - 1 && x[j + 1] <= v) ++j;
    if (v == x[j]) return y[j];
    const double slope = (y[j + 1] - y[j]) / (x[j + 1] - x[j]);
    return slope * (v - x[j]) + y[j];
}

/* Per-cell Thetis terms K, P, U, Ct, Cp (river_turbine_thetis.py:175-216). Returns 0 or an error. */
static int om_cell_terms(const om_turbines *T, int r, double depth, double u, double v, double out[5])
{
    const double *p = T->param + (size_t)r * OM_TP_N;
    const double D = p[OM_TP_D];
    const int mode = (int)p[OM_TP_MODE];
    const int *cv = T->curve + 4 * r;
    const double *tx = T->curve_x + cv[0], *ty = T->curve_y + cv[0], *px = T->curve_x + cv[2], *py = T->curve_y + cv[2];
    const double speed = hypot(u, v);
    const double area = OM_PI * (D * D) / 4;
    if (mode == OM_INCIDENT_TABLE || mode == OM_INCIDENT_CURVES) {
        if (depth < D * (1 - 1e-10)) return 2;
        const double c = OM_PI * D / (4 * depth);
        double low = tx[0], high = tx[cv[1] - 1];
        const double smin = low * .5 * (1 + sqrt(1 - c * ty[0]));
        const double smax = high * .5 * (1 + sqrt(1 - c * ty[cv[1] - 1]));
        const int active = speed >= smin && speed < smax;
        for (int it = 0; it < 44; ++it) {
            const double mid = .5 * (low + high);
            const double ct = om_lookup(tx, ty, cv[1], mid);
            const double local = mid * .5 * (1 + sqrt(1 - c * ct));
            if (local < speed) low = mid; else high = mid;
        }
        const double incident = active ? .5 * (low + high) : speed;
        const double ct = active ? om_lookup(tx, ty, cv[1], incident) : 0.;
        const double cp = active ? om_lookup(px, py, cv[3], incident) : 0.;
        const double alpha = .5 * (1 + sqrt(1 - c * ct));
        out[0] = area * ct / (2 * (alpha * alpha));
        out[1] = .5 * area * cp * (incident * incident * incident);
        out[2] = incident; out[3] = ct; out[4] = cp;
        return 0;
    }
    double ct, cp;
    if (mode == OM_CONSTANT) ct = p[OM_TP_CT];
    else ct = om_lookup(tx, ty, cv[1], speed);
    const double radicand = 1 - area * ct / (D * depth);
    if (radicand < 0) return 1;
    const double alpha = .5 * (1 + sqrt(radicand));
    const double incident = speed / alpha;
    if (mode == OM_CONSTANT) cp = p[OM_TP_CP];
    else cp = om_lookup(px, py, cv[3], incident);
    out[0] = area * ct / (2 * (alpha * alpha));
    out[1] = .5 * area * cp * (incident * incident * incident);
    out[2] = incident; out[3] = ct; out[4] = cp;
    return 0;
}

/* One rotor's sample (ThetisRotor.sample with the CoveredRotor gate) and its
 * sink coefficient per support cell. Returns 0 or an error code. */
static int om_turbine_sample(const om_ctx *m, const om_turbines *T, int r, const double *q, const double *z,
                             const double *grad, double *kcell, double *diag)
{
    const int n = m->nc, np_ = T->plane_offset[T->nr];
    const double dry = m->dry;
    const double *p = T->param + (size_t)r * OM_TP_N;
    const double D = p[OM_TP_D], tol = p[OM_TP_TOL];
    const double top = p[OM_TP_HUB] + D / 2, bottom = p[OM_TP_HUB] - D / 2;
    const int mode = (int)p[OM_TP_MODE];
    double low = INFINITY, high = -INFINITY;
    for (int j = T->plane_offset[r]; j < T->plane_offset[r + 1]; ++j) {
        const int c = T->plane_cell[j];
        const double eta = q[c] + z[c];
        const double surface = eta + grad[4 * n + c] * T->plane_delta[j] + grad[5 * n + c] * T->plane_delta[np_ + j];
        const double bed = z[c] + grad[6 * n + c] * T->plane_delta[j] + grad[7 * n + c] * T->plane_delta[np_ + j];
        low = fmin(low, fmin(surface, eta)); high = fmax(high, fmax(bed, z[c]));
    }
    int support_dry = 0, below = 0;
    double u1 = 0., depth = 0.;
    const int *cv = T->curve + 4 * r;
    for (int e = T->support_offset[r]; e < T->support_offset[r + 1]; ++e) {
        const int c = T->support_cell[e];
        const double h = q[c], u = q[n + c] / fmax(h, dry), v = q[2 * n + c] / fmax(h, dry);
        const double speed = hypot(u, v), w = T->support_weight[e];
        if (h <= dry) support_dry = 1;
        u1 += w * speed; depth += w * h;
        kcell[e] = 0.;
        if (mode != OM_CONSTANT) {
            double minimum = T->curve_x[cv[0]];
            if (mode != OM_SPEED_TABLE)
                minimum = minimum * .5 * (1 + sqrt(1 - OM_PI * D * T->curve_y[cv[0]] / (4 * h)));
            if (speed < minimum) below = 1;
        }
    }
    const double margin = low - top, clearance = bottom - high;
    int reason = OM_R_COVERED;
    if (margin < tol) reason = OM_R_DEPTH;
    else if (clearance < tol) reason = OM_R_BED;
    else if (margin + tol < p[OM_TP_SURFCLEAR]) reason = OM_R_SURFCLEAR;
    else if (clearance + tol < p[OM_TP_BEDCLEAR]) reason = OM_R_BEDCLEAR;
    else if (support_dry) reason = OM_R_DRY;
    int active = reason == OM_R_COVERED;
    if (active && u1 <= 1e-10) { active = 0; reason = u1 < 0 ? OM_R_REVERSE : OM_R_NOFLOW; }
    if (active && mode != OM_CONSTANT && below) { active = 0; reason = OM_R_CUTIN; }
    for (int k = 0; k < OM_TURB_FIELDS; ++k) diag[k] = 0.;
    diag[OM_TD_ACTIVE] = active; diag[OM_TD_REASON] = reason;
    diag[OM_TD_MARGIN] = margin; diag[OM_TD_CLEARANCE] = clearance;
    diag[OM_TD_U1] = u1; diag[OM_TD_U0] = u1; diag[OM_TD_DEPTH] = depth;
    diag[OM_TD_LOW] = low; diag[OM_TD_HIGH] = high;
    if (!active) return 0;
    double F = 0., work = 0., P = 0., incoming = 0., ctm = 0., cpm = 0.;
    for (int e = T->support_offset[r]; e < T->support_offset[r + 1]; ++e) {
        const int c = T->support_cell[e];
        const double h = q[c], u = q[n + c] / fmax(h, dry), v = q[2 * n + c] / fmax(h, dry);
        const double speed = hypot(u, v), w = T->support_weight[e], density = T->support_density[e];
        double t[5];
        const int err = om_cell_terms(T, r, h, u, v, t);
        if (err) { diag[OM_TD_ERROR] = err; return err; }
        kcell[e] = t[0] * density / m->area[c];
        F += t[0] * density * (speed * speed);
        work += t[0] * density * (speed * speed * speed);
        P += t[1] * density;
        incoming += w * t[2]; ctm += w * t[3]; cpm += w * t[4];
    }
    diag[OM_TD_FORCE] = F; diag[OM_TD_REMOVED] = work; diag[OM_TD_POWER] = P;
    diag[OM_TD_U0] = incoming; diag[OM_TD_CT] = ctm; diag[OM_TD_CP] = cpm;
    return 0;
}

/* Face traces of the hydrostatically reconstructed states (river_turbine_flow.h:39-52). */
static void om_hkt_surface_pack(const om_ctx *m, const double *local, const int *constant, double *out)
{
    const int nf = m->nf;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nf; ++i) {
        for (int k = 0; k < 10; ++k) out[k * nf + i] = 0.;
        if (m->neighbour[i] < 0) continue;
        const double hl = local[i], hr = local[4 * nf + i];
        out[i] = hl + local[3 * nf + i]; out[nf + i] = hr + local[7 * nf + i];
        out[2 * nf + i] = hl > 0. ? local[nf + i] / hl : 0.; out[3 * nf + i] = hr > 0. ? local[5 * nf + i] / hr : 0.;
        out[4 * nf + i] = hl > 0. ? hypot(local[nf + i], local[2 * nf + i]) / hl : 0.;
        out[5 * nf + i] = hr > 0. ? hypot(local[5 * nf + i], local[6 * nf + i]) / hr : 0.;
        out[6 * nf + i] = local[3 * nf + i]; out[7 * nf + i] = local[7 * nf + i];
        out[8 * nf + i] = constant[m->owner[i]]; out[9 * nf + i] = constant[m->neighbour[i]];
    }
}

/* Balanced face pressure correction (river_turbine_flow.h:54-82). */
void om_hkt_pressure(const om_ctx *m, const om_turbines *T, const double *q, const double *z, const double *trace,
                     const double *grad, const double *source, double *out, int *status)
{
    const int nf = m->nf, n = m->nc;
    const double gravity = m->grav, dry = m->dry;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nf; ++i) {
        out[i] = 0.; out[nf + i] = 0.; status[i] = 0;
        const int a = m->owner[i], b = m->neighbour[i];
        if (b < 0) continue;
        if (q[a] <= dry || q[b] <= dry) { status[i] = 1; continue; }
        const double bed = fmax(fmax(z[a], z[b]), fmax(trace[6 * nf + i], trace[7 * nf + i]));
        const double ha = fmax(0., q[a] + z[a] - bed), hb = fmax(0., q[b] + z[b] - bed);
        const double hl = fmax(0., trace[i] - bed), hr = fmax(0., trace[nf + i] - bed);
        if (fmin(fmin(ha, hb), fmin(hl, hr)) <= dry) { status[i] = 1; continue; }
        const double h = .5 * (hl + hr);
        if (fabs(hr - hl) > .005 * h) { status[i] = 2; continue; }
        const double old = .25 * gravity * (hl * hl + hr * hr);
        double po = old, pn = old;
        if (trace[8 * nf + i] != 0.) po += .5 * gravity * (ha * ha - hl * hl);
        if (trace[9 * nf + i] != 0.) pn += .5 * gravity * (hb * hb - hr * hr);
        if (fabs(po - pn) > 128. * OM_EPS * fmax(1., fmax(fabs(po), fabs(pn)))) { status[i] = 3; continue; }
        const double da = m->distance[i], db = m->distance[nf + i], d = da + db, wa = db / d, wb = da / d;
        const double sx = wa * T->mdisp[i] + wb * T->mdisp[2 * nf + i];
        const double sy = wa * T->mdisp[nf + i] + wb * T->mdisp[3 * nf + i];
        double pressure = .5 * gravity * (wa * ha * ha + wb * hb * hb);
        pressure += gravity * sx * (wa * ha * grad[4 * n + a] + wb * hb * grad[4 * n + b]);
        pressure += gravity * sy * (wa * ha * grad[5 * n + a] + wb * hb * grad[5 * n + b]);
        const double nx = m->normal[i], ny = m->normal[nf + i];
        pressure += da * db / d * ((source[n + a] - source[n + b]) * nx + (source[2 * n + a] - source[2 * n + b]) * ny);
        double delta = .5 * (po + pn) - pressure;
        const double speed = sqrt(gravity * h), theta = fmin(1., fmax(trace[4 * nf + i], trace[5 * nf + i]) / speed);
        delta -= .5 * (1. - theta) * speed * (2. * hl * hr / (hl + hr)) * (trace[3 * nf + i] - trace[2 * nf + i]);
        out[i] = delta * nx; out[nf + i] = delta * ny;
    }
}

/* Symmetric-strain ambient stress (river_hydrokinetic_stress.h:13-35). */
void om_hkt_stress(const om_ctx *m, const om_turbines *T, const double *q, const double *z, const double *grad,
                   double *out)
{
    const int nf = m->nf, n = m->nc;
    const double dry = m->dry;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nf; ++i) {
        out[i] = 0.; out[nf + i] = 0.;
        const int o = m->owner[i], j = m->neighbour[i];
        if (j < 0 || q[o] <= dry || q[j] <= dry) continue;
        double h = fmin(q[o], q[j]);
        h = fmin(h, fmax(0., .5 * (q[o] + z[o] + q[j] + z[j]) - fmax(z[o], z[j])));
        const double d = m->distance[i] + m->distance[nf + i], wo = m->distance[nf + i] / d, wj = m->distance[i] / d;
        const double visc = wo * T->nu[o] + wj * T->nu[j];
        const double nx = m->normal[i], ny = m->normal[nf + i];
        const double dx = T->xy[j] - T->xy[o], dy = T->xy[n + j] - T->xy[n + o];
        const double dn = dx * nx + dy * ny;
        const double du = q[n + j] / q[j] - q[n + o] / q[o], dv = q[2 * n + j] / q[j] - q[2 * n + o] / q[o];
        double ux = wo * grad[o] + wj * grad[j], uy = wo * grad[n + o] + wj * grad[n + j];
        double vx = wo * grad[2 * n + o] + wj * grad[2 * n + j], vy = wo * grad[3 * n + o] + wj * grad[3 * n + j];
        const double cu = (du - ux * dx - uy * dy) / dn, cv = (dv - vx * dx - vy * dy) / dn;
        ux += cu * nx; uy += cu * ny; vx += cv * nx; vy += cv * ny;
        out[i] = visc * h * (2. * ux * nx + (uy + vx) * ny);
        out[nf + i] = visc * h * ((uy + vx) * nx + 2. * vy * ny);
    }
}

/* work(1:2) = sum_k s len flux / area, then rate(1:2) += work(1:2)
 * (flow2dh_fixed_bed_kernels.h:54-60 with unit depth weights). */
static void om_face_momentum_add(const om_ctx *m, const double *flux, double *rate)
{
    const int n = m->nc, nf = m->nf;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double x = 0., y = 0.;
        for (int k = m->offset[i]; k < m->offset[i + 1]; ++k) {
            const int f = m->faces[k];
            x += m->signs[k] * m->length[f] * flux[f];
            y += m->signs[k] * m->length[f] * flux[nf + f];
        }
        rate[n + i] += (1. * x / m->area[i]);
        rate[2 * n + i] += (1. * y / m->area[i]);
    }
}

typedef struct {
    double *v, *grad, *trace, *local, *riemann, *fl, *fr, *speed, *ext_trace, *ext_flux, *work,
           *theta, *correction, *freq, *stage, *total;
    int *active, *pstatus, *constant, *kind, *rstatus, *closed, *astatus, *fstatus, *estatus;
} om_scratch;

static void *om_alloc(size_t bytes) { void *p = calloc(bytes ? bytes : 1, 1); return p; }

om_scratch *om_scratch_create(const om_ctx *m)
{
    const size_t nc = m->nc, nf = m->nf;
    om_scratch *s = (om_scratch *)om_alloc(sizeof(om_scratch));
    s->v = om_alloc(4 * nc * 8); s->grad = om_alloc(8 * nc * 8); s->trace = om_alloc(10 * nf * 8);
    s->local = om_alloc(8 * nf * 8); s->riemann = om_alloc(18 * nf * 8); s->fl = om_alloc(3 * nf * 8);
    s->fr = om_alloc(3 * nf * 8); s->speed = om_alloc(nf * 8); s->ext_trace = om_alloc(3 * nf * 8);
    s->ext_flux = om_alloc(3 * nf * 8); s->work = om_alloc((3 * nf + 3 * nc) * 8); s->theta = om_alloc(nc * 8);
    s->correction = om_alloc(2 * nf * 8); s->freq = om_alloc(nc * 8);
    s->stage = om_alloc((2 * (size_t)m->nb + 1) * 8); s->total = om_alloc(((size_t)m->nb + 1) * 8);
    s->active = om_alloc(nc * 4); s->pstatus = om_alloc(nc * 4); s->constant = om_alloc(nc * 4);
    s->kind = om_alloc(nf * 4); s->rstatus = om_alloc(nf * 4); s->closed = om_alloc(nf * 4);
    s->astatus = om_alloc(nf * 4); s->fstatus = om_alloc(nf * 4); s->estatus = om_alloc(nf * 4);
    return s;
}

void om_scratch_destroy(om_scratch *s)
{
    if (!s) return;
    void *all[] = {s->v, s->grad, s->trace, s->local, s->riemann, s->fl, s->fr, s->speed, s->ext_trace,
                   s->ext_flux, s->work, s->theta, s->correction, s->freq, s->stage, s->total, s->active,
                   s->pstatus, s->constant, s->kind, s->rstatus, s->closed, s->astatus, s->fstatus, s->estatus};
    for (size_t i = 0; i < sizeof(all) / sizeof(all[0]); ++i) free(all[i]);
    free(s);
}

/* Momentum sources of an installed rotor array, in the order of the
 * reference's add_momentum: ambient stress, actuator sinks, balanced
 * pressure (river_turbine_flow.py:230-239). Returns 0 or an error code. */
int om_turbine_momentum(const om_ctx *m, om_scratch *s, const double *q, const double *z, double *rate)
{
    om_turbines *T = (om_turbines *)m->turb;
    const int n = m->nc;
    om_hkt_gradients(m, T, q, z, T->grad);
    if (T->nu) {
        om_hkt_stress(m, T, q, z, T->grad, T->face);
        om_face_momentum_add(m, T->face, rate);
    }
    memset(T->raw, 0, sizeof(double) * 3 * (size_t)n);
    int err = 0;
    for (int r = 0; r < T->nr; ++r) {
        const int e = om_turbine_sample(m, T, r, q, z, T->grad, T->kcell, T->diag + (size_t)r * OM_TURB_FIELDS);
        if (e && !err) err = e;
        for (int k = T->support_offset[r]; k < T->support_offset[r + 1]; ++k) {
            const int c = T->support_cell[k];
            const double h = q[c], u = q[n + c] / fmax(h, m->dry), v = q[2 * n + c] / fmax(h, m->dry);
            const double speed = hypot(u, v);
            T->raw[n + c] -= T->kcell[k] * speed * u;
            T->raw[2 * n + c] -= T->kcell[k] * speed * v;
        }
    }
    if (err) return err;
    for (int i = 0; i < n; ++i) { rate[n + i] += T->raw[n + i]; rate[2 * n + i] += T->raw[2 * n + i]; }
    if (T->pressure) {
        om_hkt_surface_pack(m, s->local, s->constant, T->trace);
        om_hkt_pressure(m, T, q, z, T->trace, T->grad, T->raw, T->face, T->fstatus);
        om_face_momentum_add(m, T->face, rate);
    }
    return 0;
}

/* Rotor diagnostics of a state (the reference's hkt_diagnose): gradients, then every rotor's sample. */
int om_turbine_diagnose(const om_ctx *m, const double *q, const double *z)
{
    om_turbines *T = (om_turbines *)m->turb;
    om_hkt_gradients(m, T, q, z, T->grad);
    int err = 0;
    for (int r = 0; r < T->nr; ++r) {
        const int e = om_turbine_sample(m, T, r, q, z, T->grad, T->kcell, T->diag + (size_t)r * OM_TURB_FIELDS);
        if (e && !err) err = e;
    }
    return err;
}

/* ------------------------------------------------------------------ */
/* Exner bed update with MPM transport (one grain size)                */
/* ------------------------------------------------------------------ */
typedef struct {
    double diameter, porosity, chezy, morfac, sediment_depth;
    const int *bedbc;                                  /* (nf) 0 wall, 1 feed, 2 outflow, 3 capacity */
    const double *feed, *rock;                         /* (nf) (nc) */
    const double *dxdy, *inverse, *xy;                 /* (2,nadj) (3,nc) (2,nc) */
} om_exner_params;

typedef struct { int ok; double residual, boundary, donor, change; } om_exner_stats;

/* Koch--Flokstra slope correction, FLOW ISlope = 3 with alfabs = alfabn = 0,
 * ashld .85, bshld .5, cshld = dshld = 0 (flow_bed_slope_runtime.cu:13-144). */
static int om_slope3(double qx, double qy, double down_x, double down_y, double stress, double *cx, double *cy)
{
    *cx = qx; *cy = qy;
    if (!isfinite(qx) || !isfinite(qy) || !isfinite(down_x) || !isfinite(down_y) || !isfinite(stress) || stress < 0.0)
        return 2;
    double magnitude = sqrt(qx * qx + qy * qy);
    if (!isfinite(magnitude)) return 2;
    if (magnitude <= 1.0e-6) return 0;
    const double alfabs = 0., ashld = .85, bshld = .5;
    double dzds = down_x * qx / magnitude + down_y * qy / magnitude;
    const double tan_phi = tan((double)(30.0f / 180.0f) * acos(-1.0));
    dzds = fmin((double)0.9f * tan_phi, dzds);
    double ftheta = 0.0;
    if (stress != 0.0) ftheta = ashld * pow(stress, bshld) * pow(1.0, 0.0) * pow(1.0, 0.0);
    double dirx, diry;
    if (down_x != 0.0 || down_y != 0.0) { dirx = ftheta * qx / magnitude + down_x; diry = ftheta * qy / magnitude + down_y; }
    else { dirx = qx / magnitude; diry = qy / magnitude; }
    const double norm = sqrt(dirx * dirx + diry * diry);
    if (!isfinite(norm) || norm <= 2.2250738585072014e-308) return 3;
    magnitude = magnitude * (1.0 + alfabs * dzds);
    *cx = magnitude * dirx / norm; *cy = magnitude * diry / norm;
    if (!isfinite(*cx) || !isfinite(*cy)) { *cx = qx; *cy = qy; return 4; }
    return 0;
}

/* One bed update over dt (seconds of hydraulics; morfac applied here).
 * q is the accepted state, z0 the bed; writes ztrial (nc). */
int om_exner(const om_ctx *m, const om_exner_params *ex, const double *q, const double *z0, double dt,
             double *ztrial, om_exner_stats *st)
{
    const int n = m->nc, nf = m->nf, na = m->nadj;
    const double d = ex->diameter, phi = 1.0 - ex->porosity, dtm = dt * ex->morfac;
    double *safe = om_alloc(sizeof(double) * 3 * (size_t)n), *gz = om_alloc(sizeof(double) * 2 * (size_t)n);
    double *cell = om_alloc(sizeof(double) * 6 * (size_t)n), *flux = om_alloc(sizeof(double) * nf);
    double *fac = om_alloc(sizeof(double) * n);
    int *wet = om_alloc(sizeof(int) * n), bad = 0;
    /* single-grain mixture: D90 by the log-linear bisection, hiding factor */
    double hiding, d90;
    {
        const double logd = log(d), lo = logd + 1.25 * log(.75), hi = logd + 1.25 * log(1.5);
        const double mean = d * 1. / 1., r = d / fmax(mean, 1.e-4), v = 1.27875360095283;
        hiding = pow(v / (v + log10(r)), 2.);
        double low = lo, high = hi;
        for (int it = 0; it < 60; ++it) {
            const double mid = .5 * (low + high);
            double f = 0.;
            if (mid >= hi) f = 1.;
            else if (mid > logd) f = .5 + .5 * (mid - logd) / (hi - logd);
            else if (mid > lo) f = .5 * (mid - lo) / (logd - lo);
            const double cdf = 1. / 1. * f;
            if (cdf < .9) low = mid; else high = mid;
        }
        d90 = exp(.5 * (low + high));
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        wet[i] = q[i] > ex->sediment_depth;
        safe[i] = wet[i] ? q[i] : .001001;
        safe[n + i] = wet[i] ? q[n + i] : 0.;
        safe[2 * n + i] = wet[i] ? q[2 * n + i] : 0.;
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        /* bed gradient of the flow engines' LS metric (bend_methods_v1_kernels.h:23-39, z row) */
        double bx = 0., by = 0.;
        for (int s = m->offset[i]; s < m->offset[i + 1]; ++s) {
            const int j = om_other(m, s);
            if (j < 0) continue;
            const double dx = ex->dxdy[s], dy = ex->dxdy[na + s], wt = 1. / (dx * dx + dy * dy);
            bx += wt * dx * (z0[j] - z0[i]); by += wt * dy * (z0[j] - z0[i]);
        }
        gz[i] = ex->inverse[i] * bx + ex->inverse[n + i] * by;
        gz[n + i] = ex->inverse[n + i] * bx + ex->inverse[2 * n + i] * by;
        /* MPM (river_mpm.h:32-46) with hI = 0 */
        const double h = safe[i], u = safe[n + i] / h, vv = safe[2 * n + i] / h;
        const double ue = safe[n + i] / safe[i], ve = safe[2 * n + i] / safe[i], c = ex->chezy;
        const double speed = hypot(ue, ve), theta = speed * speed / (c * c * 1.65 * d);
        const double grain = 18. * log10(12. * fmax(fmax(.01, safe[i]) / d90, 1.)), mu = fmin(1., pow(c / grain, 1.5));
        const double excess = fmax(0., mu * theta - .047 * hiding);
        const double mag = 2650. * 8. * sqrt(9.81 * 1.65 * d * excess) * d * excess;
        const double x = speed > 0. ? mag * ue / speed : 0., y = speed > 0. ? mag * ve / speed : 0.;
        const double us = hypot(u, vv), alpha = us > 0. && mag > 0. ? 12.5 * (1. - sqrt(9.81) / (.4 * c)) * (0. / h) / us : 0.;
        const double bxr = u + alpha * vv, byr = vv - alpha * u, bs = hypot(bxr, byr);
        cell[i] = x; cell[n + i] = y; cell[2 * n + i] = theta;
        cell[3 * n + i] = bs > 0. ? mag * bxr / bs : 0.; cell[4 * n + i] = bs > 0. ? mag * byr / bs : 0.;
        cell[5 * n + i] = alpha;
    }
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int f = 0; f < nf; ++f) {
        /* face inputs (flow2dh_mobile_kernels.h:13-38) */
        const int o = m->owner[f], j = m->neighbour[f];
        const double nx = m->normal[f], ny = m->normal[nf + f];
        double x = cell[3 * n + o], y = cell[4 * n + o], gx = gz[o], gy = gz[n + o];
        double stress = cell[2 * n + o] * sqrt(1. + cell[5 * n + o] * cell[5 * n + o]);
        if (j >= 0) {
            const double dd = m->distance[f] + m->distance[nf + f], wo = m->distance[nf + f] / dd, wj = m->distance[f] / dd;
            const double a = x * nx + y * ny, b = cell[3 * n + j] * nx + cell[4 * n + j] * ny;
            const double un = (a > 0. && b > 0.) ? a : ((a < 0. && b < 0.) ? b : .5 * (a + b));
            const double ut = wo * (-x * ny + y * nx) + wj * (-cell[3 * n + j] * ny + cell[4 * n + j] * nx);
            x = un * nx - ut * ny; y = un * ny + ut * nx;
            gx = wo * gx + wj * gz[j]; gy = wo * gy + wj * gz[n + j];
            const double dx = ex->xy[j] - ex->xy[o], dy = ex->xy[n + j] - ex->xy[n + o], dn = dx * nx + dy * ny;
            const double correction = (z0[j] - z0[o] - gx * dx - gy * dy) / dn;
            gx += correction * nx; gy += correction * ny;
            stress = wo * stress + wj * cell[2 * n + j] * sqrt(1. + cell[5 * n + j] * cell[5 * n + j]);
        } else {
            const double normal_slope = gx * nx + gy * ny;
            gx -= normal_slope * nx; gy -= normal_slope * ny;
        }
        double cx, cy;
        if (om_slope3(x, y, -gx, -gy, stress, &cx, &cy)) bad |= 1;
        /* bed flux and its boundaries (flow2dh_mobile_kernels.h:41-53) */
        double fl = (cx * nx + cy * ny) / 2650.;
        if (j < 0) {
            const int bc = ex->bedbc[f];
            if (bc == 1) fl = -ex->feed[f];
            else if (bc == 2) fl = fmax(0., fl);
            else if (bc == 3) {}
            else fl = 0.;
        }
        /* no bed flux across a face with a dry side (shoreline_solver.py:214-215) */
        const int active = wet[o] && (j >= 0 ? wet[j] : 1);
        flux[f] = fl * active;
    }
    /* donor limiter of the solid stock (bend_methods_v1_kernels.h:396-405) */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double outgoing = 0.;
        for (int k = m->offset[i]; k < m->offset[i + 1]; ++k) {
            const int f = m->faces[k];
            outgoing += fmax(0., m->signs[k] * flux[f]) * m->length[f];
        }
        const double available = phi * (z0[i] - ex->rock[i]);
        fac[i] = outgoing > 0. ? fmin(1., fmax(0., available) * m->area[i] / (dtm * outgoing)) : 1.;
    }
    for (int f = 0; f < nf; ++f) {
        const int j = flux[f] >= 0. ? m->owner[f] : m->neighbour[f];
        if (j >= 0) flux[f] *= fac[j];
    }
    double donor = 1., change = 0., residual = 0., boundary = 0.;
    int finite = 1, above = 1;
    for (int i = 0; i < n; ++i) {
        double r = 0.;
        for (int k = m->offset[i]; k < m->offset[i + 1]; ++k) r -= m->signs[k] * m->length[m->faces[k]] * flux[m->faces[k]];
        r = r / m->area[i];
        ztrial[i] = z0[i] + (dtm / phi) * r;
        donor = fmin(donor, fac[i]);
        if (!isfinite(ztrial[i])) finite = 0;
        if (ztrial[i] < ex->rock[i] - 1e-13) above = 0;
        change = fmax(change, fabs(ztrial[i] - z0[i]) / fmax(q[i], ex->sediment_depth));
        residual += phi * (ztrial[i] - z0[i]) * m->area[i];
    }
    for (int f = 0; f < nf; ++f)
        if (m->neighbour[f] < 0 && m->bid[f] >= 0) boundary -= dtm * flux[f] * m->length[f];
    residual -= boundary;
    st->ok = !bad && finite && above && fabs(residual) <= 1e-10 && change <= .05;
    st->residual = residual; st->boundary = boundary; st->donor = donor; st->change = change;
    free(safe); free(gz); free(cell); free(flux); free(fac); free(wet);
    return bad ? OM_REJECT_SPATIAL : (st->ok ? OM_OK : OM_REJECT_BUDGET);
}

/* One spatial residual (RiverMidpoint.rate + RiverExplicit.rate).
 * q is the stage state, base the interval-start stock. Writes rate (3,nc)
 * and the limited water flux (nf); *freq_out gets the max CFL frequency. */
/* Conservative wet-bank viscosity of a state (shoreline_viscosity.py:57-72):
 * the velocity gradients of the safe state (dry columns: depth 0.001001,
 * no momentum; secondary_vector_ops.py:39-48) by the flow engines' least
 * squares (bend_methods_v1_kernels.h:23-39, rows u and v), the shared-face
 * stress of wet columns (shoreline_viscosity.h:14-33), gathered as
 * sum(s len stress) / area with unit weights (flow2dh_fixed_bed_kernels.h:
 * 54-60) into the momentum rate. */
void om_shoreline_viscosity(const om_ctx *m, const double *q, const double *z, double *rate)
{
    const int n = m->nc, nf = m->nf, na = m->nadj;
    const double dry = m->dry, nu = m->visc;
    double *grad = m->vgrad, *out = m->vface;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const int wi = q[i] > dry;
        const double hi = wi ? q[i] : .001001;
        const double x[2] = {(wi ? q[n + i] : 0.) / hi, (wi ? q[2 * n + i] : 0.) / hi};
        double bx[2] = {0., 0.}, by[2] = {0., 0.};
        for (int k = m->offset[i]; k < m->offset[i + 1]; ++k) {
            const int f = m->faces[k], j = m->owner[f] == i ? m->neighbour[f] : m->owner[f];
            if (j < 0) continue;
            const double dx = m->vdxdy[k], dy = m->vdxdy[na + k], wt = 1. / (dx * dx + dy * dy);
            const int wj = q[j] > dry;
            const double hj = wj ? q[j] : .001001;
            const double y[2] = {(wj ? q[n + j] : 0.) / hj, (wj ? q[2 * n + j] : 0.) / hj};
            for (int c = 0; c < 2; ++c) { bx[c] += wt * dx * (y[c] - x[c]); by[c] += wt * dy * (y[c] - x[c]); }
        }
        for (int c = 0; c < 2; ++c) {
            grad[(2 * c) * n + i] = m->vinv[i] * bx[c] + m->vinv[n + i] * by[c];
            grad[(2 * c + 1) * n + i] = m->vinv[n + i] * bx[c] + m->vinv[2 * n + i] * by[c];
        }
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nf; ++i) {
        out[i] = 0.; out[nf + i] = 0.;
        const int o = m->owner[i], j = m->neighbour[i];
        if (j < 0 || q[o] <= dry || q[j] <= dry) continue;
        double h = fmin(q[o], q[j]);
        h = fmin(h, fmax(0., .5 * (q[o] + z[o] + q[j] + z[j]) - fmax(z[o], z[j])));
        const double d = m->distance[i] + m->distance[nf + i], wo = m->distance[nf + i] / d, wj = m->distance[i] / d;
        const double nx = m->normal[i], ny = m->normal[nf + i], dx = m->xy[j] - m->xy[o], dy = m->xy[n + j] - m->xy[n + o];
        const double dn = dx * nx + dy * ny;
        const double tx = dx - dn * nx, ty = dy - dn * ny;
        const double du = q[n + j] / q[j] - q[n + o] / q[o], dv = q[2 * n + j] / q[j] - q[2 * n + o] / q[o];
        const double ux = wo * grad[o] + wj * grad[j], uy = wo * grad[n + o] + wj * grad[n + j];
        const double vx = wo * grad[2 * n + o] + wj * grad[2 * n + j], vy = wo * grad[3 * n + o] + wj * grad[3 * n + j];
        out[i] = nu * h * (du - ux * tx - uy * ty) / dn;
        out[nf + i] = nu * h * (dv - vx * tx - vy * ty) / dn;
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double x = 0., y = 0.;
        for (int k = m->offset[i]; k < m->offset[i + 1]; ++k) {
            const int f = m->faces[k];
            x += m->signs[k] * m->length[f] * out[f];
            y += m->signs[k] * m->length[f] * out[nf + f];
        }
        rate[n + i] += 1. * x / m->area[i];
        rate[2 * n + i] += 1. * y / m->area[i];
    }
}

int om_rate(om_ctx *m, om_scratch *s, const double *q, const double *z, const double *base,
            double dt, double time, double *rate, double *water, double *freq_out)
{
    const int nc = m->nc, nf = m->nf;
    *freq_out = 0.0;
    for (int i = 0; i < 3 * nc; ++i)
        if (!isfinite(q[i])) return OM_REJECT_SPATIAL;
    for (int i = 0; i < nc; ++i)
        if (q[i] < 0) return OM_REJECT_SPATIAL;
    if (m->nb > 0) {
        const int ex = om_exterior(m, q, z, time, s->ext_trace, s->ext_flux, s->estatus, s->work, s->stage, s->total);
        if (ex == OM_EXTERIOR_FATAL) return OM_FAIL;
        if (ex) return OM_REJECT_SPATIAL;
        om_outlet_feasibility(m, base, dt, s->ext_flux, s->ext_trace, s->work);
        if (om_has_inlet(m)) om_inlet_feasibility(m, base, dt, s->ext_flux, s->ext_trace, s->work);
    }
    om_primitive(m, q, z, s->v, s->active, s->pstatus);
    om_cells(m, q, s->v, s->active, s->grad, s->constant);
    om_faces(m, q, s->v, s->grad, s->constant, s->trace, s->kind, s->rstatus);
    for (int f = 0; f < nf; ++f)
        if (om_open(m, f)) for (int j = 0; j < 3; ++j) s->trace[j * nf + f] = s->ext_trace[j * nf + f];
    om_prepare(m, s->trace, q, z, s->kind, s->local, s->closed);
    om_fwave(m, s->local, s->riemann, s->astatus);
    om_assemble(m, s->trace, s->local, s->riemann, q, z, s->kind, s->constant, s->closed,
                s->fl, s->fr, s->speed, s->fstatus);
    for (int f = 0; f < nf; ++f)
        if (om_open(m, f)) {
            for (int j = 0; j < 3; ++j) { s->fl[j * nf + f] = s->ext_flux[j * nf + f]; s->fr[j * nf + f] = s->ext_flux[j * nf + f]; }
            s->fstatus[f] = s->estatus[f];
        }
    for (int c = 0; c < nc; ++c) if (s->pstatus[c]) return OM_REJECT_SPATIAL;
    for (int f = 0; f < nf; ++f)
        if (s->rstatus[f] || s->astatus[f] || s->fstatus[f]) return OM_REJECT_SPATIAL;
    om_gather(m, q, s->fl, s->fr, s->active, rate);
    memcpy(water, s->fl, sizeof(double) * nf);
    om_inventory(m, dt, base, water, s->theta);
    if (m->nb > 0 && om_reserve(m, dt, base, water, s->theta)) return OM_REJECT_BUDGET;
    om_limit_faces(m, q, s->theta, water, s->correction);
    om_limit_gather(m, water, s->correction, rate);
    if (m->turb && om_turbine_momentum(m, s, q, z, rate)) return OM_FAIL;
    if (m->visc > 0.) om_shoreline_viscosity(m, q, z, rate);
    for (int i = 0; i < 3 * nc; ++i) if (!isfinite(rate[i])) return OM_REJECT_SPATIAL;
    const double freq = om_frequency(m, q, s->speed, s->ext_trace, s->freq);
    *freq_out = freq;
    if (!isfinite(freq) || dt * freq > m->cfl * (1 + 1e-12)) return OM_REJECT_CFL;
    return OM_OK;
}

/* One SSPRK(2,2) substep with Strang-split drag (RiverExplicit._single).
 * out gets q2; water (nf) gets the stage-mean limited water flux;
 * *peak the larger stage frequency seen (also on rejection). */
int om_single(om_ctx *m, om_scratch *s, const double *base, const double *z, double dt, double time,
              double *out, double *water, double *peak, double *tmp /* 9*nc + 2*nf */)
{
    const int nc = m->nc, nf = m->nf;
    double *work = tmp, *r = tmp + 3 * (size_t)nc, *q1 = tmp + 6 * (size_t)nc;
    double *w1 = tmp + 9 * (size_t)nc, *w2 = w1 + nf;
    double f1 = 0.0, f2 = 0.0;
    *peak = 0.0;
    memcpy(work, base, sizeof(double) * 3 * nc);
    om_drag(m, .5 * dt, work);
    int st = om_rate(m, s, work, z, work, dt, time, r, w1, &f1);
    if (isfinite(f1) && f1 > *peak) *peak = f1;
    if (st) return st;
    for (int i = 0; i < 3 * nc; ++i) q1[i] = work[i] + dt * r[i];
    for (int i = 0; i < nc; ++i) if (q1[i] < 0) return OM_REJECT_SPATIAL;
    for (int i = 0; i < nc; ++i) if (q1[i] <= m->dry) { q1[nc + i] = 0.; q1[2 * nc + i] = 0.; }
    st = om_rate(m, s, q1, z, q1, dt, time + dt, r, w2, &f2);
    if (isfinite(f2) && f2 > *peak) *peak = f2;
    if (st) return st;
    for (int i = 0; i < 3 * nc; ++i) out[i] = .5 * work[i] + .5 * (q1[i] + dt * r[i]);
    for (int i = 0; i < 3 * nc; ++i) if (!isfinite(out[i])) return OM_REJECT_SPATIAL;
    for (int i = 0; i < nc; ++i) if (out[i] < 0) return OM_REJECT_SPATIAL;
    for (int i = 0; i < nc; ++i) if (out[i] <= m->dry) { out[nc + i] = 0.; out[2 * nc + i] = 0.; }
    om_drag(m, .5 * dt, out);
    for (int f = 0; f < nf; ++f) water[f] = .5 * (w1[f] + w2[f]);
    return OM_OK;
}

typedef struct {
    int substeps, rejections, status;
    double min_dt, max_dt, accepted_cfl_max, hint;
} om_stats;

/* Adaptive substep loop over one outer interval dt (RiverExplicit.advance).
 * q is advanced in place; water_mean (nf) gets the time-mean water flux.
 * *hint carries the controller's step hint between calls (<= 0: none). */
int om_advance(om_ctx *m, double *q, const double *z, double dt, double time, double *hint,
               double *water_mean, om_stats *stats)
{
    const int nc = m->nc, nf = m->nf;
    om_scratch *s = om_scratch_create(m);
    double *tmp = om_alloc(sizeof(double) * (9 * (size_t)nc + 2 * (size_t)nf));
    double *next = om_alloc(sizeof(double) * 3 * (size_t)nc), *w = om_alloc(sizeof(double) * nf);
    double elapsed = 0.0, h = *hint > 0 ? *hint : dt;
    const double floor_ = dt * ldexp(1.0, -20);
    memset(stats, 0, sizeof(*stats));
    memset(water_mean, 0, sizeof(double) * nf);
    int status = OM_OK;
    while (stats->substeps == 0 || elapsed < dt - 1e-13 * fmax(1., dt)) {
        const double trial = fmin(h, dt - elapsed);
        const int truncated = trial < h * (1 - 1e-12);
        double peak = 0.0;
        const int st = om_single(m, s, q, z, trial, time + elapsed, next, w, &peak, tmp);
        if (st) {
            stats->rejections++;
            h = peak > 0 ? fmin(.5 * trial, .98 * m->cfl / peak) : .5 * trial;
            if (h < floor_ || stats->rejections > 100) { status = st; break; }
            continue;
        }
        memcpy(q, next, sizeof(double) * 3 * nc);
        for (int f = 0; f < nf; ++f) water_mean[f] += trial * w[f];
        elapsed += trial;
        stats->substeps++;
        if (stats->substeps == 1 || trial < stats->min_dt) stats->min_dt = trial;
        if (trial > stats->max_dt) stats->max_dt = trial;
        if (trial * peak > stats->accepted_cfl_max) stats->accepted_cfl_max = trial * peak;
        const double growth = truncated ? h : 2 * trial;
        h = peak > 0 ? fmin(growth, .98 * m->cfl / peak) : growth;
        if (stats->substeps > 4096) { status = OM_FAIL; break; }
    }
    for (int f = 0; f < nf; ++f) water_mean[f] /= dt;
    *hint = h;
    stats->hint = h;
    stats->status = status;
    free(tmp); free(next); free(w);
    om_scratch_destroy(s);
    return status;
}

/* ------------------------------------------------------------------ */
/* HLLC / MUSCL-Hancock option                                          */
/*   orchestration  src/braids_core/hydraulics/hllc.py:76-149           */
/*   kernels        src/braids_core/hydraulics/hllc.h:15-155            */
/*   rotor pressure src/braids_core/hydraulics/hllc_turbines.h:13-31    */
/*   rotor momentum src/braids_core/hydraulics/river_turbines.py:27-36  */
/* ------------------------------------------------------------------ */

/* Cell incidence in the HLLC operator's own order (each cell's faces in
 * ascending face number, hllc.py:29-34), its least-squares inverse (walls
 * mirrored, open faces left out, hllc.py:35-43) and the open-face flags. */
typedef struct {
    const int *off, *faces, *signs;
    const double *xy, *mid, *inverse;   /* (2,nc) (2,nf) (3,nc) */
    const int *selected;                /* (nf) */
} om_hllc_geo;

/* Limited MUSCL gradients of (eta, u, v, b) and the half-step predictor
 * (hllc.h:15-50). dt is the predictor's full interval (2 * 0.5 * dt). */
void om_hllc_reconstruct(const om_ctx *m, const om_hllc_geo *G, double dt, const double *q, const double *z,
                         double *grad, double *half, double *qhalf, int *status)
{
    const int n = m->nc, nf = m->nf;
    const double dry = m->dry, g = m->grav;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const double h0 = q[i];
        double c[4] = {h0 + z[i], h0 > dry ? q[n + i] / h0 : 0., h0 > dry ? q[2 * n + i] / h0 : 0., z[i]};
        double bx[4] = {0., 0., 0., 0.}, by[4] = {0., 0., 0., 0.}, lo[4], hi[4], gr[8];
        for (int k = 0; k < 4; ++k) lo[k] = hi[k] = c[k];
        for (int e = G->off[i]; e < G->off[i + 1]; ++e) {
            const int f = G->faces[e], j = m->owner[f] == i ? m->neighbour[f] : m->owner[f];
            double dx, dy, o[4];
            if (j >= 0) {
                const double hj = q[j];
                dx = G->xy[j] - G->xy[i];
                dy = G->xy[n + j] - G->xy[n + i];
                o[0] = hj + z[j]; o[1] = hj > dry ? q[n + j] / hj : 0.; o[2] = hj > dry ? q[2 * n + j] / hj : 0.;
                o[3] = z[j];
                if (o[0] - o[3] <= dry && o[3] >= c[0]) o[0] = c[0];     /* dry bank above the water line */
            } else {
                if (G->selected[f]) continue;
                const double nx = m->normal[f], ny = m->normal[nf + f];
                const double dist = (G->mid[f] - G->xy[i]) * nx + (G->mid[nf + f] - G->xy[n + i]) * ny;
                dx = 2. * dist * nx; dy = 2. * dist * ny;
                for (int k = 0; k < 4; ++k) o[k] = c[k];
                const double un = c[1] * nx + c[2] * ny;           /* mirrored wall ghost */
                o[1] -= 2. * un * nx; o[2] -= 2. * un * ny;
            }
            const double d2 = dx * dx + dy * dy;
            if (d2 <= 0.) continue;
            for (int k = 0; k < 4; ++k) {
                const double d = o[k] - c[k];
                bx[k] += d * dx / d2; by[k] += d * dy / d2;
                lo[k] = fmin(lo[k], o[k]); hi[k] = fmax(hi[k], o[k]);
            }
        }
        const double i0 = G->inverse[i], i1 = G->inverse[n + i], i2 = G->inverse[2 * n + i];
        for (int k = 0; k < 4; ++k) {
            const double gx = i0 * bx[k] + i1 * by[k], gy = i1 * bx[k] + i2 * by[k];
            double lim = 1.;
            for (int e = G->off[i]; e < G->off[i + 1]; ++e) {
                const int f = G->faces[e];
                const double d = gx * (G->mid[f] - G->xy[i]) + gy * (G->mid[nf + f] - G->xy[n + i]);
                if (d > 0.) lim = fmin(lim, (hi[k] - c[k]) / d);
                else if (d < 0.) lim = fmin(lim, (lo[k] - c[k]) / d);
            }
            gr[2 * k] = lim * gx; gr[2 * k + 1] = lim * gy;
        }
        const double h = c[0] - c[3];
        if (h <= dry) for (int k = 0; k < 6; ++k) gr[k] = 0.;
        for (int k = 0; k < 8; ++k) grad[(size_t)k * n + i] = gr[k];
        const double u = c[1], w = c[2];
        double eta = c[0] - .5 * dt * (u * (gr[0] - gr[6]) + w * (gr[1] - gr[7]) + h * (gr[2] + gr[5]));
        double uh = u - .5 * dt * (u * gr[2] + w * gr[3] + g * gr[0]);
        double wh = w - .5 * dt * (u * gr[4] + w * gr[5] + g * gr[1]);
        if (eta < c[3]) { eta = c[0]; uh = u; wh = w; }
        if (h <= dry) { eta = c[0]; uh = 0.; wh = 0.; }
        half[i] = eta; half[n + i] = uh; half[2 * n + i] = wh; half[3 * n + i] = c[3];
        const double hh = fmax(0., eta - c[3]);
        qhalf[i] = hh; qhalf[n + i] = hh * uh; qhalf[2 * n + i] = hh * wh;
        status[i] = !isfinite(eta) || !isfinite(uh) || !isfinite(wh);
    }
}

/* HLLC flux of one rotated face, HLLE where a side is dry or the contact
 * state is inadmissible (hllc.h:52-78). */
static void om_hllc_flux(double hl, double ul, double vl, double hr, double ur, double vr, double g, double dry,
                         double out[3], double *speed)
{
    const double cl = sqrt(g * hl), cr = sqrt(g * hr);
    double sl = fmin(ul - cl, ur - cr), sr = fmax(ul + cl, ur + cr);
    if (hl <= dry) sl = ur - 2. * cr;
    if (hr <= dry) sr = ul + 2. * cl;
    *speed = fmax(fabs(sl), fabs(sr));
    const double fL[3] = {hl * ul, hl * ul * ul + .5 * g * hl * hl, hl * ul * vl};
    const double fR[3] = {hr * ur, hr * ur * ur + .5 * g * hr * hr, hr * ur * vr};
    if (hl <= dry && hr <= dry) { out[0] = out[1] = out[2] = 0.; *speed = 0.; return; }
    if (sl >= 0.) { for (int k = 0; k < 3; ++k) out[k] = fL[k]; return; }
    if (sr <= 0.) { for (int k = 0; k < 3; ++k) out[k] = fR[k]; return; }
    const double a = hl * (sl - ul), b = hr * (sr - ur), den = a - b;
    const double sm = fabs(den) > 1e-30 ? (.5 * g * (hr * hr - hl * hl) + a * ul - b * ur) / den : 0.;
    if (hl > dry && hr > dry && sl < sm && sm < sr) {
        const double hs = sm >= 0. ? a / (sl - sm) : b / (sr - sm);
        if (hs >= 0. && isfinite(hs)) {
            if (sm >= 0.) {
                out[0] = fL[0] + sl * (hs - hl); out[1] = fL[1] + sl * (hs * sm - hl * ul);
                out[2] = fL[2] + sl * (hs * vl - hl * vl);
            } else {
                out[0] = fR[0] + sr * (hs - hr); out[1] = fR[1] + sr * (hs * sm - hr * ur);
                out[2] = fR[2] + sr * (hs * vr - hr * vr);
            }
            return;
        }
    }
    const double uL[3] = {hl, hl * ul, hl * vl}, uR[3] = {hr, hr * ur, hr * vr};
    for (int k = 0; k < 3; ++k) out[k] = (sr * fL[k] - sl * fR[k] + sl * sr * (uR[k] - uL[k])) / (sr - sl);
}

/* Half-step momentum source on the predicted state (hllc.h:74-77). */
void om_hllc_predict_source(int n, double dry, double dt, const double *rate, double *half, double *qhalf)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const double h = qhalf[i];
        qhalf[n + i] += .5 * dt * rate[n + i];
        qhalf[2 * n + i] += .5 * dt * rate[2 * n + i];
        half[n + i] = h > dry ? qhalf[n + i] / h : 0.;
        half[2 * n + i] = h > dry ? qhalf[2 * n + i] / h : 0.;
    }
}

/* Face extrapolation of the predicted primitive m of cell c to face f. */
static inline double om_hllc_face_value(const om_ctx *m, const om_hllc_geo *G, const double *half,
                                        const double *grad, int k, int c, int f)
{
    const int n = m->nc, nf = m->nf;
    return half[(size_t)k * n + c] + grad[(size_t)2 * k * n + c] * (G->mid[f] - G->xy[c]) +
           grad[(size_t)(2 * k + 1) * n + c] * (G->mid[nf + f] - G->xy[n + c]);
}

/* Face fluxes (hllc.h:80-114): open faces take the exterior flux with the
 * cell-reference pressure removed; others the hydrostatically reconstructed
 * HLLC flux with the cell-reference pressure quadrature. */
void om_hllc_faces(const om_ctx *m, const om_hllc_geo *G, const double *half, const double *grad,
                   const double *external, const double *ext_trace, double *fl, double *fr, double *speed)
{
    const int n = m->nc, nf = m->nf;
    const double g = m->grav, dry = m->dry;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nf; ++i) {
        const int l = m->owner[i], r = m->neighbour[i];
        const double nx = m->normal[i], ny = m->normal[nf + i];
        if (G->selected[i]) {
            const double h = fmax(0., half[l] - half[3 * n + l]);
            fl[i] = fr[i] = external[i];
            fl[nf + i] = fr[nf + i] = external[nf + i] - .5 * g * h * h * nx;
            fl[2 * nf + i] = fr[2 * nf + i] = external[2 * nf + i] - .5 * g * h * h * ny;
            const double hb = ext_trace[i];
            const double ub = hb > dry ? (ext_trace[nf + i] * nx + ext_trace[2 * nf + i] * ny) / hb : 0.;
            speed[i] = fmax(fabs(half[n + l] * nx + half[2 * n + l] * ny) + sqrt(g * h),
                            fabs(ub) + sqrt(g * fmax(hb, 0.)));
            continue;
        }
        double L[4], R[4];
        for (int k = 0; k < 4; ++k) {
            L[k] = om_hllc_face_value(m, G, half, grad, k, l, i);
            R[k] = r < 0 ? L[k] : om_hllc_face_value(m, G, half, grad, k, r, i);
        }
        const int ldry = half[l] - half[3 * n + l] <= dry, rdry = r >= 0 && half[r] - half[3 * n + r] <= dry;
        if (ldry || rdry) { L[3] = half[3 * n + l]; R[3] = r < 0 ? L[3] : half[3 * n + r]; }
        if (ldry) { L[0] = L[3]; L[1] = L[2] = 0.; }
        if (rdry) { R[0] = R[3]; R[1] = R[2] = 0.; }
        if (r < 0) { const double un = R[1] * nx + R[2] * ny; R[1] -= 2. * un * nx; R[2] -= 2. * un * ny; }
        const double top = fmax(L[3], R[3]), hl = fmax(0., L[0] - L[3]), hr = fmax(0., R[0] - R[3]);
        const double hls = fmax(0., L[0] - top), hrs = fmax(0., R[0] - top);
        double out[3], s;
        om_hllc_flux(hls, L[1] * nx + L[2] * ny, -L[1] * ny + L[2] * nx,
                     hrs, R[1] * nx + R[2] * ny, -R[1] * ny + R[2] * nx, g, dry, out, &s);
        const double el = fmax(0., half[l] - L[3]), er = r < 0 ? el : fmax(0., half[r] - R[3]);
        const double pl = .5 * g * (hl * hl - hls * hls - el * el), pr = .5 * g * (hr * hr - hrs * hrs - er * er);
        fl[i] = fr[i] = r < 0 ? 0. : out[0];
        fl[nf + i] = (out[1] + pl) * nx - out[2] * ny; fl[2 * nf + i] = (out[1] + pl) * ny + out[2] * nx;
        fr[nf + i] = (out[1] + pr) * nx - out[2] * ny; fr[2 * nf + i] = (out[1] + pr) * ny + out[2] * nx;
        speed[i] = s;
    }
}

/* Low-Froude acoustic correction on fully wet, small-jump interior faces
 * of a rotor array's mesh (hllc_turbines.h:13-31). */
void om_hllc_turbine_pressure(const om_ctx *m, const om_hllc_geo *G, const double *half, const double *grad,
                              double *fl, double *fr)
{
    const int n = m->nc, nf = m->nf;
    const double g = m->grav, dry = m->dry;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nf; ++i) {
        const int a = m->owner[i], b = m->neighbour[i];
        if (b < 0) continue;
        if (half[a] - half[3 * n + a] <= dry || half[b] - half[3 * n + b] <= dry) continue;
        double L[4], R[4];
        for (int k = 0; k < 4; ++k) {
            L[k] = om_hllc_face_value(m, G, half, grad, k, a, i);
            R[k] = om_hllc_face_value(m, G, half, grad, k, b, i);
        }
        const double bed = fmax(L[3], R[3]), hl = L[0] - bed, hr = R[0] - bed, h = .5 * (hl + hr);
        if (fmin(hl, hr) <= dry || fabs(hr - hl) > .005 * h) continue;
        const double c = sqrt(g * h), theta = fmin(1., fmax(hypot(L[1], L[2]), hypot(R[1], R[2])) / c);
        const double nx = m->normal[i], ny = m->normal[nf + i];
        const double du = (R[1] - L[1]) * nx + (R[2] - L[2]) * ny;
        const double delta = .5 * (1. - theta) * c * (2. * hl * hr / (hl + hr)) * du;
        fl[nf + i] += delta * nx; fr[nf + i] += delta * nx;
        fl[2 * nf + i] += delta * ny; fr[2 * nf + i] += delta * ny;
    }
}

/* Donor budget and CFL frequency per cell (hllc.h:116-132): prescribed
 * exterior debits are reserved first; theta = -1 marks an unfunded one. */
void om_hllc_budget(const om_ctx *m, const om_hllc_geo *G, double dt, const double *q, const double *fl,
                    const double *speed, const int *pstatus, double *theta, double *freq)
{
    const int n = m->nc;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double outgoing = 0., prescribed = 0., sum = 0.;
        for (int e = G->off[i]; e < G->off[i + 1]; ++e) {
            const int f = G->faces[e];
            const double debit = fmax(0., G->signs[e] * fl[f]) * m->length[f];
            if (G->selected[f]) prescribed += debit; else outgoing += debit;
            sum += speed[f] * m->length[f];
        }
        freq[i] = pstatus[i] ? INFINITY : sum / m->area[i];
        theta[i] = 1.;
        const double available = q[i] * m->area[i] / dt;
        if (prescribed > available) theta[i] = -1.;
        else if (outgoing > 0. && outgoing >= available - prescribed)
            theta[i] = fmin(1., (available - prescribed) / outgoing) * (1. - 32. * OM_EPS);
    }
}

/* Donor limiting of interior faces; unfunded exterior debits flag their face (hllc.h:134-143). */
void om_hllc_limit(const om_ctx *m, const om_hllc_geo *G, const double *q, const double *theta,
                   double *fl, double *fr, int *fstatus)
{
    const int n = m->nc, nf = m->nf;
    const double dry = m->dry;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nf; ++i) {
        fstatus[i] = 0;
        const double water = fl[i];
        const int donor = water < 0. ? m->neighbour[i] : m->owner[i];
        if (donor < 0 || water == 0.) continue;
        if (G->selected[i]) { fstatus[i] = theta[donor] < 0. ? 1 : 0; continue; }
        if (theta[donor] >= 1.) continue;
        const double factor = fmax(0., theta[donor]), delta = (factor - 1.) * water;
        fl[i] = fr[i] = water * factor;
        if (q[donor] > dry)
            for (int k = 1; k < 3; ++k) {
                const double d = delta * q[(size_t)k * n + donor] / q[donor];
                fl[(size_t)k * nf + i] += d; fr[(size_t)k * nf + i] += d;
            }
    }
}

/* Conservative update from the limited fluxes (hllc.h:145-155). */
void om_hllc_update(const om_ctx *m, const om_hllc_geo *G, double dt, const double *q, const double *fl,
                    const double *fr, const int *fstatus, double *next, int *status)
{
    const int n = m->nc, nf = m->nf;
    const double dry = m->dry;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double v[3] = {q[i], q[n + i], q[2 * n + i]};
        int bad = 0;
        for (int e = G->off[i]; e < G->off[i + 1]; ++e) {
            const int f = G->faces[e], s = G->signs[e];
            const double a = dt * s * m->length[f] / m->area[i];
            const double *src = s > 0 ? fl : fr;
            for (int k = 0; k < 3; ++k) v[k] -= a * src[(size_t)k * nf + f];
            bad = bad || fstatus[f];
        }
        if (v[0] <= dry) v[1] = v[2] = 0.;
        for (int k = 0; k < 3; ++k) { next[(size_t)k * n + i] = v[k]; bad = bad || !isfinite(v[k]); }
        status[i] = bad || v[0] < 0.;
    }
}

typedef struct {
    double *grad, *half, *qhalf, *fl, *fr, *speed, *theta, *freq, *next, *rate, *work;
    int *pstatus, *fstatus, *status;
} om_hllc_scratch;

static om_hllc_scratch *om_hllc_scratch_create(const om_ctx *m)
{
    const size_t nc = m->nc, nf = m->nf;
    om_hllc_scratch *S = (om_hllc_scratch *)om_alloc(sizeof(*S));
    S->grad = om_alloc(8 * nc * 8); S->half = om_alloc(4 * nc * 8); S->qhalf = om_alloc(3 * nc * 8);
    S->fl = om_alloc(3 * nf * 8); S->fr = om_alloc(3 * nf * 8); S->speed = om_alloc(nf * 8);
    S->theta = om_alloc(nc * 8); S->freq = om_alloc(nc * 8); S->next = om_alloc(3 * nc * 8);
    S->rate = om_alloc(3 * nc * 8); S->work = om_alloc(3 * nc * 8);
    S->pstatus = om_alloc(nc * 4); S->fstatus = om_alloc(nf * 4); S->status = om_alloc(nc * 4);
    return S;
}

static void om_hllc_scratch_destroy(om_hllc_scratch *S)
{
    void *all[] = {S->grad, S->half, S->qhalf, S->fl, S->fr, S->speed, S->theta, S->freq, S->next, S->rate,
                   S->work, S->pstatus, S->fstatus, S->status};
    for (size_t i = 0; i < sizeof(all) / sizeof(all[0]); ++i) free(all[i]);
    free(S);
}

/* One Hancock substep (HLLCHydraulics._spatial_step with predictor 0.5):
 * Strang drag, predictor, half-time rotor source, exterior at t + dt/2
 * with the outlet stock cap, faces, budget, CFL check, limiter, update,
 * rotor source at the half state, drag. *peak is the reference's
 * frequency_peak (0 before the budget; possibly inf or NaN). */
int om_hllc_single(om_ctx *m, const om_hllc_geo *G, om_scratch *s, om_hllc_scratch *S, const double *q,
                   const double *z, double dt, double time, double *out, double *water, double *peak)
{
    const int n = m->nc, nf = m->nf;
    *peak = 0.;
    memcpy(S->work, q, sizeof(double) * 3 * n);
    om_drag(m, .5 * dt, S->work);
    om_hllc_reconstruct(m, G, dt, S->work, z, S->grad, S->half, S->qhalf, S->pstatus);
    if (m->turb) {
        memset(S->rate, 0, sizeof(double) * 3 * n);
        if (om_turbine_momentum(m, s, S->work, z, S->rate)) return OM_FAIL;
        om_hllc_predict_source(n, m->dry, dt, S->rate, S->half, S->qhalf);
    }
    const double *ext = s->ext_flux, *ext_trace = s->ext_trace;
    if (m->nb > 0) {
        const int ex = om_exterior(m, S->qhalf, z, time + .5 * dt, s->ext_trace, s->ext_flux, s->estatus, s->work,
                                   s->stage, s->total);
        if (ex == OM_EXTERIOR_FATAL) return OM_FAIL;
        if (ex) return OM_REJECT_SPATIAL;
        om_outlet_feasibility(m, S->work, dt, s->ext_flux, s->ext_trace, s->work);
        if (om_has_inlet(m)) om_inlet_feasibility(m, S->work, dt, s->ext_flux, s->ext_trace, s->work);
    }
    om_hllc_faces(m, G, S->half, S->grad, ext, ext_trace, S->fl, S->fr, S->speed);
    if (m->turb) om_hllc_turbine_pressure(m, G, S->half, S->grad, S->fl, S->fr);
    om_hllc_budget(m, G, dt, S->work, S->fl, S->speed, S->pstatus, S->theta, S->freq);
    double f = -INFINITY;
    int nan = 0;
    for (int i = 0; i < n; ++i) { if (isnan(S->freq[i])) nan = 1; else if (S->freq[i] > f) f = S->freq[i]; }
    if (nan) f = NAN;                           /* numpy max propagates NaN */
    *peak = f;
    if (!isfinite(f) || dt * f > m->cfl * (1 + 1e-12)) return OM_REJECT_CFL;
    om_hllc_limit(m, G, S->work, S->theta, S->fl, S->fr, S->fstatus);
    om_hllc_update(m, G, dt, S->work, S->fl, S->fr, S->fstatus, S->next, S->status);
    for (int i = 0; i < n; ++i) if (S->status[i]) return OM_REJECT_BUDGET;
    memcpy(out, S->next, sizeof(double) * 3 * n);
    if (m->turb) {
        memset(S->rate, 0, sizeof(double) * 3 * n);
        if (om_turbine_momentum(m, s, S->qhalf, z, S->rate)) return OM_FAIL;
        for (int i = 0; i < 3 * n; ++i) out[i] += dt * S->rate[i];
        for (int i = 0; i < 3 * n; ++i) if (!isfinite(out[i])) return OM_REJECT_SPATIAL;
    }
    om_drag(m, .5 * dt, out);
    memcpy(water, S->fl, sizeof(double) * nf);
    return OM_OK;
}

/* Adaptive Hancock substeps over one outer interval (HLLCHydraulics.advance,
 * hllc.py:131-149): no substep cap; a rejection halves the trial (bounded by
 * the CFL estimate of the frequency seen); more than 100 rejections or a
 * hint below dt / 2^20 fail the interval. */
int om_hllc_advance(om_ctx *m, const om_hllc_geo *G, double *q, const double *z, double dt, double time,
                    double *hint, double *water_mean, om_stats *stats)
{
    const int n = m->nc, nf = m->nf;
    om_scratch *s = om_scratch_create(m);
    om_hllc_scratch *S = om_hllc_scratch_create(m);
    double *next = om_alloc(sizeof(double) * 3 * (size_t)n), *w = om_alloc(sizeof(double) * nf);
    double elapsed = 0., h = *hint > 0 ? *hint : dt;
    memset(stats, 0, sizeof(*stats));
    memset(water_mean, 0, sizeof(double) * nf);
    /* the HLLC owner's rotor momentum has no balanced-pressure term
     * (hydrostatic HLLC pressure; river_turbines.py:27-36) */
    om_turbines *T = (om_turbines *)m->turb;
    const int pressure = T ? T->pressure : 0;
    if (T) T->pressure = 0;
    int status = OM_OK;
    while (stats->substeps == 0 || elapsed < dt - 1e-13 * fmax(1., dt)) {
        const double trial = fmin(h, dt - elapsed);
        const int truncated = trial < h * (1 - 1e-12);
        double peak = 0.;
        const int st = om_hllc_single(m, G, s, S, q, z, trial, time + elapsed, next, w, &peak);
        if (st == OM_FAIL) { status = st; break; }
        if (st) {
            stats->rejections++;
            h = peak > 0 ? fmin(.5 * trial, .98 * m->cfl / peak) : .5 * trial;
            if (stats->rejections > 100 || h < dt * ldexp(1., -20)) { status = st; break; }
            continue;
        }
        memcpy(q, next, sizeof(double) * 3 * n);
        for (int f = 0; f < nf; ++f) water_mean[f] += trial * w[f];
        elapsed += trial;
        stats->substeps++;
        if (stats->substeps == 1 || trial < stats->min_dt) stats->min_dt = trial;
        if (trial > stats->max_dt) stats->max_dt = trial;
        if (trial * peak > stats->accepted_cfl_max) stats->accepted_cfl_max = trial * peak;
        const double growth = truncated ? h : 2 * trial;
        h = peak > 0 ? fmin(growth, .98 * m->cfl / peak) : growth;
    }
    if (T) T->pressure = pressure;
    for (int f = 0; f < nf; ++f) water_mean[f] /= dt;
    *hint = h;
    stats->hint = h;
    stats->status = status;
    free(next); free(w);
    om_hllc_scratch_destroy(S);
    om_scratch_destroy(s);
    return status;
}

/* One Hancock step from q with its internals copied out (any output may be NULL). */
int om_hllc_step(om_ctx *m, const om_hllc_geo *G, const double *q, const double *z, double dt, double time,
                 double *out, double *water, double *peak, double *grad, double *half, double *qhalf,
                 double *fl, double *fr, double *speed, double *theta, double *freq, double *next)
{
    const size_t n = m->nc, nf = m->nf;
    om_scratch *s = om_scratch_create(m);
    om_hllc_scratch *S = om_hllc_scratch_create(m);
    double *res = om_alloc(sizeof(double) * 3 * n), *w = om_alloc(sizeof(double) * nf);
    om_turbines *T = (om_turbines *)m->turb;
    const int pressure = T ? T->pressure : 0;
    if (T) T->pressure = 0;
    const int st = om_hllc_single(m, G, s, S, q, z, dt, time, res, w, peak);
    if (T) T->pressure = pressure;
#define OM_COPY(dst, src, count) if (dst) memcpy(dst, src, sizeof(double) * (count))
    OM_COPY(out, res, 3 * n); OM_COPY(water, w, nf); OM_COPY(grad, S->grad, 8 * n);
    OM_COPY(half, S->half, 4 * n); OM_COPY(qhalf, S->qhalf, 3 * n); OM_COPY(fl, S->fl, 3 * nf);
    OM_COPY(fr, S->fr, 3 * nf); OM_COPY(speed, S->speed, nf); OM_COPY(theta, S->theta, n);
    OM_COPY(freq, S->freq, n); OM_COPY(next, S->next, 3 * n);
#undef OM_COPY
    free(res); free(w);
    om_hllc_scratch_destroy(S);
    om_scratch_destroy(s);
    return st;
}

size_t om_hllc_geo_size(void) { return sizeof(om_hllc_geo); }

void om_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) { omp_set_dynamic(0); omp_set_num_threads(n); }
#else
    (void)n;
#endif
}

size_t om_ctx_size(void) { return sizeof(om_ctx); }
size_t om_stats_size(void) { return sizeof(om_stats); }
size_t om_turbines_size(void) { return sizeof(om_turbines); }
size_t om_exner_size(void) { return sizeof(om_exner_params); }
