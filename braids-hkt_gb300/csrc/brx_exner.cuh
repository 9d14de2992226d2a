// Exner bed update with Meyer-Peter-Mueller transport, one grain size, once per
// outer interval (FP64 in both arithmetic forms; compiled in the FP64 unit):
//
//   finish / bed_faces    src/braids_core/sediment/shoreline_solver.py:209-240,
//                         flow2dh_mobile_bed.py:101-109
//   MPM capacity          river_mpm.h:32-46 (hI = 0: no secondary-flow spiral)
//   bed gradient          bend_methods_v1_kernels.h:23-39 (z row)
//   face inputs, flux     flow2dh_mobile_kernels.h:13-53
//   slope correction      src/braids_gpu/flow_bed_slope_runtime.cu:13-144 (ISlope 3)
//   donor limit, div      bend_methods_v1_kernels.h:389-405
//
// Cells, faces, donor factors, flux limit and trial bed are grid-stride sweeps
// over every scenario with a bed model; one CTA per scenario then reduces the
// budget residual, boundary volume, donor minimum and relative change in a
// fixed order, and a last sweep commits the trial bed where the checks pass.
#pragma once
#include "brx_common.cuh"

namespace brx {

enum { EP_D = 0, EP_POROSITY, EP_CHEZY, EP_MORFAC, EP_SEDDEPTH, EP_D90, EP_HIDING, EP_N = 8 };
enum { ES_OK = 0, ES_RESIDUAL, ES_BOUNDARY, ES_DONOR, ES_CHANGE, ES_BAD, ES_N = 8 };

struct ExnerDev {
    const int *enabled;          // (nscen)
    const double *param;         // (nscen, 8)
    const int *bedbc;            // (nf) 0 wall, 1 feed, 2 outflow, 3 capacity
    const double *feed, *rock;   // (nf) (nc)
    const double *dxdy, *inverse, *xy;
    double *cell;                // (6, nc) MPM output
    double *gz;                  // (2, nc) bed gradient
    double *flux;                // (nf) solid volume flux per length
    double *fac;                 // (nc) donor factors
    double *ztrial;              // (nc)
    double *stats;               // (nscen, 8)
    int *wet;                    // (nc)
    int *bad;                    // (nscen) slope operator status
    const double *dt;            // (nscen) interval of each scenario (seconds of hydraulics)
};

__global__ void __launch_bounds__(256) k_ex_cells(MeshDev m, ExnerDev e, const double *q, const double *z)
{
    const int n = m.nc, na = m.nadj;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int sid = m.cell_sid[i];
        if (!e.enabled[sid]) continue;
        const double *p = e.param + (size_t)sid * EP_N;
        const double d = p[EP_D], c = p[EP_CHEZY], d90 = p[EP_D90], hide = p[EP_HIDING];
        // division-safe state at the sediment working depth (secondary_vector_ops.safe)
        const bool wet = q[i] > p[EP_SEDDEPTH];
        e.wet[i] = wet;
        const double h = wet ? q[i] : .001001, hu = wet ? q[n + i] : 0., hv = wet ? q[2 * n + i] : 0.;
        double bx = 0., by = 0.;
        for (int s = m.offset[i]; s < m.offset[i + 1]; ++s) {
            const int f = m.faces[s];
            const int j = m.signs[s] < 0 ? m.owner[f] : m.neighbour[f];
            if (j < 0) continue;
            const double dx = e.dxdy[s], dy = e.dxdy[na + s], wt = 1. / (dx * dx + dy * dy);
            bx += wt * dx * (z[j] - z[i]); by += wt * dy * (z[j] - z[i]);
        }
        e.gz[i] = e.inverse[i] * bx + e.inverse[n + i] * by;
        e.gz[n + i] = e.inverse[n + i] * bx + e.inverse[2 * n + i] * by;
        const double u = hu / h, v = hv / h, ue = hu / h, ve = hv / h;
        const double speed = hypot(ue, ve), theta = speed * speed / (c * c * 1.65 * d);
        const double grain = 18. * log10(12. * fmax(fmax(.01, h) / d90, 1.)), mu = fmin(1., pow(c / grain, 1.5));
        const double excess = fmax(0., mu * theta - .047 * hide);
        const double mag = 2650. * 8. * sqrt(9.81 * 1.65 * d * excess) * d * excess;
        const double x = speed > 0. ? mag * ue / speed : 0., y = speed > 0. ? mag * ve / speed : 0.;
        const double us = hypot(u, v);
        const double alpha = us > 0. && mag > 0. ? 12.5 * (1. - sqrt(9.81) / (.4 * c)) * (0. / h) / us : 0.;
        const double rx = u + alpha * v, ry = v - alpha * u, bs = hypot(rx, ry);
        e.cell[i] = x; e.cell[n + i] = y; e.cell[2 * n + i] = theta;
        e.cell[3 * n + i] = bs > 0. ? mag * rx / bs : 0.; e.cell[4 * n + i] = bs > 0. ? mag * ry / bs : 0.;
        e.cell[5 * n + i] = alpha;
    }
}

// Koch--Flokstra slope correction, FLOW ISlope 3 with alfabs = alfabn = 0,
// ashld .85, bshld .5, cshld = dshld = 0. Returns 0 or the operator's status.
__device__ __forceinline__ int slope_ks3(double qx, double qy, double down_x, double down_y, double stress,
                                         double &cx, double &cy)
{
    cx = qx; cy = qy;
    if (!isfinite(qx) || !isfinite(qy) || !isfinite(down_x) || !isfinite(down_y) || !isfinite(stress) || stress < 0.0)
        return 2;
    double magnitude = sqrt(qx * qx + qy * qy);
    if (!isfinite(magnitude)) return 2;
    if (magnitude <= 1.0e-6) return 0;
    double dzds = down_x * qx / magnitude + down_y * qy / magnitude;
    // FLOW's default-real literals rounded to FP32 before promotion
    const double tan_phi = tan((double)(30.0f / 180.0f) * acos(-1.0));
    dzds = fmin((double)0.9f * tan_phi, dzds);
    const double ftheta = stress != 0.0 ? .85 * pow(stress, .5) * pow(1.0, 0.0) * pow(1.0, 0.0) : 0.0;
    double dirx, diry;
    if (down_x != 0.0 || down_y != 0.0) { dirx = ftheta * qx / magnitude + down_x; diry = ftheta * qy / magnitude + down_y; }
    else { dirx = qx / magnitude; diry = qy / magnitude; }
    const double norm = sqrt(dirx * dirx + diry * diry);
    if (!isfinite(norm) || norm <= 2.2250738585072014e-308) return 3;
    magnitude = magnitude * (1.0 + 0. * dzds);
    cx = magnitude * dirx / norm; cy = magnitude * diry / norm;
    if (!isfinite(cx) || !isfinite(cy)) { cx = qx; cy = qy; return 4; }
    return 0;
}

__global__ void __launch_bounds__(128) k_ex_faces(MeshDev m, ExnerDev e, const double *z)
{
    const int n = m.nc, nf = m.nf;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
        const int sid = m.face_sid[f];
        if (!e.enabled[sid]) continue;
        const int o = m.owner[f], j = m.neighbour[f];
        const double nx = m.normal[f], ny = m.normal[nf + f];
        double x = e.cell[3 * n + o], y = e.cell[4 * n + o], gx = e.gz[o], gy = e.gz[n + o];
        double stress = e.cell[2 * n + o] * sqrt(1. + e.cell[5 * n + o] * e.cell[5 * n + o]);
        if (j >= 0) {
            const double dd = m.distance[f] + m.distance[nf + f], wo = m.distance[nf + f] / dd, wj = m.distance[f] / dd;
            const double a = x * nx + y * ny, b = e.cell[3 * n + j] * nx + e.cell[4 * n + j] * ny;
            // upwind sign rule in the face-normal basis, tangential part interpolated
            const double un = (a > 0. && b > 0.) ? a : ((a < 0. && b < 0.) ? b : .5 * (a + b));
            const double ut = wo * (-x * ny + y * nx) + wj * (-e.cell[3 * n + j] * ny + e.cell[4 * n + j] * nx);
            x = un * nx - ut * ny; y = un * ny + ut * nx;
            gx = wo * gx + wj * e.gz[j]; gy = wo * gy + wj * e.gz[n + j];
            const double dx = e.xy[j] - e.xy[o], dy = e.xy[n + j] - e.xy[n + o], dn = dx * nx + dy * ny;
            const double correction = (z[j] - z[o] - gx * dx - gy * dy) / dn;
            gx += correction * nx; gy += correction * ny;
            stress = wo * stress + wj * e.cell[2 * n + j] * sqrt(1. + e.cell[5 * n + j] * e.cell[5 * n + j]);
        } else {
            const double normal_slope = gx * nx + gy * ny;
            gx -= normal_slope * nx; gy -= normal_slope * ny;
        }
        double cx, cy;
        if (slope_ks3(x, y, -gx, -gy, stress, cx, cy)) atomicOr(&e.bad[sid], 1);
        double fl = (cx * nx + cy * ny) / 2650.;
        if (j < 0) {
            const int bc = e.bedbc[f];
            if (bc == 1) fl = -e.feed[f];
            else if (bc == 2) fl = fmax(0., fl);
            else if (bc != 3) fl = 0.;
        }
        // no bed flux across a face with a dry side
        const bool active = e.wet[o] && (j >= 0 ? e.wet[j] : true);
        e.flux[f] = fl * (active ? 1. : 0.);
    }
}

__global__ void __launch_bounds__(256) k_ex_donor(MeshDev m, ExnerDev e, const double *z)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m.nc; i += gridDim.x * blockDim.x) {
        const int sid = m.cell_sid[i];
        if (!e.enabled[sid]) continue;
        const double *p = e.param + (size_t)sid * EP_N;
        const double dtm = e.dt[sid] * p[EP_MORFAC], phi = 1.0 - p[EP_POROSITY];
        double outgoing = 0.;
        for (int k = m.offset[i]; k < m.offset[i + 1]; ++k) {
            const int f = m.faces[k];
            outgoing += fmax(0., m.signs[k] * e.flux[f]) * m.length[f];
        }
        const double available = phi * (z[i] - e.rock[i]);
        e.fac[i] = outgoing > 0. ? fmin(1., fmax(0., available) * m.area[i] / (dtm * outgoing)) : 1.;
    }
}

__global__ void __launch_bounds__(256) k_ex_limit(MeshDev m, ExnerDev e)
{
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < m.nf; f += gridDim.x * blockDim.x) {
        if (!e.enabled[m.face_sid[f]]) continue;
        const int j = e.flux[f] >= 0. ? m.owner[f] : m.neighbour[f];
        if (j >= 0) e.flux[f] *= e.fac[j];
    }
}

__global__ void __launch_bounds__(256) k_ex_trial(MeshDev m, ExnerDev e, const double *z)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m.nc; i += gridDim.x * blockDim.x) {
        const int sid = m.cell_sid[i];
        if (!e.enabled[sid]) continue;
        const double *p = e.param + (size_t)sid * EP_N;
        const double dtm = e.dt[sid] * p[EP_MORFAC], phi = 1.0 - p[EP_POROSITY];
        double r = 0.;
        for (int k = m.offset[i]; k < m.offset[i + 1]; ++k) r -= m.signs[k] * m.length[m.faces[k]] * e.flux[m.faces[k]];
        r = r / m.area[i];
        e.ztrial[i] = z[i] + (dtm / phi) * r;
    }
}

// One CTA per scenario: budget residual, boundary volume, donor minimum,
// relative change and the positivity / finiteness checks, in a fixed order.
__global__ void __launch_bounds__(256) k_ex_reduce(MeshDev m, ExnerDev e, const double *q, const double *z,
                                                   const int *cell_offset, const int *face_offset)
{
    __shared__ double red[4][256];
    __shared__ int flags[2];
    const int sid = blockIdx.x, tid = threadIdx.x;
    if (!e.enabled[sid]) return;
    const double *p = e.param + (size_t)sid * EP_N;
    const double dtm = e.dt[sid] * p[EP_MORFAC], phi = 1.0 - p[EP_POROSITY], sd = p[EP_SEDDEPTH];
    if (tid < 2) flags[tid] = 0;
    __syncthreads();
    double res = 0., bnd = 0., donor = 1., change = 0.;
    bool bad = false;
    for (int i = cell_offset[sid] + tid; i < cell_offset[sid + 1]; i += blockDim.x) {
        const double zt = e.ztrial[i];
        if (!isfinite(zt) || zt < e.rock[i] - 1e-13) bad = true;
        res += phi * (zt - z[i]) * m.area[i];
        donor = fmin(donor, e.fac[i]);
        change = fmax(change, fabs(zt - z[i]) / fmax(q[i], sd));
    }
    for (int f = face_offset[sid] + tid; f < face_offset[sid + 1]; f += blockDim.x)
        if (m.neighbour[f] < 0 && m.bid[f] >= 0) bnd -= dtm * e.flux[f] * m.length[f];
    if (bad) atomicOr(&flags[0], 1);
    red[0][tid] = res; red[1][tid] = bnd; red[2][tid] = donor; red[3][tid] = change;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (tid < w) {
            red[0][tid] += red[0][tid + w]; red[1][tid] += red[1][tid + w];
            red[2][tid] = fmin(red[2][tid], red[2][tid + w]); red[3][tid] = fmax(red[3][tid], red[3][tid + w]);
        }
        __syncthreads();
    }
    if (tid == 0) {
        double *s = e.stats + (size_t)sid * ES_N;
        const double residual = red[0][0] - red[1][0];
        const bool slope_bad = e.bad[sid] != 0;
        s[ES_OK] = (!flags[0] && !slope_bad && fabs(residual) <= 1e-10 && red[3][0] <= .05) ? 1. : 0.;
        s[ES_RESIDUAL] = residual; s[ES_BOUNDARY] = red[1][0]; s[ES_DONOR] = red[2][0]; s[ES_CHANGE] = red[3][0];
        s[ES_BAD] = slope_bad ? 1. : 0.;
    }
}

__global__ void __launch_bounds__(256) k_ex_commit(MeshDev m, ExnerDev e, double *z)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m.nc; i += gridDim.x * blockDim.x) {
        const int sid = m.cell_sid[i];
        if (e.enabled[sid] && e.stats[(size_t)sid * ES_N + ES_OK] != 0.) z[i] = e.ztrial[i];
    }
}

}  // namespace brx
