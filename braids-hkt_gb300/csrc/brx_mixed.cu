// Mixed-precision form of the river step.
//
// Same algorithm as the FP64 form (the reference's reconstruction, hydrostatic
// reconstruction at the common face bed, augmented f-wave, flux assembly,
// donor limiter and SSPRK(2,2) update), rearranged for a GPU whose FP64 rate
// is a small fraction of its FP32 rate: the cell, face and gather sweeps do
// no FP64 arithmetic per neighbour or per face.
//
//   * The kernels that produce a stage input (the drag half-step and the
//     first-stage update) also write a 32-byte FP32 primitive record per cell:
//     depth, velocities, a wet bit decided on the FP64 depth, and the FP64
//     stage eta = h + b as an unevaluated pair of FP32 numbers (hi, lo).
//     Differences (hi_n - hi_c) + (lo_n - lo_c) carry the FP64 stage to FP32
//     accuracy of the difference and vanish exactly for equal stages, so the
//     stage reconstruction keeps FP64 information at wet/dry faces.
//   * Bed differences per CSR entry and per face, and the limited bed gradient
//     (it depends on the bed alone, except beside a stage outlet), are tables
//     rebuilt from the FP64 bed at the start of every call.
//   * Every reconstructed face value is an FP32 increment relative to its
//     cell. The hydrostatic part of the momentum flux minus the gathering
//     cell's own pressure is evaluated in perturbation form,
//        1/2 g [ (hL - h)(hL + h) + (h + raw) d_b ],
//     with separately rounded products, which cancels exactly for a surface
//     at rest.
//   * The Riemann solve, limiter, projection, gather sums and drag run in
//     FP32. The donor factor carries a margin that covers the FP32 outflow
//     sum, so the FP64 depth update stays nonnegative.
//   * Mass bookkeeping (limited water flux, the depth update) uses FP64
//     signed weights s*len/area, so mass telescopes exactly.
//
// This unit is compiled with FMA contraction and fast FP32 division / sqrt.
#include <algorithm>
#include "brx_launch.h"
#include "brx_fwave.cuh"

namespace brx_mx {
using namespace brx;

constexpr float FEPS = 1.1920928955078125e-07f;

// FP32 primitives of one stage input, one sector per cell.
struct __align__(16) MxPrim {
    float ehi, elo;   // eta = h + b (FP64) as ehi = fl32(eta), elo = fl32(eta - ehi)
    float h, u, v;    // depth, velocities (0 when dry)
    int wet;          // h > dry, decided on the FP64 depth
    float pad0, pad1;
};
static_assert(sizeof(MxPrim) == 32, "primitive record is one sector");

// Cell record of the face sweep, 64 bytes.
struct __align__(16) MxRec {
    float h;
    int flags;                   // bit0 flatten, bit1 active, bit2 wet
    float ehi, elo;
    float u, v;
    float gx[4], gy[4];          // eta, u, v, b
    float pad0, pad1;
};
static_assert(sizeof(MxRec) == 64, "mixed record is half a line");

struct __align__(16) MxLim {
    double water;                // limited mass flux (FP64: both cells use this value)
    float cx, cy;                // momentum correction
};

// Bit-level tests and conversions of FP64 values on the integer pipe. This
// part issues FP64 instructions (compares and conversions included) at about
// two lanes per clock per SM, a few percent of its integer rate, and the
// update and drag sweeps spent most of their FP64 issue slots on compares
// and conversions between the FP32 sweep values and the FP64 state. The
// 64-bit register is split and joined with inline mov.b64, which the
// optimizer treats as opaque, so it cannot fold these tests back into FP64
// compares and conversions.
__device__ __forceinline__ void dsplit(double x, unsigned &hi, unsigned &lo)
{
    asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(x));
}
__device__ __forceinline__ double djoin(unsigned hi, unsigned lo)
{
    double x;
    asm("mov.b64 %0, {%1, %2};" : "=d"(x) : "r"(lo), "r"(hi));
    return x;
}

// x is neither infinite nor NaN
__device__ __forceinline__ bool finite64(double x)
{
    unsigned hi, lo;
    dsplit(x, hi, lo);
    return (hi & 0x7ff00000u) != 0x7ff00000u;
}

// x <= threshold for a positive finite threshold, as a signed 64-bit compare
// of the bit patterns (the order of non-NaN doubles against a positive
// value; a NaN depth fails the state's finiteness check wherever this is used)
__device__ __forceinline__ bool le_threshold(double x, double threshold)
{
    unsigned xh, xl, th, tl;
    dsplit(x, xh, xl);
    dsplit(threshold, th, tl);
    return (int)xh < (int)th || (xh == th && xl <= tl);
}

// x < 0 (false for -0 and NaN, as the FP64 compare): the sign bit with a
// magnitude in (0, inf]
__device__ __forceinline__ bool lt_zero(double x)
{
    unsigned hi, lo;
    dsplit(x, hi, lo);
    const unsigned mh = hi & 0x7fffffffu;
    return (int)hi < 0 && (mh | lo) != 0u && (mh < 0x7ff00000u || (mh == 0x7ff00000u && lo == 0u));
}

// float -> double, exact (every float is a double): the sign, the exponent
// rebased by 1023 - 127, the 23 fraction bits at the top of the 52;
// subnormals normalised; infinities and NaN keep their payload.
__device__ __forceinline__ double f2d(float f)
{
    const unsigned b = __float_as_uint(f);
    const unsigned sign = b & 0x80000000u, e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
    unsigned hi = sign | ((e + 896u) << 20) | (m >> 3), lo = m << 29;
    if (e == 0xffu) hi = sign | 0x7ff00000u | (m >> 3);
    if (e == 0u) {
        if (m == 0u) { hi = sign; lo = 0u; }
        else {
            const int p = 31 - __clz(m);                       // leading bit of the subnormal fraction
            const unsigned long long frac = (unsigned long long)(m ^ (1u << p)) << (52 - p);
            hi = sign | ((unsigned)(p + 874) << 20) | (unsigned)(frac >> 32);
            lo = (unsigned)frac;
        }
    }
    return djoin(hi, lo);
}

// double -> float, to nearest with ties to even, as this unit's flush-to-zero
// conversion: the top 23 of the 52 fraction bits kept and the low 29 deciding
// the rounding (a carry into the exponent is the correct result, up to
// infinity); results below the float normal range flush to a signed zero,
// results above it are infinite, NaN stays NaN.
__device__ __forceinline__ float d2f(double x)
{
    unsigned hi, lo;
    dsplit(x, hi, lo);
    const unsigned sign = hi & 0x80000000u, e = (hi >> 20) & 0x7ffu;
    const unsigned top = ((hi & 0xfffffu) << 3) | (lo >> 29), rem = lo & 0x1fffffffu;
    unsigned r = sign | (((e - 896u) & 0xffu) << 23) | top;
    if (rem > 0x10000000u || (rem == 0x10000000u && (top & 1u))) r += 1u;
    if (e < 896u || (r & 0x7f800000u) == 0u) r = sign;                        // flushed
    if (e > 1150u) r = sign | 0x7f800000u;                                     // overflow
    if (e == 0x7ffu && ((hi & 0xfffffu) | lo)) r = sign | 0x7fc00000u;        // NaN
    return __uint_as_float(r);
}

// Stage 2 skips a scenario whose first stage failed (status, or the CFL test
// evaluated once per scenario after the first gather).
__device__ __forceinline__ bool mx_skip(const Ctrl &c, int stage)
{
    if (!c.active || c.done) return true;
    return stage == 2 && (c.status1 != 0u || c.cfl1 != 0);
}

// FP32 primitives of a cell state; returns whether the state is a valid sweep input.
__device__ __forceinline__ bool put_prim(MxPrim *P, int c, double h, double hu, double hv, double z, double dry)
{
    const double eta = h + z;
    MxPrim p;
    p.ehi = d2f(eta);
    p.elo = d2f(eta - f2d(p.ehi));
    p.h = d2f(h);
    const bool wet = !le_threshold(h, dry);
    p.u = wet ? d2f(hu) / p.h : 0.f;
    p.v = wet ? d2f(hv) / p.h : 0.f;
    p.wet = wet;
    p.pad0 = 0.f; p.pad1 = 0.f;
    P[c] = p;
    return !lt_zero(h) && finite64(h) && finite64(hu) && finite64(hv) && finite64(z);
}

// Per-scenario CFL peak: FP32 warp maximum, one atomic per scenario group.
__device__ __forceinline__ void warp_max_peak_f(unsigned long long *peak_of_sid0, size_t stride_bytes, int sid,
                                                bool valid, float v)
{
    const unsigned bits = valid ? __float_as_uint(v) : 0u;     // nonnegative floats order like their bits
    const unsigned same = __match_any_sync(0xffffffffu, valid ? sid : -1);
    const unsigned top = __reduce_max_sync(same, bits);
    if (valid && (int)(threadIdx.x & 31) == __ffs(same) - 1) {
        unsigned long long *addr = (unsigned long long *)((char *)peak_of_sid0 + stride_bytes * (size_t)sid);
        atomicMax(addr, (unsigned long long)__double_as_longlong(f2d(__uint_as_float(top))));
    }
}

// ---------------------------------------------------------------------------
// Gradient bounds: the directional projection limiter on a set of slabs
//     -bm[j] <= (ux[j], uy[j]) . g <= bp[j]      (entries j of one cell)
// ---------------------------------------------------------------------------
template <int N>
struct Slabs {
    float ux[N], uy[N], bp[N], bm[N];
    unsigned mask;   // enabled entries
};

template <int N>
__device__ __forceinline__ bool slabs_feasible(const Slabs<N> &S, float x, float y)
{
    bool ok = true;
#pragma unroll (N <= 4 ? N : 1)
    for (int j = 0; j < N; ++j)
        if (S.mask >> j & 1u) {
            const float t = S.ux[j] * x + S.uy[j] * y;
            const float a = fabsf(S.ux[j] * x) + fabsf(S.uy[j] * y);
            if (t > S.bp[j] + (2.e-14f + 16.f * FEPS * (a + S.bp[j]))) ok = false;
            if (-t > S.bm[j] + (2.e-14f + 16.f * FEPS * (a + S.bm[j]))) ok = false;
        }
    return ok;
}

// Nearest feasible point: the best feasible candidate among single-side
// projections and pairwise vertices. The polygon contains the origin (all
// bounds >= 0) and is convex, so its nearest point is unique and lies on a
// side the unlimited gradient violates: only violated sides seed candidates.
template <int N>
__device__ __forceinline__ void slabs_project(const Slabs<N> &S, float &x, float &y)
{
    const float rx = x, ry = y;
    float bx = 0.f, by = 0.f, best = rx * rx + ry * ry;
#pragma unroll (N <= 4 ? N : 1)
    for (int i = 0; i < N; ++i) {
        if (!(S.mask >> i & 1u)) continue;
        const float t = S.ux[i] * rx + S.uy[i] * ry;
        float ax, ay, b;
        if (t - S.bp[i] > 0.f) { ax = S.ux[i]; ay = S.uy[i]; b = S.bp[i]; }
        else if (-t - S.bm[i] > 0.f) { ax = -S.ux[i]; ay = -S.uy[i]; b = S.bm[i]; }
        else continue;
        const float dot = ax * rx + ay * ry - b;
        float cx = rx - dot * ax, cy = ry - dot * ay;
        float d = (cx - rx) * (cx - rx) + (cy - ry) * (cy - ry);
        if (d < best && slabs_feasible(S, cx, cy)) { bx = cx; by = cy; best = d; }
#pragma unroll (N <= 4 ? N : 1)
        for (int j = 0; j < N; ++j) {
            if (j == i || !(S.mask >> j & 1u)) continue;
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                const float jx = side ? -S.ux[j] : S.ux[j], jy = side ? -S.uy[j] : S.uy[j];
                const float jb = side ? S.bm[j] : S.bp[j];
                const float det = ax * jy - ay * jx;
                if (fabsf(det) < 1.e-12f) continue;
                cx = (b * jy - ay * jb) / det;
                cy = (ax * jb - b * jx) / det;
                d = (cx - rx) * (cx - rx) + (cy - ry) * (cy - ry);
                if (d < best && slabs_feasible(S, cx, cy)) { bx = cx; by = cy; best = d; }
            }
        }
    }
    x = bx; y = by;
}

// ---------------------------------------------------------------------------
// Bed-derived tables (once per call: the bed may change between calls)
// ---------------------------------------------------------------------------
template <int MAXF>
__global__ void __launch_bounds__(128) km_bed(MeshDev m, StateDev s, MixedGeo g)
{
    const int nc = m.nc, nf = m.nf, n = nc > nf ? nc : nf;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (i < nf) {
            const int o = m.neighbour[i];
            g.fdb[i] = o >= 0 ? float(s.z[o] - s.z[m.owner[i]]) : 0.f;
        }
        if (i >= nc) continue;
        const int c = i, k0 = m.offset[c], deg = m.offset[c + 1] - k0;
        const double zc = s.z[c];
        float bx = 0.f, by = 0.f, lo = 0.f, hi = 0.f;
        for (int k = k0; k < k0 + deg; ++k) {
            const int o = g.cidx[k].x;
            float d = 0.f;
            if (o >= 0) {
                d = float(s.z[o] - zc);
                const float4 ge = g.cent[k];
                bx += ge.x * d; by += ge.y * d;
                lo = fminf(lo, d); hi = fmaxf(hi, d);
            }
            g.cdb[k] = d;
        }
        if (g.hent)          // the HLLC incidence (faces ascending per cell)
            for (int k = k0; k < k0 + deg; ++k) {
                const int o = g.hent[k].y;
                g.hcdb[k] = o >= 0 ? float(s.z[o] - zc) : 0.f;
            }
        float2 gb = make_float2(0.f, 0.f);
        const float4 inv = g.cinv[c];
        if (inv.x != 0.f || inv.y != 0.f || inv.z != 0.f) {
            float gx = inv.x * bx + inv.y * by, gy = inv.y * bx + inv.z * by;
            Slabs<MAXF> S{};
            const float bp = fmaxf(0.f, hi), bm = fmaxf(0.f, -lo);
#pragma unroll (MAXF <= 4 ? MAXF : 1)
            for (int j = 0; j < MAXF; ++j) {
                if (j >= deg) continue;      // (a break would stop the unrolling)
                if (g.cidx[k0 + j].y & 4) continue;          // walls do not bound the bed
                const float4 ge = g.cent[k0 + j];
                const float len = sqrtf(ge.z * ge.z + ge.w * ge.w);
                if (len <= 0.f) continue;
                const float il = 1.f / len;
                S.ux[j] = ge.z * il; S.uy[j] = ge.w * il; S.bp[j] = bp * il; S.bm[j] = bm * il;
                S.mask |= 1u << j;
            }
            if (!slabs_feasible(S, gx, gy)) slabs_project(S, gx, gy);
            gb = make_float2(gx, gy);
        }
        g.gbed[c] = gb;
    }
}

// ---------------------------------------------------------------------------
// Cells: limited gradients and the cell record
// ---------------------------------------------------------------------------
// resident blocks per SM the register allocation of the cell sweep is fitted to
#ifndef BRX_CELLS_MIN_BLOCKS
#define BRX_CELLS_MIN_BLOCKS 8
#endif

// Wet least-squares gradients of u, v and the surface for the rotor face
// terms (river_turbine_flow.h:13-35): wet neighbours only, weights 1/|d|^2 of
// the flow metric's centre offsets. Called in the cell sweep's tail, after
// the cell record is written, so its sums are not live in the limiter; the
// neighbour primitives were just read and come from L1.
template <class Nbr>
__device__ __forceinline__ void hkt_cell_gradients(const MeshDev &m, const MixedGeo &g, const Nbr &nb,
                                                   const MxPrim &pc, int c, int nc)
{
    float xx = 0.f, xy = 0.f, yy = 0.f, bx[3] = {0.f, 0.f, 0.f}, by[3] = {0.f, 0.f, 0.f};
    if (pc.wet)
        for (int k0 = m.offset[c], k = k0; k < m.offset[c + 1]; ++k) {
            const int n = nb.id(k, k - k0).x;
            if (n < 0) continue;
            const MxPrim pn = nb.prim(n);
            if (!pn.wet) continue;
            const float2 d = g.hdxy[k];
            const float w = 1.f / (d.x * d.x + d.y * d.y);
            xx += w * d.x * d.x; xy += w * d.x * d.y; yy += w * d.y * d.y;
            const float dv[3] = {pn.u - pc.u, pn.v - pc.v, (pn.ehi - pc.ehi) + (pn.elo - pc.elo)};
#pragma unroll
            for (int p = 0; p < 3; ++p) { bx[p] += w * d.x * dv[p]; by[p] += w * d.y * dv[p]; }
        }
    const float det = xx * yy - xy * xy;
    const bool solve = det > 1e-6f * fmaxf(1.f, xx * yy);
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        g.hgrad[(2 * p) * nc + c] = solve ? (yy * bx[p] - xy * by[p]) / det : 0.f;
        g.hgrad[(2 * p + 1) * nc + c] = solve ? (xx * by[p] - xy * bx[p]) / det : 0.f;
    }
}

// Neighbour access of the cell record: entry j (global entry k) of the cell
// and the primitive record of the neighbour it names. The grid sweep reads
// the mesh's entries and the stage primitives in global memory.
struct GlobalNbr {
    const int2 *cidx;
    const MxPrim *P;
    __device__ __forceinline__ int2 id(int k, int) const { return cidx[k]; }
    __device__ __forceinline__ MxPrim prim(int n) const { return P[n]; }
};

// Cell record of one cell (limited gradients and flags) from its primitives
// pc and its neighbours' through nb: the body of the cell sweep.
template <int MAXF, class Nbr>
__device__ __forceinline__ MxRec mx_record(const MeshDev &m, const StateDev &s, const Ctrl &ct, const MixedGeo &g,
                                           const MxPrim &pc, int c, int k0, int deg, const Nbr &nb)
{
    {
        const float dry = ct.dryf;
        const bool wet = pc.wet != 0;
        const float hf = pc.h, u = pc.u, v = pc.v;
        const bool outlet = g.ccls[c] & 1;   // a stage outlet face: the bed gradient is formed here
        // bounds of eta and b relative to the cell (centre = 0), of u and v absolute
        float lo[4] = {0.f, u, v, 0.f}, hi[4] = {0.f, u, v, 0.f};
        float bx[4] = {0.f, 0.f, 0.f, 0.f}, by[4] = {0.f, 0.f, 0.f, 0.f};
        bool active = wet;
        for (int k = k0; k < k0 + deg; ++k) {
            const int2 id = nb.id(k, k - k0);
            const int n = id.x;
            if (n < 0) {
                if (id.y & 1) active = true;
                else if ((id.y & 4) && wet) {
                    // a wall bounds the velocities by the mirrored cell velocity
                    const float2 nn = g.fnorm[m.faces[k]];
                    const float un = u * nn.x + v * nn.y;
                    const float mx = u - 2.f * un * nn.x, my = v - 2.f * un * nn.y;
                    lo[1] = fminf(lo[1], mx); hi[1] = fmaxf(hi[1], mx);
                    lo[2] = fminf(lo[2], my); hi[2] = fmaxf(hi[2], my);
                }
                continue;
            }
            const MxPrim pn = nb.prim(n);
            const bool wetn = pn.wet != 0;
            if (wetn) active = true;
            const float ddb = g.cdb[k];
            float d[4];
            d[0] = (pn.ehi - pc.ehi) + (pn.elo - pc.elo);
            d[1] = pn.u - u;
            d[2] = pn.v - v;
            d[3] = ddb;
            // a dry neighbour whose bed rises above the wet surface contributes the surface
            if (wet && !wetn && ddb >= hf) d[0] = 0.f;
            const float4 ge = g.cent[k];     // LS weight * (dx, dy), face displacement
#pragma unroll
            for (int p = 0; p < 3; ++p) {
                bx[p] += ge.x * d[p];
                by[p] += ge.y * d[p];
                const float val = (p == 1 || p == 2) ? d[p] + (p == 1 ? u : v) : d[p];
                lo[p] = fminf(lo[p], val); hi[p] = fmaxf(hi[p], val);
            }
            if (outlet) {
                bx[3] += ge.x * d[3]; by[3] += ge.y * d[3];
                lo[3] = fminf(lo[3], d[3]); hi[3] = fmaxf(hi[3], d[3]);
            }
        }
        float gx[4] = {0.f, 0.f, 0.f, 0.f}, gy[4] = {0.f, 0.f, 0.f, 0.f};
        const float4 inv = g.cinv[c];
        if (active && (inv.x != 0.f || inv.y != 0.f || inv.z != 0.f)) {
#pragma unroll
            for (int p = 0; p < 3; ++p) {
                gx[p] = inv.x * bx[p] + inv.y * by[p];
                gy[p] = inv.y * bx[p] + inv.z * by[p];
            }
            float bedtol = 0.f, sq = 0.f;
            if (outlet) {
                gx[3] = inv.x * bx[3] + inv.y * by[3];
                gy[3] = inv.y * bx[3] + inv.z * by[3];
                bedtol = 64.f * FEPS * fmaxf(1.f, fabsf(float(s.z[c])));
                sq = wet ? sqrtf(ct.gravf * hf) : 0.f;
            } else {
                const float2 gb = g.gbed[c];
                gx[3] = gb.x; gy[3] = gb.y;
            }
            float theta1 = 1.f, theta2 = 1.f;
            // one slab set, filled for the surface, then (stage-outlet cells
            // only) refilled for the bed: half the live registers of two sets
            Slabs<MAXF> S{};
            const float b0p = fmaxf(0.f, hi[0]), b0m = fmaxf(0.f, -lo[0]);
#pragma unroll (MAXF <= 4 ? MAXF : 1)
            for (int j = 0; j < MAXF; ++j) {
                if (j >= deg) continue;      // (a break would stop the unrolling)
                const int k = k0 + j;
                const float4 ge = g.cent[k];
                const float rx = ge.z, ry = ge.w;
                if (outlet && (nb.id(k, j).y & 2) && wet) {
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
                const float il = 1.f / len;
                S.ux[j] = rx * il; S.uy[j] = ry * il; S.bp[j] = b0p * il; S.bm[j] = b0m * il;
                S.mask |= 1u << j;
            }
            if (!slabs_feasible(S, gx[0], gy[0])) slabs_project(S, gx[0], gy[0]);
            if (outlet) {
                const float b3p = fmaxf(0.f, hi[3]), b3m = fmaxf(0.f, -lo[3]);
                S.mask = 0u;
#pragma unroll (MAXF <= 4 ? MAXF : 1)
                for (int j = 0; j < MAXF; ++j) {
                    if (j >= deg) continue;
                    const int k = k0 + j;
                    const int fl = nb.id(k, j).y;
                    const float4 ge = g.cent[k];
                    const float rx = ge.z, ry = ge.w;
                    if ((fl & 2) && wet) {
                        const float2 nn = g.fnorm[m.faces[k]];
                        if (fabsf(u * nn.x + v * nn.y) < sq && fabsf(gx[3] * rx + gy[3] * ry) > bedtol) continue;
                    }
                    const float len = sqrtf(rx * rx + ry * ry);
                    if (len <= 0.f || (fl & 4)) continue;          // walls do not bound the bed
                    const float il = 1.f / len;
                    S.ux[j] = rx * il; S.uy[j] = ry * il; S.bp[j] = b3p * il; S.bm[j] = b3m * il;
                    S.mask |= 1u << j;
                }
                if (!slabs_feasible(S, gx[3], gy[3])) slabs_project(S, gx[3], gy[3]);
            }
            gx[1] *= fmaxf(0.f, theta1); gy[1] *= fmaxf(0.f, theta1);
            gx[2] *= fmaxf(0.f, theta2); gy[2] *= fmaxf(0.f, theta2);
        }
        bool flatten = !wet;
        if (!flatten) {
            for (int k = k0; k < k0 + deg; ++k) {
                const float4 ge = g.cent[k];
                const float de = gx[0] * ge.z + gy[0] * ge.w, db = gx[3] * ge.z + gy[3] * ge.w;
                if (hf + (de - db) <= dry || fabsf(db) >= hf) { flatten = true; break; }
            }
        }
        MxRec r;
        r.h = hf;
        r.flags = (flatten ? 1 : 0) | (active ? 2 : 0) | (wet ? 4 : 0);
        r.ehi = pc.ehi; r.elo = pc.elo; r.u = u; r.v = v;
#pragma unroll
        for (int p = 0; p < 4; ++p) { r.gx[p] = gx[p]; r.gy[p] = gy[p]; }
        r.pad0 = 0.f; r.pad1 = 0.f;
        return r;
    }
}

template <int MAXF>
__global__ void __launch_bounds__(128, BRX_CELLS_MIN_BLOCKS) km_cells(MeshDev m, StateDev s, Ctrl *ctrl, Work w,
                                                                      MixedGeo g, int stage, TurbDev t, int turb)
{
    const int nc = m.nc;
    MxRec *rec = reinterpret_cast<MxRec *>(w.rec);
    const MxPrim *P = reinterpret_cast<const MxPrim *>((stage == 1 ? g.prim[0] : g.prim[1]));
    const GlobalNbr nb{g.cidx, P};
    FOR_ACTIVE_CELLS(m.act, c) {
        const Ctrl &ct = ctrl[m.cell_sid[c]];
        if (mx_skip(ct, stage)) continue;
        const MxPrim pc = P[c];
        const int k0 = m.offset[c], deg = m.offset[c + 1] - k0;
        rec[c] = mx_record<MAXF>(m, s, ct, g, pc, c, k0, deg, nb);
        if (turb && t.hkt[m.cell_sid[c]]) hkt_cell_gradients(m, g, nb, pc, c, nc);
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
    const float hf = r.h;
    const bool constant = r.flags & 1, wet = r.flags & 4;
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
    if (!wet || (constant && raw <= dry)) depth = 0.f;
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

// Rotor face terms of one interior face between two wet cells (the balanced
// pressure correction and the ambient stress, river_turbine_flow.h:13-82,
// river_hydrokinetic_stress.h:13-35), from the cell records and the face's
// hydrostatic traces t0 (hl, hr, common bed, constant flags) and t1 (un_l,
// un_r, |u|_l, |u|_r): computed in the face sweep's tail, so the traces never
// leave registers. Heights are relative to the owner's bed; the hydrostatic
// part of the pressure correction is written in difference form,
//   1/4 g [(hl-ha)(hl+ha) + (hr-hb)(hr+hb)] + 1/4 g (da-db)/d (ha-hb)(ha+hb)
//   + 1/4 g [ca (ha-hl)(ha+hl) + cb (hb-hr)(hb+hr)]
// (algebraically the reference's 1/2 (po + pn) - 1/2 g (wa ha^2 + wb hb^2)),
// so a surface at rest gives exactly zero and FP32 carries only the small
// differences.
__device__ __forceinline__ void hkt_face_terms(const MxRec &pa, const MxRec &pb, float4 t0, float4 t1, int f, int a,
                                               int b, int sid, float gravity, float dry, const MixedGeo &g,
                                               const TurbDev &t, int nc, float2 &pr, float2 &st)
{
    const float2 nn = g.fnorm[f], di = g.fdist[f];
    const float nx = nn.x, ny = nn.y, da = di.x, db = di.y, d = da + db, wa = db / d, wb = da / d;
    const float zb = g.fdb[f];
    const float ea = pa.h, eb = pa.h + ((pb.ehi - pa.ehi) + (pb.elo - pa.elo));
    if (t.stress[sid]) {
        float h = fminf(pa.h, pb.h);
        h = fminf(h, fmaxf(0.f, .5f * (ea + eb) - fmaxf(0.f, zb)));
        const float visc = wa * float(t.nu[a]) + wb * float(t.nu[b]);
        const float2 dd = g.hcc[f];
        const float dn = dd.x * nx + dd.y * ny;
        const float du = pb.u - pa.u, dv = pb.v - pa.v;
        const float *G = g.hgrad;
        float ux = wa * G[a] + wb * G[b], uy = wa * G[nc + a] + wb * G[nc + b];
        float vx = wa * G[2 * nc + a] + wb * G[2 * nc + b], vy = wa * G[3 * nc + a] + wb * G[3 * nc + b];
        const float cu = (du - ux * dd.x - uy * dd.y) / dn, cv = (dv - vx * dd.x - vy * dd.y) / dn;
        ux += cu * nx; uy += cu * ny; vx += cv * nx; vy += cv * ny;
        st = make_float2(visc * h * (2.f * ux * nx + (uy + vx) * ny), visc * h * ((uy + vx) * nx + 2.f * vy * ny));
    }
    const int cf = __float_as_int(t0.w);
    const float top = t0.z, bed = fmaxf(fmaxf(0.f, zb), top);
    const float ha = fmaxf(0.f, ea - bed), hb = fmaxf(0.f, eb - bed);
    const float hl = fmaxf(0.f, (top + t0.x) - bed), hr = fmaxf(0.f, (top + t0.y) - bed);
    const float h = .5f * (hl + hr);
    const float qg = .25f * gravity;
    const float ca = (cf & 1) ? qg * __fmul_rn(ha - hl, ha + hl) : 0.f;
    const float cb = (cf & 2) ? qg * __fmul_rn(hb - hr, hb + hr) : 0.f;
    const float scale = qg * (hl * hl + hr * hr);                       // |po|, |pn| to first order
    if (!(fminf(fminf(ha, hb), fminf(hl, hr)) <= dry) && !(fabsf(hr - hl) > .005f * h) &&
        !(fabsf(2.f * (ca - cb)) > 128.f * FEPS * fmaxf(1.f, scale))) {
        const float4 md = g.hmd[f];
        const float sx = wa * md.x + wb * md.z, sy = wa * md.y + wb * md.w;
        const float *G = g.hgrad;
        float delta = qg * (__fmul_rn(hl - ha, hl + ha) + __fmul_rn(hr - hb, hr + hb)) +
                      qg * ((da - db) / d) * __fmul_rn(ha - hb, ha + hb) + (ca + cb);
        delta -= gravity * sx * (wa * ha * G[4 * nc + a] + wb * hb * G[4 * nc + b]);
        delta -= gravity * sy * (wa * ha * G[5 * nc + a] + wb * hb * G[5 * nc + b]);
        // the actuator sink difference: FP64 rates, zero outside the rotor
        // support cells, so only faces touching one read and subtract them
        if (t.foot[a] | t.foot[b])
            delta -= da * db / d * (float(t.raw[a] - t.raw[b]) * nx + float(t.raw[nc + a] - t.raw[nc + b]) * ny);
        const float speed = sqrtf(gravity * h), theta = fminf(1.f, fmaxf(t1.z, t1.w) / speed);
        delta -= .5f * (1.f - theta) * speed * (2.f * hl * hr / (hl + hr)) * (t1.y - t1.x);
        pr = make_float2(delta * nx, delta * ny);
    }
}

// Fluxes of one interior or wall face from its cells' records (the body of
// the face sweep): the FP32 water flux and CFL speed, both sides' momentum
// fluxes; the rotor face terms go to g.hp / g.hs. n < 0: a wall (rn unused).
struct MxFaceOut {
    float water, speed, gl1, gl2, gr1, gr2;
};

__device__ __forceinline__ MxFaceOut mx_face(const MeshDev &m, const StateDev &s, Ctrl &ct, const MixedGeo &g,
                                             int stage, const TurbDev &t, bool rotors, int sid, int f, int c, int n,
                                             const MxRec &rc, const MxRec &rn)
{
    const int nc = m.nc;
    const float dry = ct.dryf, grav = ct.gravf;
    const float half_g = 0.5f * grav;
    const float2 nn = g.fnorm[f];
    const float nx = nn.x, ny = nn.y;
    const float hc = rc.h;
    {
        const bool wc = rc.flags & 4, wn = n >= 0 && (rn.flags & 4);
        int kind = n >= 0 ? 1 : 2;
        if (!wc && !wn) kind = 0;
        unsigned bad = 0;
        const float4 dsp = g.fdisp[f];
        const MxSide L = mx_side(rc, dsp.x, dsp.y, dry, kind == 0, bad);
        MxSide R = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const float hn = n >= 0 ? rn.h : 0.f;
        if (n >= 0) R = mx_side(rn, dsp.z, dsp.w, dry, kind == 0, bad);
        float water = 0.f, speed = 0.f;
        float gl1 = 0.f, gl2 = 0.f, gr1 = 0.f, gr2 = 0.f;
        bool rotor_face = false;       // the rotor face terms were formed in the flux branch
        if (kind != 0) {
            float hL = L.h, xL = L.hu, yL = L.hv;
            float hR = R.h, xR = R.hu, yR = R.hv;
            // surfaces and beds relative to the owner's surface / bed; both sides
            // share the owner's depth as base, so a surface at rest gives
            // bit-identical hydrostatic depths on the two sides
            const float bLr = L.db;
            float bRr = n >= 0 ? g.fdb[f] + R.db : L.db;
            const float sL = hc + L.de;
            float sR = n >= 0 ? hc + (((rn.ehi - rc.ehi) + (rn.elo - rc.elo)) + R.de) : sL;
            if (kind == 2) { hR = hL; xR = xL; yR = yL; bRr = bLr; sR = sL; }
            float xRr = xR, yRr = yR;
            if (kind == 2) {
                const float dot = xL * nx + yL * ny;
                xRr = xL - 2.f * dot * nx; yRr = yL - 2.f * dot * ny;
            }
            const float unL = xL * nx + yL * ny, utL = xL * (-ny) + yL * nx;
            const float unR = xRr * nx + yRr * ny, utR = xRr * (-ny) + yRr * nx;
            float loc[8] = {hL, unL, utL, 0.f, hR, unR, utR, 0.f};
            float top_bed = 0.f;           // the face's common bed (kind 1), for the rotor terms
            if (kind == 1) {
                const float top = fmaxf(bLr, bRr);
                float hl = hL > 0.f ? fmaxf(0.f, sL - top) : 0.f, hr = hR > 0.f ? fmaxf(0.f, sR - top) : 0.f;
                // The FP32 depths above the common bed are differences of
                // values relative to the owner's bed, good to a few FP32 ulps
                // of those values. Within that band of the dry threshold the
                // decision is taken in FP64 from the FP64 state and bed, with
                // the reference's roundoff tolerance (16 eps of the absolute
                // elevations, face_activity.py:33-37); outside it, FP32 and
                // FP64 agree. A film just above the dry depth is then active
                // in both forms (an elevation-scaled FP32 tolerance would
                // close it, and the face would carry a different flux every
                // substep).
                const float band = 16.f * FEPS * fmaxf(dry, fmaxf(fmaxf(fabsf(sL), fabsf(sR)), fabsf(top)));
                if ((hl > 0.f && fabsf(hl - dry) <= band) || (hr > 0.f && fabsf(hr - dry) <= band)) {
                    const double *q = stage == 1 ? s.work : s.q1;
                    const double zc = s.z[c], zn = s.z[n];
                    const double etaL = zc + q[c] + double(L.de), etaR = zn + q[n] + double(R.de);
                    const double topd = fmax(zc + double(L.db), zn + double(R.db));
                    const double tol64 = 16. * EPS * fmax(ct.dry, fmax(fabs(topd), fmax(fabs(etaL), fabs(etaR))));
                    const double hld = hL > 0.f ? fmax(0., etaL - topd) : 0., hrd = hR > 0.f ? fmax(0., etaR - topd) : 0.;
                    hl = hld <= ct.dry + tol64 ? 0.f : float(hld);
                    hr = hrd <= ct.dry + tol64 ? 0.f : float(hrd);
                } else {
                    if (hl <= dry) hl = 0.f;
                    if (hr <= dry) hr = 0.f;
                }
                loc[0] = hl; loc[4] = hr;
                const float sl = hL > dry ? __fdividef(hl, hL) : 0.f, sr = hR > dry ? __fdividef(hr, hR) : 0.f;
                loc[1] = unL * sl;
                loc[2] = utL * sl;
                loc[5] = unR * sr;
                loc[6] = utR * sr;
                top_bed = top;
            }
            bool closed = false;
            if (kind == 1 && !(fminf(hc, hn) > dry)) {
                // wet/dry face: the shared surface from distance-weighted cell stages (FP64, rare)
                const double *q = stage == 1 ? s.work : s.q1;
                const double zc = s.z[c], zn = s.z[n], hcd = q[c], hnd = q[n];
                const float2 di = g.fdist[f];
                const double dc = di.x, dn = di.y;
                double shared;
                if (dc + dn > 0.0)
                    shared = (dn * (zc + hcd) + dc * (zn + hnd)) / (dc + dn) - fmax(zc, zn);
                else
                    shared = 0.5 * ((zc + hcd) + (zn + hnd)) - fmax(zc, zn);
                closed = shared <= ct.dry;
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
                if (starL > dry) { const float r = __fdividef(loc[1], starL); dl0 = loc[1]; dl1 = loc[1] * r; dl2 = loc[2] * r; }
                if (starR > dry) { const float r = __fdividef(loc[5], starR); dr0 = loc[5]; dr1 = loc[5] * r; dr2 = loc[6] * r; }
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
            if (rotors && kind == 1 && wc && wn) {
                // traces for the rotor pressure correction (beds relative to the
                // owner's; loc holds the hydrostatic face states, fwave reads it only)
                const float hl = loc[0], hr = loc[4];
                const float4 t0 = make_float4(hl, hr, top_bed, __int_as_float((rc.flags & 1) | ((rn.flags & 1) << 1)));
                const float4 t1 = make_float4(hl > 0.f ? loc[1] / hl : 0.f, hr > 0.f ? loc[5] / hr : 0.f,
                                              hl > 0.f ? hypotf(loc[1], loc[2]) / hl : 0.f,
                                              hr > 0.f ? hypotf(loc[5], loc[6]) / hr : 0.f);
                float2 pr = make_float2(0.f, 0.f), st = make_float2(0.f, 0.f);
                hkt_face_terms(rc, rn, t0, t1, f, c, n, sid, grav, dry, g, t, nc, pr, st);
                g.hp[f] = pr;
                if (t.stress[sid]) g.hs[f] = st;
                rotor_face = true;
            }
        } else {
            // dry face: zero flux, the cells' own pressure still enters the gather
            gl1 = -half_g * hc * hc * nx; gl2 = -half_g * hc * hc * ny;
            gr1 = -half_g * hn * hn * nx; gr2 = -half_g * hn * hn * ny;
        }
        if (bad) raise_status(ct, stage, ST_SPATIAL);
        if (rotors && !rotor_face) {
            g.hp[f] = make_float2(0.f, 0.f);
            if (t.stress[sid]) g.hs[f] = make_float2(0.f, 0.f);
        }
        return MxFaceOut{water, speed, gl1, gl2, gr1, gr2};
    }
}

// Open face: the exterior owner's flux and the owner/exterior CFL speed (FP64, few faces).
__device__ __forceinline__ void mx_open_face(const MeshDev &m, const StateDev &s, const BoundaryDev &b, const Ctrl &ct,
                                             int stage, int f, int c, int slot, float2 &wsf, float4 &gff)
{
    const int nf = m.nf, nc = m.nc;
    const double *q = stage == 1 ? s.work : s.q1;
    const double dn = m.normal[f], dm = m.normal[nf + f], gd = ct.grav, dd = ct.dry;
    const double fl0 = b.flux[slot], fl1 = b.flux[(size_t)b.nslot + slot], fl2 = b.flux[2 * (size_t)b.nslot + slot];
    const double hb = b.trace[slot], hq = q[c];
    const double pc = .5 * gd * hq * hq;
    const double a = hq > dd ? fabs((q[nc + c] * dn + q[2 * nc + c] * dm) / hq) + sqrt(gd * hq) : 0.;
    const double bb = hb > dd ? fabs((b.trace[(size_t)b.nslot + slot] * dn + b.trace[2 * (size_t)b.nslot + slot] * dm) / hb) +
                                    sqrt(gd * hb) : 0.;
    wsf = make_float2(float(fl0), float(fmax(a, bb)));
    gff = make_float4(float(fl1 - pc * dn), float(fl2 - pc * dm), 0.f, 0.f);
}

// resident blocks per SM the register allocation of the face sweep is fitted to
#ifndef BRX_FACES_MIN_BLOCKS
#define BRX_FACES_MIN_BLOCKS 8
#endif

__global__ void __launch_bounds__(128, BRX_FACES_MIN_BLOCKS) km_faces(MeshDev m, StateDev s, BoundaryDev b, Ctrl *ctrl, Work w,
                                                MixedGeo g, int stage, TurbDev t, int turb)
{
    const MxRec *rec = reinterpret_cast<const MxRec *>(w.rec);
    float2 *ws = reinterpret_cast<float2 *>(w.ws);
    float4 *gf = reinterpret_cast<float4 *>(w.gf);
    FOR_ACTIVE_FACES(m.act, f) {
        const int sid = m.face_sid[f];
        Ctrl &ct = ctrl[sid];
        if (mx_skip(ct, stage)) continue;
        const bool rotors = turb && t.hkt[sid];
        const int c = m.owner[f], n = m.neighbour[f];
        const int slot = m.bslot[f];
        if (slot >= 0) {
            float2 wsf;
            float4 gff;
            mx_open_face(m, s, b, ct, stage, f, c, slot, wsf, gff);
            ws[f] = wsf;
            gf[f] = gff;
            if (rotors) {
                g.hp[f] = make_float2(0.f, 0.f);
                if (t.stress[sid]) g.hs[f] = make_float2(0.f, 0.f);
            }
            continue;
        }
        const MxRec rc = rec[c];
        MxRec rn;
        if (n >= 0) rn = rec[n];
        const MxFaceOut o = mx_face(m, s, ct, g, stage, t, rotors, sid, f, c, n, rc, rn);
        ws[f] = make_float2(o.water, o.speed);
        gf[f] = make_float4(o.gl1, o.gl2, o.gr1, o.gr2);
    }
}

// ---------------------------------------------------------------------------
// Gather: momentum rate, donor factor, CFL frequency (FP32 sums)
// ---------------------------------------------------------------------------
// Margin of the donor factor over the FP32 outflow sum: a sum of m products
// of rounded weights carries a relative error below (m + 2) eps32, and cells
// have at most MAX_CELL_FACES faces.
constexpr double DONOR_MARGIN = 64.0 * (double)FEPS;

// Face values of a cell's entries for the gather: the grid sweep reads the
// face sweep's arrays through the cell's face list.
struct GlobalFaces {
    const int *faces;
    const float2 *ws;
    const float4 *gf;
    __device__ __forceinline__ float2 ws_at(int k) const { return ws[faces[k]]; }
    __device__ __forceinline__ float4 gf_at(int k) const { return gf[faces[k]]; }
};

// Gather of one cell (the body of the gather sweep): its momentum rates and
// donor factor into rate32 / theta32 and its face-sum CFL frequency in fr;
// hf = the record's (depth, flags). Returns whether fr is valid.
template <class FaceAt>
__device__ __forceinline__ bool mx_gather_cell(const MeshDev &m, const StateDev &s, Ctrl &ct, const MixedGeo &g,
                                               int stage, int c, float2 hf, const FaceAt &fa, float *rate32,
                                               float *theta32, float &fr)
{
    const int nc = m.nc;
    const bool active = __float_as_int(hf.y) & 2;
    const bool owns_open = m.cflags[c] & 1;
    float out = 0.f, ext = 0.f, interior = 0.f, sum1 = 0.f, sum2 = 0.f, freq = 0.f;
    for (int k = m.offset[c]; k < m.offset[c + 1]; ++k) {
        const float wk = g.cw4[k];            // s * len / area
        const float2 wsf = fa.ws_at(k);
        const float4 gff = fa.gf_at(k);
        const float debit = fmaxf(wk * wsf.x, 0.f);   // outward water rate of this cell
        if (wk > 0.f) { sum1 += wk * gff.x; sum2 += wk * gff.y; }
        else { sum1 += wk * gff.z; sum2 += wk * gff.w; }
        out += debit;
        if (owns_open) { if (m.bslot[m.faces[k]] >= 0) ext += debit; else interior += debit; }
        freq += fabsf(wk) * wsf.y;
    }
    rate32[c] = active ? -sum1 : 0.f;
    rate32[nc + c] = active ? -sum2 : 0.f;
    float theta = 1.f;
    // donor factor: an FP32 test that is conservative, the value in FP64
    if (out > 0.f && ct.trialf * out >= 0.999f * hf.x) {
        const double hb = (stage == 1 ? s.work : s.q1)[c];
        const double cap = ct.trial * double(out) * (1. + DONOR_MARGIN);
        if (cap >= hb) theta = float(fmin(1., hb / cap) * (1. - 32. * EPS));
    }
    if (owns_open) {
        const double hb = (stage == 1 ? s.work : s.q1)[c];
        const double available = hb / ct.trial;
        const double e = double(ext), e_hi = e * (1. + DONOR_MARGIN);
        const double in_hi = double(interior) * (1. + DONOR_MARGIN);
        if (e > available) raise_status(ct, stage, ST_BUDGET);
        const double factor = fmin(1., (available - e_hi) / fmax(in_hi, 1e-300)) * (1. - 32. * EPS);
        theta = (interior > 0.f && in_hi >= available - e_hi) ? float(fmax(factor, 0.)) : 1.f;
    }
    theta32[c] = theta;
    fr = freq;
    if (isnan(fr)) { raise_status(ct, stage, ST_FREQ); return false; }
    return true;
}

__global__ void __launch_bounds__(256) km_gather(MeshDev m, StateDev s, Ctrl *ctrl, Work w, MixedGeo g, int stage)
{
    const int nc = m.nc;
    const MxRec *rec = reinterpret_cast<const MxRec *>(w.rec);
    float *rate32 = reinterpret_cast<float *>(w.rate);      // (2, nc) momentum rates
    float *theta32 = reinterpret_cast<float *>(w.theta);
    const GlobalFaces fa{m.faces, reinterpret_cast<const float2 *>(w.ws), reinterpret_cast<const float4 *>(w.gf)};
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
            if (!mx_skip(ct, stage))
                have = mx_gather_cell(m, s, ct, g, stage, c, *reinterpret_cast<const float2 *>(&rec[c]), fa, rate32,
                                      theta32, fr);
        }
        unsigned long long *peak0 = stage == 1 ? &ctrl[0].peak1 : &ctrl[0].peak2;
        warp_max_peak_f(peak0, sizeof(Ctrl), sid, have, fr);
    }
}

// ---------------------------------------------------------------------------
// Tile sweep: cells, faces and gather of one stage over cell tiles staged in
// shared memory
// ---------------------------------------------------------------------------
// Neighbour access of a tile's cells: the entry's local slot and flags from
// the tile tables, the neighbour's primitives from shared memory.
struct TileNbr {
    const int2 *ent;         // the cell's entries, in entry order
    const MxPrim *sP;
    __device__ __forceinline__ int2 id(int, int j) const { return ent[j]; }
    __device__ __forceinline__ MxPrim prim(int l) const { return sP[l]; }
};

// Face values of a tile cell's entries: the tile's face buffers in shared memory.
struct TileFaces {
    const int *tfslot;
    const float2 *sW;
    const float4 *sG;
    __device__ __forceinline__ float2 ws_at(int k) const { return sW[tfslot[k]]; }
    __device__ __forceinline__ float4 gf_at(int k) const { return sG[tfslot[k]]; }
};

// One block per tile (grid-stride over the tiles). The tile's primitives,
// with two rings of neighbours, go to shared memory; the block forms the
// records of its cells and of the first ring (whose records its edge faces
// read), then every face of its cells, then its cells' gathers, all from
// shared memory. The arithmetic of each record, face and gather is the
// separate sweeps' own (mx_record, mx_face, mx_gather_cell), so the results
// are theirs; a face on a tile edge is formed by both tiles alike. Only what
// the update reads leaves the block: the water flux and CFL speed per face,
// the momentum rates and donor factor per cell, the rotor face terms.
template <int MAXF>
__global__ void __launch_bounds__(TILE_THREADS, 4) km_tile(MeshDev m, StateDev s, BoundaryDev b, Ctrl *ctrl, Work w,
                                                           MixedGeo g, int stage, TurbDev t, int turb, TileDev td)
{
    extern __shared__ __align__(16) unsigned char smem[];
    MxPrim *sP = reinterpret_cast<MxPrim *>(smem);
    MxRec *sR = reinterpret_cast<MxRec *>(sP + td.cap_prims);
    float2 *sW = reinterpret_cast<float2 *>(sR + td.cap_recs);
    float4 *sG = reinterpret_cast<float4 *>(sW + td.cap_faces);
    const MxPrim *P = reinterpret_cast<const MxPrim *>((stage == 1 ? g.prim[0] : g.prim[1]));
    float2 *ws = reinterpret_cast<float2 *>(w.ws);
    float *rate32 = reinterpret_cast<float *>(w.rate);
    float *theta32 = reinterpret_cast<float *>(w.theta);
    unsigned long long *peak0 = stage == 1 ? &ctrl[0].peak1 : &ctrl[0].peak2;
    const TileFaces fa{td.tfslot, sW, sG};
    for (int tile = blockIdx.x; tile < td.ntiles; tile += gridDim.x) {
        const int4 I = td.info[tile], I2 = td.info2[tile];
        const int c0 = I.x, nt = I.y - I.x, n1 = I2.x, n2 = I2.y, nface = I2.z;
        const int sid = m.cell_sid[c0];
        Ctrl &ct = ctrl[sid];
        if (mx_skip(ct, stage)) continue;                 // uniform over the block
        const bool rotors = turb && t.hkt[sid];
        // primitives of the tile and its two rings
        for (int i = threadIdx.x; i < nt + n1 + n2; i += blockDim.x)
            sP[i] = P[i < nt ? c0 + i : td.halo[I.z + i - nt]];
        __syncthreads();
        // records of the tile's cells and of ring 1
        for (int i = threadIdx.x; i < nt + n1; i += blockDim.x) {
            const int c = i < nt ? c0 + i : td.halo[I.z + i - nt];
            const int k0 = m.offset[c], deg = m.offset[c + 1] - k0;
            const TileNbr nb{i < nt ? td.tent + k0 : td.hent + 4 * (I2.w + i - nt), sP};
            sR[i] = mx_record<MAXF>(m, s, ct, g, sP[i], c, k0, deg, nb);
            if (rotors) hkt_cell_gradients(m, g, nb, sP[i], c, m.nc);
        }
        __syncthreads();
        // every face of the tile's cells
        for (int j = threadIdx.x; j < nface; j += blockDim.x) {
            const int4 F = td.tface[I.w + j];
            const int f = F.x, c = m.owner[f], n = m.neighbour[f];
            const int slot = m.bslot[f];
            float2 wsf;
            float4 gff;
            if (slot >= 0) {
                mx_open_face(m, s, b, ct, stage, f, c, slot, wsf, gff);
                if (rotors) {
                    g.hp[f] = make_float2(0.f, 0.f);
                    if (t.stress[sid]) g.hs[f] = make_float2(0.f, 0.f);
                }
            } else {
                const MxRec rc = sR[F.y];
                MxRec rn;
                if (F.z >= 0) rn = sR[F.z];
                const MxFaceOut o = mx_face(m, s, ct, g, stage, t, rotors, sid, f, c, n, rc, rn);
                wsf = make_float2(o.water, o.speed);
                gff = make_float4(o.gl1, o.gl2, o.gr1, o.gr2);
            }
            sW[j] = wsf;
            sG[j] = gff;
            ws[f] = wsf;
        }
        __syncthreads();
        // gathers of the tile's cells (warp-uniform trip count for the CFL peak)
        for (int first = 0; first < nt; first += blockDim.x) {
            const int i = first + (int)threadIdx.x;
            bool have = false;
            float fr = 0.f;
            if (i < nt)
                have = mx_gather_cell(m, s, ct, g, stage, c0 + i, make_float2(sR[i].h, __int_as_float(sR[i].flags)),
                                      fa, rate32, theta32, fr);
            warp_max_peak_f(peak0, sizeof(Ctrl), sid, have, fr);
        }
        __syncthreads();                                  // the next tile refills the buffers
    }
}

// Donor-limited water flux (FP64) and the momentum it carries. After the
// first gather, block 0 also evaluates each scenario's first-stage CFL test.
__global__ void __launch_bounds__(256) km_limit(MeshDev m, Ctrl *ctrl, Work w, MixedGeo g, int stage)
{
    const int nf = m.nf;
    if (stage == 1 && blockIdx.x == 0)
        for (int i = threadIdx.x; i < m.nscen; i += blockDim.x) {
            Ctrl &c = ctrl[i];
            c.cfl1 = c.trial * bits_to_double(c.peak1) > c.cfl * (1 + 1e-12);
        }
    const float2 *ws = reinterpret_cast<const float2 *>(w.ws);
    const float *theta32 = reinterpret_cast<const float *>(w.theta);
    const MxPrim *P = reinterpret_cast<const MxPrim *>((stage == 1 ? g.prim[0] : g.prim[1]));
    MxLim *lim = reinterpret_cast<MxLim *>(w.lim);
    FOR_ACTIVE_FACES(m.act, f) {
        const Ctrl &ct = ctrl[m.face_sid[f]];
        if (mx_skip(ct, stage)) continue;
        const float wf = ws[f].x;
        double water = double(wf);
        float cx = 0.f, cy = 0.f;
        if (wf != 0.f && m.bslot[f] < 0) {
            const int donor = wf < 0.f ? m.neighbour[f] : m.owner[f];
            if (donor >= 0) {
                const float th = theta32[donor];
                if (th != 1.f) {
                    const float delta = (th - 1.f) * wf;
                    water = double(wf) * double(th);          // exact product
                    const MxPrim pd = P[donor];
                    if (pd.wet) { cx = delta * pd.u; cy = delta * pd.v; }
                }
            }
        }
        MxLim l;
        l.water = water; l.cx = cx; l.cy = cy;
        lim[f] = l;
    }
}

__device__ __forceinline__ void drag_f(const Ctrl &ct, float dtf, double &h, double &hu, double &hv)
{
    if (le_threshold(h, ct.dry)) { hu = 0.; hv = 0.; return; }
    const float hf = d2f(h), uf = d2f(hu), vf = d2f(hv);
    float c;
    const float val = ct.roughf;
    if (ct.roughness_mode == 1) c = val;
    else if (ct.roughness_mode == 2) c = powf(hf, 1.f / 6.f) / val;
    else if (ct.roughness_mode == 3) c = sqrtf(9.81f) / .41f * log1pf(30.f * hf / (2.718281828459045f * val));
    else c = 18.f * log10f(12.f * fmaxf(.5f, hf / val));
    const float speed = sqrtf(uf * uf + vf * vf) / hf;
    const float factor = 1.f / (1.f + dtf * ct.gravf * speed / (c * c * hf));
    const double fd = f2d(factor);
    hu *= fd;
    hv *= fd;
}

// Update (owner computes): each cell forms the donor-limited water flux of
// its faces itself (river_midpoint.h:30-41) from the face sweep's FP32 water
// and the donor's factor, exactly as the face pass km_limit does: both cells
// of a face compute the same FP64 value double(w) * double(theta), so mass
// still telescopes, and no limited-flux buffer goes through memory. After
// the first gather, block 0 also evaluates each scenario's first-stage CFL
// test (the second stage's kernels read it).
__global__ void __launch_bounds__(256) km_update(MeshDev m, StateDev s, Ctrl *ctrl, Work w, MixedGeo g, int stage,
                                                 double *rate_out, TurbDev t, int turb)
{
    const int nc = m.nc;
    if (stage == 1 && blockIdx.x == 0)
        for (int i = threadIdx.x; i < m.nscen; i += blockDim.x) {
            Ctrl &c = ctrl[i];
            c.cfl1 = c.trial * bits_to_double(c.peak1) > c.cfl * (1 + 1e-12);
        }
    const float2 *ws = reinterpret_cast<const float2 *>(w.ws);
    const float *theta32 = reinterpret_cast<const float *>(w.theta);
    const float *rate32 = reinterpret_cast<const float *>(w.rate);
    const MxPrim *P = reinterpret_cast<const MxPrim *>((stage == 1 ? g.prim[0] : g.prim[1]));
    MxPrim *P2 = reinterpret_cast<MxPrim *>(g.prim[1]);
    FOR_ACTIVE_CELLS(m.act, c) {
        const int sid = m.cell_sid[c];
        Ctrl &ct = ctrl[sid];
        if (mx_skip(ct, stage)) continue;
        double mass = 0.;
        float mx = 0.f, my = 0.f;
        for (int k = m.offset[c]; k < m.offset[c + 1]; ++k) {
            const float wf = ws[m.faces[k]].x;
            const float wk = g.cw4[k];
            double water = f2d(wf);
            if (wf != 0.f) {
                const int2 id = g.cidx[k];
                // the donor is the owner for outward (positive) water, else the neighbour
                const int donor = (wf > 0.f) == ((id.y & 16) != 0) ? c : id.x;
                if (!(id.y & 8) && donor >= 0) {
                    const float th = theta32[donor];
                    if (th != 1.f) {
                        const float delta = (th - 1.f) * wf;
                        water = f2d(wf) * f2d(th);                // exact product
                        const MxPrim pd = P[donor];
                        if (pd.wet) { mx -= wk * (delta * pd.u); my -= wk * (delta * pd.v); }
                    }
                }
            }
            mass -= g.cw8[k] * water;
        }
        float f1 = rate32[c] + mx, f2 = rate32[nc + c] + my;
        double r1, r2;
        if (turb && t.hkt[sid]) {
            // ambient stress and balanced pressure (FP32 face sums, added in
            // FP32), then the FP64 actuator sink of a support cell: one
            // conversion per component
            const int k0 = m.offset[c], k1 = m.offset[c + 1];
            if (t.stress[sid]) {
                float x = 0.f, y = 0.f;
                for (int k = k0; k < k1; ++k) { const float2 v = g.hs[m.faces[k]]; x += g.cw4[k] * v.x; y += g.cw4[k] * v.y; }
                f1 += x; f2 += y;
            }
            float x = 0.f, y = 0.f;
            for (int k = k0; k < k1; ++k) { const float2 v = g.hp[m.faces[k]]; x += g.cw4[k] * v.x; y += g.cw4[k] * v.y; }
            r1 = f2d(f1 + x);
            r2 = f2d(f2 + y);
            if (t.foot[c]) { r1 += t.raw[c]; r2 += t.raw[nc + c]; }
        } else {
            r1 = f2d(f1);
            r2 = f2d(f2);
        }
        if (w.visc.nu && w.visc.nu[sid] > 0.) {
            // the wet-bank viscosity's FP64 face stresses, FP64 signed weights
            double x = 0., y = 0.;
            for (int k = m.offset[c]; k < m.offset[c + 1]; ++k) {
                const int f = m.faces[k];
                x += g.cw8[k] * w.visc.face[f];
                y += g.cw8[k] * w.visc.face[m.nf + f];
            }
            r1 += x; r2 += y;
        }
        if (!finite64(mass) || !finite64(r1) || !finite64(r2)) raise_status(ct, stage, ST_RATE);
        if (rate_out) { rate_out[c] = mass; rate_out[nc + c] = r1; rate_out[2 * nc + c] = r2; continue; }
        const double dt = ct.trial, dry = ct.dry;
        if (stage == 1) {
            const double h = s.work[c] + dt * mass;
            double hu = s.work[nc + c] + dt * r1, hv = s.work[2 * nc + c] + dt * r2;
            if (lt_zero(h)) raise_status(ct, 1, ST_ENDPOINT);
            if (le_threshold(h, dry)) { hu = 0.; hv = 0.; }
            s.q1[c] = h; s.q1[nc + c] = hu; s.q1[2 * nc + c] = hv;
            // the second stage's input; an invalid one fails that stage
            if (!put_prim(P2, c, h, hu, hv, s.z[c], dry) && !lt_zero(h)) raise_status(ct, 2, ST_SPATIAL);
        } else {
            double h = .5 * s.work[c] + .5 * (s.q1[c] + dt * mass);
            double hu = .5 * s.work[nc + c] + .5 * (s.q1[nc + c] + dt * r1);
            double hv = .5 * s.work[2 * nc + c] + .5 * (s.q1[2 * nc + c] + dt * r2);
            if (!finite64(h) || !finite64(hu) || !finite64(hv) || lt_zero(h)) raise_status(ct, 2, ST_ENDPOINT);
            if (le_threshold(h, dry)) { hu = 0.; hv = 0.; }
            drag_f(ct, .5f * ct.trialf, h, hu, hv);
            double *qn = ct.cur ? s.q[0] : s.q[1];
            qn[c] = h; qn[nc + c] = hu; qn[2 * nc + c] = hv;
        }
    }
}

// First drag half-step: work = drag(accepted, trial/2), and the first stage's
// primitives. The drag factor scales the FP64 momenta; the FP32 velocities
// of the primitives are the FP32 momenta times the same factor over the
// depth, so the scaled FP64 momenta are not converted back (two fewer FP64-
// pipe conversions per cell in this FP64-pipe-bound sweep).
__global__ void __launch_bounds__(256) km_open_drag(MeshDev m, StateDev s, Ctrl *ctrl, MixedGeo g)
{
    const int nc = m.nc;
    MxPrim *P1 = reinterpret_cast<MxPrim *>(g.prim[0]);
    FOR_ACTIVE_CELLS(m.act, c) {
        Ctrl &ct = ctrl[m.cell_sid[c]];
        if (!ct.active || ct.done) continue;
        const double *q = ct.cur ? s.q[1] : s.q[0];
        const double h = q[c], z = s.z[c];
        double hu = q[nc + c], hv = q[2 * nc + c];
        const bool wet = !le_threshold(h, ct.dry);
        const float hf = d2f(h);
        float uf = 0.f, vf = 0.f;
        if (!wet) { hu = 0.; hv = 0.; }
        else {
            const float mu = d2f(hu), mv = d2f(hv);
            float cz;
            const float val = ct.roughf;
            if (ct.roughness_mode == 1) cz = val;
            else if (ct.roughness_mode == 2) cz = powf(hf, 1.f / 6.f) / val;
            else if (ct.roughness_mode == 3) cz = sqrtf(9.81f) / .41f * log1pf(30.f * hf / (2.718281828459045f * val));
            else cz = 18.f * log10f(12.f * fmaxf(.5f, hf / val));
            const float speed = sqrtf(mu * mu + mv * mv) / hf;
            const float factor = 1.f / (1.f + .5f * ct.trialf * ct.gravf * speed / (cz * cz * hf));
            const double fd = f2d(factor);
            hu *= fd; hv *= fd;
            uf = mu * factor / hf; vf = mv * factor / hf;
        }
        s.work[c] = h; s.work[nc + c] = hu; s.work[2 * nc + c] = hv;
        const double eta = h + z;
        MxPrim p;
        p.ehi = d2f(eta);
        p.elo = d2f(eta - f2d(p.ehi));
        p.h = hf; p.u = uf; p.v = vf; p.wet = wet;
        p.pad0 = 0.f; p.pad1 = 0.f;
        P1[c] = p;
        if (!(!lt_zero(h) && finite64(h) && finite64(hu) && finite64(hv) && finite64(z))) raise_status(ct, 1, ST_SPATIAL);
    }
}

// First stage's primitives of a state placed in work directly (single residual).
__global__ void __launch_bounds__(256) km_prim(MeshDev m, StateDev s, Ctrl *ctrl, MixedGeo g)
{
    const int nc = m.nc;
    MxPrim *P1 = reinterpret_cast<MxPrim *>(g.prim[0]);
    FOR_ACTIVE_CELLS(m.act, c) {
        Ctrl &ct = ctrl[m.cell_sid[c]];
        if (!ct.active || ct.done) continue;
        if (!put_prim(P1, c, s.work[c], s.work[nc + c], s.work[2 * nc + c], s.z[c], ct.dry))
            raise_status(ct, 1, ST_SPATIAL);
    }
}

// Limited water flux of the last stage into a caller buffer.
__global__ void km_water_out(MeshDev m, Work w, double *water)
{
    const MxLim *lim = reinterpret_cast<const MxLim *>(w.lim);
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < m.nf; f += gridDim.x * blockDim.x) water[f] = lim[f].water;
}

#include "brx_hllc_mixed.cuh"

}  // namespace brx_mx

// The boundary CTA of the mixed form is the FP64 kernel (few faces, FP64 sums).
#define BRX_NS brx_mixb
#include "brx_kernels.cuh"

namespace brx {

int mixed_max_block(int kind, int maxdeg)
{
    const bool small = maxdeg <= 4;
    const void *fn = nullptr;
    switch (kind) {
    case K_DRAG: fn = (const void *)brx_mx::km_open_drag; break;
    case K_CELLS: fn = small ? (const void *)brx_mx::km_cells<4> : (const void *)brx_mx::km_cells<MAX_CELL_FACES>; break;
    case K_FACES: fn = (const void *)brx_mx::km_faces; break;
    case K_GATHER: fn = (const void *)brx_mx::km_gather; break;
    case K_LIMIT: fn = (const void *)brx_mx::km_limit; break;
    case K_UPDATE: fn = (const void *)brx_mx::km_update; break;
    case KH_CELLS: fn = (const void *)brx_mx::km_hllc_cells; break;
    case KH_PREDICT: fn = (const void *)brx_mx::km_hllc_predict; break;
    case KH_FACES: fn = (const void *)brx_mx::km_hllc_faces; break;
    case KH_BUDGET: fn = (const void *)brx_mx::km_hllc_budget; break;
    case KH_UPDATE: fn = (const void *)brx_mx::km_hllc_update; break;
    case K_TILE: return small ? TILE_THREADS : 0;          // the block is fixed; the grid cap is tunable
    default: return 0;
    }
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, fn) != cudaSuccess) return 0;
    return a.maxThreadsPerBlock;
}

int mixed_hllc_kernel(const Launch &L, int kind)
{
    cudaStream_t st = L.stream;
    const int nc = L.mesh.nc, nf = L.mesh.nf;
    brx_mx::HCellF *rec = reinterpret_cast<brx_mx::HCellF *>(L.work.rec);
#define SHAPE(kind_, n_) shape_grid(L, kind_, n_), L.shape[kind_].block
    switch (kind) {
    case KH_CELLS:
        brx_mx::km_hllc_cells<<<SHAPE(KH_CELLS, nc), 0, st>>>(L.mesh, L.state, L.ctrl, L.mx, rec);
        return 1;
    case KH_PREDICT:
        if (!L.has_turb) return 0;
        brx_mx::km_hllc_predict<<<SHAPE(KH_PREDICT, nc), 0, st>>>(L.mesh, L.state, L.turb, L.ctrl, rec);
        return 1;
    case KH_FACES:
        brx_mx::km_hllc_faces<<<SHAPE(KH_FACES, nf), 0, st>>>(L.mesh, L.state, L.bnd, L.ctrl, L.work, L.mx, L.turb,
                                                              L.has_turb, rec);
        return 1;
    case KH_BUDGET:
        brx_mx::km_hllc_budget<<<SHAPE(KH_BUDGET, nc), 0, st>>>(L.mesh, L.state, L.ctrl, L.work, L.mx);
        return 1;
    case KH_UPDATE:
        brx_mx::km_hllc_update<<<SHAPE(KH_UPDATE, nc), 0, st>>>(L.mesh, L.state, L.ctrl, L.work, L.mx, L.turb,
                                                                L.has_turb);
        return 1;
    }
#undef SHAPE
    return 0;
}

int mixed_kernel(const Launch &L, int kind, int stage, double *out)
{
    cudaStream_t st = L.stream;
    const bool small = L.maxdeg <= 4;
    const int nc = L.mesh.nc, nf = L.mesh.nf;
#define SHAPE(kind_, n_) shape_grid(L, kind_, n_), L.shape[kind_].block
    switch (kind) {
    case K_DRAG:
        brx_mx::km_open_drag<<<SHAPE(K_DRAG, nc), 0, st>>>(L.mesh, L.state, L.ctrl, L.mx);
        return 1;
    case K_BOUNDARY:
        if (!L.nslot) return 0;
        brx_mixb::k_boundary<float><<<L.nscen, 256, 0, st>>>(L.mesh, L.state, L.bnd, L.ctrl, stage);
        return 1;
    case K_CELLS:
        if (small)
            brx_mx::km_cells<4><<<SHAPE(K_CELLS, nc), 0, st>>>(L.mesh, L.state, L.ctrl, L.work, L.mx, stage, L.turb,
                                                              L.has_turb);
        else
            brx_mx::km_cells<MAX_CELL_FACES><<<SHAPE(K_CELLS, nc), 0, st>>>(L.mesh, L.state, L.ctrl, L.work, L.mx,
                                                                            stage, L.turb, L.has_turb);
        return 1;
    case K_FACES:
        brx_mx::km_faces<<<SHAPE(K_FACES, nf), 0, st>>>(L.mesh, L.state, L.bnd, L.ctrl, L.work, L.mx, stage, L.turb,
                                                    L.has_turb);
        return 1;
    case K_GATHER:
        brx_mx::km_gather<<<SHAPE(K_GATHER, nc), 0, st>>>(L.mesh, L.state, L.ctrl, L.work, L.mx, stage);
        return 1;
    case K_TILE: {
        const int grid = std::max(1, std::min(L.tiles.ntiles, L.shape[K_TILE].per_sm * L.sms));
        brx_mx::km_tile<4><<<grid, TILE_THREADS, L.tile_smem, st>>>(L.mesh, L.state, L.bnd, L.ctrl, L.work, L.mx,
                                                                   stage, L.turb, L.has_turb, L.tiles);
        return 1;
    }
    case K_LIMIT:
        brx_mx::km_limit<<<SHAPE(K_LIMIT, nf), 0, st>>>(L.mesh, L.ctrl, L.work, L.mx, stage);
        return 1;
    case K_UPDATE:
        brx_mx::km_update<<<SHAPE(K_UPDATE, nc), 0, st>>>(L.mesh, L.state, L.ctrl, L.work, L.mx, stage, out, L.turb,
                                                     L.has_turb);
        return 1;
    case K_PRIM:
        brx_mx::km_prim<<<L.grid_c256, 256, 0, st>>>(L.mesh, L.state, L.ctrl, L.mx);
        return 1;
    case K_BED: {
        const int grid = L.grid_c > L.grid_f ? L.grid_c : L.grid_f;
        if (small) brx_mx::km_bed<4><<<grid, 128, 0, st>>>(L.mesh, L.state, L.mx);
        else brx_mx::km_bed<MAX_CELL_FACES><<<grid, 128, 0, st>>>(L.mesh, L.state, L.mx);
        return 1;
    }
    case K_WATER:
        brx_mx::km_water_out<<<L.grid_f256, 256, 0, st>>>(L.mesh, L.work, out);
        return 1;
    case K_HKT_GRAD:        // fused into the cell sweep's tail
        return 0;
    case K_HKT_FACES:       // fused into the face sweep's tail
        return 0;
    }
#undef SHAPE
    return 0;
}

int mixed_tile_smem(int cap_prims, int cap_recs, int cap_faces)
{
    return (int)(sizeof(brx_mx::MxPrim) * cap_prims + sizeof(brx_mx::MxRec) * cap_recs +
                 (sizeof(float2) + sizeof(float4)) * cap_faces);
}

int mixed_tile_prepare(int smem_bytes)
{
    return (int)cudaFuncSetAttribute(brx_mx::km_tile<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
}

}  // namespace brx
