// Face-local shallow-water Riemann arithmetic for the river step, templated on
// the flux precision F (double for the FP64 form, float for the mixed form).
//
// Algorithms (restated from the published method and from the reference's
// FP64 port, whose operation order the FP64 instantiation keeps so that it
// reproduces the reference bit for bit when compiled with -fmad=false):
//   * GeoClaw Riemann type estimate and augmented f-wave solver of
//     George (2008, J. Comput. Phys. 227:3089), one iteration, no rarefaction
//     corrector: src/braids_support/gpu_fwave/augmented_fwave.cu:28-262.
//   * rpn2 wrapper with dry-state wall reflection and wave/fluctuation split:
//     augmented_fwave.cu:264-334.
//   * exact shallow-water reflecting-wall pressure (bracketed Newton on the
//     shock Hugoniot): src/braids_core/sediment/reflecting_wall.py:10-31.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace brx {

// Division of the Riemann arithmetic. The FP64 form keeps the reference's
// correctly rounded division (its operation order decides bits); the FP32
// form uses the fast reciprocal-multiply (2 ulp; every divisor here is a
// depth, a speed sum or a wave-speed difference well inside its range).
template <class F> __device__ __forceinline__ F quo(F a, F b) { return a / b; }
template <> __device__ __forceinline__ float quo<float>(float a, float b) { return __fdividef(a, b); }

template <class F> struct RType { F hm, s1m, s2m; };

template <class F>
__device__ __forceinline__ RType<F> riemann_type(F hL, F hR, F uL, F uR, F drytol, F g)
{
    const F two = F(2), three = F(3), half = F(0.5);
    RType<F> o;
    const F hmin = fmin(hR, hL), hmax = fmax(hR, hL), delu = uR - uL;
    if (hmin <= drytol) {
        o.hm = F(0);
        o.s1m = uR + uL - two * sqrt(g * hR) + two * sqrt(g * hL);
        o.s2m = o.s1m;
        return o;
    }
    const F fmn = delu + two * (sqrt(g * hmin) - sqrt(g * hmax));
    const F fmx = delu + (hmax - hmin) * sqrt(quo<F>(half * g * (hmax + hmin), hmax * hmin));
    if (fmn > F(0)) {
        const F root = fmax(F(0), -delu + two * (sqrt(g * hL) + sqrt(g * hR)));
        o.hm = quo<F>(F(1), F(16) * g) * (root * root);
        o.s1m = uL + two * sqrt(g * hL) - three * sqrt(g * o.hm);
        o.s2m = uR - two * sqrt(g * hR) + three * sqrt(g * o.hm);
    } else if (fmx <= F(0)) {
        F h0 = hmax;
        const F gL = sqrt(half * g * (quo<F>(F(1), h0) + quo<F>(F(1), hL)));
        const F gR = sqrt(half * g * (quo<F>(F(1), h0) + quo<F>(F(1), hR)));
        const F F0 = delu + (h0 - hL) * gL + (h0 - hR) * gR;
        const F dfdh = gL - quo<F>(g * (h0 - hL), F(4) * (h0 * h0) * gL) +
                       gR - quo<F>(g * (h0 - hR), F(4) * (h0 * h0) * gR);
        const F slope = two * sqrt(h0) * dfdh;
        const F root = sqrt(h0) - quo<F>(F0, slope);
        h0 = root * root;
        o.hm = h0;
        const F u1m = uL - (o.hm - hL) * sqrt((half * g) * (quo<F>(F(1), o.hm) + quo<F>(F(1), hL)));
        const F u2m = uR + (o.hm - hR) * sqrt((half * g) * (quo<F>(F(1), o.hm) + quo<F>(F(1), hR)));
        o.s1m = u1m - sqrt(g * o.hm);
        o.s2m = u2m + sqrt(g * o.hm);
    } else {
        F h0 = hmin;
        const F F0 = delu + two * (sqrt(g * h0) - sqrt(g * hmax)) +
                     (h0 - hmin) * sqrt(half * g * (quo<F>(F(1), h0) + quo<F>(F(1), hmin)));
        const F slope = quo<F>(fmx - F0, hmax - hmin);
        h0 = h0 - quo<F>(F0, slope);
        o.hm = h0;
        if (hL > hR) {
            o.s1m = uL + two * sqrt(g * hL) - three * sqrt(g * o.hm);
            o.s2m = uL + two * sqrt(g * hL) - sqrt(g * o.hm);
        } else {
            o.s2m = uR - two * sqrt(g * hR) + three * sqrt(g * o.hm);
            o.s1m = uR - two * sqrt(g * hR) + sqrt(g * o.hm);
        }
    }
    return o;
}

// 3x3 determinant with the cofactor expansion along the first row.
template <class F>
__device__ __forceinline__ F det3(F a00, F a01, F a02, F a10, F a11, F a12, F a20, F a21, F a22)
{
    const F d1 = a00 * (a11 * a22 - a12 * a21);
    const F d2 = a01 * (a10 * a22 - a12 * a20);
    const F d3 = a02 * (a10 * a21 - a11 * a20);
    return d1 - d2 + d3;
}

// Fluctuations and speeds of one face in the local frame.
// in: hL, huL (normal), hvL (tangent), bL, hR, huR, hvR, bR.
// Returns the status word: 0 ok, bit 0 negative depth clamped, bit 1
// nonfinite result, -1 nonfinite input.
template <class F>
struct FWaveOut { F amdq[3], apdq[3], s[3]; };

template <class F>
__device__ __forceinline__ int fwave(const F in[8], F grav, F drytol, FWaveOut<F> &out)
{
    const F zero = F(0), half = F(0.5), two = F(2);
#pragma unroll
    for (int c = 0; c < 3; ++c) { out.amdq[c] = zero; out.apdq[c] = zero; out.s[c] = zero; }
    int status = 0;
    bool finite = true;
#pragma unroll
    for (int r = 0; r < 8; ++r) finite = finite && isfinite(in[r]);
    if (!finite) return -1;
    F hL = in[0], huL = in[1], hvL = in[2], bL = in[3];
    F hR = in[4], huR = in[5], hvR = in[6], bR = in[7];
    if (hL < zero) { hL = zero; huL = zero; hvL = zero; status |= 1; }
    if (hR < zero) { hR = zero; huR = zero; hvR = zero; status |= 1; }
    if (hL <= drytol && hR <= drytol) return status;
    F uL, uR, vL, vR, phiL, phiR;
    if (hR > drytol) {
        uR = quo<F>(huR, hR); vR = quo<F>(hvR, hR);
        phiR = half * grav * (hR * hR) + quo<F>(huR * huR, hR);
    } else { hR = zero; huR = zero; hvR = zero; uR = zero; vR = zero; phiR = zero; }
    if (hL > drytol) {
        uL = quo<F>(huL, hL); vL = quo<F>(hvL, hL);
        phiL = half * grav * (hL * hL) + quo<F>(huL * huL, hL);
    } else { hL = zero; huL = zero; hvL = zero; uL = zero; vL = zero; phiL = zero; }
    F w0 = F(1), w1 = F(1), w2 = F(1);
    if (hR <= drytol) {
        const RType<F> t = riemann_type<F>(hL, hL, uL, -uL, drytol, grav);
        const F hstar = fmax(hL, t.hm);
        if (hstar + bL < bR) {
            w1 = zero; w2 = zero;
            hR = hL; huR = -huL; bR = bL; phiR = phiL; uR = -uL; vR = vL;
        } else if (hL + bL < bR) bR = hL + bL;
    } else if (hL <= drytol) {
        const RType<F> t = riemann_type<F>(hR, hR, -uR, uR, drytol, grav);
        const F hstar = fmax(hR, t.hm);
        if (hstar + bR < bL) {
            w0 = zero; w1 = zero;
            hL = hR; huL = -huR; bL = bR; phiL = phiR; uL = -uR; vL = vR;
        } else if (hR + bR < bL) bL = hR + bR;
    }
    const F sqL = sqrt(grav * hL), sqR = sqrt(grav * hR);
    const F sL = uL - sqL, sR = uR + sqR;
    const F uhat = quo<F>(sqL * uL + sqR * uR, sqR + sqL);
    const F chat = sqrt(grav * half * (hR + hL));
    F sE1 = fmin(sL, uhat - chat), sE2 = fmax(sR, uhat + chat);

    const F g = grav;
    const F delh = hR - hL, delhu = huR - huL, delphi = phiR - phiL, delb = bR - bL;
    const RType<F> t = riemann_type<F>(hL, hR, uL, uR, drytol, g);
    const F s1m = t.s1m, s2m = t.s2m;
    const F lam0 = fmin(sE1, s2m);
    const F lam2 = fmax(sE2, s1m);
    sE1 = lam0;
    sE2 = lam2;
    const F hstarHLL = fmax(quo<F>(huL - huR + sE2 * hR - sE1 * hL, sE2 - sE1), zero);
    // eigenvectors: r(:,0) = (1, lam0, lam0^2), r(:,1) = (0, 0, 1), r(:,2) = (1, lam2, lam2^2)
    const F r10 = lam0, r20 = lam0 * lam0, r12 = lam2, r22 = lam2 * lam2;
    const F lam1 = half * (lam0 + lam2);

    const F crit = fmax(drytol * g, F(1.0e-6));
    const F crit2 = sqrt(crit);
    const F hbar = fmax(half * (hL + hR), zero);
    const F usum = uL + uR;
    const F s1s2bar = F(0.25) * (usum * usum) - g * hbar;
    const F s1s2tilde = fmax(zero, uL * uR) - g * hbar;
    bool sonic;
    if (fabs(s1s2bar) <= crit) sonic = true;
    else if (s1s2bar * s1s2tilde <= crit * crit) sonic = true;
    else if (s1s2bar * sE1 * sE2 <= crit * crit) sonic = true;
    else if (fmin(fabs(sE1), fabs(sE2)) < crit2) sonic = true;
    else if (sE1 < crit2 && s1m > -crit2) sonic = true;
    else if (sE2 > -crit2 && s2m < crit2) sonic = true;
    else if ((uL + sqL) * (uR + sqR) < zero) sonic = true;
    else if ((uL - sqL) * (uR - sqR) < zero) sonic = true;
    else sonic = false;

    F deldelh = sonic ? -delb : quo<F>(delb * g * hbar, s1s2bar);
    if (sE1 < -crit && sE2 > crit) {
        deldelh = fmin(deldelh, quo<F>(hstarHLL * (sE2 - sE1), sE2));
        deldelh = fmax(deldelh, quo<F>(hstarHLL * (sE2 - sE1), sE1));
    } else if (sE1 >= crit) {
        deldelh = fmin(deldelh, quo<F>(hstarHLL * (sE2 - sE1), sE1));
        deldelh = fmax(deldelh, -hL);
    } else if (sE2 <= -crit) {
        deldelh = fmin(deldelh, hR);
        deldelh = fmax(deldelh, quo<F>(hstarHLL * (sE2 - sE1), sE2));
    }
    F deldelphi = sonic ? -g * hbar * delb : quo<F>(-delb * g * hbar * s1s2tilde, s1s2bar);
    deldelphi = fmin(deldelphi, g * fmax(-hL * delb, -hR * delb));
    deldelphi = fmax(deldelphi, g * fmin(-hL * delb, -hR * delb));
    const F d0 = delh - deldelh, d1 = delhu, d2 = delphi - deldelphi;
    // Cramer's rule on [r0 r1 r2] beta = delta. The FP64 form evaluates the
    // cofactor expansions with their unit and zero entries as the reference
    // does; the FP32 form folds them (det = lam0 - lam2).
    const F one = F(1);
    F beta0, beta1, beta2;
    if constexpr (sizeof(F) == 4) {
        const F rdet = quo<F>(one, r10 - r12);
        beta0 = (d1 - d0 * r12) * rdet;
        beta1 = ((d1 * r22 - r12 * d2) - d0 * (r10 * r22 - r12 * r20) + (r10 * d2 - d1 * r20)) * rdet;
        beta2 = (d0 * r10 - d1) * rdet;
    } else {
        const F det = det3<F>(one, zero, one, r10, zero, r12, r20, one, r22);
        beta0 = det3<F>(d0, zero, one, d1, zero, r12, d2, one, r22) / det;
        beta1 = det3<F>(one, d0, one, r10, d1, r12, r20, d2, r22) / det;
        beta2 = det3<F>(one, zero, d0, r10, zero, d1, r20, one, d2) / det;
    }
    F fw00 = beta0 * r10, fw01 = beta0 * r20, fw02 = beta0 * r10;
    F fw10 = beta1 * zero, fw11 = beta1 * one;
    F fw20 = beta2 * r12, fw21 = beta2 * r22, fw22 = beta2 * r12;
    fw02 = fw02 * vL;
    fw22 = fw22 * vR;
    F fw12 = zero;
    const F hustar = huL + fw00;
    if (hustar <= zero)
        fw02 = fw02 + (hR * uR * vR - hL * uL * vL - fw02 - fw22);
    else
        fw22 = fw22 + (hR * uR * vR - hL * uL * vL - fw02 - fw22);

    const F s[3] = {lam0 * w0, lam1 * w1, lam2 * w2};
    const F fw[3][3] = {{fw00 * w0, fw01 * w0, fw02 * w0}, {fw10 * w1, fw11 * w1, fw12 * w1},
                        {fw20 * w2, fw21 * w2, fw22 * w2}};
    F am[3] = {zero, zero, zero}, ap[3] = {zero, zero, zero};
#pragma unroll
    for (int w = 0; w < 3; ++w) {
        out.s[w] = s[w];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const F v = fw[w][c];
            if (!isfinite(v)) status |= 2;
            if (s[w] < F(-1.0e-14)) am[c] = am[c] + v;
            else if (s[w] > F(1.0e-14)) ap[c] = ap[c] + v;
            else { am[c] = am[c] + half * v; ap[c] = ap[c] + half * v; }
        }
        if (!isfinite(s[w])) status |= 2;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        out.amdq[c] = am[c]; out.apdq[c] = ap[c];
        if (!isfinite(am[c]) || !isfinite(ap[c])) status |= 2;
    }
    return status;
}

template <class F>
__device__ __forceinline__ F wall_pressure(F h, F momentum, F g, F dry)
{
    if (h <= dry) return F(0);
    const F c = sqrt(g * h), v = quo<F>(quo<F>(momentum, h), c);
    F ratio;
    if (v <= F(0)) { const F a = fmax(F(0), F(1) + F(0.5) * v); ratio = a * a; }
    else {
        F lo = F(1), hi = F(1) + sqrt(F(2)) * v, rr = F(1) + v;
        for (int k = 0; k < 32; ++k) {
            const F s = sqrt(F(0.5) * (F(1) + quo<F>(F(1), rr)));
            const F f = (rr - F(1)) * s - v;
            if (fabs(f) <= F(2.e-15) * fmax(F(1), v)) break;
            if (f > F(0)) hi = rr; else lo = rr;
            const F df = s - quo<F>(rr - F(1), F(4) * s * rr * rr);
            const F trial = rr - quo<F>(f, df);
            rr = (trial > lo && trial < hi) ? trial : F(0.5) * (lo + hi);
        }
        ratio = rr;
    }
    const F star = h * ratio;
    return F(0.5) * g * star * star;
}

}  // namespace brx
