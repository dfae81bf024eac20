// bs_math.cuh -- device arithmetic: complex numbers, the reference's
// recurrences (rts/math/legendre.h, rts/math/spherical_bessel.h) and
// double-precision spherical Bessel functions for the Mie coefficients and
// the lookup tables.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "bs_internal.h"

namespace bs {

template <class T>
struct cpx {
    T re, im;
};
using zd = cpx<double>;

template <class T>
__host__ __device__ __forceinline__ cpx<T> mk(T r, T i) {
    cpx<T> z;
    z.re = r;
    z.im = i;
    return z;
}
template <class T>
__host__ __device__ __forceinline__ cpx<T> operator+(cpx<T> a, cpx<T> b) { return mk(a.re + b.re, a.im + b.im); }
template <class T>
__host__ __device__ __forceinline__ cpx<T> operator-(cpx<T> a, cpx<T> b) { return mk(a.re - b.re, a.im - b.im); }
template <class T>
__host__ __device__ __forceinline__ cpx<T> operator*(cpx<T> a, cpx<T> b) {
    return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <class T>
__host__ __device__ __forceinline__ cpx<T> operator*(cpx<T> a, T s) { return mk(a.re * s, a.im * s); }
template <class T>
__host__ __device__ __forceinline__ cpx<T> operator*(T s, cpx<T> a) { return mk(a.re * s, a.im * s); }
template <class T>
__host__ __device__ __forceinline__ cpx<T> operator/(cpx<T> a, cpx<T> b) {
    // Smith's algorithm: scale by the larger component of b to avoid overflow
    if (fabs(b.re) >= fabs(b.im)) {
        T r = b.im / b.re, den = b.re + b.im * r;
        return mk((a.re + a.im * r) / den, (a.im - a.re * r) / den);
    }
    T r = b.re / b.im, den = b.re * r + b.im;
    return mk((a.re * r + a.im) / den, (a.im * r - a.re) / den);
}
template <class T>
__host__ __device__ __forceinline__ T cabs2(cpx<T> a) { return a.re * a.re + a.im * a.im; }

__device__ __forceinline__ double zabs(zd a) { return hypot(a.re, a.im); }

// sin, cos of a complex argument (rts/math/complex.h:379-395)
__device__ __forceinline__ zd zsin(zd z) { return mk(sin(z.re) * cosh(z.im), cos(z.re) * sinh(z.im)); }
__device__ __forceinline__ zd zcos(zd z) { return mk(cos(z.re) * cosh(z.im), -(sin(z.re) * sinh(z.im))); }

// i^l
__device__ __forceinline__ zd ipow(int l) {
    switch (l & 3) {
        case 0: return mk(1.0, 0.0);
        case 1: return mk(0.0, 1.0);
        case 2: return mk(-1.0, 0.0);
        default: return mk(0.0, -1.0);
    }
}

// ---------------------------------------------------------------------------
// The reference's three-term recurrences
// ---------------------------------------------------------------------------
// P_n from P_{n-1}, P_{n-2} (rts/math/legendre.h:17-25)
__device__ __forceinline__ void legendre_step(int n, double x, double& P0, double& P1) {
    double Pn = ((2 * n - 1) * x * P1 - (n - 1) * P0) / n;
    P0 = P1;
    P1 = Pn;
}

// j_n upward with the "convergence" clamp of spherical_bessel.h:102-119:
// once n > x, a value outside [0.0145, 0.4] is replaced by zero.
__device__ __forceinline__ void sbesselj_step(int n, double x, double& b0, double& b1) {
    double bn = ((2 * n - 1) * b1) / x - b0;
    if (n > x && (bn < CONV_MIN || bn > CONV_MAX)) bn = 0.0;
    b0 = b1;
    b1 = bn;
}

// complex-argument version: the clamp tests the real parts
__device__ __forceinline__ void sbesselj_step_c(int n, zd x, zd& b0, zd& b1) {
    zd bn = (((double)(2 * n - 1)) * b1) / x - b0;
    if (n > x.re && (bn.re < CONV_MIN || bn.re > CONV_MAX)) bn = mk(0.0, 0.0);
    b0 = b1;
    b1 = bn;
}

// y_n upward with the floor/sign clamp of spherical_bessel.h:121-141
__device__ __forceinline__ void sbessely_step(int n, double x, double& b0, double& b1) {
    double bn = ((2 * n - 1) * b1) / x - b0;
    if (bn < Y_FLOOR || (n > x && bn > 0)) {
        bn = 0;
        b1 = 0;
    }
    b0 = b1;
    b1 = bn;
}

// ---------------------------------------------------------------------------
// Accurate spherical Bessel functions, double precision.
//   j_l: upward from j_0, j_1 while l < x, otherwise Miller's downward
//        recurrence from a start order well above max(l, x), normalised to
//        j_0 = sin z / z (or j_1 when |j_1| > |j_0|);
//   y_l: upward from y_0, y_1 (stable).
// The reference scales J_{l+1/2} with sqrt(PI/(2x)), PI = 3.14159
// (bessjy.cpp:719-723), so every value carries the factor sqrt(3.14159/pi).
// Its Zhang & Jin routines stop at the order where J falls below 1e-200 (the
// MSTA1 estimate) and leave higher entries unset; those entries are zero here.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int miller_start(int N, double ax) {
    double m = fmax((double)N, ax);
    return (int)(m + 16.0 + sqrt(60.0 * (m + 1.0)));
}

__device__ __forceinline__ double digits_at(int n, double x) {
    return 0.5 * log10(6.28 * n) - n * log10(1.36 * x / n);
}

// Order where J_n(x) ~ 10^-mp, by secant iteration on digits_at: routine MSTA1 of
// S. Zhang and J. Jin, Computation of Special Functions (Wiley, 1996), which the
// reference's bessjy.cpp:268-290 also follows (its constants 6.28, 1.36, 1.1).
__device__ inline int order_cutoff(double x, int mp) {
    double a = fabs(x);
    int lo = (int)(1.1 * a) + 1, hi = lo + 5;
    double flo = digits_at(lo, a) - mp, fhi = digits_at(hi, a) - mp;
    int nn = hi;
    for (int it = 0; it < 20; it++) {
        nn = (int)(hi - (hi - lo) / (1.0 - flo / fhi));
        double f = digits_at(nn, a) - mp;
        if (abs(nn - hi) < 1) break;
        lo = hi;
        flo = fhi;
        hi = nn;
        fhi = f;
    }
    return nn;
}

// j[l], y[l] for l = 0..N (stride `st` between orders) of a real x > 0.
__device__ inline void sph_real(int N, double x, double* j, double* y, int st) {
    const double cs = sqrt(PI_BES / TRUE_PI);
    if (x < 1e-15) {
        double sc = sqrt(PI_BES / (x * 2.0));
        for (int l = 0; l <= N; l++) {
            j[l * st] = 0.0 * sc;
            y[l * st] = -1e308 * sc;
        }
        return;
    }
    int Nv = N;
    if (N >= 2 && N > (int)(0.9 * x)) {
        int m = order_cutoff(x, 200);
        if (m < N) Nv = m;
    }
    double s, c;
    sincos(x, &s, &c);
    double j0 = s / x, j1 = s / (x * x) - c / x;
    if (Nv < x) {
        j[0] = j0;
        if (Nv >= 1) j[st] = j1;
        double a = j0, b = j1;
        for (int l = 2; l <= Nv; l++) {
            double t = (2 * l - 1) / x * b - a;
            a = b;
            b = t;
            j[l * st] = t;
        }
    } else {
        int M = miller_start(Nv, x);
        double fp = 0.0, fc = 1e-300;
        if (M <= Nv) j[M * st] = fc;
        for (int l = M; l >= 1; l--) {
            double fm = (2 * l + 1) / x * fc - fp;
            fp = fc;
            fc = fm;
            if (l - 1 <= Nv) j[(l - 1) * st] = fm;
            if (fabs(fc) > 1e250) {
                for (int q = l - 1; q <= Nv; q++) j[q * st] *= 1e-250;
                fc *= 1e-250;
                fp *= 1e-250;
            }
        }
        double sc = (fabs(j0) >= fabs(j1)) ? j0 / j[0] : j1 / j[st];
        for (int l = 0; l <= Nv; l++) j[l * st] *= sc;
    }
    double ya = -c / x, yb = -c / (x * x) - s / x;
    y[0] = ya;
    if (Nv >= 1) y[st] = yb;
    for (int l = 2; l <= Nv; l++) {
        double t = (2 * l - 1) / x * yb - ya;
        ya = yb;
        yb = t;
        y[l * st] = t;
    }
    for (int l = 0; l <= N; l++) {
        if (l > Nv) {
            j[l * st] = 0.0;
            y[l * st] = 0.0;
        } else {
            j[l * st] *= cs;
            y[l * st] *= cs;
        }
    }
}

// Complex argument.  j, jp required; y, yp may be null.  `quirk` adds j_0 to
// y_0 when |z| > 12: the reference's cbessjyva writes cpz*csk + cqz + cck
// where cqz*cck was meant (cbessjy.cpp:541), which for order 1/2 (cqz = 0,
// cpz = 1) adds J_{1/2}(z) to Y_{1/2}(z).
__device__ inline void sph_complex(int N, zd z, bool quirk, zd* j, zd* y, zd* jp, zd* yp) {
    const double cs = sqrt(PI_BES / TRUE_PI);
    double az = zabs(z);
    int Nv = N;
    if (N >= 2 && N > (int)(0.25 * az)) {
        int m = order_cutoff(az, 200);
        if (m < N) Nv = m;
    }
    zd s = zsin(z), c = zcos(z);
    zd j0 = s / z, j1 = s / (z * z) - c / z;
    int M = miller_start(N, az);
    zd fp = mk(0.0, 0.0), fc = mk(1e-300, 0.0);
    if (M <= N) j[M] = fc;
    for (int l = M; l >= 1; l--) {
        zd fm = ((double)(2 * l + 1)) * fc / z - fp;
        fp = fc;
        fc = fm;
        if (l - 1 <= N) j[l - 1] = fm;
        if (zabs(fc) > 1e250) {
            for (int q = l - 1; q <= N; q++) j[q] = j[q] * 1e-250;
            fc = fc * 1e-250;
            fp = fp * 1e-250;
        }
    }
    zd sc = (zabs(j0) >= zabs(j1)) ? j0 / j[0] : j1 / j[1 <= N ? 1 : 0];
    for (int l = 0; l <= N; l++) j[l] = j[l] * sc;
    zd ya = zd{0, 0} - c / z;
    zd yb = zd{0, 0} - c / (z * z) - s / z;
    if (quirk && az > 12.0) ya = ya + j0;
    if (y) {
        y[0] = ya;
        if (N >= 1) y[1] = yb;
        for (int l = 2; l <= N; l++) {
            zd t = ((double)(2 * l - 1)) * yb / z - ya;
            ya = yb;
            yb = t;
            y[l] = t;
        }
    }
    for (int l = 0; l <= N; l++) {
        if (l > Nv) {
            j[l] = mk(0.0, 0.0);
            if (y) y[l] = mk(0.0, 0.0);
        } else {
            j[l] = j[l] * cs;
            if (y) y[l] = y[l] * cs;
        }
    }
    // j_0' = -j_1, j_l' = j_{l-1} - (l+1)/z j_l (the derivative cbessjyva
    // and cbessjyva_sph form, cbessjy.cpp:590-593 and 726-733)
    if (jp) {
        jp[0] = zd{0, 0} - (N >= 1 ? j[1] : j1 * cs);
        for (int l = 1; l <= N; l++) jp[l] = j[l - 1] - ((double)(l + 1)) * j[l] / z;
    }
    if (yp && y) {
        yp[0] = zd{0, 0} - (N >= 1 ? y[1] : yb * cs);
        for (int l = 1; l <= N; l++) yp[l] = y[l - 1] - ((double)(l + 1)) * y[l] / z;
    }
}

}  // namespace bs
