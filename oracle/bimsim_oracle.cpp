// bimsim_oracle.cpp -- TEST INFRASTRUCTURE, not product code.
//
// A double-precision CPU restatement of the reference's near-field-to-detector
// path.  The reference computes on the GPU in single precision
// (dataTypes.h:6) and evaluates its special functions on the host in double;
// this file keeps the reference's formulas, constants, loop bounds and quirks
// and evaluates all of them in double.  Only the tests, the smoke check and
// the bench's CPU baseline call it.  Built with -ffp-contract=off so that the
// same source gives the same bits on x86-64 and aarch64.
#include "bimsim_oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using cd = std::complex<double>;

// dataTypes.h:17 defines PI as the float literal 3.14159f; every use in the
// kernels and in sphere.cpp/nearfield.cpp sees that float value.
constexpr double PI_REF = (double)3.14159f;
// bessjy.cpp:18 and cbessjy.cpp:16 define PI as the double literal 3.14159;
// it scales J_{n+1/2} into spherical functions (bessjy.cpp:719-723).
constexpr double PI_BES = 3.14159;
constexpr double TRUE_PI = 3.14159265358979323846;
// nearfield.h:11
constexpr double EPS_FLOAT = (double)0.000001f;
// rts/math/spherical_bessel.h:8-10
constexpr double CONV_MIN = 0.0145;
constexpr double CONV_MAX = 0.4;
constexpr double Y_FLOOR = -1e33;

struct V3 {
    double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double len(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 v3(const double* p) { return {p[0], p[1], p[2]}; }

// ---------------------------------------------------------------------------
// Geometry: rts/math/quad.h and rts/math/triangle.h
// ---------------------------------------------------------------------------
struct Quad {
    V3 A, X, Y;
};

// quad(pMin, pMax, normal), rts/math/quad.h:55-84
Quad quad_from(V3 pmin, V3 pmax, V3 normal) {
    V3 v0 = pmax - pmin;
    V3 v1 = cross(v0, normal);
    V3 B = pmin + v0 * 0.5 + v1 * 0.5;
    V3 C = pmin + v0 * 0.5 - v1 * 0.5;
    return {pmin, B - pmin, C - pmin};
}

// quad * scalar, rts/math/quad.h:162-177
Quad quad_scale(const Quad& q, double s) {
    V3 c = q.A + q.X * 0.5 + q.Y * 0.5;
    Quad r;
    r.X = q.X * s;
    r.Y = q.Y * s;
    r.A = c - r.X * 0.5 - r.Y * 0.5;
    return r;
}

inline V3 quad_at(const Quad& q, double u, double v) { return q.A + q.X * u + q.Y * v; }

// triangle::nearest, rts/math/triangle.h:62-177, including its shortcut
// regions 2, 4 and 6 (corner points without edge minimisation).
V3 tri_nearest(V3 A, V3 B, V3 C, V3 p) {
    V3 E0 = B - A, E1 = C - A, D = A - p;
    double a = dot(E0, E0), b = dot(E0, E1), c = dot(E1, E1), d = dot(E0, D), e = dot(E1, D);
    double det = a * c - b * b;
    double s = b * e - c * d;
    double t = b * d - a * e;
    if (s + t <= det) {
        if (s < 0) {
            if (t < 0) {
                s = 0;
                t = 0;
            } else {
                s = 0;
                t = (e >= 0 ? 0 : (-e >= c ? 1 : -e / c));
            }
        } else if (t < 0) {
            s = (d >= 0 ? 0 : (-d >= a ? 1 : -d / a));
            t = 0;
        } else {
            double inv = 1.0 / det;
            s *= inv;
            t *= inv;
        }
    } else {
        if (s < 0) {
            s = 0;
            t = 1;
        } else if (t < 0) {
            s = 1;
            t = 0;
        } else {
            double numer = c + e - b - d;
            if (numer <= 0) {
                s = 0;
            } else {
                double denom = a - 2 * b + c;
                s = (numer >= denom ? 1 : numer / denom);
            }
            t = 1 - s;
        }
    }
    return A + E0 * s + E1 * t;
}

// quad::dist, rts/math/quad.h:179-195
double quad_dist(const Quad& q, V3 p) {
    V3 n0 = tri_nearest(q.A, q.A + q.X, q.A + q.Y, p);
    V3 n1 = tri_nearest(q.A + q.X + q.Y, q.A + q.X, q.A + q.Y, p);
    double d0 = len(p - n0), d1 = len(p - n1);
    return d0 < d1 ? d0 : d1;
}

// quad::dist_max, rts/math/quad.h:197-205
double quad_dist_max(const Quad& q, V3 p) {
    double da = len(q.A - p), db = len(q.A + q.X - p), dc = len(q.A + q.Y - p),
           dd = len(q.A + q.X + q.Y - p);
    return std::max(da, std::max(db, std::max(dc, dd)));
}

// ---------------------------------------------------------------------------
// Recurrences of rts/math/legendre.h and rts/math/spherical_bessel.h
// ---------------------------------------------------------------------------
inline void shift_legendre(int n, double x, double& P0, double& P1) {  // legendre.h:17-25
    double Pn = ((2 * n - 1) * x * P1 - (n - 1) * P0) / n;
    P0 = P1;
    P1 = Pn;
}

// shift_sbesselj for a real argument, spherical_bessel.h:102-119
inline void shift_sbesselj(int n, double x, double* b) {
    double bn = ((2 * n - 1) * b[1]) / x - b[0];
    if (n > x)
        if (bn < CONV_MIN || bn > CONV_MAX) bn = 0.0;
    b[0] = b[1];
    b[1] = bn;
}

// shift_sbesselj for a complex argument (clamp on the real part)
inline void shift_sbesselj_c(int n, cd x, cd* b) {
    cd bn = (double)(2 * n - 1) * b[1] / x - b[0];
    if (n > x.real())
        if (bn.real() < CONV_MIN || bn.real() > CONV_MAX) bn = 0.0;
    b[0] = b[1];
    b[1] = bn;
}

// shift_sbessely, spherical_bessel.h:121-141
inline void shift_sbessely(int n, double x, double* b) {
    double bn = ((2 * n - 1) * b[1]) / x - b[0];
    if (bn < Y_FLOOR || (n > x && bn > 0)) {
        bn = 0;
        b[1] = 0;
    }
    b[0] = b[1];
    b[1] = bn;
}

// rts::complex sin/cos (complex.h:379-395)
inline cd csin(cd z) { return {std::sin(z.real()) * std::cosh(z.imag()), std::cos(z.real()) * std::sinh(z.imag())}; }
inline cd ccos(cd z) { return {std::cos(z.real()) * std::cosh(z.imag()), -(std::sin(z.real()) * std::sinh(z.imag()))}; }

inline cd ipow(int l) {  // i^l
    switch (l & 3) {
        case 0: return {1, 0};
        case 1: return {0, 1};
        case 2: return {-1, 0};
        default: return {0, -1};
    }
}

// ---------------------------------------------------------------------------
// Accurate spherical Bessel functions (Zhang & Jin's role in bessjy.cpp /
// cbessjy.cpp).  Written from the textbook method: j_l by Miller's downward
// recurrence normalised to j_0 or j_1 (upward when l < x), y_l by upward
// recurrence.  The reference's spherical scaling uses PI = 3.14159, so every
// value is the true function times sqrt(3.14159/pi).
// ---------------------------------------------------------------------------
inline int miller_start(int N, double ax) {
    double m = std::max((double)N, ax);
    return (int)(m + 16.0 + std::sqrt(60.0 * (m + 1.0)));
}

// Zhang & Jin's MSTA1 estimate: the order n at which J_n(x) has fallen to
// about 10^-mp, found by secant iteration on
//     0.5 log10(6.28 n) - n log10(1.36 x / n) = mp.
// The reference's bessjyv/cbessjyva stop at that order when it is below the
// requested one and leave the higher entries unset (bessjy.cpp:631-633,
// cbessjy.cpp:599-601); this restatement defines those entries as zero.
inline double envj_digits(int n, double x) { return 0.5 * std::log10(6.28 * n) - n * std::log10(1.36 * x / n); }

int order_cutoff(double x, int mp) {
    double a = std::fabs(x);
    int lo = (int)(1.1 * a) + 1;
    int hi = lo + 5;
    double flo = envj_digits(lo, a) - mp, fhi = envj_digits(hi, a) - mp;
    int nn = hi;
    for (int it = 0; it < 20; it++) {
        nn = (int)(hi - (hi - lo) / (1.0 - flo / fhi));
        double f = envj_digits(nn, a) - mp;
        if (std::abs(nn - hi) < 1) break;
        lo = hi;
        flo = fhi;
        hi = nn;
        fhi = f;
    }
    return nn;
}

void sph_real(int N, double x, double* j, double* y) {
    const double cs = std::sqrt(PI_BES / TRUE_PI);
    if (x < 1e-15) {
        // bessjyv's x < 1e-15 branch leaves J_{n+1/2} = 0 and Y = -1e308
        // (bessjy.cpp:554-567); the spherical scaling sqrt(PI/(2x))
        // (bessjy.cpp:719-720) then gives 0*inf at x = 0.
        double sc = std::sqrt(PI_BES / (x * 2.0));
        for (int l = 0; l <= N; l++) {
            j[l] = 0.0 * sc;
            y[l] = -1e308 * sc;
        }
        return;
    }
    int Nv = N;  // orders actually evaluated
    if (N >= 2 && N > (int)(0.9 * x)) {
        int m = order_cutoff(x, 200);
        if (m < N) Nv = m;
    }
    double s = std::sin(x), c = std::cos(x);
    double j0 = s / x, j1 = s / (x * x) - c / x;
    if (Nv < x) {
        j[0] = j0;
        if (Nv >= 1) j[1] = j1;
        for (int l = 2; l <= Nv; l++) j[l] = (2 * l - 1) / x * j[l - 1] - j[l - 2];
    } else {
        int M = miller_start(Nv, x);
        std::vector<double> f(M + 2, 0.0);
        double fp = 0.0, fc = 1e-300;
        f[M + 1] = 0.0;
        f[M] = fc;
        for (int l = M; l >= 1; l--) {
            double fm = (2 * l + 1) / x * fc - fp;
            fp = fc;
            fc = fm;
            f[l - 1] = fm;
            if (std::fabs(fc) > 1e250) {  // rescale to avoid overflow
                for (int q = l - 1; q <= M; q++) f[q] *= 1e-250;
                fc *= 1e-250;
                fp *= 1e-250;
            }
        }
        double sc = (std::fabs(j0) >= std::fabs(j1)) ? j0 / f[0] : j1 / f[1];
        for (int l = 0; l <= Nv; l++) j[l] = f[l] * sc;
    }
    y[0] = -c / x;
    if (Nv >= 1) y[1] = -c / (x * x) - s / x;
    for (int l = 2; l <= Nv; l++) y[l] = (2 * l - 1) / x * y[l - 1] - y[l - 2];
    for (int l = 0; l <= N; l++) {
        if (l > Nv) {
            j[l] = 0.0;
            y[l] = 0.0;
            continue;
        }
        j[l] *= cs;
        y[l] *= cs;
    }
}

void sph_complex(int N, cd z, bool typo, cd* j, cd* y, cd* jp, cd* yp) {
    const double cs = std::sqrt(PI_BES / TRUE_PI);
    double az = std::abs(z);
    int Nv = N;
    if (N >= 2 && N > (int)(0.25 * az)) {
        int m = order_cutoff(az, 200);
        if (m < N) Nv = m;
    }
    cd s = std::sin(z), c = std::cos(z);
    cd j0 = s / z, j1 = s / (z * z) - c / z;
    int M = miller_start(N, az);
    std::vector<cd> f(M + 2);
    cd fp = 0.0, fc = 1e-300;
    f[M + 1] = 0.0;
    f[M] = fc;
    for (int l = M; l >= 1; l--) {
        cd fm = (double)(2 * l + 1) / z * fc - fp;
        fp = fc;
        fc = fm;
        f[l - 1] = fm;
        if (std::abs(fc) > 1e250) {
            for (int q = l - 1; q <= M; q++) f[q] *= 1e-250;
            fc *= 1e-250;
            fp *= 1e-250;
        }
    }
    cd sc = (std::abs(j0) >= std::abs(j1)) ? j0 / f[0] : j1 / f[1];
    for (int l = 0; l <= N; l++) j[l] = f[l] * sc;
    cd y0 = -c / z;
    cd y1 = -c / (z * z) - s / z;
    // cbessjy.cpp:541 writes cyv0 = ca0*(cpz*csk+cqz+cck) for |z| > 12; with
    // order 1/2 (cqz = 0, cpz = 1) the extra ca0*cck is J_{1/2}(z), so the
    // reference's y_0 becomes y_0 + j_0 while y_1 stays exact.
    if (typo && az > 12.0) y0 += j0;
    y[0] = y0;
    if (N >= 1) y[1] = y1;
    for (int l = 2; l <= N; l++) y[l] = (double)(2 * l - 1) / z * y[l - 1] - y[l - 2];
    for (int l = 0; l <= N; l++) {
        if (l > Nv) {
            j[l] = 0.0;
            y[l] = 0.0;
            continue;
        }
        j[l] *= cs;
        y[l] *= cs;
    }
    // derivatives as cbessjyva + cbessjyva_sph produce them: j_0' = -j_1,
    // j_l' = j_{l-1} - (l+1)/z j_l (cbessjy.cpp:590-593, 726-733)
    if (N >= 1) {
        jp[0] = -j[1];
        yp[0] = -y[1];
    } else {
        cd j1s = j1 * cs, y1s = y1 * cs;
        jp[0] = -j1s;
        yp[0] = -y1s;
    }
    for (int l = 1; l <= N; l++) {
        jp[l] = j[l - 1] - (double)(l + 1) / z * j[l];
        yp[l] = y[l - 1] - (double)(l + 1) / z * y[l];
    }
}

// ---------------------------------------------------------------------------
// glibc rand(): TYPE_3 additive generator, r_i = r_{i-3} + r_{i-31} mod 2^32,
// seeded by the 16807 Lehmer sequence, first 310 outputs discarded.
// ---------------------------------------------------------------------------
struct GlibcRand {
    uint32_t r[34];
    int pos;
    std::vector<uint32_t> hist;
    explicit GlibcRand(unsigned seed) {
        if (seed == 0) seed = 1;
        hist.reserve(512);
        int64_t w = seed;
        hist.push_back((uint32_t)w);
        for (int i = 1; i < 31; i++) {
            w = (16807LL * w) % 2147483647LL;
            if (w < 0) w += 2147483647LL;
            hist.push_back((uint32_t)w);
        }
        for (int i = 31; i < 34; i++) hist.push_back(hist[i - 31]);
        for (int i = 34; i < 344; i++) hist.push_back(hist[i - 31] + hist[i - 3]);
        pos = 344;
    }
    int next() {
        uint32_t v = hist[pos - 31] + hist[pos - 3];
        hist.push_back(v);
        pos++;
        return (int)(v >> 1);
    }
};

// ---------------------------------------------------------------------------
// Parameters and per-sphere derivation
// ---------------------------------------------------------------------------
struct Geom {
    int R, res, ss, pad, crop_res, crop_off;
    Quad det, nf;
    double kmag, sub_amp, cos_a, cos_b;
};

Geom derive(const bs_params& p) {
    Geom g;
    g.res = p.resolution;
    g.ss = std::max(1, (int)p.supersample);
    g.pad = p.padding;
    g.R = g.res * g.ss * (2 * g.pad + 1);        // microscope.cu:700-718
    g.crop_res = g.res * g.ss;
    g.crop_off = g.pad * g.crop_res;              // microscope.cu:641-655
    g.det = quad_from(v3(p.plane_min), v3(p.plane_max), v3(p.plane_normal));
    g.nf = quad_scale(g.det, (double)(2 * g.pad + 1));
    g.kmag = 2 * PI_REF / p.lambda;
    g.cos_a = std::cos(std::asin(p.condenser[0]));  // nfScalarUf.cu:197-198
    g.cos_b = std::cos(std::asin(p.condenser[1]));
    // nfScalarUpLut.cu:365-379
    if (p.plane_wave)
        g.sub_amp = p.amplitude;
    else
        g.sub_amp = 2 * PI_REF * p.amplitude * ((1 - g.cos_b) - (1 - g.cos_a));
    return g;
}

int calc_nl(double a_d, double lambda_d) {  // sphere.h:71-74, single precision
    volatile float a = (float)a_d, lam = (float)lambda_d;
    volatile float pi = 3.14159f;
    volatile float t = 2.0f * pi;
    t = t * a;
    t = t / lam;
    volatile float third = (float)(1.0 / 3.0);
    volatile float pw = std::pow((float)t, (float)third);
    volatile float four = 4.0f * pw;
    volatile float v = t + four;
    v = v + 2.0f;
    return (int)std::ceil((float)v);
}

struct SphereGeom {
    int Nl, aR, dR, thetaR;
    double dmin, dmax, r0;
};

SphereGeom sphere_derive(const bs_params& p, const Geom& g, const bs_sphere& s) {
    SphereGeom sg;
    sg.Nl = calc_nl(s.a, p.lambda);
    V3 c{s.x, s.y, s.z};
    sg.dmin = quad_dist(g.nf, c);      // sphere.cpp:227
    sg.dmax = quad_dist_max(g.nf, c);  // sphere.cpp:228
    double a_inter = 0;
    if (sg.dmin < s.a) a_inter = std::sqrt(s.a - sg.dmin);  // sphere.cpp:231-233 (sic)
    double diag = len(g.nf.X + g.nf.Y);                     // |nfPlane(0,0) - nfPlane(1,1)|
    sg.aR = (int)(1 + 2.0 * g.R * a_inter / diag);          // sphere.cpp:237
    sg.dR = p.us_lut_r > 0 ? p.us_lut_r : 2 * g.R;          // sphere.cpp:238
    sg.thetaR = p.us_lut_theta > 0 ? p.us_lut_theta : 1000; // sphere.cpp:239, defaults.h:83
    sg.r0 = std::max(s.a, sg.dmin);
    return sg;
}

// Mie coefficients, sphere.cpp:21-97
void mie(double k, double a, cd n, int Nl, cd* A, cd* B) {
    cd kna = n * k * a;
    cd ka(k * a, 0.0);
    std::vector<cd> ja(Nl + 1), ya(Nl + 1), jpa(Nl + 1), ypa(Nl + 1);
    std::vector<cd> jn(Nl + 1), yn(Nl + 1), jpn(Nl + 1), ypn(Nl + 1);
    sph_complex(Nl, ka, true, ja.data(), ya.data(), jpa.data(), ypa.data());
    sph_complex(Nl, kna, true, jn.data(), yn.data(), jpn.data(), ypn.data());
    const cd I(0, 1);
    for (int l = 0; l <= Nl; l++) {
        cd h = ja[l] + I * ya[l];
        cd hp = jpa[l] + I * ypa[l];
        cd an = ja[l] * hp - jpa[l] * h;
        cd bn = jn[l] * hp - h * jpn[l] * n;
        A[l] = (2.0 * l + 1.0) * ipow(l) * (an / bn);
        cd cn = ja[l] * jpn[l] * n - jn[l] * jpa[l];
        cd dn = jn[l] * hp - h * jpn[l] * n;
        B[l] = (2.0 * l + 1.0) * ipow(l) * (cn / dn);
    }
}

// Per-sphere LUTs Usp(r, theta), Uip(r, theta), radial-major, filled on
// first use.  Values are those of gpuScalarUsp / gpuScalarUip
// (sphere.cu:4-99) on the Bessel/Hankel tables of sphere.cpp:99-203.
struct SphereLut {
    SphereGeom sg;
    double a;
    std::vector<cd> A, B;
    std::vector<cd> h;  // dR x (Nl+1)
    std::vector<cd> jt; // aR x (Nl+1)
    std::vector<double> ctheta;  // thetaR
    cd* usp = nullptr;           // dR x thetaR
    cd* uip = nullptr;           // aR x thetaR
    std::atomic<uint8_t>* usp_ok = nullptr;
    std::atomic<uint8_t>* uip_ok = nullptr;

    ~SphereLut() {
        std::free(usp);
        std::free(uip);
        std::free(usp_ok);
        std::free(uip_ok);
    }

    void build(const Geom& g, const bs_sphere& s, const SphereGeom& sgeo, double lambda) {
        sg = sgeo;
        a = s.a;
        int L = sg.Nl + 1;
        A.resize(L);
        B.resize(L);
        double k = 2 * PI_REF / lambda;  // sphere.cpp:135 / :310
        mie(k, s.a, cd(s.n_re, s.n_im), sg.Nl, A.data(), B.data());
        // calcHankelLut, sphere.cpp:154-203
        h.resize((size_t)sg.dR * L);
        std::vector<double> jj(L), yy(L);
        double dr = (sg.dmax - sg.r0) / (sg.dR - 1);
        for (int ir = 0; ir < sg.dR; ir++) {
            double r = ir * dr + sg.r0;
            sph_real(sg.Nl, k * r, jj.data(), yy.data());
            for (int l = 0; l < L; l++) h[(size_t)ir * L + l] = cd(jj[l], yy[l]);
        }
        // calcBesselLut, sphere.cpp:99-152
        jt.resize((size_t)sg.aR * L);
        std::vector<cd> cj(L), cy(L), cjp(L), cyp(L);
        double da = s.a / (sg.aR - 1);
        cd n(s.n_re, s.n_im);
        for (int ia = 0; ia < sg.aR; ia++) {
            if (ia == 0) {
                for (int l = 0; l < L; l++) jt[l] = (l == 0) ? cd(1, 0) : cd(0, 0);
                continue;
            }
            double r = ia * da;
            cd knr = k * n * r;
            sph_complex(sg.Nl, knr, true, cj.data(), cy.data(), cjp.data(), cyp.data());
            for (int l = 0; l < L; l++) jt[(size_t)ia * L + l] = cj[l];
        }
        // theta samples, sphere.cu:16-21: the step (PI) / (thetaR - 1) is the float literal PI
        // over an int, a single-precision quotient even in the reference's double build
        ctheta.resize(sg.thetaR);
        double dtheta = (double)(3.14159f / (float)(sg.thetaR - 1));
        for (int it = 0; it < sg.thetaR; it++) ctheta[it] = std::cos(dtheta * it);
        size_t nu = (size_t)sg.dR * sg.thetaR, ni = (size_t)sg.aR * sg.thetaR;
        usp = (cd*)std::calloc(nu, sizeof(cd));
        uip = (cd*)std::calloc(ni, sizeof(cd));
        usp_ok = (std::atomic<uint8_t>*)std::calloc(nu, 1);
        uip_ok = (std::atomic<uint8_t>*)std::calloc(ni, 1);
    }

    // sum over orders with the Legendre recurrence, sphere.cu:24-39
    cd order_sum(const cd* coef, const cd* tab, int it) const {
        double x = ctheta[it];
        double P0 = 1, P1 = x;
        cd U(0, 0);
        for (int l = 0; l <= sg.Nl; l++) {
            if (l == 0) {
                U += coef[0] * tab[0] * P0;
            } else {
                if (l > 1) shift_legendre(l, x, P0, P1);
                U += coef[l] * tab[l] * P1;
            }
        }
        return U;
    }

    cd Usp(int ir, int it) {
        size_t idx = (size_t)ir * sg.thetaR + it;
        if (!usp_ok[idx].load(std::memory_order_acquire)) {
            usp[idx] = order_sum(B.data(), &h[(size_t)ir * (sg.Nl + 1)], it);
            usp_ok[idx].store(1, std::memory_order_release);
        }
        return usp[idx];
    }
    cd Uip(int ia, int it) {
        size_t idx = (size_t)ia * sg.thetaR + it;
        if (!uip_ok[idx].load(std::memory_order_acquire)) {
            uip[idx] = order_sum(A.data(), &jt[(size_t)ia * (sg.Nl + 1)], it);
            uip_ok[idx].store(1, std::memory_order_release);
        }
        return uip[idx];
    }

    // Linear filtering with unnormalised coordinates (x + 0.5, y + 0.5) and
    // clamp addressing, with exact weights (nfScalarUpLut.cu:83,89).
    template <class F>
    static cd bilerp(F get, double x, double y, int W, int H) {
        x = std::min(std::max(x, 0.0), (double)(W - 1));
        y = std::min(std::max(y, 0.0), (double)(H - 1));
        int i = (int)std::floor(x), j = (int)std::floor(y);
        double al = x - i, be = y - j;
        int i1 = std::min(i + 1, W - 1), j1 = std::min(j + 1, H - 1);
        return (1 - al) * (1 - be) * get(i, j) + al * (1 - be) * get(i1, j) +
               (1 - al) * be * get(i, j1) + al * be * get(i1, j1);
    }
};

// ---------------------------------------------------------------------------
// Incident field
// ---------------------------------------------------------------------------
// gpuScalarUf, nfScalarUf.cu:46-175
cd uf_direct(const bs_params& p, const Geom& g, V3 pt) {
    V3 f = v3(p.focus), k = v3(p.k_dir);
    V3 r = pt - f;
    double d = len(r);
    if (d < EPS_FLOAT) return cd(p.amplitude * 2 * PI_REF * (g.cos_a - g.cos_b), 0);
    r = r * (1.0 / d);
    double kd = g.kmag * d;
    double j[2] = {std::sin(kd) / kd, 0};
    j[1] = j[0] / kd - std::cos(kd) / kd;
    double cth = dot(k, r);
    double P[2] = {1, cth};
    double Pa[3] = {1, g.cos_a, 1}, Pb[3] = {1, g.cos_b, 1};
    cd sum(0, 0), il(1, 0);
    for (int l = 0; l <= p.field_order; l++) {
        double jl, Pl;
        if (l == 0) {
            jl = j[0];
            Pl = P[0];
        } else if (l == 1) {
            jl = j[1];
            Pl = P[1];
            Pa[2] = Pa[0];
            shift_legendre(l + 1, g.cos_a, Pa[0], Pa[1]);
            Pb[2] = Pb[0];
            shift_legendre(l + 1, g.cos_b, Pb[0], Pb[1]);
        } else {
            shift_sbesselj(l, kd, j);
            shift_legendre(l, cth, P[0], P[1]);
            jl = j[1];
            Pl = P[1];
            Pa[2] = Pa[0];
            shift_legendre(l + 1, g.cos_a, Pa[0], Pa[1]);
            Pb[2] = Pb[0];
            shift_legendre(l + 1, g.cos_b, Pb[0], Pb[1]);
        }
        sum += il * jl * Pl * (Pa[1] - Pa[2] - Pb[1] + Pb[2]);
        il *= cd(0, 1);
    }
    return sum * 2.0 * PI_REF * p.amplitude;
}

// gpuScalarUfp, nfScalarUf.cu:9-44
cd uf_plane(const bs_params& p, const Geom& g, V3 pt) {
    V3 r = pt - v3(p.focus);
    double kdr = g.kmag * dot(v3(p.k_dir), r);
    return std::exp(cd(0, kdr)) * p.amplitude;
}

struct UfTable {
    double dmin, dmax;
    int dR, m;
    std::vector<double> j;  // dR x (m+1)
};

// nearfieldStruct::calcBesselLut, nearfield.cpp:222-283
UfTable uf_table(const bs_params& p, const Geom& g) {
    UfTable t;
    V3 f = v3(p.focus);
    t.dmin = quad_dist(g.nf, f);
    t.dmax = quad_dist_max(g.nf, f);
    t.dR = p.uf_lut_r > 0 ? p.uf_lut_r : 2 * g.R;
    t.m = p.field_order;
    int L = t.m + 1;
    t.j.resize((size_t)t.dR * L);
    std::vector<double> jj(L), yy(L);
    double dr = (t.dmax - t.dmin) / (t.dR - 1);
    for (int id = 0; id < t.dR; id++) {
        double d = id * dr + t.dmin;
        double kd = g.kmag * d;
        sph_real(t.m, kd, jj.data(), yy.data());
        for (int l = 0; l < L; l++) {
            double jv = jj[l];
            if (std::isnan(jv) || std::isinf(jv)) jv = (kd == 0 && l == 0) ? 1 : 0;
            t.j[(size_t)id * L + l] = jv;
        }
    }
    return t;
}

// gpuScalarUfLut, nfScalarUfLut.cu:11-123
cd uf_lut(const bs_params& p, const Geom& g, const UfTable& t, V3 pt) {
    V3 f = v3(p.focus), k = v3(p.k_dir);
    V3 r = pt - f;
    double d = len(r);
    if (d == 0) return cd(p.amplitude * 2 * PI_REF * (g.cos_a - g.cos_b), 0);
    r = r * (1.0 / d);
    double cth = dot(k, r);
    double P[2] = {1, cth};
    double Pa[3] = {1, g.cos_a, 1}, Pb[3] = {1, g.cos_b, 1};
    cd sum(0, 0), il(1, 0);
    int L = t.m + 1;
    double di = ((d - t.dmin) / (t.dmax - t.dmin)) * (t.dR - 1);
    double y = std::min(std::max(di, 0.0), (double)(t.dR - 1));
    int i0 = (int)std::floor(y);
    double be = y - i0;
    int i1 = std::min(i0 + 1, t.dR - 1);
    for (int l = 0; l <= t.m; l++) {
        double jl = (1 - be) * t.j[(size_t)i0 * L + l] + be * t.j[(size_t)i1 * L + l];
        double Pl;
        if (l == 0) {
            Pl = P[0];
        } else if (l == 1) {
            Pl = P[1];
            Pa[2] = Pa[0];
            shift_legendre(l + 1, g.cos_a, Pa[0], Pa[1]);
            Pb[2] = Pb[0];
            shift_legendre(l + 1, g.cos_b, Pb[0], Pb[1]);
        } else {
            shift_legendre(l, cth, P[0], P[1]);
            Pl = P[1];
            Pa[2] = Pa[0];
            shift_legendre(l + 1, g.cos_a, Pa[0], Pa[1]);
            Pb[2] = Pb[0];
            shift_legendre(l + 1, g.cos_b, Pb[0], Pb[1]);
        }
        sum += il * jl * Pl * (Pa[1] - Pa[2] - Pb[1] + Pb[2]);
        il *= cd(0, 1);
    }
    return sum * 2.0 * PI_REF * p.amplitude;
}

// ---------------------------------------------------------------------------
// Scattered field, direct (--recursive): calc_Us / calc_Ui, nfScalarUs.cu
// ---------------------------------------------------------------------------
cd calc_us(double kd, double cth, int Nl, const cd* B) {  // nfScalarUs.cu:50-95
    double j[2], y[2];
    j[0] = std::sin(kd) / kd;
    j[1] = j[0] / kd - std::cos(kd) / kd;
    y[0] = -std::cos(kd) / kd;
    y[1] = y[0] / kd - std::sin(kd) / kd;
    double P[2] = {1, cth};
    cd U(0, 0);
    for (int l = 0; l <= Nl; l++) {
        if (l == 0) {
            U += B[0] * cd(j[0], y[0]) * P[0];
        } else {
            if (l > 1) {
                shift_legendre(l, cth, P[0], P[1]);
                shift_sbesselj(l, kd, j);
                shift_sbessely(l, kd, y);
            }
            U += B[l] * cd(j[1], y[1]) * P[1];
        }
    }
    return U;
}

cd calc_ui(cd knd, double cth, int Nl, const cd* A) {  // nfScalarUs.cu:201-245
    if (knd.real() < EPS_FLOAT) return A[0];
    cd j[2];
    j[0] = csin(knd) / knd;
    j[1] = j[0] / knd - ccos(knd) / knd;
    double P[2] = {1, cth};
    cd U(0, 0);
    for (int l = 0; l <= Nl; l++) {
        if (l == 0) {
            U += A[0] * j[0] * P[0];
        } else {
            if (l > 1) {
                shift_legendre(l, cth, P[0], P[1]);
                shift_sbesselj_c(l, knd, j);
            }
            U += A[l] * j[1] * P[1];
        }
    }
    return U;
}

// ---------------------------------------------------------------------------
// The whole near field for a set of rows
// ---------------------------------------------------------------------------
struct Scene {
    bs_params p;
    Geom g;
    std::vector<bs_sphere> s;
    std::vector<SphereGeom> sg;
    std::vector<SphereLut*> lut;  // LUT mode
    std::vector<std::vector<cd>> A, B;  // direct mode
    std::vector<V3> waves;
    UfTable uft;
    int nk;

    ~Scene() {
        for (auto* l : lut) delete l;
    }
};

void scene_init(Scene& sc, const bs_params& p, const bs_sphere* s, int ns, const double* waves, int nk) {
    sc.p = p;
    sc.g = derive(p);
    sc.s.assign(s, s + ns);
    if (p.plane_wave) {
        sc.waves.assign(1, v3(p.k_dir));  // nfScalarUpLut.cu:365-371
        sc.nk = 1;
    } else {
        sc.nk = nk;
        sc.waves.resize(nk);
        for (int w = 0; w < nk; w++) sc.waves[w] = v3(waves + 3 * w);
    }
    bool scalar_us = p.scalar != 0;
    for (int i = 0; i < ns; i++) {
        SphereGeom sg = sphere_derive(p, sc.g, s[i]);
        sc.sg.push_back(sg);
        if (!scalar_us) continue;
        if (p.lut_us) {
            auto* L = new SphereLut();
            L->build(sc.g, s[i], sg, p.lambda);
            sc.lut.push_back(L);
        } else {
            std::vector<cd> A(sg.Nl + 1), B(sg.Nl + 1);
            mie(2 * PI_REF / p.lambda, s[i].a, cd(s[i].n_re, s[i].n_im), sg.Nl, A.data(), B.data());
            sc.A.push_back(A);
            sc.B.push_back(B);
        }
    }
    if (p.lut_uf && !p.plane_wave) sc.uft = uf_table(p, sc.g);
}

cd incident(const Scene& sc, V3 pt) {
    const bs_params& p = sc.p;
    if (!p.scalar && p.lut_uf) return cd(0, 0);  // nfVectorUfLut.cu:7-10 is empty
    if (p.plane_wave) return uf_plane(p, sc.g, pt);
    if (p.lut_uf) return uf_lut(p, sc.g, sc.uft, pt);
    return uf_direct(p, sc.g, pt);
}

cd scattered(Scene& sc, V3 pt) {
    const bs_params& p = sc.p;
    const Geom& g = sc.g;
    cd U(0, 0);
    int ns = (int)sc.s.size();
    if (!p.scalar || ns == 0) return U;  // nearfield.cpp:160-165 (vector: nothing)
    V3 f = v3(p.focus);
    // the reference's weight 1.0f/nk is a single-precision quotient (nfScalarUs.cu:457,
    // nfScalarUpLut.cu:83,89): in its own double-precision build it stays float-rounded
    double scale_amp = (double)(1.0f / (float)sc.nk) * g.sub_amp;
    for (int is = 0; is < ns; is++) {
        const bs_sphere& s = sc.s[is];
        V3 ps{s.x, s.y, s.z};
        V3 r = pt - ps;
        V3 c = ps - f;
        double d = len(r);
        cd sum(0, 0);
        if (p.lut_us) {
            // gpuScalarUpLut, nfScalarUpLut.cu:11-97
            SphereLut& L = *sc.lut[is];
            const SphereGeom& sg = L.sg;
            double di = ((d - sg.r0) / (sg.dmax - sg.r0)) * (sg.dR - 1);
            double ai = ((d - sg.dmin) / (s.a - sg.dmin)) * (sg.aR - 1);
            V3 rn = r * (1.0 / d);
            for (int w = 0; w < sc.nk; w++) {
                V3 kw = sc.waves[w];
                double cth = (d == 0) ? 1.0 : dot(kw, rn);
                if (cth < -1) cth = -1;
                if (cth > 1) cth = 1;
                double ti = (std::acos(cth) / PI_REF) * (sg.thetaR - 1);
                cd phase = std::exp(cd(0, g.kmag * dot(kw, c)));
                cd T;
                if (d < s.a)
                    T = SphereLut::bilerp([&](int i, int j) { return L.Uip(i, j); }, ai, ti, sg.aR, sg.thetaR);
                else
                    T = SphereLut::bilerp([&](int i, int j) { return L.Usp(i, j); }, di, ti, sg.dR, sg.thetaR);
                sum += scale_amp * phase * T;
            }
        } else {
            // optPc_gpuScalarUsp / gpuScalarUsp, nfScalarUs.cu:333-391,447-491
            const int Nl = sc.sg[is].Nl;
            const cd* A = sc.A[is].data();
            const cd* B = sc.B[is].data();
            V3 rn = r * (1.0 / d);
            cd knd = g.kmag * d * cd(s.n_re, s.n_im);
            double kd = g.kmag * d;
            for (int w = 0; w < sc.nk; w++) {
                V3 kw = sc.waves[w];
                double cth = dot(kw, rn);
                cd phase = std::exp(cd(0, g.kmag * dot(kw, c)));
                if (d <= s.a)
                    sum += scale_amp * phase * calc_ui(knd, cth, Nl, A);
                else
                    sum += scale_amp * phase * calc_us(kd, cth, Nl, B);
            }
        }
        U += sum;
    }
    return U;
}

// nfSumUf.cu:6-49: is the point outside every sphere?
bool outside_all(const Scene& sc, V3 pt) {
    for (const auto& s : sc.s) {
        V3 r = pt - V3{s.x, s.y, s.z};
        if (len(r) < s.a) return false;
    }
    return true;
}

void nearfield_rows(Scene& sc, int row0, int row1, int nthreads, cd* U, cd* Uf) {
    const int R = sc.g.R;
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
#endif
    for (long long pix = (long long)row0 * R; pix < (long long)row1 * R; pix++) {
        {
            const int iv = (int)(pix / R), iu = (int)(pix % R);
            double u = (double)iu / R, v = (double)iv / R;
            V3 pt = quad_at(sc.g.nf, u, v);
            cd uf = incident(sc, pt);
            cd us = scattered(sc, pt);
            cd tot;
            if (sc.s.empty())
                tot = uf;  // nfSumUf.cu:59-68 (plain copy)
            else
                tot = us + (outside_all(sc, pt) ? uf : cd(0, 0));
            size_t o = (size_t)(iv - row0) * R + iu;
            if (U) U[o] = tot;
            if (Uf) Uf[o] = uf;
        }
    }
}

// ---------------------------------------------------------------------------
// FFT (double): mixed radix for small prime factors, Bluestein otherwise
// ---------------------------------------------------------------------------
void fft_any(std::vector<cd>& a, int sign);

void fft_rec(const cd* in, cd* out, int n, int stride, int sign, const cd* tw, int twn) {
    // out[k] = sum_j in[j*stride] * exp(sign*2*pi*i*j*k/n); tw has twn entries of
    // exp(sign*2*pi*i*e/twn) and n divides twn.
    if (n == 1) {
        out[0] = in[0];
        return;
    }
    int p = 2;
    while (p * p <= n && n % p) p++;
    if (n % p) p = n;
    int m = n / p;
    for (int r = 0; r < p; r++) fft_rec(in + r * stride, out + r * m, m, stride * p, sign, tw, twn);
    int step = twn / n;
    std::vector<cd> t(p), o(p);
    for (int k = 0; k < m; k++) {
        for (int r = 0; r < p; r++) t[r] = out[r * m + k] * tw[((size_t)r * k * step) % twn];
        for (int q = 0; q < p; q++) {
            cd acc(0, 0);
            for (int r = 0; r < p; r++) acc += t[r] * tw[((size_t)r * q * m * step) % twn];
            o[q] = acc;
        }
        for (int q = 0; q < p; q++) out[q * m + k] = o[q];
    }
}

int largest_prime(int n) {
    int lp = 1;
    for (int p = 2; (long)p * p <= n; p++)
        while (n % p == 0) {
            lp = p;
            n /= p;
        }
    if (n > 1) lp = std::max(lp, n);
    return lp;
}

void fft_smooth(std::vector<cd>& a, int sign) {
    int n = (int)a.size();
    std::vector<cd> tw(n), out(n);
    for (int e = 0; e < n; e++) {
        long double ang = (long double)sign * 2.0L * 3.14159265358979323846264338327950288L * e / n;
        tw[e] = cd((double)std::cos(ang), (double)std::sin(ang));
    }
    fft_rec(a.data(), out.data(), n, 1, sign, tw.data(), n);
    a.swap(out);
}

void fft_any(std::vector<cd>& a, int sign) {
    int n = (int)a.size();
    if (n <= 1) return;
    if (largest_prime(n) <= 31) {
        fft_smooth(a, sign);
        return;
    }
    // Bluestein: chirp z-transform through a power-of-two convolution
    int m = 1;
    while (m < 2 * n - 1) m <<= 1;
    std::vector<cd> w(n), A(m, 0.0), B(m, 0.0);
    for (int k = 0; k < n; k++) {
        long long kk = ((long long)k * k) % (2LL * n);
        long double ang = (long double)sign * 3.14159265358979323846264338327950288L * kk / n;
        w[k] = cd((double)std::cos(ang), (double)std::sin(ang));
    }
    for (int k = 0; k < n; k++) A[k] = a[k] * w[k];
    B[0] = std::conj(w[0]);
    for (int k = 1; k < n; k++) B[k] = B[m - k] = std::conj(w[k]);
    fft_smooth(A, -1);
    fft_smooth(B, -1);
    for (int k = 0; k < m; k++) A[k] *= B[k];
    fft_smooth(A, +1);
    for (int k = 0; k < n; k++) a[k] = A[k] * w[k] / (double)m;
}

void fft2(std::vector<cd>& f, int R, int sign) {
    std::vector<cd> line(R);
    for (int r = 0; r < R; r++) {
        for (int c = 0; c < R; c++) line[c] = f[(size_t)r * R + c];
        fft_any(line, sign);
        for (int c = 0; c < R; c++) f[(size_t)r * R + c] = line[c];
    }
    for (int c = 0; c < R; c++) {
        for (int r = 0; r < R; r++) line[r] = f[(size_t)r * R + c];
        fft_any(line, sign);
        for (int r = 0; r < R; r++) f[(size_t)r * R + c] = line[r];
    }
}

// applyBackpropagation's factor -exp(i kz d) at spectrum bin (iu, iv) of an
// R x R near field (microscope.cu:423-488), in that kernel's arithmetic:
//     float Kx = 2*PI * uR * du;  float dkx = Kx / uR;  kx = (ptype)iu * dkx
//     (or -(ptype)(uR - 1 - iu) * dkx above uR / 2, stored in a float);
//     float k = 2*PI / lambda;  if (kx*kx + ky*ky < k*k) kz = sqrt(k*k - kx*kx - ky*ky)
//     shift = -exp(i (kz * d)), d a float; else 0
// with PI = 3.14159f and du, dv, lambda the double-precision build's ptype.
cd backprop_factor(int iu, int iv, int R, double du, double dv, double lambda, float d) {
    const float two_pi = 2 * (float)PI_REF;
    const float Kx = (float)((double)(two_pi * (float)R) * du);
    const float Ky = (float)((double)(two_pi * (float)R) * dv);
    const float dkx = Kx / (float)R, dky = Ky / (float)R;
    float kx, ky;
    if (iu <= R / 2) kx = (float)((double)iu * dkx);
    else kx = (float)(-(double)(R - 1 - iu) * dkx);
    if (iv <= R / 2) ky = (float)((double)iv * dky);
    else ky = (float)(-(double)(R - 1 - iv) * dky);
    const float kx_sq = kx * kx, ky_sq = ky * ky;
    const float k = (float)((double)two_pi / lambda);
    const float k_sq = k * k;
    if (!(kx_sq + ky_sq < k_sq)) return 0.0;
    const float kz = std::sqrt(k * k - kx * kx - ky * ky);
    const float ph = kz * d;
    return cd(-std::cos((double)ph), -std::sin((double)ph));
}

// applyBandpass / bandpass / getFarField / integrateDetector
// (microscope.cu:495-526, 608-662; fieldslice.cpp:25-94; fieldslice.cu:71-108,319-338)
// bp: propagation distance of applyBackpropagation (microscope.cu:423-488,
// 592-605), or null: the spectrum times backprop_factor (the reference
// transforms back and forth between the two steps, fromAngularSpectrum
// dividing by R^2, which is the identity here).
std::vector<cd> bandpassed(const bs_params& p, const Geom& g, const cd* U, const double* bp = nullptr) {
    const int R = g.R;
    std::vector<cd> f(U, U + (size_t)R * R);
    fft2(f, R, -1);
    double du = 1.0 / len(g.nf.X), dv = 1.0 / len(g.nf.Y);
    double lo = p.objective[0] / p.lambda, hi = p.objective[1] / p.lambda;
    for (int iv = 0; iv < R; iv++) {
        double v = (iv <= R / 2) ? iv * dv : -(double)(R - 1 - iv) * dv;
        for (int iu = 0; iu < R; iu++) {
            double u = (iu <= R / 2) ? iu * du : -(double)(R - 1 - iu) * du;
            if (bp) f[(size_t)iv * R + iu] *= backprop_factor(iu, iv, R, du, dv, p.lambda, (float)*bp);
            double fm = std::sqrt(u * u + v * v);
            if (fm < lo || fm > hi) f[(size_t)iv * R + iu] = 0.0;
        }
    }
    fft2(f, R, +1);
    return f;
}

void detector(const bs_params& p, const Geom& g, const cd* U, double* D, const double* bp = nullptr) {
    const int R = g.R;
    std::vector<cd> f = bandpassed(p, g, U, bp);
    double sc = 1.0 / ((double)R * R);
    int cr = g.crop_res, off = g.crop_off, ss = g.ss, res = g.res;
    for (int iv = 0; iv < res; iv++)
        for (int iu = 0; iu < res; iu++) {
            double I = 0;
            for (int ix = 0; ix < ss; ix++)
                for (int iy = 0; iy < ss; iy++) {
                    int cu = iu * ss + ix, cv = iv * ss + iy;
                    cd val = f[(size_t)(off + cv) * R + (off + cu)] * sc;
                    double m = std::abs(val);
                    I += m * m;
                }
            (void)cr;
            D[(size_t)iv * res + iu] = I / (ss * ss);
        }
}

// ---------------------------------------------------------------------------
// Ring point sources (--interpolate 1, 2, 3).  The reference samples rotated
// images through linearly filtered textures with border addressing; here the
// sample coordinates are formed in single precision as the reference's kernels
// form them (each operation rounded on its own), cosines and sines are double
// values rounded to float, and the bilinear weights are exact (zero outside).
// ---------------------------------------------------------------------------
template <class V>
V bilinear_at(const V* f, int W, int H, float x, float y) {
    const float fx = std::floor(x), fy = std::floor(y);
    const int i0 = (int)fx, j0 = (int)fy;
    const double a = (double)(x - fx), e = (double)(y - fy);
    auto at = [&](int i, int j) -> V { return (i >= 0 && i < W && j >= 0 && j < H) ? f[(size_t)j * W + i] : V(0); };
    return (1 - a) * (1 - e) * at(i0, j0) + a * (1 - e) * at(i0 + 1, j0) + (1 - a) * e * at(i0, j0 + 1) +
           a * e * at(i0 + 1, j0 + 1);
}

// Position of pixel (iu, iv) rotated by (c, s) about (uc, uc):
// uc + (iu - uc) c - (iv - uc) s, uc + (iu - uc) s + (iv - uc) c
// (nfInterpolate.cu:28-29, microscope.cu:101-102).
void rotated_xy(int iu, int iv, float uc, float c, float s, float& x, float& y) {
    const float du = (float)iu - uc, dv = (float)iv - uc;
    x = (uc + du * c) - dv * s;
    y = (uc + du * s) + dv * c;
}

// gpuInterpolateU / gpuInterpolateUf (nfInterpolate.cu:13-66): centre (int)(R/2)
// for U, R/2 for Uf.
void rotate_field(int R, float c, float s, bool int_centre, const cd* src, cd* dst) {
    const float uc = int_centre ? (float)(int)(R / 2.0) : (float)(R / 2.0);
    for (int iv = 0; iv < R; iv++)
        for (int iu = 0; iu < R; iu++) {
            float x, y;
            rotated_xy(iu, iv, uc, c, s, x, y);
            dst[(size_t)iv * R + iu] = bilinear_at(src, R, R, x, y);
        }
}

// InterpolateAndIntegrateUd / Ufd (microscope.cu:89-135): dst += src rotated
// about ((int)(res/2), (int)(res/2)).
void rotate_add_image(int res, float c, float s, const double* src, double* dst) {
    const float uc = (float)(int)(res / 2.0);
    for (int iv = 0; iv < res; iv++)
        for (int iu = 0; iu < res; iu++) {
            float x, y;
            rotated_xy(iu, iv, uc, c, s, x, y);
            dst[(size_t)iv * res + iu] += bilinear_at(src, res, res, x, y);
        }
}

// simRing_Ud / simRing_Ufd (microscope.cu:138-250): for each radius r < L,
// line[r] += the sum of the image at (uc + r cos t_k, uc - r sin t_k),
// t_k = (2 pi / points)(k + 1) formed in double and rounded to float, added in
// the reference's shared-memory tree (steps points/2, points/4, ..., 1; with a
// count that is not a power of two some samples never reach the sum).
void ring_line(int res, int points, int L, const double* img, double* line) {
    const float uc = (float)(int)(res / 2.0);
    std::vector<float> cs(2 * (size_t)points);
    for (int k = 0; k < points; k++) {
        const float t = (float)((2.0 * PI_REF / points) * (k + 1));
        cs[2 * k] = (float)std::cos((double)t);
        cs[2 * k + 1] = (float)std::sin((double)t);
    }
    std::vector<double> sh(points);
    for (int r = 0; r < L; r++) {
        for (int k = 0; k < points; k++) {
            const float x = uc + (float)r * cs[2 * k], y = uc - (float)r * cs[2 * k + 1];
            sh[k] = bilinear_at(img, res, res, x, y);
        }
        for (unsigned step = (unsigned)points / 2; step >= 1; step >>= 1)
            for (unsigned k = 0; k < step; k++) sh[k] += sh[k + step];
        line[r] += sh[0];
    }
}

// InterpolateAndIntegrateUdFromLine / UfdFromLine (microscope.cu:37-85): D at
// distance r = sqrt((iu-uc)^2 + (iv-uc)^2) (single precision) from the centre
// is the line linearly interpolated at r, zero beyond its L entries.
void line_image(int res, int L, const double* line, double* D) {
    const float uc = (float)(int)(res / 2.0);
    for (int iv = 0; iv < res; iv++)
        for (int iu = 0; iu < res; iu++) {
            const float du = (float)iu - uc, dv = (float)iv - uc;
            const float r = std::sqrt(du * du + dv * dv);
            const float fr = std::floor(r);
            const int i0 = (int)fr;
            const double a = (double)(r - fr);
            const double v0 = i0 < L ? line[i0] : 0.0, v1 = i0 + 1 < L ? line[i0 + 1] : 0.0;
            D[(size_t)iv * res + iu] = (1 - a) * v0 + a * v1;
        }
}

// Ring angles of generatePointSources (microscope.cu:1298-1325): t_0 = 2 pi / points
// in float, each next one the float sum of the previous and that step.
std::vector<float> ring_angles(int points) {
    const float step = 2 * (float)PI_REF / (float)points;
    std::vector<float> t(points);
    float th = step;
    for (int i = 0; i < points; i++) {
        t[i] = th;
        th += step;
    }
    return t;
}

// ---------------------------------------------------------------------------
// ENVI
// ---------------------------------------------------------------------------
std::string fmt_g(double v) {
    std::ostringstream os;
    os << v;
    return os.str();
}

std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && s[a] == ' ') a++;
    while (b > a && s[b - 1] == ' ') b--;
    return s.substr(a, b - a);
}

struct EnviHdr {
    std::string description;
    unsigned samples = 0, lines = 0, bands = 0, offset = 0;
    std::string file_type = "ENVI Standard";
    int data_type = 4;
    std::string interleave = "bsq";
    std::string sensor = "Unknown";
    int byte_order = 0;
    double x_start = 0, y_start = 0;
    std::string wl_units = "Unknown";
    std::string zt0 = "Unknown", zt1 = "Unknown";
    double px0 = 1, px1 = 1;
    std::vector<std::string> band_names;
    std::vector<double> wl;
};

std::vector<std::string> split_commas(const std::string& s) {
    std::vector<std::string> out;
    std::string cur;
    std::stringstream ss(s);
    while (std::getline(ss, cur, ',')) out.push_back(trim(cur));
    if (!s.empty() && s.back() == ',') out.push_back("");
    return out;
}

bool envi_load(const std::string& name, EnviHdr& h) {
    std::ifstream in(name);
    if (!in) return false;
    std::string first;
    in >> first;
    if (first != "ENVI") return false;
    std::string line;
    std::getline(in, line);
    while (std::getline(in, line)) {
        size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        std::string key = trim(line.substr(0, eq > 0 ? eq - 1 : 0));
        std::string val = trim(line.substr(eq + 1));
        if (val.find('{') != std::string::npos) {
            std::string acc = val.substr(val.find('{') + 1);
            while (acc.find('}') == std::string::npos && std::getline(in, line)) acc += line;
            acc = trim(acc.substr(0, acc.find('}')));
            if (key == "description") h.description = acc;
            else if (key == "band names") h.band_names = split_commas(acc);
            else if (key == "wavelength") {
                h.wl.clear();
                for (auto& e : split_commas(acc)) h.wl.push_back(std::atof(e.c_str()));
            } else if (key == "pixel size") {
                auto v = split_commas(acc);
                if (v.size() >= 2) {
                    h.px0 = std::atof(v[0].c_str());
                    h.px1 = std::atof(v[1].c_str());
                }
            } else if (key == "z plot titles") {
                auto v = split_commas(acc);
                if (v.size() >= 2) {
                    h.zt0 = v[0];
                    h.zt1 = v[1];
                }
            }
            continue;
        }
        if (key == "samples") h.samples = std::atoi(val.c_str());
        else if (key == "lines") h.lines = std::atoi(val.c_str());
        else if (key == "bands") h.bands = std::atoi(val.c_str());
        else if (key == "header offset") h.offset = std::atoi(val.c_str());
        else if (key == "file type") h.file_type = val;
        else if (key == "data type") h.data_type = std::atoi(val.c_str());
        else if (key == "interleave") h.interleave = val;
        else if (key == "sensor type") h.sensor = val;
        else if (key == "byte order") h.byte_order = std::atoi(val.c_str());
        else if (key == "x start") h.x_start = std::atof(val.c_str());
        else if (key == "y start") h.y_start = std::atof(val.c_str());
        else if (key == "wavelength units") h.wl_units = val;
    }
    return true;
}

bool envi_save(const std::string& name, const EnviHdr& h) {
    std::ofstream o(name);
    if (!o) return false;
    o << "ENVI\n";
    o << "description = {\n";
    o << "  " << h.description << "}\n";
    o << "samples = " << h.samples << "\n";
    o << "lines = " << h.lines << "\n";
    o << "bands = " << h.bands << "\n";
    o << "header offset = " << h.offset << "\n";
    o << "file type = " << h.file_type << "\n";
    o << "data type = " << h.data_type << "\n";
    o << "interleave = " << h.interleave << "\n";
    o << "sensor type = " << h.sensor << "\n";
    o << "byte order = " << h.byte_order << "\n";
    o << "x start = " << fmt_g(h.x_start) << "\n";
    o << "y start = " << fmt_g(h.y_start) << "\n";
    o << "wavelength units = " << h.wl_units << "\n";
    o << "z plot titles = {" << h.zt0 << ", " << h.zt1 << "}\n";
    o << "pixel size = {" << fmt_g(h.px0) << ", " << fmt_g(h.px1) << ", units=Meters}\n";
    if (!h.band_names.empty()) {
        o << "band names = {\n";
        for (size_t i = 0; i < h.band_names.size(); i++) {
            o << h.band_names[i];
            if (i + 1 < h.band_names.size()) o << ", ";
        }
        o << "}\n";
    }
    o << "wavelength = {\n";
    for (size_t i = 0; i + 1 < h.wl.size(); i++) o << fmt_g(h.wl[i]) << ", ";
    if (!h.wl.empty()) o << fmt_g(h.wl.back());
    o << "}\n";
    return (bool)o;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int bso_derive(const bs_params* p, bso_geom* out) {
    Geom g = derive(*p);
    out->R = g.R;
    out->det_res = g.res;
    out->crop_res = g.crop_res;
    out->crop_off = g.crop_off;
    const V3* v[3] = {&g.nf.A, &g.nf.X, &g.nf.Y};
    double* dst[3] = {out->A, out->X, out->Y};
    for (int i = 0; i < 3; i++) {
        dst[i][0] = v[i]->x;
        dst[i][1] = v[i]->y;
        dst[i][2] = v[i]->z;
    }
    out->kmag = g.kmag;
    out->sub_amp = g.sub_amp;
    out->cos_alpha = g.cos_a;
    out->cos_beta = g.cos_b;
    return 0;
}

int bso_sphere_derive(const bs_params* p, const bs_sphere* s, bso_sphere_geom* out) {
    Geom g = derive(*p);
    SphereGeom sg = sphere_derive(*p, g, *s);
    out->Nl = sg.Nl;
    out->aR = sg.aR;
    out->dR = sg.dR;
    out->thetaR = sg.thetaR;
    out->d_min = sg.dmin;
    out->d_max = sg.dmax;
    return 0;
}

int bso_calc_nl(double a, double lambda) { return calc_nl(a, lambda); }

int bso_sbessel_real(int N, double x, double* j, double* y) {
    sph_real(N, x, j, y);
    return 0;
}

int bso_sbessel_complex(int N, double zr, double zi, int typo, double* j, double* y, double* jp, double* yp) {
    std::vector<cd> a(N + 1), b(N + 1), c(N + 1), d(N + 1);
    sph_complex(N, cd(zr, zi), typo != 0, a.data(), b.data(), c.data(), d.data());
    for (int l = 0; l <= N; l++) {
        j[2 * l] = a[l].real(); j[2 * l + 1] = a[l].imag();
        y[2 * l] = b[l].real(); y[2 * l + 1] = b[l].imag();
        jp[2 * l] = c[l].real(); jp[2 * l + 1] = c[l].imag();
        yp[2 * l] = d[l].real(); yp[2 * l + 1] = d[l].imag();
    }
    return 0;
}

int bso_mie(double k, double a, double n_re, double n_im, int Nl, double* A, double* B) {
    std::vector<cd> a_(Nl + 1), b_(Nl + 1);
    mie(k, a, cd(n_re, n_im), Nl, a_.data(), b_.data());
    for (int l = 0; l <= Nl; l++) {
        A[2 * l] = a_[l].real(); A[2 * l + 1] = a_[l].imag();
        B[2 * l] = b_[l].real(); B[2 * l + 1] = b_[l].imag();
    }
    return 0;
}

int bso_glibc_rand(unsigned seed, int n, int* out) {
    GlibcRand g(seed);
    for (int i = 0; i < n; i++) out[i] = g.next();
    return 0;
}

// mcSampleNA (montecarlo.cpp:9-71) after srand(NULL) (nearfield.cpp:102);
// every operation in single precision, in the reference's order.
int bso_mc_sample(int nk, const double* kd, double na_in, double na_out, double* out) {
    GlibcRand rng(0);
    volatile float kx = (float)kd[0], ky = (float)kd[1], kz = (float)kd[2];
    float M[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};  // column-major M[c*3+r]
    volatile float cos_angle = 0.0f;
    cos_angle = cos_angle + kx * 0.0f;
    cos_angle = cos_angle + ky * 0.0f;
    cos_angle = cos_angle + kz * 1.0f;
    if (cos_angle != 1.0f) {
        volatile float ax = 0.0f * kz - 1.0f * ky, ay = 1.0f * kx - 0.0f * kz, az = 0.0f * ky - 0.0f * kx;
        volatile float sq = 0.0f;
        sq = sq + ax * ax;
        sq = sq + ay * ay;
        sq = sq + az * az;
        volatile float l = std::sqrt((float)sq);
        ax = ax / l;
        ay = ay / l;
        az = az / l;
        volatile float angle = std::acos((float)cos_angle);
        volatile float w = (float)std::cos((double)angle / 2.0);
        volatile float s2 = (float)std::sin((double)angle / 2.0);
        volatile float x = ax * s2, y = ay * s2, z = az * s2;
        volatile float x2 = x + x, y2 = y + y, z2 = z + z;
        volatile float xx = x * x2, xy = x * y2, xz = x * z2;
        volatile float yy = y * y2, yz = y * z2, zz = z * z2;
        volatile float wx = w * x2, wy = w * y2, wz = w * z2;
        auto set = [&](int r, int c, float v) { M[c * 3 + r] = v; };
        set(0, 0, 1.0f - (yy + zz));
        set(0, 1, xy - wz);
        set(0, 2, xz + wy);
        set(1, 0, xy + wz);
        set(1, 1, 1.0f - (xx + zz));
        set(1, 2, yz - wx);
        set(2, 0, xz - wy);
        set(2, 1, yz + wx);
        set(2, 2, 1.0f - (xx + yy));
    }
    volatile float inPhi = std::asin((float)na_in), outPhi = std::asin((float)na_out);
    volatile float inZ = std::cos((float)inPhi), outZ = std::cos((float)outPhi);
    volatile float rangeZ = inZ - outZ;
    const float RM = (float)2147483647;
    const float PIf = 3.14159f;
    for (int i = 0; i < nk; i++) {
        volatile float q = (float)rng.next() / RM;
        volatile float z = q * rangeZ;
        z = z + outZ;
        volatile float q2 = (float)rng.next() / RM;
        volatile float theta = q2 * 2.0f;
        theta = theta * PIf;
        volatile float phi = std::acos((float)z);
        volatile float c0 = 1.0f * std::cos((float)theta);
        c0 = c0 * std::sin((float)phi);
        volatile float c1 = 1.0f * std::sin((float)theta);
        c1 = c1 * std::sin((float)phi);
        volatile float c2 = 1.0f * std::cos((float)phi);
        float v[3] = {c0, c1, c2};
        for (int r = 0; r < 3; r++) {
            volatile float acc = 0.0f;
            for (int c = 0; c < 3; c++) {
                volatile float t = M[c * 3 + r] * v[c];
                acc = acc + t;
            }
            out[3 * i + r] = acc;
        }
    }
    return 0;
}

int bso_sphere_luts(const bs_params* p, const bs_sphere* s, double* usp, double* uip) {
    Geom g = derive(*p);
    SphereGeom sg = sphere_derive(*p, g, *s);
    SphereLut L;
    L.build(g, *s, sg, p->lambda);
    for (int ir = 0; ir < sg.dR; ir++)
        for (int it = 0; it < sg.thetaR; it++) {
            cd v = L.Usp(ir, it);
            size_t o = ((size_t)ir * sg.thetaR + it) * 2;
            usp[o] = v.real();
            usp[o + 1] = v.imag();
        }
    for (int ia = 0; ia < sg.aR; ia++)
        for (int it = 0; it < sg.thetaR; it++) {
            cd v = L.Uip(ia, it);
            size_t o = ((size_t)ia * sg.thetaR + it) * 2;
            uip[o] = v.real();
            uip[o + 1] = v.imag();
        }
    return 0;
}

int bso_uf_table(const bs_params* p, double* table, double* dmin, double* dmax) {
    Geom g = derive(*p);
    UfTable t = uf_table(*p, g);
    std::memcpy(table, t.j.data(), t.j.size() * sizeof(double));
    *dmin = t.dmin;
    *dmax = t.dmax;
    return 0;
}

int bso_nearfield_rows(const bs_params* p, const bs_sphere* s, int ns, const double* waves, int nk,
                       int nthreads, int row0, int row1, double* U) {
    Scene sc;
    scene_init(sc, *p, s, ns, waves, nk);
    nearfield_rows(sc, row0, row1, nthreads, reinterpret_cast<cd*>(U), nullptr);
    return 0;
}

// Timed band for CPU baselines: times[0] = scene set-up (Mie coefficients and
// the Bessel/Hankel rows, serial per sphere as the reference builds them on the
// host), times[1] = every LUT entry of every sphere (OpenMP over entries),
// times[2] = the near field of rows [row0, row1) with the tables complete.  A
// whole slice then costs times[0] + times[1] + times[2] * R / (row1 - row0).
int bso_nearfield_rows_timed(const bs_params* p, const bs_sphere* s, int ns, const double* waves, int nk,
                             int nthreads, int row0, int row1, double* U, double* times) {
    auto now = [] { return std::chrono::steady_clock::now(); };
    auto sec = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
        return std::chrono::duration<double>(b - a).count();
    };
    auto t0 = now();
    Scene sc;
    scene_init(sc, *p, s, ns, waves, nk);
    auto t1 = now();
    for (SphereLut* L : sc.lut) {
        const long long nu = (long long)L->sg.dR * L->sg.thetaR, ni = (long long)L->sg.aR * L->sg.thetaR;
#ifdef _OPENMP
        int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
#endif
        for (long long e = 0; e < nu + ni; e++) {
            if (e < nu)
                L->Usp((int)(e / L->sg.thetaR), (int)(e % L->sg.thetaR));
            else
                L->Uip((int)((e - nu) / L->sg.thetaR), (int)((e - nu) % L->sg.thetaR));
        }
    }
    auto t2 = now();
    nearfield_rows(sc, row0, row1, nthreads, reinterpret_cast<cd*>(U), nullptr);
    auto t3 = now();
    times[0] = sec(t0, t1);
    times[1] = sec(t1, t2);
    times[2] = sec(t2, t3);
    return 0;
}

// the far field Ud: band-passed field on the crop, scaled by 1/R^2 (getFarField, microscope.cu:641-655)
int bso_far_field(const bs_params* p, const double* U, double* out) {
    Geom g = derive(*p);
    std::vector<cd> f = bandpassed(*p, g, reinterpret_cast<const cd*>(U));
    const double sc = 1.0 / ((double)g.R * g.R);
    for (int v = 0; v < g.crop_res; v++)
        for (int u = 0; u < g.crop_res; u++) {
            cd val = f[(size_t)(g.crop_off + v) * g.R + (g.crop_off + u)] * sc;
            out[2 * ((size_t)v * g.crop_res + u)] = val.real();
            out[2 * ((size_t)v * g.crop_res + u) + 1] = val.imag();
        }
    return 0;
}

int bso_detector(const bs_params* p, const double* U, const double* Uf, double* D, double* Di) {
    Geom g = derive(*p);
    if (D) detector(*p, g, reinterpret_cast<const cd*>(U), D);
    if (Di) detector(*p, g, reinterpret_cast<const cd*>(Uf), Di);
    return 0;
}

// The detector with applyBackpropagation over distance d on U (Uf is not propagated).
int bso_detector_bp(const bs_params* p, const double* U, const double* Uf, double d, double* D, double* Di) {
    Geom g = derive(*p);
    if (D) detector(*p, g, reinterpret_cast<const cd*>(U), D, &d);
    if (Di) detector(*p, g, reinterpret_cast<const cd*>(Uf), Di);
    return 0;
}

int bso_simulate(const bs_params* p, const bs_sphere* s, int ns, const double* waves, int nk, int nthreads,
                 double* U, double* Uf, double* D, double* Di) {
    Scene sc;
    scene_init(sc, *p, s, ns, waves, nk);
    const int R = sc.g.R;
    std::vector<cd> u((size_t)R * R), uf((size_t)R * R);
    nearfield_rows(sc, 0, R, nthreads, u.data(), uf.data());
    if (U) std::memcpy(U, u.data(), u.size() * sizeof(cd));
    if (Uf) std::memcpy(Uf, uf.data(), uf.size() * sizeof(cd));
    if (D) detector(*p, sc.g, u.data(), D);
    if (Di) detector(*p, sc.g, uf.data(), Di);
    return 0;
}

// The reference's ring drivers: mode 3 SimulateExtendedSourceWithInterpolation
// (microscope.cu:1189-1253), mode 1 SimulateExtendedSourceInterpAtDetector
// (:1004-1093), mode 2 SimulateExtendedSourceInterpLineAtDetector (:1097-1183).
int bso_simulate_rings(const bs_params* p, const bs_sphere* s, int ns, const double* waves, int nk, int nthreads,
                       int mode, int points, int rings, double* D, double* Di) {
    if (points < 1 || rings < 1 || (mode != 1 && mode != 2 && mode != 3)) return 1;
    const Geom g = derive(*p);
    const int R = g.R, res = g.res;
    const size_t nf = (size_t)R * R, ni = (size_t)res * res;
    std::vector<cd> u(nf), uf(nf), ur(nf), ufr(nf);
    std::vector<double> d(ni), di(ni), t(ni);
    std::fill(D, D + ni, 0.0);
    std::fill(Di, Di + ni, 0.0);
    auto source = [&](bs_params q) {
        bso_simulate(&q, s, ns, waves, nk, nthreads, reinterpret_cast<double*>(u.data()),
                     reinterpret_cast<double*>(uf.data()), d.data(), di.data());
    };
    if (mode == 2) {
        // every source's image feeds the radial line; the detector is the line
        std::vector<double> line(rings, 0.0), linei(rings, 0.0);
        bs_params q = *p;
        q.amplitude = 1;
        for (int j = 0; j < rings; j++) {
            if (j > 0) {
                q.focus[0] = j;
                q.focus[1] = 0;
                q.focus[2] = 0;
            }
            source(q);
            ring_line(res, points, rings, d.data(), line.data());
            ring_line(res, points, rings, di.data(), linei.data());
        }
        line_image(res, rings, line.data(), D);
        line_image(res, rings, linei.data(), Di);
        return 0;
    }
    source(*p);
    for (size_t i = 0; i < ni; i++) {
        D[i] += d[i];
        Di[i] += di[i];
    }
    for (int ring = 1; ring < rings; ring++) {
        const std::vector<float> th = ring_angles(points);
        bs_params q = *p;
        q.focus[0] = (float)std::cos((double)th[0]) * (float)ring;
        q.focus[1] = (float)std::sin((double)th[0]) * (float)ring;
        q.focus[2] = 0;
        q.amplitude = 1;
        source(q);
        for (size_t i = 0; i < ni; i++) {
            D[i] += d[i];
            Di[i] += di[i];
        }
        for (int k = 1; k < points; k++) {
            const float c = (float)std::cos((double)th[k]), sn = (float)std::sin((double)th[k]);
            if (mode == 3) {
                rotate_field(R, c, sn, true, u.data(), ur.data());
                rotate_field(R, c, sn, false, uf.data(), ufr.data());
                detector(*p, g, ur.data(), t.data());
                for (size_t i = 0; i < ni; i++) D[i] += t[i];
                detector(*p, g, ufr.data(), t.data());
                for (size_t i = 0; i < ni; i++) Di[i] += t[i];
            } else {
                rotate_add_image(res, c, sn, d.data(), D);
                rotate_add_image(res, c, sn, di.data(), Di);
            }
        }
    }
    return 0;
}

// material::computeN (rts/optics/material.h:257-432) from the resampled kappa:
// chi2 = -alpha n0 / k with float k = 2 PI / lambda and float alpha = kappa 2k,
// zero-padded to M = pf N points, forward FFT, x i for 0 < f < M/2.0, x -i for
// f >= M/2.0, DC zeroed, inverse FFT / M, n = Re chi1 / (2 n0) + n0.
int bso_kk_transform(int N, int pf, double n0, const double* lambdas, const double* kappas, double* n_out) {
    const int M = N * pf;
    std::vector<cd> a(M, cd(0, 0));
    for (int i = 0; i < N; i++) {
        const float k = (float)(2 * (float)PI_REF / lambdas[i]);
        const float alpha = (float)(kappas[i] * (double)(2 * k));
        a[i] = cd(-(double)alpha * (n0 / (double)k), 0);
    }
    fft_any(a, -1);
    for (int f = 0; f < M; f++) {
        if (f == 0) a[f] = 0;
        else if (f < M / 2.0) a[f] *= cd(0, 1);
        else a[f] *= cd(0, -1);
    }
    fft_any(a, +1);
    for (int i = 0; i < N; i++) n_out[i] = (a[i].real() / M) / (2 * n0) + n0;
    return 0;
}

int bso_fft(int n, int sign, double* data) {
    std::vector<cd> a(n);
    for (int i = 0; i < n; i++) a[i] = cd(data[2 * i], data[2 * i + 1]);
    fft_any(a, sign);
    for (int i = 0; i < n; i++) {
        data[2 * i] = a[i].real();
        data[2 * i + 1] = a[i].imag();
    }
    return 0;
}

// scalarslice::toEnvi (scalarslice.cu:146-166) + EnviFile (rts/envi/envi.h)
int bso_envi_add_band(const char* path, const float* band, int samples, int lines, double wavelength, int append) {
    std::string data(path), hdr = data + ".hdr";
    EnviHdr h;
    bool locked = false;
    if (append) {
        envi_load(hdr, h);
        FILE* t = std::fopen(path, "rb");
        if (t) {
            std::fseek(t, 0, SEEK_END);
            locked = std::ftell(t) > 0;
            std::fclose(t);
        }
    }
    if (locked && (h.lines != (unsigned)lines || h.samples != (unsigned)samples)) return 1;
    FILE* f = std::fopen(path, append ? "ab" : "wb");
    if (!f) return 2;
    h.bands++;
    h.samples = samples;
    h.lines = lines;
    h.wl.push_back(wavelength);
    std::fwrite(band, sizeof(float), (size_t)samples * lines, f);
    std::fclose(f);
    return envi_save(hdr, h) ? 0 : 3;
}

}  // extern "C"
