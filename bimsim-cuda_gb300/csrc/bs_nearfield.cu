// bs_nearfield.cu -- near-field kernels: incident field Uf, Mie coefficients,
// per-sphere lookup tables, and the scattered field Us summed over spheres
// and Monte Carlo plane waves, with the Uf + Us assembly of nfSumUf.cu fused
// into the epilogue.
#include <cuda_runtime.h>

#include <climits>

#include "bs_kernels.h"
#include "bs_math.cuh"

namespace bs {

// Geometry that feeds a discrete decision (inside/outside a sphere, d == 0,
// d < 1e-6) is rounded operation by operation in the order of the host
// restatement, with no fused multiply-add, so the GPU and the double
// precision reference agree on every boundary pixel.
__device__ __forceinline__ void pixel_pos(const Scene& sc, int iu, int iv, double p[3]) {
    // quad::operator()(u, v) = (A + X u) + Y v with u = iu / R (nfScalarUf.cu:66-71)
    double u = __ddiv_rn((double)iu, (double)sc.R), v = __ddiv_rn((double)iv, (double)sc.R);
#pragma unroll
    for (int c = 0; c < 3; c++) p[c] = __dadd_rn(__dadd_rn(sc.A[c], __dmul_rn(sc.X[c], u)), __dmul_rn(sc.Y[c], v));
}

// |p - c| as sqrt((x*x + y*y) + z*z), each operation rounded separately
__device__ __forceinline__ double dist_exact(const double p[3], const double c[3], double r[3]) {
    r[0] = __dsub_rn(p[0], c[0]);
    r[1] = __dsub_rn(p[1], c[1]);
    r[2] = __dsub_rn(p[2], c[2]);
    double s = __dadd_rn(__dadd_rn(__dmul_rn(r[0], r[0]), __dmul_rn(r[1], r[1])), __dmul_rn(r[2], r[2]));
    return __dsqrt_rn(s);
}

// ---------------------------------------------------------------------------
// Incident field (double precision; stored as T)
// ---------------------------------------------------------------------------
// gpuScalarUf, nfScalarUf.cu:46-175: Debye-focused field as a Legendre series
// over l = 0..m with the clamped upward j_l recurrence.
// w[l] = (P_{l+1} - P_{l-1})(cos a) - (P_{l+1} - P_{l-1})(cos b) of the condenser
// aperture does not depend on the pixel: the host computes it once per run.
__device__ zd uf_direct(const Scene& sc, const double* __restrict__ w, const double p[3]) {
    double r[3];
    double d = dist_exact(p, sc.focus, r);
    if (d < EPS_FLOAT) return mk(sc.amp * 2 * PI_REF * (sc.cos_a - sc.cos_b), 0.0);
    double inv = 1.0 / d;
    double cth = sc.kdir[0] * (r[0] * inv) + sc.kdir[1] * (r[1] * inv) + sc.kdir[2] * (r[2] * inv);
    double kd = sc.kmag * d;
    double s, c;
    sincos(kd, &s, &c);
    double j0 = s / kd, j1 = j0 / kd - c / kd;
    double P0 = 1, P1 = cth;
    zd sum = mk(0.0, 0.0), il = mk(1.0, 0.0);
    for (int l = 0; l <= sc.m; l++) {
        double jl, Pl;
        if (l == 0) {
            jl = j0;
            Pl = P0;
        } else if (l == 1) {
            jl = j1;
            Pl = P1;
        } else {
            sbesselj_step(l, kd, j0, j1);
            legendre_step(l, cth, P0, P1);
            jl = j1;
            Pl = P1;
        }
        sum = sum + il * (jl * Pl * w[l]);
        il = il * mk(0.0, 1.0);
    }
    return sum * (2.0 * PI_REF * sc.amp);
}

// gpuScalarUfLut, nfScalarUfLut.cu:11-123: j_l(k d) read from the table with
// linear filtering along d (texture y) and exact order (texture x = l + 0.5).
__device__ zd uf_lut(const Scene& sc, const double* __restrict__ tab, const double* __restrict__ w,
                     const double p[3]) {
    double r[3];
    double d = dist_exact(p, sc.focus, r);
    if (d == 0) return mk(sc.amp * 2 * PI_REF * (sc.cos_a - sc.cos_b), 0.0);
    double inv = 1.0 / d;
    double cth = sc.kdir[0] * (r[0] * inv) + sc.kdir[1] * (r[1] * inv) + sc.kdir[2] * (r[2] * inv);
    int L = sc.m + 1;
    double y = ((d - sc.uf_dmin) / (sc.uf_dmax - sc.uf_dmin)) * (sc.uf_dR - 1);
    y = fmin(fmax(y, 0.0), (double)(sc.uf_dR - 1));
    int i0 = (int)floor(y);
    double be = y - i0;
    int i1 = min(i0 + 1, sc.uf_dR - 1);
    const double* t0 = tab + (size_t)i0 * L;
    const double* t1 = tab + (size_t)i1 * L;
    double P0 = 1, P1 = cth;
    zd sum = mk(0.0, 0.0), il = mk(1.0, 0.0);
    for (int l = 0; l <= sc.m; l++) {
        double jl = (1 - be) * t0[l] + be * t1[l];
        double Pl;
        if (l == 0) {
            Pl = P0;
        } else {
            if (l > 1) legendre_step(l, cth, P0, P1);
            Pl = P1;
        }
        sum = sum + il * (jl * Pl * w[l]);
        il = il * mk(0.0, 1.0);
    }
    return sum * (2.0 * PI_REF * sc.amp);
}

template <class T>
__global__ void uf_kernel(Scene sc, const double* __restrict__ tab, const double* __restrict__ w,
                          cpx<T>* __restrict__ Uf) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= sc.R * sc.R) return;
    double p[3];
    pixel_pos(sc, idx % sc.R, idx / sc.R, p);
    zd v;
    if (!sc.scalar && sc.lut_uf) {
        v = mk(0.0, 0.0);  // nfVectorUfLut.cu:7-10 is empty
    } else if (sc.plane_wave) {
        // gpuScalarUfp, nfScalarUf.cu:9-44
        double kr = sc.kmag * (sc.kdir[0] * (p[0] - sc.focus[0]) + sc.kdir[1] * (p[1] - sc.focus[1]) +
                               sc.kdir[2] * (p[2] - sc.focus[2]));
        double s, c;
        sincos(kr, &s, &c);
        v = mk(c * sc.amp, s * sc.amp);
    } else if (sc.lut_uf) {
        v = uf_lut(sc, tab, w, p);
    } else {
        v = uf_direct(sc, w, p);
    }
    Uf[idx] = mk((T)v.re, (T)v.im);
}

// nearfieldStruct::calcBesselLut (nearfield.cpp:222-283): j_l(k d) for
// d in [dmin, dmax], NaN/Inf replaced by 0 (1 for l = 0 at k d = 0).
__global__ void uf_table_kernel(Scene sc, double* __restrict__ tab, double* __restrict__ scratch) {
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= sc.uf_dR) return;
    int L = sc.m + 1;
    double dr = (sc.uf_dmax - sc.uf_dmin) / (sc.uf_dR - 1);
    double d = id * dr + sc.uf_dmin;
    double kd = sc.kmag * d;
    double* j = tab + (size_t)id * L;
    double* y = scratch + (size_t)id * L;
    sph_real(sc.m, kd, j, y, 1);
    for (int l = 0; l < L; l++) {
        double v = j[l];
        if (isnan(v) || isinf(v)) j[l] = (kd == 0 && l == 0) ? 1.0 : 0.0;
    }
}

// ---------------------------------------------------------------------------
// Mie coefficients (sphere::calcCoeff, sphere.cpp:21-97), one thread per sphere
// ---------------------------------------------------------------------------
__global__ void mie_kernel(const Sphere* __restrict__ sph, int ns, double k, zd* __restrict__ scratch, int lstride,
                           zd* __restrict__ A, zd* __restrict__ B) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ns) return;
    Sphere S = sph[s];
    int N = S.Nl;
    zd* ja = scratch + (size_t)s * 6 * lstride;
    zd* ya = ja + lstride;
    zd* jpa = ya + lstride;
    zd* ypa = jpa + lstride;
    zd* jn = ypa + lstride;
    zd* jpn = jn + lstride;
    zd n = mk(S.n_re, S.n_im);
    zd ka = mk(k * S.a, 0.0);
    zd kna = (n * k) * S.a;
    sph_complex(N, ka, true, ja, ya, jpa, ypa);
    sph_complex(N, kna, true, jn, nullptr, jpn, nullptr);
    for (int l = 0; l <= N; l++) {
        zd h = mk(ja[l].re - ya[l].im, ja[l].im + ya[l].re);      // j + i y
        zd hp = mk(jpa[l].re - ypa[l].im, jpa[l].im + ypa[l].re);
        zd an = ja[l] * hp - jpa[l] * h;
        zd bn = jn[l] * hp - (h * jpn[l]) * n;
        zd cn = (ja[l] * jpn[l]) * n - jn[l] * jpa[l];
        zd f = mk(2.0 * l + 1.0, 0.0) * ipow(l);
        A[S.coef_off + l] = f * (an / bn);
        B[S.coef_off + l] = f * (cn / bn);
    }
}

// Per-row order coefficients of the spheres [s0, s0 + n) in one launch:
//   rows [0, dR):  C_l(r) = B_l (j_l + i y_l)(k r),  r in [r0, dmax]  (sphere.cpp:154-203)
//   rows [dR, dR+aR): D_l(r) = A_l j_l(k n r),       r in [0, a]      (sphere.cpp:99-152)
// Thread g takes global row g; starts[i] / starts[n + 1 + i] are sphere i's
// first global row and its first coefficient in tab (rows of Nl + 1
// coefficients; starts[n], the total row count, bounds the grid).  The scratch
// holds 2 (Nl + 1) doubles per row.
__global__ void coef_rows_batch_kernel(const Sphere* __restrict__ sph, int s0, int n,
                                       const long long* __restrict__ starts, double k, const zd* __restrict__ A,
                                       const zd* __restrict__ B, zd* __restrict__ tab,
                                       double* __restrict__ scratch) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= starts[n]) return;
    int lo = 0, hi = n - 1;  // last sphere whose first row is <= g
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (starts[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    const Sphere& S = sph[s0 + lo];
    const int row = (int)(g - starts[lo]);
    const int L = S.Nl + 1;
    const long long c0 = starts[n + 1 + lo] + (long long)row * L;
    zd* out = tab + c0;
    double* sj = scratch + 2 * c0;
    if (row < S.dR) {
        double dr = (S.dmax - S.r0) / (S.dR - 1);
        double r = row * dr + S.r0;
        sph_real(S.Nl, k * r, sj, sj + L, 1);
        for (int l = 0; l < L; l++) out[l] = B[S.coef_off + l] * mk(sj[l], sj[L + l]);
    } else {
        int ia = row - S.dR;
        if (ia == 0) {
            for (int l = 0; l < L; l++) out[l] = (l == 0) ? A[S.coef_off] * mk(1.0, 0.0) : A[S.coef_off + l] * mk(0.0, 0.0);
            return;
        }
        double da = S.a / (S.aR - 1);
        double r = ia * da;
        zd knr = (mk(S.n_re, S.n_im) * k) * r;
        sph_complex(S.Nl, knr, true, out, nullptr, nullptr, nullptr);
        for (int l = 0; l < L; l++) out[l] = A[S.coef_off + l] * out[l];
    }
}

// P_l(cos theta_t), theta_t = t * dtheta (sphere.cu:16-21).  The reference's step
// (PI) / (thetaR - 1) divides the float literal PI by an int: a single-precision
// quotient in every build, kept here.
__global__ void legendre_table_kernel(int thetaR, int Lmax, double* __restrict__ P) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= thetaR) return;
    double dtheta = (double)__fdiv_rn(3.14159f, (float)(thetaR - 1));
    double x = cos(dtheta * t);
    double* row = P + (size_t)t * Lmax;
    double P0 = 1, P1 = x;
    row[0] = P0;
    if (Lmax > 1) row[1] = P1;
    for (int l = 2; l < Lmax; l++) {
        legendre_step(l, x, P0, P1);
        row[l] = P1;
    }
}

// ---------------------------------------------------------------------------
// LUT build: T(r, t) = sum_l coef_l(r) P_l(cos theta_t) (gpuScalarUsp /
// gpuScalarUip, sphere.cu:4-99), then stored as bilinear patches
//     {T00, T10 - T00, T01 - T00, T11 - T10 - T01 + T00}
// at (r, t), with r+1 and t+1 clamped, so that one 32-byte (float) or 64-byte
// (double) load gives a whole bilinear cell.
// ---------------------------------------------------------------------------
constexpr int LB_TR = 8, LB_TT = 32;

template <class T>
__global__ void __launch_bounds__(256) lut_build_kernel(const zd* __restrict__ tab, int rows, int L,
                                                        const double* __restrict__ P, int Pstride, int thetaR,
                                                        Patch<T>* __restrict__ out) {
    __shared__ zd sv[LB_TR + 1][LB_TT + 1];
    int r0 = blockIdx.y * LB_TR, t0 = blockIdx.x * LB_TT;
    for (int e = threadIdx.x; e < (LB_TR + 1) * (LB_TT + 1); e += blockDim.x) {
        int i = e / (LB_TT + 1), j = e % (LB_TT + 1);
        int r = min(r0 + i, rows - 1), t = min(t0 + j, thetaR - 1);
        const zd* c = tab + (size_t)r * L;
        const double* pl = P + (size_t)t * Pstride;
        zd acc = mk(0.0, 0.0);
        for (int l = 0; l < L; l++) acc = acc + c[l] * pl[l];
        sv[i][j] = acc;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < LB_TR * LB_TT; e += blockDim.x) {
        int i = e / LB_TT, j = e % LB_TT;
        int r = r0 + i, t = t0 + j;
        if (r >= rows || t >= thetaR) continue;
        zd a = sv[i][j], b = sv[i + 1][j], c = sv[i][j + 1], d = sv[i + 1][j + 1];
        Patch<T> pt;
        pt.v[0] = (T)a.re;
        pt.v[1] = (T)a.im;
        pt.v[2] = (T)(b.re - a.re);
        pt.v[3] = (T)(b.im - a.im);
        pt.v[4] = (T)(c.re - a.re);
        pt.v[5] = (T)(c.im - a.im);
        pt.v[6] = (T)(d.re - b.re - c.re + a.re);
        pt.v[7] = (T)(d.im - b.im - c.im + a.im);
        out[(size_t)r * thetaR + t] = pt;
    }
}

// Per (sphere, wave): (subA / nk) exp(i k k_w . (p_s - f)) (nfScalarUpLut.cu:71,84,90)
template <class T>
__global__ void phase_kernel(Scene sc, const Sphere* __restrict__ sph, const double* __restrict__ waves,
                             cpx<T>* __restrict__ ph, float4* __restrict__ kw4) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < sc.nk && kw4) {
        kw4[idx] = make_float4((float)waves[3 * idx], (float)waves[3 * idx + 1], (float)waves[3 * idx + 2], 0.f);
    }
    if (idx >= sc.ns * sc.nk) return;
    int s = idx / sc.nk, w = idx % sc.nk;
    const double* k = waves + 3 * w;
    double c0 = sph[s].p[0] - sc.focus[0], c1 = sph[s].p[1] - sc.focus[1], c2 = sph[s].p[2] - sc.focus[2];
    double arg = sc.kmag * (k[0] * c0 + k[1] * c1 + k[2] * c2);
    double sn, cs;
    sincos(arg, &sn, &cs);
    ph[idx] = mk((T)(sc.wave_amp * cs), (T)(sc.wave_amp * sn));
}

// ---------------------------------------------------------------------------
// Scattered field from the LUTs (gpuScalarUpLut, nfScalarUpLut.cu:11-97),
// all spheres of [s0, s1) in one launch, then Uf added where the pixel is
// outside every sphere (nfSumUf.cu:6-49).
// ---------------------------------------------------------------------------
struct TableSel {
    int64_t off;
    int rows;
    double x;  // fractional row index
};

__device__ __forceinline__ TableSel select_table(const Sphere& S, double d) {
    TableSel t;
    if (d < S.a) {  // internal field, ai = (d - dmin)/(a - dmin) (aR - 1)  (nfScalarUpLut.cu:54)
        t.off = S.uip_off;
        t.rows = S.aR;
        t.x = ((d - S.dmin) / (S.a - S.dmin)) * (S.aR - 1);
    } else {        // scattered field, di = (d - r0)/(dmax - r0) (dR - 1)  (nfScalarUpLut.cu:53)
        t.off = S.usp_off;
        t.rows = S.dR;
        t.x = ((d - S.r0) / (S.dmax - S.r0)) * (S.dR - 1);
    }
    // unnormalised texture coordinates with clamp addressing = clamped index
    t.x = fmin(fmax(t.x, 0.0), (double)(t.rows - 1));
    return t;
}

// select_table with the per-sphere scales (rows - 1) / (range) of the host in
// place of the division: the index may differ in its last bit, which moves a
// sample across a row boundary only where the bilinear value is continuous.
__device__ __forceinline__ TableSel select_table_scaled(const Sphere& S, double d) {
    TableSel t;
    if (d < S.a) {
        t.off = S.uip_off;
        t.rows = S.aR;
        t.x = (d - S.dmin) * S.xs_uip;
    } else {
        t.off = S.usp_off;
        t.rows = S.dR;
        t.x = (d - S.r0) * S.xs_usp;
    }
    t.x = fmin(fmax(t.x, 0.0), (double)(t.rows - 1));
    return t;
}

// plain double precision, one pixel per thread
__global__ void __launch_bounds__(128) us_lut_f64_kernel(Scene sc, const Sphere* __restrict__ sph, int s0, int s1,
                                                          int accumulate, int finalize,
                                                          const double* __restrict__ waves,
                                                          const zd* __restrict__ ph, const Patch<double>* __restrict__ lut,
                                                          const zd* __restrict__ Uf, zd* __restrict__ U) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= sc.R * sc.R) return;
    double p[3];
    pixel_pos(sc, idx % sc.R, idx / sc.R, p);
    zd total = accumulate ? U[idx] : mk(0.0, 0.0);
    const double tscale = 1.0 / PI_REF;
    for (int s = s0; s < s1; s++) {
        const Sphere& S = sph[s];
        double r[3];
        double d = dist_exact(p, S.p, r);
        TableSel ts = select_table(S, d);
        int ir = (int)floor(ts.x);
        double al = ts.x - ir;
        const Patch<double>* row = lut + ts.off + (size_t)ir * S.thetaR;
        double rn[3] = {0, 0, 0}, cb = 1.0;  // d == 0: cos(theta) := 1
        if (d != 0) {
            rn[0] = r[0] / d;
            rn[1] = r[1] / d;
            rn[2] = r[2] / d;
            cb = 0.0;
        }
        double tmax = S.thetaR - 1;
        zd sum = mk(0.0, 0.0);
        const zd* phs = ph + (size_t)s * sc.nk;
        for (int w = 0; w < sc.nk; w++) {
            const double* k = waves + 3 * w;
            double c = (d != 0) ? (k[0] * rn[0] + k[1] * rn[1] + k[2] * rn[2]) : cb;
            c = fmin(fmax(c, -1.0), 1.0);
            double t = (acos(c) * tscale) * tmax;
            t = fmin(t, tmax);
            int it = (int)floor(t);
            double be = t - it;
            const Patch<double>& q = row[it];
            double vr = (q.v[0] + al * q.v[2]) + be * (q.v[4] + al * q.v[6]);
            double vi = (q.v[1] + al * q.v[3]) + be * (q.v[5] + al * q.v[7]);
            zd pw = phs[w];
            sum = sum + pw * mk(vr, vi);
        }
        total = total + sum;
    }
    if (finalize) {
        bool outside = true;
        for (int s = 0; s < sc.ns; s++) {
            const Sphere& S = sph[s];
            double r[3];
            if (dist_exact(p, S.p, r) < S.a) outside = false;
        }
        if (outside) total = total + Uf[idx];
    }
    U[idx] = total;
}

// Mixed precision: per-(pixel, sphere) geometry in double, per-wave work in
// float, per-chunk partial sums combined with Kahan compensation.
//
// A block owns a 16 x 16 pixel tile, one or two pixels per thread.  The waves arrive
// grouped by direction into compact chunks of `chunk` waves (64, 32 or 16) and
// are processed chunk by chunk; the host gives each chunk a bounding cone
// (axis c_k, half-angle beta_k).  For a
// tile whose pixels all lie outside the sphere and see it within an angle
// gamma of the tile-centre direction r_c, every lookup angle of a chunk lies
// in angle(c_k, r_c) +- (beta_k + gamma) (triangle inequality on the sphere of
// directions).  The table values of the tile's rows times that angular window
// (float2, at most lut_stage_entries(chunk) of them) are copied to shared memory once per
// chunk and the bilinear cells are read from there.  Chunks whose window does
// not fit, and tiles touching or containing the sphere, read the cells through
// the texture path instead: the tables also live in CUDA arrays (block-linear
// layout, real and imaginary float planes, x = angle, y = radius) and
// tex2Dgather returns the cell's four texels, (i, j+1), (i+1, j+1), (i+1, j),
// (i, j) in x, y, z, w.  Both paths interpolate with the same single-precision
// formula, so they give the same bits; edge cells clamp like the reference's
// texture fetch.
constexpr int UST_TILE = 256;           // 16 x 16 pixel tile
// Pixels per thread of the staged kernel.  With 64-wave chunks two pixels per thread (128 threads
// at 128 registers, 4 blocks per SM) are fastest: 730 ms on the 1024^2, 50-sphere slice against
// 755 ms for one pixel (four: 19 % slower; two at 96 registers and 5 blocks per SM: 11 %), 697 ms
// with 51 KB windows and the wave loop unrolled 16 deep.  With 16- and 32-wave chunks the
// per-chunk barriers and window copies weigh more and one pixel per thread on 8 warps is faster
// (512^2 slice at 3x the table rows per tile: 307 against 366 ms with 16-wave chunks).
constexpr int UST_TWO_PIXEL_MIN_CHUNK = 64;

// Fractional LUT angle index t = acos(c) tsc for c in [-1, 1] (c is clamped),
// tsc = (thetaR - 1) / PI_REF, tscpi = tsc * pi.  acos(x) = sqrt(1 - x) g(x)
// on [0, 1] with g analytic there (the square-root factorisation of acos at
// x = 1, as in Abramowitz & Stegun 4.4.45-46), and acos(-x) = pi - acos(x).
// g is our own degree-7 least-squares fit on 4000 Chebyshev nodes of [0, 1],
// weighted for absolute error; evaluated in single precision the angle is
// within 3.5e-7 rad of acos over [-1, 1] (about 1e-4 of one table column at
// thetaR = 1024).
__device__ __forceinline__ float theta_index(float c, float tsc, float tscpi) {
    const float ax = fminf(fabsf(c), 1.f);
    float s;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(s) : "f"(1.f - ax));
    float g = -1.411853940e-03f;
    g = fmaf(g, ax, 7.149144541e-03f);
    g = fmaf(g, ax, -1.768672466e-02f);
    g = fmaf(g, ax, 3.125903755e-02f);
    g = fmaf(g, ax, -5.028845742e-02f);
    g = fmaf(g, ax, 8.899561316e-02f);
    g = fmaf(g, ax, -2.145996839e-01f);
    g = fmaf(g, ax, 1.570796371e+00f);
    const float v = (s * tsc) * g;
    return c < 0.f ? tscpi - v : v;
}

// 8-byte global -> shared copy that does not go through registers (cp.async)
__device__ __forceinline__ void copy_async8(float2* dst, const float2* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}

__device__ __forceinline__ void copy_async16(float4* dst, const float4* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}

__device__ __forceinline__ void copy_async4(float* dst, const float* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}

// Two single-precision lanes in one 64-bit register pair (low lane first), worked
// on by Blackwell's packed f32x2 instructions; each lane rounds exactly like the
// scalar instruction (round to nearest, no flush).
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 f2_splat(float a) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %1};" : "=l"(r) : "f"(a));
    return r;
}
__device__ __forceinline__ f32x2 f2_sub(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 f2_fma(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ f32x2 f2_pack(float a, float b) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ f32x2 f2_mul(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ float2 f2_unpack(f32x2 v) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}

// theta_index of two pixels with the polynomial and the final products in packed
// f32x2 instructions; every lane rounds as the scalar instruction, so t0, t1 are
// theta_index(c0, ...), theta_index(c1, ...) bit for bit.
__device__ __forceinline__ void theta_index2(float c0, float c1, float tsc, float tscpi, float& t0, float& t1) {
    const float ax0 = fminf(fabsf(c0), 1.f), ax1 = fminf(fabsf(c1), 1.f);
    float s0, s1;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(s0) : "f"(1.f - ax0));
    asm("sqrt.approx.f32 %0, %1;" : "=f"(s1) : "f"(1.f - ax1));
    const f32x2 ax = f2_pack(ax0, ax1);
    f32x2 g = f2_splat(-1.411853940e-03f);
    g = f2_fma(g, ax, f2_splat(7.149144541e-03f));
    g = f2_fma(g, ax, f2_splat(-1.768672466e-02f));
    g = f2_fma(g, ax, f2_splat(3.125903755e-02f));
    g = f2_fma(g, ax, f2_splat(-5.028845742e-02f));
    g = f2_fma(g, ax, f2_splat(8.899561316e-02f));
    g = f2_fma(g, ax, f2_splat(-2.145996839e-01f));
    g = f2_fma(g, ax, f2_splat(1.570796371e+00f));
    const float2 v = f2_unpack(f2_mul(f2_mul(f2_pack(s0, s1), f2_splat(tsc)), g));
    t0 = c0 < 0.f ? tscpi - v.x : v.x;
    t1 = c1 < 0.f ? tscpi - v.y : v.y;
}

__device__ __forceinline__ void copy_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
constexpr int UST_CHUNK = WAVE_CHUNK_MAX;  // shared arrays; the run's chunk may be smaller
constexpr float UST_MARGIN = LUT_STAGE_MARGIN;

// Block-uniform values of one (tile, sphere) pair, kept in shared memory so
// that they are re-read per chunk instead of holding registers through the
// wave loops.
struct TileSphere {
    float cx, cy, cz;  // unit direction from the sphere to the tile centre
    float gam;         // angular radius of the tile seen from the sphere, plus margin
    float tsc, tscpi;
    int rlo, nrows;    // staged table rows [rlo, rlo + nrows); nrows = 0: texture path only
    int thetaR, lin_stride;
    long long off;     // first entry of the table in the linear pool
};

// Window of a wave chunk with bounding cone `cone` for the block's (tile, sphere):
// first column and width, width 0 when the block does not stage this sphere or
// the window does not fit.  Columns go up to thetaR: the linear rows carry a
// copy of the last column there.
__device__ __forceinline__ int2 chunk_plan(const float4 cone, const TileSphere& ts, int stage_cap) {
    if (ts.nrows == 0) return make_int2(0, 0);
    const float tsc = ts.tsc, gam = ts.gam;
    const float thc = acosf(fminf(fmaxf(cone.x * ts.cx + cone.y * ts.cy + cone.z * ts.cz, -1.f), 1.f));
    const int t_lo = max(0, (int)floorf((thc - cone.w - gam) * tsc) - 1);
    const int t_hi = min(ts.thetaR, (int)floorf((thc + cone.w + gam) * tsc) + 2);
    int W = t_hi - t_lo + 1;
    if (W < 2 || ts.nrows * lut_stage_stride(W) > stage_cap) W = 0;
    return make_int2(t_lo, W);
}

// STAGE = false: texture path only, no dynamic shared memory (the L1 keeps
// its full size for the texture cache) and 6 blocks per SM.  PPT pixels per
// thread: the tile's eight 4 x 8 warp blocks are spread over 8 / PPT warps, and
// each wave's direction and phase (shared-memory broadcasts) are read once for
// the thread's PPT pixels.  Every pixel's arithmetic is the same for any PPT.
// stage_cap: float2 entries of the dynamic shared memory (lut_stage_entries).
// Blocks per SM: the one-pixel staged kernel runs 3 (its 72 KB stage) and may
// take 80 registers (config 3 262 against 266 ms per band at 64); the two-pixel
// one 4; the texture-only one 6 (5, at 48 registers without spills, measured
// no faster).
template <bool STAGE, int PPT>
__global__ void __launch_bounds__(UST_TILE / PPT, STAGE ? (PPT == 1 ? 3 : 4) : 6) us_lut_tex_kernel(Scene sc, const Sphere* __restrict__ sph, int s0, int s1,
                                                                    int accumulate, int finalize,
                                                                    const float4* __restrict__ kw4,
                                                                    const float4* __restrict__ cones,
                                                                    const cpx<float>* __restrict__ ph,
                                                                    const unsigned long long* __restrict__ tex,
                                                                    const float2* __restrict__ lin,
                                                                    const cpx<float>* __restrict__ Uf,
                                                                    cpx<float>* __restrict__ U,
                                                                    unsigned long long* __restrict__ counters,
                                                                    float2* __restrict__ kcmp, int chunk,
                                                                    int stage_cap) {
    constexpr int NT = UST_TILE / PPT, NWARP = NT / 32;
    static_assert(NT >= UST_CHUNK && NT % 32 == 0, "one thread per wave of a chunk");
    extern __shared__ float2 s_stage[];
    __shared__ float4 s_k[UST_CHUNK];
    __shared__ float2 s_p[UST_CHUNK];
    __shared__ int s_red[4][NWARP];
    __shared__ TileSphere s_ts;
    __shared__ int2 s_plan;  // staged window of the next chunk: first column, width (0: texture path)
    __shared__ double s_pa[3][16], s_pb[3][16];  // pixel position = s_pa[.][column] + s_pb[.][row]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // the tile is covered by eight 4 x 8 pixel blocks (half-warps 4 x 4): the compact footprint of
    // one load instruction has the fewest shared-memory bank conflicts (8 x 4 blocks: 1 % slower,
    // 16 x 2: 22 %).  Pixel j of a thread lies in block warp + NWARP j.
    const int tiles_u = (sc.R + 15) / 16;
    const int tu = (blockIdx.x % tiles_u) * 16, tv = (blockIdx.x / tiles_u) * 16;
    int iu[PPT], iv[PPT], lu[PPT], lv[PPT];
    bool valid[PPT];
#pragma unroll
    for (int j = 0; j < PPT; j++) {
        const int blk = warp + NWARP * j;
        iu[j] = tu + (lane & 3) + 4 * (blk & 3);
        iv[j] = tv + (lane >> 2) + 8 * (blk >> 2);
        valid[j] = iu[j] < sc.R && iv[j] < sc.R;
        lu[j] = min(iu[j], sc.R - 1) - tu;
        lv[j] = min(iv[j], sc.R - 1) - tv;
    }
    // pixel_pos computes (A + X u) + Y v: the terms of the tile's 16 columns and 16 rows, once
    if (threadIdx.x < 32) {
        const int k = threadIdx.x & 15;
        const double t = __ddiv_rn((double)min((threadIdx.x < 16 ? tu : tv) + k, sc.R - 1), (double)sc.R);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            if (threadIdx.x < 16) s_pa[c][k] = __dadd_rn(sc.A[c], __dmul_rn(sc.X[c], t));
            else s_pb[c][k] = __dmul_rn(sc.Y[c], t);
        }
    }
    __syncthreads();
    float tot_r[PPT], tot_i[PPT], cmp_r[PPT], cmp_i[PPT];  // Kahan sums over chunk partials
#pragma unroll
    for (int j = 0; j < PPT; j++) {
        tot_r[j] = tot_i[j] = cmp_r[j] = cmp_i[j] = 0.f;
        if (accumulate && valid[j]) {
            tot_r[j] = U[iv[j] * sc.R + iu[j]].re;
            tot_i[j] = U[iv[j] * sc.R + iu[j]].im;
            if (kcmp) {  // the Kahan compensation the previous sphere chunk left: the sum goes on as in one launch
                cmp_r[j] = kcmp[iv[j] * sc.R + iu[j]].x;
                cmp_i[j] = kcmp[iv[j] * sc.R + iu[j]].y;
            }
        }
    }
    const int nchunks = (sc.nk + chunk - 1) / chunk;
    unsigned staged_chunks = 0;
    for (int s = s0; s < s1; s++) {
        const Sphere& S = sph[s];
        float rx[PPT], ry[PPT], rz[PPT], cb[PPT], al[PPT], y[PPT];
        int ir[PPT], ktex[PPT];
        bool far[PPT];  // outside the sphere, d > 0
#pragma unroll
        for (int j = 0; j < PPT; j++) {
            double p[3], r[3];
#pragma unroll
            for (int c = 0; c < 3; c++) p[c] = __dadd_rn(s_pa[c][lu[j]], s_pb[c][lv[j]]);
            const double d = dist_exact(p, S.p, r);
            const TableSel ts = select_table_scaled(S, d);
            ir[j] = (int)floor(ts.x);
            al[j] = (float)(ts.x - ir[j]);
            y[j] = (float)ir[j] + 1.0f;  // gather footprint rows ir, ir + 1
            ktex[j] = 4 * (s - s0) + (d < S.a ? 2 : 0);
            rx[j] = ry[j] = rz[j] = 0.f;
            cb[j] = 1.f;  // d == 0: cos(theta) := 1
            if (d != 0) {
                const float inv = 1.f / (float)d;
                rx[j] = (float)r[0] * inv;
                ry[j] = (float)r[1] * inv;
                rz[j] = (float)r[2] * inv;
                cb[j] = 0.f;
            }
            far[j] = d >= S.a && d != 0;
        }
        // every pixel of a staged tile lies outside the sphere: its table is Usp (dR rows)
        const int rows = S.dR;
        // ---- tile bounds: table rows and angular radius gamma ----
        int rlo = 0, rhi = 0, ok = 0;
        if (!STAGE) {
            __syncthreads();  // s_ts is reused for every sphere
            if (threadIdx.x == 0) {
                s_ts.tsc = (float)((S.thetaR - 1) / PI_REF);
                s_ts.tscpi = (float)((S.thetaR - 1) / PI_REF * TRUE_PI);
                s_ts.nrows = 0;
            }
        } else {
            // tile centre in single precision (bounds only, covered by the margins)
            const float u = ((float)tu + 7.5f) / (float)sc.R, v = ((float)tv + 7.5f) / (float)sc.R;
            float cx = (float)sc.A[0] + (float)sc.X[0] * u + (float)sc.Y[0] * v - (float)S.p[0];
            float cy = (float)sc.A[1] + (float)sc.X[1] * u + (float)sc.Y[1] * v - (float)S.p[1];
            float cz = (float)sc.A[2] + (float)sc.X[2] * u + (float)sc.Y[2] * v - (float)S.p[2];
            const float cl = sqrtf(cx * cx + cy * cy + cz * cz);
            bool far_ok = cl > 0.f;
            float gam = 0.f;
            if (cl > 0.f) {
                cx /= cl;
                cy /= cl;
                cz /= cl;
            }
            rlo = INT_MAX;
            rhi = INT_MIN;
#pragma unroll
            for (int j = 0; j < PPT; j++) {
                if (!valid[j]) continue;
                far_ok = far_ok && far[j];
                if (cl > 0.f)
                    gam = fmaxf(gam, acosf(fminf(fmaxf(rx[j] * cx + ry[j] * cy + rz[j] * cz, -1.f), 1.f)));
                rlo = min(rlo, ir[j]);
                rhi = max(rhi, ir[j]);
            }
            rlo = __reduce_min_sync(0xffffffffu, rlo);
            rhi = __reduce_max_sync(0xffffffffu, rhi);
            int gbits = (int)__reduce_max_sync(0xffffffffu, (unsigned)__float_as_int(gam));
            ok = __all_sync(0xffffffffu, far_ok);
            __syncthreads();  // s_red and s_ts are reused for every sphere
            if (lane == 0) {
                s_red[0][warp] = rlo;
                s_red[1][warp] = rhi;
                s_red[2][warp] = gbits;
                s_red[3][warp] = ok;
            }
            __syncthreads();
#pragma unroll
            for (int w = 0; w < NWARP; w++) {
                rlo = min(rlo, s_red[0][w]);
                rhi = max(rhi, s_red[1][w]);
                gbits = max(gbits, s_red[2][w]);
                ok = ok && s_red[3][w];
            }
            if (threadIdx.x == 0) {
                s_ts.cx = cx;
                s_ts.cy = cy;
                s_ts.cz = cz;
                s_ts.gam = __int_as_float(gbits) + UST_MARGIN;
                s_ts.tsc = (float)((S.thetaR - 1) / PI_REF);
                s_ts.tscpi = (float)((S.thetaR - 1) / PI_REF * TRUE_PI);
                // staged rows: [rlo, rhi + 1] clamped to the table
                s_ts.rlo = rlo;
                s_ts.nrows = ok ? min(rhi + 1, rows - 1) - rlo + 1 : 0;
                s_ts.thetaR = S.thetaR;
                s_ts.lin_stride = S.lin_stride;
                s_ts.off = S.usp_off;
                s_plan = chunk_plan(cones[0], s_ts, stage_cap);
            }
        }
        // local rows of each pixel in the staged block (clamped, so always in bounds)
        const int nrows_b = ok ? min(rhi + 1, rows - 1) - rlo + 1 : 1;
        int lr0[PPT], drow0[PPT];
#pragma unroll
        for (int j = 0; j < PPT; j++) {
            lr0[j] = min(max(ir[j] - rlo, 0), max(nrows_b, 1) - 1);
            drow0[j] = min(max(min(ir[j] + 1, rows - 1) - rlo, 0), max(nrows_b, 1) - 1) - lr0[j];
        }
        for (int ch = 0; ch < nchunks; ch++) {
            const int w0 = ch * chunk;
            const int nw = min(chunk, sc.nk - w0);
            __syncthreads();  // the previous chunk's readers are done; s_ts is written
            const int nrows = s_ts.nrows;
            // window of this chunk: planned by thread 0 (before the first chunk, or while the
            // previous chunk was summed)
            const int2 pl = STAGE ? s_plan : make_int2(0, 0);
            const int t_lo = pl.x, W = pl.y, Ws = lut_stage_stride(W);
            const bool staged = STAGE && W > 0;
            if (threadIdx.x < nw) {
                copy_async16(&s_k[threadIdx.x], kw4 + w0 + threadIdx.x);
                copy_async8(&s_p[threadIdx.x], reinterpret_cast<const float2*>(ph + (size_t)s * sc.nk + w0) + threadIdx.x);
            }
            if (STAGE && staged) {
                // asynchronous copies, one table row per warp at a time, all in flight together
                const float2* table = lin + s_ts.off + (size_t)s_ts.rlo * s_ts.lin_stride + t_lo;
                const int ls = s_ts.lin_stride;
                for (int rr = warp; rr < nrows; rr += NWARP) {
                    const float2* src = table + (size_t)rr * ls;
                    float2* dst = s_stage + rr * Ws;
                    for (int tt = lane; tt < W; tt += 32) copy_async8(dst + tt, src + tt);
                }
            }
            copy_async_wait_all();
            __syncthreads();
            if (STAGE && threadIdx.x == 0 && ch + 1 < nchunks) s_plan = chunk_plan(cones[ch + 1], s_ts, stage_cap);
            // t < thetaR - 1 + 1e-3 (PI_REF < pi): the last column is repeated in the staged rows and
            // clamped in the texture planes, so t past thetaR - 1 reads the last column, as a clamp would
            const float tsc = s_ts.tsc, tscpi = s_ts.tscpi;
            // the chunk's sum of pw v as sum(pw.x v) and sum(pw.y v), each a (re, im) pair:
            // Re = x.re - y.im, Im = x.im + y.re
            float2 sx[PPT], sy[PPT];
            if (STAGE && staged) {
                staged_chunks++;
                const unsigned lt_max = (unsigned)(W - 2);
                const float2* row0[PPT];
                int drow[PPT];
                f32x2 alp[PPT], ax[PPT], ay[PPT];
#pragma unroll
                for (int j = 0; j < PPT; j++) {
                    row0[j] = s_stage + lr0[j] * Ws;
                    drow[j] = drow0[j] * Ws;
                    alp[j] = f2_splat(al[j]);
                    ax[j] = ay[j] = 0ull;
                }
                // one lookup of pixel j at angle index t, wave weight (pwx, pwy)
                auto lookup = [&](int j, float t, f32x2 pwx, f32x2 pwy) {
                    const float tf = floorf(t);
                    const float be = t - tf;
                    // in the window by construction; the unsigned clamp only keeps a bad bound in bounds
                    const unsigned lt = min((unsigned)((int)tf - t_lo), lt_max);
                    const f32x2* q = reinterpret_cast<const f32x2*>(row0[j] + lt);
                    const f32x2 e00 = q[0], e01 = q[1], e10 = q[drow[j]], e11 = q[drow[j] + 1];
                    const f32x2 bep = f2_splat(be);
                    const f32x2 a0 = f2_fma(bep, f2_sub(e01, e00), e00);
                    const f32x2 a1 = f2_fma(bep, f2_sub(e11, e10), e10);
                    const f32x2 v = f2_fma(alp[j], f2_sub(a1, a0), a0);
                    ax[j] = f2_fma(pwx, v, ax[j]);
                    ay[j] = f2_fma(pwy, v, ay[j]);
                };
                // cb = 0 here: every d > 0.  The angle indices of two lookups at a time (the thread's
                // two pixels, or one pixel's two consecutive waves) in packed instructions; the lookups
                // and their sums run in wave order, so the bits are those of one at a time.
                // 32 lookups per thread per unrolled step (config 2: 697 ms; 8: 721 ms, 16: 700 ms,
                // 64: 792 ms)
                if (PPT == 2) {
#pragma unroll 16
                    for (int w = 0; w < nw; w++) {
                        const float4 kk = s_k[w];
                        const float2 pw = s_p[w];
                        const f32x2 pwx = f2_splat(pw.x), pwy = f2_splat(pw.y);
                        float t0, t1;
                        theta_index2(fmaf(kk.x, rx[0], fmaf(kk.y, ry[0], kk.z * rz[0])),
                                     fmaf(kk.x, rx[PPT - 1], fmaf(kk.y, ry[PPT - 1], kk.z * rz[PPT - 1])), tsc,
                                     tscpi, t0, t1);
                        lookup(0, t0, pwx, pwy);
                        lookup(PPT - 1, t1, pwx, pwy);
                    }
                } else {
                    int w = 0;
#pragma unroll 16
                    for (; w + 1 < nw; w += 2) {
                        const float4 k0 = s_k[w], k1 = s_k[w + 1];
                        const float2 p0 = s_p[w], p1 = s_p[w + 1];
                        float t0, t1;
                        theta_index2(fmaf(k0.x, rx[0], fmaf(k0.y, ry[0], k0.z * rz[0])),
                                     fmaf(k1.x, rx[0], fmaf(k1.y, ry[0], k1.z * rz[0])), tsc, tscpi, t0, t1);
                        lookup(0, t0, f2_splat(p0.x), f2_splat(p0.y));
                        lookup(0, t1, f2_splat(p1.x), f2_splat(p1.y));
                    }
                    if (w < nw) {
                        const float4 kk = s_k[w];
                        const float2 pw = s_p[w];
                        lookup(0, theta_index(fmaf(kk.x, rx[0], fmaf(kk.y, ry[0], kk.z * rz[0])), tsc, tscpi),
                               f2_splat(pw.x), f2_splat(pw.y));
                    }
                }
#pragma unroll
                for (int j = 0; j < PPT; j++) {
                    sx[j] = f2_unpack(ax[j]);
                    sy[j] = f2_unpack(ay[j]);
                }
            } else {
                cudaTextureObject_t tre[PPT], tim[PPT];
#pragma unroll
                for (int j = 0; j < PPT; j++) {
                    sx[j] = sy[j] = make_float2(0.f, 0.f);
                    tre[j] = tex[ktex[j]];
                    tim[j] = tex[ktex[j] + 1];
                }
#pragma unroll 1
                for (int w = 0; w < nw; w++) {
                    const float4 kk = s_k[w];
                    const float2 pw = s_p[w];
#pragma unroll
                    for (int j = 0; j < PPT; j++) {
                        const float c = fmaf(kk.x, rx[j], fmaf(kk.y, ry[j], fmaf(kk.z, rz[j], cb[j])));
                        const float t = theta_index(c, tsc, tscpi);
                        const float tf = floorf(t);
                        const float be = t - tf;
                        const float4 gr = tex2Dgather<float4>(tre[j], tf + 1.0f, y[j], 0);
                        const float4 gi = tex2Dgather<float4>(tim[j], tf + 1.0f, y[j], 0);
                        const float ar0 = fmaf(be, gr.z - gr.w, gr.w), ar1 = fmaf(be, gr.y - gr.x, gr.x);
                        const float ai0 = fmaf(be, gi.z - gi.w, gi.w), ai1 = fmaf(be, gi.y - gi.x, gi.x);
                        const float vr = fmaf(al[j], ar1 - ar0, ar0);
                        const float vi = fmaf(al[j], ai1 - ai0, ai0);
                        sx[j].x = fmaf(pw.x, vr, sx[j].x);
                        sx[j].y = fmaf(pw.x, vi, sx[j].y);
                        sy[j].x = fmaf(pw.y, vr, sy[j].x);
                        sy[j].y = fmaf(pw.y, vi, sy[j].y);
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < PPT; j++) {
                const float ar = sx[j].x - sy[j].y, ai = sx[j].y + sy[j].x;
                // Kahan: add the chunk partial to the running total
                const float yr = ar - cmp_r[j], yi = ai - cmp_i[j];
                const float tr = tot_r[j] + yr, ti = tot_i[j] + yi;
                cmp_r[j] = (tr - tot_r[j]) - yr;
                cmp_i[j] = (ti - tot_i[j]) - yi;
                tot_r[j] = tr;
                tot_i[j] = ti;
            }
        }
    }
    if (threadIdx.x == 0 && counters) {
        atomicAdd(counters, (unsigned long long)staged_chunks);
        atomicAdd(counters + 1, (unsigned long long)(s1 - s0) * nchunks);
    }
#pragma unroll
    for (int j = 0; j < PPT; j++) {
        if (!valid[j]) continue;
        const int idx = iv[j] * sc.R + iu[j];
        if (finalize) {
            double p[3];
#pragma unroll
            for (int c = 0; c < 3; c++) p[c] = __dadd_rn(s_pa[c][lu[j]], s_pb[c][lv[j]]);
            bool outside = true;
            for (int s = 0; s < sc.ns && outside; s++) {
                const Sphere& S = sph[s];
                // clearly outside in single precision (0.1 % margin on d^2), else the exact test
                const float dx = (float)(p[0] - S.p[0]), dy = (float)(p[1] - S.p[1]), dz = (float)(p[2] - S.p[2]);
                const float af = (float)S.a;
                if (dx * dx + dy * dy + dz * dz > 1.001f * af * af) continue;
                double r[3];
                if (dist_exact(p, S.p, r) < S.a) outside = false;
            }
            if (outside) {
                tot_r[j] += Uf[idx].re - cmp_r[j];
                tot_i[j] += Uf[idx].im - cmp_i[j];
            }
        } else if (kcmp) {
            kcmp[idx] = make_float2(cmp_r[j], cmp_i[j]);
        }
        U[idx] = mk(tot_r[j], tot_i[j]);
    }
}

// LUT build into the real and imaginary planes of a CUDA array pair (same
// sums as lut_build_kernel, written through surfaces) and into the linear
// float2 table used for staging.  `rows` counts one spare row of the planes
// that repeats the last table row.
__device__ __forceinline__ void lut_build_tex_entry(const zd* __restrict__ tab, int rows, int L,
                                                    const double* __restrict__ P, int Pstride, int thetaR,
                                                    cudaSurfaceObject_t sre, cudaSurfaceObject_t sim,
                                                    float2* __restrict__ lin, int lin_stride, int r, int t) {
    if (t >= thetaR || r >= rows) return;
    const zd* c = tab + (size_t)min(r, rows - 2) * L;  // the last row written repeats the one before
    const double* pl = P + (size_t)t * Pstride;
    zd acc = mk(0.0, 0.0);
    for (int l = 0; l < L; l++) acc = acc + c[l] * pl[l];
    surf2Dwrite((float)acc.re, sre, t * (int)sizeof(float), r);
    surf2Dwrite((float)acc.im, sim, t * (int)sizeof(float), r);
    if (r < rows - 1) {
        const float2 v = make_float2((float)acc.re, (float)acc.im);
        lin[(size_t)r * lin_stride + t] = v;
        if (t == thetaR - 1) lin[(size_t)r * lin_stride + thetaR] = v;  // clamped neighbour of the last column
    }
}

// Tables of a sphere batch in one launch: blockIdx.z picks the table,
// blockIdx.y its block of 8 rows (blocks past the table's rows return) and
// blockIdx.x a block of 32 angles, as the one-table grid would.
__global__ void __launch_bounds__(256) lut_build_tex_batch_kernel(const LutBuildJob* __restrict__ jobs,
                                                                    const zd* __restrict__ tab,
                                                                    const double* __restrict__ P, int Pstride,
                                                                    float2* __restrict__ lin) {
    const LutBuildJob& j = jobs[blockIdx.z];
    const int r = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (r >= j.rows) return;
    lut_build_tex_entry(tab + j.tab_off, j.rows, j.L, P, Pstride, j.thetaR, j.sre, j.sim, lin + j.lin_off,
                        j.lin_stride, r, blockIdx.x * 32 + (threadIdx.x & 31));
}

// ---------------------------------------------------------------------------
// Direct scattered field through the addition theorem of spherical harmonics.
// The per-pixel sum over waves, sum_w pw_w sum_l c_l P_l(k_w . r^), is
// sum_l c_l Q_l(r^) with Q_l(r^) = sum_w pw_w P_l(k_w . r^).  With the Schmidt
// semi-normalised associated Legendre functions S_l^m (S_l^m = sqrt(e_m (l-m)!
// / (l+m)!) P_l^m, e_0 = 1, e_m = 2), P_l(cos g) = sum_{m<=l} S_l^m(cos t1)
// S_l^m(cos t2) cos(m (f1 - f2)), so
//   Q_l(r^) = sum_m S_l^m(r_z) (cos(m f_r) C_lm + sin(m f_r) S_lm),
//   (C_lm, S_lm) = sum_w pw_w S_l^m(k_wz) (cos, sin)(m f_w)   per sphere,
// with f the azimuth about z.  A (pixel, sphere) pair then costs L (L + 1) / 2
// terms instead of nk L, and the result is the same sum up to rounding.
// Tables are in (m, l) order: index(m, l) = m L - m (m - 1) / 2 + (l - m).
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ int sh_index(int L, int m, int l) { return m * L - m * (m - 1) / 2 + (l - m); }

// Recurrence factors: rec[index(m, l)] = (a, b) with S_l^m = a x S_{l-1}^m - b S_{l-2}^m
// for l >= m + 2 (a = (2l - 1) / sqrt(l^2 - m^2), b = sqrt((l-1)^2 - m^2) / sqrt(l^2 - m^2)),
// a = sqrt(2m + 1) for l = m + 1, and for l = m the diagonal factor
// S_m^m = a sin(t) S_{m-1}^{m-1} (a = 1 for m = 1, sqrt((2m - 1) / (2m)) above).
__global__ void sh_recur_kernel(int L, double2* __restrict__ rec) {
    const int m = blockIdx.x, l = m + threadIdx.x;
    if (m >= L || l >= L) return;
    double a = 0, b = 0;
    if (l == m) a = m == 0 ? 1.0 : (m == 1 ? 1.0 : sqrt((2.0 * m - 1.0) / (2.0 * m)));
    else if (l == m + 1) a = sqrt(2.0 * m + 1.0);
    else {
        const double den = sqrt((double)l * l - (double)m * m);
        a = (2.0 * l - 1.0) / den;
        b = sqrt((double)(l - 1) * (l - 1) - (double)m * m) / den;
    }
    rec[sh_index(L, m, l)] = make_double2(a, b);
}

// Per wave: tab[w][index(m, l)] = S_l^m(k_z) (cos, sin)(m f_k).
__global__ void sh_wave_kernel(int nk, int L, const double* __restrict__ waves, const double2* __restrict__ rec,
                               double2* __restrict__ tab) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nk) return;
    const double kx = waves[3 * w], ky = waves[3 * w + 1], kz = waves[3 * w + 2];
    const double rho = sqrt(kx * kx + ky * ky);
    const double cf = rho > 0 ? kx / rho : 1.0, sf = rho > 0 ? ky / rho : 0.0;
    double2* out = tab + (size_t)w * (L * (L + 1) / 2);
    double cm = 1, sm = 0, smm = 1;  // cos(m f), sin(m f), S_m^m
    for (int m = 0; m < L; m++) {
        if (m > 0) {
            smm *= rec[sh_index(L, m, m)].x * rho;
            const double c2 = cm * cf - sm * sf;
            sm = sm * cf + cm * sf;
            cm = c2;
        }
        double p2 = 0, p1 = smm;
        for (int l = m; l < L; l++) {
            double v;
            if (l == m) v = smm;
            else if (l == m + 1) v = rec[sh_index(L, m, l)].x * kz * smm;
            else {
                const double2 ab = rec[sh_index(L, m, l)];
                v = ab.x * kz * p1 - ab.y * p2;
            }
            if (l > m) {
                p2 = p1;
                p1 = v;
            }
            out[sh_index(L, m, l)] = make_double2(v * cm, v * sm);
        }
    }
}

// Per sphere s and table index: coef[s][index] = (C, S) = sum_w pw_{s,w} tab[w][index], with the
// phase pw of phase_kernel in double precision.
constexpr int SH_WAVES = 128;
__global__ void sh_coef_kernel(Scene sc, const Sphere* __restrict__ sph, int L, const double* __restrict__ waves,
                               const double2* __restrict__ tab, zd* __restrict__ coef) {
    __shared__ zd s_pw[SH_WAVES];
    const int s = blockIdx.y, nlm = L * (L + 1) / 2;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double c0 = sph[s].p[0] - sc.focus[0], c1 = sph[s].p[1] - sc.focus[1], c2 = sph[s].p[2] - sc.focus[2];
    zd ac = mk(0.0, 0.0), as = mk(0.0, 0.0);
    for (int w0 = 0; w0 < sc.nk; w0 += SH_WAVES) {
        const int nw = min(SH_WAVES, sc.nk - w0);
        __syncthreads();
        for (int t = threadIdx.x; t < nw; t += blockDim.x) {
            const double* k = waves + 3 * (w0 + t);
            const double arg = sc.kmag * (k[0] * c0 + k[1] * c1 + k[2] * c2);
            double sn, cs;
            sincos(arg, &sn, &cs);
            s_pw[t] = mk(sc.wave_amp * cs, sc.wave_amp * sn);
        }
        __syncthreads();
        if (i < nlm)
            for (int t = 0; t < nw; t++) {
                const double2 v = tab[(size_t)(w0 + t) * nlm + i];
                ac = ac + s_pw[t] * v.x;
                as = as + s_pw[t] * v.y;
            }
    }
    if (i < nlm) {
        coef[((size_t)s * nlm + i) * 2] = ac;
        coef[((size_t)s * nlm + i) * 2 + 1] = as;
    }
}

// Per pixel: U = sum_s sum_l c_l(r) Q_l(r^) (+ Uf outside every sphere)
// (--recursive; nfScalarUs.cu:17-95, 201-245, 333-491).  The Bessel recurrences
// depend on (pixel, sphere) only, so they run once per pair in double and give
//   outside (d > a):  c_l = B_l (j_l + i y_l)(k d)   with the reference clamps
//   inside  (d <= a): c_l = A_l j_l(k n d)           (c_0 = A_0 only when
//                                                      Re(k n d) < 1e-6)
// where the reference re-runs them for every wave (nfScalarUs.cu:69-93).  All
// in double precision, stored as T.
constexpr int SH_BLOCK = 64;
template <class T>
__global__ void __launch_bounds__(SH_BLOCK) us_sh_kernel(Scene sc, const Sphere* __restrict__ sph, int L,
                                                         const zd* __restrict__ A, const zd* __restrict__ B,
                                                         const double2* __restrict__ rec, const zd* __restrict__ coef,
                                                         const cpx<T>* __restrict__ Uf, cpx<T>* __restrict__ U) {
    extern __shared__ unsigned char smem_raw[];
    zd* cl = reinterpret_cast<zd*>(smem_raw);  // [L][SH_BLOCK]
    const int tid = threadIdx.x, nlm = L * (L + 1) / 2;
    int idx = blockIdx.x * SH_BLOCK + tid;
    const bool valid = idx < sc.R * sc.R;
    if (!valid) idx = sc.R * sc.R - 1;
    double p[3];
    pixel_pos(sc, idx % sc.R, idx / sc.R, p);
    zd tot = mk(0.0, 0.0), cmp = mk(0.0, 0.0);
    bool outside = true;
    for (int s = 0; s < sc.ns; s++) {
        const Sphere& S = sph[s];
        double r[3];
        const double d = dist_exact(p, S.p, r);
        if (d < S.a) outside = false;
        const int Ls = S.Nl + 1;
        int Leff = Ls;
        if (d <= S.a) {
            const zd* co = A + S.coef_off;
            const zd knd = mk(sc.kmag * d * S.n_re, sc.kmag * d * S.n_im);
            if (knd.re < EPS_FLOAT) {
                Leff = 1;
                cl[tid] = co[0];
            } else {
                zd j0 = zsin(knd) / knd;
                zd j1 = j0 / knd - zcos(knd) / knd;
                for (int l = 0; l < Ls; l++) {
                    zd jl;
                    if (l == 0) {
                        jl = j0;
                    } else {
                        if (l > 1) sbesselj_step_c(l, knd, j0, j1);
                        jl = j1;
                    }
                    cl[l * SH_BLOCK + tid] = co[l] * jl;
                }
            }
        } else {
            const zd* co = B + S.coef_off;
            const double kd = sc.kmag * d;
            double sn, cs;
            sincos(kd, &sn, &cs);
            double j0 = sn / kd, j1 = j0 / kd - cs / kd;
            double y0 = -cs / kd, y1 = y0 / kd - sn / kd;
            for (int l = 0; l < Ls; l++) {
                double jl, yl;
                if (l == 0) {
                    jl = j0;
                    yl = y0;
                } else {
                    if (l > 1) {
                        sbesselj_step(l, kd, j0, j1);
                        sbessely_step(l, kd, y0, y1);
                    }
                    jl = j1;
                    yl = y1;
                }
                cl[l * SH_BLOCK + tid] = co[l] * mk(jl, yl);
            }
        }
        // direction of the pixel from the sphere; at d == 0 only l = 0 remains
        double x = 0, rho = 0, cf = 1, sf = 0;
        if (d != 0) {
            const double rx = r[0] / d, ry = r[1] / d;
            x = r[2] / d;
            rho = sqrt(rx * rx + ry * ry);
            if (rho > 0) {
                cf = rx / rho;
                sf = ry / rho;
            }
        }
        const zd* cs_ = coef + (size_t)s * nlm * 2;
        zd acc = mk(0.0, 0.0);
        double cm = 1, sm = 0, smm = 1;
        for (int m = 0; m < Leff; m++) {
            if (m > 0) {
                smm *= rec[sh_index(L, m, m)].x * rho;
                const double c2 = cm * cf - sm * sf;
                sm = sm * cf + cm * sf;
                cm = c2;
            }
            double p2 = 0, p1 = smm;
            for (int l = m; l < Leff; l++) {
                double v;
                if (l == m) v = smm;
                else if (l == m + 1) v = rec[sh_index(L, m, l)].x * x * smm;
                else {
                    const double2 ab = rec[sh_index(L, m, l)];
                    v = ab.x * x * p1 - ab.y * p2;
                }
                if (l > m) {
                    p2 = p1;
                    p1 = v;
                }
                const int k = sh_index(L, m, l);
                const zd C = cs_[2 * k], Sn = cs_[2 * k + 1];
                const zd q = mk(cm * C.re + sm * Sn.re, cm * C.im + sm * Sn.im) * v;
                acc = acc + cl[l * SH_BLOCK + tid] * q;
            }
        }
        // Kahan over spheres
        const zd y = acc - cmp;
        const zd t = tot + y;
        cmp = (t - tot) - y;
        tot = t;
    }
    if (!valid) return;
    if (outside) tot = tot + (mk((double)Uf[idx].re, (double)Uf[idx].im) - cmp);
    U[idx] = mk((T)tot.re, (T)tot.im);
}

// Vector stub of the reference: no scattered field, U = Uf outside every sphere.
template <class T>
__global__ void sum_only_kernel(Scene sc, const Sphere* __restrict__ sph, const cpx<T>* __restrict__ Uf,
                                cpx<T>* __restrict__ U) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= sc.R * sc.R) return;
    double p[3];
    pixel_pos(sc, idx % sc.R, idx / sc.R, p);
    bool outside = true;
    for (int s = 0; s < sc.ns; s++) {
        const Sphere& S = sph[s];
        double r[3];
        if (dist_exact(p, S.p, r) < S.a) outside = false;
    }
    U[idx] = outside ? Uf[idx] : mk((T)0, (T)0);
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
static inline unsigned blocks_for(long long n, int b) { return (unsigned)((n + b - 1) / b); }

template <class T>
void launch_uf(const Scene& sc, const double* tab, const double* w, cpx<T>* Uf, cudaStream_t st) {
    long long n = (long long)sc.R * sc.R;
    uf_kernel<T><<<blocks_for(n, 128), 128, 0, st>>>(sc, tab, w, Uf);
}

void launch_uf_table(const Scene& sc, double* tab, double* scratch, cudaStream_t st) {
    uf_table_kernel<<<blocks_for(sc.uf_dR, 128), 128, 0, st>>>(sc, tab, scratch);
}

void launch_mie(const Sphere* sph, int ns, double k, zd* scratch, int lstride, zd* A, zd* B, cudaStream_t st) {
    mie_kernel<<<blocks_for(ns, 64), 64, 0, st>>>(sph, ns, k, scratch, lstride, A, B);
}

void launch_coef_rows_batch(const Sphere* sph, int s0, int n, const long long* starts, long long total_rows,
                            double k, const zd* A, const zd* B, zd* tab, double* scratch, cudaStream_t st) {
    coef_rows_batch_kernel<<<(unsigned)((total_rows + 127) / 128), 128, 0, st>>>(sph, s0, n, starts, k, A, B, tab,
                                                                               scratch);
}

void launch_legendre_table(int thetaR, int Lmax, double* P, cudaStream_t st) {
    legendre_table_kernel<<<blocks_for(thetaR, 128), 128, 0, st>>>(thetaR, Lmax, P);
}

template <class T>
void launch_lut_build(const zd* tab, int rows, int L, const double* P, int Pstride, int thetaR, Patch<T>* out,
                      cudaStream_t st) {
    dim3 grid(blocks_for(thetaR, LB_TT), blocks_for(rows, LB_TR));
    lut_build_kernel<T><<<grid, 256, 0, st>>>(tab, rows, L, P, Pstride, thetaR, out);
}

template <class T>
void launch_phase(const Scene& sc, const Sphere* sph, const double* waves, cpx<T>* ph, float4* kw4, cudaStream_t st) {
    long long n = std::max<long long>((long long)sc.ns * sc.nk, sc.nk);
    phase_kernel<T><<<blocks_for(n, 128), 128, 0, st>>>(sc, sph, waves, ph, kw4);
}

void launch_us_lut_f64(const Scene& sc, const Sphere* sph, int s0, int s1, int accumulate, int finalize,
                       const double* waves, const zd* ph, const Patch<double>* lut, const zd* Uf, zd* U,
                       cudaStream_t st) {
    long long n = (long long)sc.R * sc.R;
    us_lut_f64_kernel<<<blocks_for(n, 128), 128, 0, st>>>(sc, sph, s0, s1, accumulate, finalize, waves, ph, lut,
                                                           Uf, U);
}

void launch_us_lut_tex(const Scene& sc, const Sphere* sph, int s0, int s1, int accumulate, int finalize,
                       const float4* kw4, const float4* cones, const cpx<float>* ph, const unsigned long long* tex,
                       const float2* lin, const cpx<float>* Uf, cpx<float>* U, unsigned long long* counters,
                       float2* kcmp, bool stage, int chunk, cudaStream_t st) {
    int tiles = (sc.R + 15) / 16;
    if (!stage) {
        us_lut_tex_kernel<false, 1><<<(unsigned)tiles * tiles, UST_TILE, 0, st>>>(sc, sph, s0, s1, accumulate, finalize,
                                                                                 kw4, cones, ph, tex, lin, Uf, U,
                                                                                 counters, kcmp, chunk, 0);
        return;
    }
    const bool two = chunk >= UST_TWO_PIXEL_MIN_CHUNK;
    const int cap = lut_stage_entries(chunk), smem = cap * (int)sizeof(float2);
    // per device and cheap; a failure shows up as the launch error
    auto kernel = two ? us_lut_tex_kernel<true, 2> : us_lut_tex_kernel<true, 1>;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    kernel<<<(unsigned)tiles * tiles, two ? UST_TILE / 2 : UST_TILE, smem, st>>>(sc, sph, s0, s1, accumulate, finalize,
                                                                               kw4, cones, ph, tex, lin, Uf, U,
                                                                               counters, kcmp, chunk, cap);
}

void launch_lut_build_tex_batch(const LutBuildJob* jobs, int njobs, int max_rows, int max_theta, const zd* tab,
                                const double* P, int Pstride, float2* lin, cudaStream_t st) {
    if (njobs < 1 || max_rows < 1) return;
    dim3 grid(blocks_for(max_theta, 32), blocks_for(max_rows, 8), (unsigned)njobs);
    lut_build_tex_batch_kernel<<<grid, 256, 0, st>>>(jobs, tab, P, Pstride, lin);
}

void launch_sh_tables(const Scene& sc, const Sphere* sph, int L, const double* waves, double2* rec, double2* tab,
                      zd* coef, cudaStream_t st) {
    sh_recur_kernel<<<L, ((L + 31) / 32) * 32, 0, st>>>(L, rec);
    sh_wave_kernel<<<blocks_for(sc.nk, 64), 64, 0, st>>>(sc.nk, L, waves, rec, tab);
    const int nlm = L * (L + 1) / 2;
    dim3 grid(blocks_for(nlm, 128), sc.ns);
    sh_coef_kernel<<<grid, 128, 0, st>>>(sc, sph, L, waves, tab, coef);
}

template <class T>
void launch_us_sh(const Scene& sc, const Sphere* sph, int L, const zd* A, const zd* B, const double2* rec,
                  const zd* coef, const cpx<T>* Uf, cpx<T>* U, cudaStream_t st) {
    const size_t smem = (size_t)L * SH_BLOCK * sizeof(zd);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(us_sh_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const long long n = (long long)sc.R * sc.R;
    us_sh_kernel<T><<<blocks_for(n, SH_BLOCK), SH_BLOCK, smem, st>>>(sc, sph, L, A, B, rec, coef, Uf, U);
}


template <class T>
void launch_sum_only(const Scene& sc, const Sphere* sph, const cpx<T>* Uf, cpx<T>* U, cudaStream_t st) {
    long long n = (long long)sc.R * sc.R;
    sum_only_kernel<T><<<blocks_for(n, 128), 128, 0, st>>>(sc, sph, Uf, U);
}

// ---------------------------------------------------------------------------
// Near-field rotation (gpuInterpolateU / gpuInterpolateUf, nfInterpolate.cu:13-58):
// dst(iu, iv) = src sampled at the pixel rotated by an angle about the slice
// centre, bilinear, zero outside the slice (border addressing).  The centre is
// (int)(R/2) for U and R/2 for Uf, as in the reference; coordinates are formed
// in single precision like the reference's (cosine and sine of the angle come
// from the host rounded to float; every operation is rounded on its own, no
// fused multiply-add), the weights are exact.
// ---------------------------------------------------------------------------
template <class T>
__global__ void rotate_fields_kernel(int R, float c, float s, const cpx<T>* __restrict__ src,
                                     cpx<T>* __restrict__ dst) {
    const int iu = blockIdx.x * blockDim.x + threadIdx.x, iv = blockIdx.y;
    const int b = blockIdx.z;  // 0: U, 1: Uf
    if (iu >= R) return;
    const float uc = b == 0 ? (float)(int)(R / 2.0) : (float)(R / 2.0);
    const float du = __fsub_rn((float)iu, uc), dv = __fsub_rn((float)iv, uc);
    const float nx = __fsub_rn(__fadd_rn(uc, __fmul_rn(du, c)), __fmul_rn(dv, s));
    const float ny = __fadd_rn(__fadd_rn(uc, __fmul_rn(du, s)), __fmul_rn(dv, c));
    const cpx<T>* f = src + (size_t)b * R * R;
    const float fx = floorf(nx), fy = floorf(ny);
    const int i0 = (int)fx, j0 = (int)fy;
    const T a = (T)(nx - fx), e = (T)(ny - fy);
    auto at = [&](int i, int j) -> cpx<T> {
        return (i >= 0 && i < R && j >= 0 && j < R) ? f[(size_t)j * R + i] : mk((T)0, (T)0);
    };
    const cpx<T> v00 = at(i0, j0), v01 = at(i0 + 1, j0), v10 = at(i0, j0 + 1), v11 = at(i0 + 1, j0 + 1);
    const T w00 = (1 - a) * (1 - e), w01 = a * (1 - e), w10 = (1 - a) * e, w11 = a * e;
    dst[(size_t)b * R * R + (size_t)iv * R + iu] =
        mk(w00 * v00.re + w01 * v01.re + w10 * v10.re + w11 * v11.re,
           w00 * v00.im + w01 * v01.im + w10 * v10.im + w11 * v11.im);
}

template <class T>
void launch_rotate_fields(int R, float c, float s, const cpx<T>* src, cpx<T>* dst, cudaStream_t st) {
    dim3 grid(blocks_for(R, 128), R, 2);
    rotate_fields_kernel<T><<<grid, 128, 0, st>>>(R, c, s, src, dst);
}

// Loads every kernel of this file (cudaFuncGetAttributes), see preload_kernels.
template <class T>
static void preload_nearfield_t() {
    cudaFuncAttributes a;
    cudaFuncGetAttributes(&a, uf_kernel<T>);
    cudaFuncGetAttributes(&a, lut_build_kernel<T>);
    cudaFuncGetAttributes(&a, phase_kernel<T>);
    cudaFuncGetAttributes(&a, us_sh_kernel<T>);
    cudaFuncGetAttributes(&a, sum_only_kernel<T>);
    cudaFuncGetAttributes(&a, rotate_fields_kernel<T>);
}
void preload_nearfield_kernels() {
    preload_nearfield_t<float>();
    preload_nearfield_t<double>();
    cudaFuncAttributes a;
    cudaFuncGetAttributes(&a, uf_table_kernel);
    cudaFuncGetAttributes(&a, mie_kernel);
    cudaFuncGetAttributes(&a, coef_rows_batch_kernel);
    cudaFuncGetAttributes(&a, legendre_table_kernel);
    cudaFuncGetAttributes(&a, us_lut_f64_kernel);
    cudaFuncGetAttributes(&a, us_lut_tex_kernel<false, 1>);
    cudaFuncGetAttributes(&a, us_lut_tex_kernel<true, 1>);
    cudaFuncGetAttributes(&a, us_lut_tex_kernel<true, 2>);
    cudaFuncGetAttributes(&a, lut_build_tex_batch_kernel);
    cudaFuncGetAttributes(&a, sh_recur_kernel);
    cudaFuncGetAttributes(&a, sh_wave_kernel);
    cudaFuncGetAttributes(&a, sh_coef_kernel);
}

#define BS_INST(T)                                                                                              \
    template void launch_rotate_fields<T>(int, float, float, const cpx<T>*, cpx<T>*, cudaStream_t);             \
    template void launch_uf<T>(const Scene&, const double*, const double*, cpx<T>*, cudaStream_t);              \
    template void launch_lut_build<T>(const zd*, int, int, const double*, int, int, Patch<T>*, cudaStream_t);   \
    template void launch_phase<T>(const Scene&, const Sphere*, const double*, cpx<T>*, float4*, cudaStream_t);  \
    template void launch_us_sh<T>(const Scene&, const Sphere*, int, const zd*, const zd*, const double2*,       \
                                  const zd*, const cpx<T>*, cpx<T>*, cudaStream_t);                           \
    template void launch_sum_only<T>(const Scene&, const Sphere*, const cpx<T>*, cpx<T>*, cudaStream_t);
BS_INST(float)
BS_INST(double)

}  // namespace bs
