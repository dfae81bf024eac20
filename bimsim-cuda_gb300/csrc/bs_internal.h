// bs_internal.h -- structures shared by the host code and the CUDA kernels.
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace bs {

// dataTypes.h:17 defines PI = 3.14159f; the kernels and sphere.cpp /
// nearfield.cpp see that float value.
constexpr double PI_REF = 3.1415901184082031250;
// bessjy.cpp:18 / cbessjy.cpp:16 use the double literal 3.14159 to scale
// cylindrical J, Y into spherical functions.
constexpr double PI_BES = 3.14159;
constexpr double TRUE_PI = 3.14159265358979323846;
// nearfield.h:11 EPSILON_FLOAT = 0.000001f
constexpr double EPS_FLOAT = 9.99999997475242707877e-07;
// rts/math/spherical_bessel.h:8-10
constexpr double CONV_MIN = 0.0145;
constexpr double CONV_MAX = 0.4;
constexpr double Y_FLOOR = -1e33;

constexpr int MAX_ORDER = 512;  // largest Nl or field order accepted

// Slice and optics, as seen by every kernel.
struct Scene {
    double A[3], X[3], Y[3];  // near-field quad nf.pos = pos * (2p+1)
    double focus[3];
    double kdir[3];
    double kmag;              // 2*PI_REF/lambda
    double amp;               // nf.A
    double wave_amp;          // subA / nk (MC) or A (plane wave)
    double cos_a, cos_b;      // cos(asin(NA_in)), cos(asin(NA_out)) of the condenser
    int R;                    // near-field pixels per side
    int nk;                   // plane waves used by Us
    int ns;                   // spheres
    int m;                    // incident-field order
    int plane_wave, lut_uf, lut_us, scalar;
    // incident-field LUT (nearfield.cpp:222-283)
    double uf_dmin, uf_dmax;
    int uf_dR;
    int pad_;
};

// Per-sphere data (sphere.h:14-92 plus the LUT geometry of sphere.cpp:222-240).
struct Sphere {
    double p[3];
    double a;
    double n_re, n_im;
    double dmin, dmax, r0;   // r0 = max(a, dmin)
    int Nl, aR, dR, thetaR;
    int64_t usp_off;         // first patch of Usp in the LUT pool
    int64_t uip_off;         // first patch of Uip in the LUT pool
    int coef_off;            // first order of this sphere in the coefficient arrays
    int lin_stride;          // mixed path: row stride of the linear float2 tables (thetaR + 1, even)
    double xs_usp, xs_uip;   // (dR - 1) / (dmax - r0) and (aR - 1) / (a - dmin): radial index scales
};

// Host helpers (bs_host.cpp).
// Material files: parse (sorted by wavelength) and evaluate n + ik at lambda (um), in the
// precision T of the reference's rts::material<T> (float: the CLI's materials; double: the
// instantiation its Kramers-Kronig routine works in).  Instantiated for float and double.
template <class T>
bool material_load(const std::string& text, std::vector<T>& lam, std::vector<T>& re, std::vector<T>& im,
                   std::string& err);
template <class T>
void material_eval(const std::vector<T>& lam, const std::vector<T>& re, const std::vector<T>& im, T l, T& n_re,
                   T& n_im);

struct V3 {
    double x, y, z;
};

struct Quad {
    V3 A, X, Y;
};

Quad quad_from(const double* pmin, const double* pmax, const double* normal);
Quad quad_scale(const Quad& q, double s);
double quad_dist(const Quad& q, V3 p);
double quad_dist_max(const Quad& q, V3 p);
double v3_len(V3 a);
int calc_nl(double a, double lambda);
void mc_sample_compat(int nk, const double* kdir, double na_in, double na_out, double* out);
int envi_add_band(const char* path, const float* band, int samples, int lines, double wavelength,
                  int append, char* err, size_t errlen);

}  // namespace bs
