// ref_shim.cpp -- TEST INFRASTRUCTURE.  Compiled together with the
// reference's own host sources (bessjy.cpp, cbessjy.cpp, gamma.cpp,
// sphere.cpp, montecarlo.cpp, nearfield.cpp, read in place from the
// reference checkout) into oracle/_ref/libref_bimsim.so by oracle/Makefile.
// It gives the oracle checks C entry points into the reference's code and
// supplies no-op bodies for the GPU-side members those sources reference but
// that the checks never call.  No reference code is copied here.
#include <cstdlib>
#include <cstring>
#include <complex>

// material::computeN (the Kramers-Kronig routine) is compiled only with FFTW;
// its calls resolve to the stand-in ref_stub/fftw3.h.  Only this translation
// unit instantiates it.
#define FFTW_AVAILABLE
#include <fftw3.h>

#include "sphere.h"
#include "nearfield.h"
#include "montecarlo.h"
#include "rts/envi/envi.h"

bool verbose = false;

int bessjyv_sph(int v, double z, double& vm, double* cjv, double* cyv, double* cjvp, double* cyvp);
int cbessjyva_sph(int v, std::complex<double> z, double& vm, std::complex<double>* cjv,
                  std::complex<double>* cyv, std::complex<double>* cjvp, std::complex<double>* cyvp);

// ---- members with GPU bodies in the reference's .cu files; never called ----
fieldslice::fieldslice() { R[0] = R[1] = 0; x_hat = y_hat = z_hat = NULL; scalarField = true; }
fieldslice::~fieldslice() {}
void fieldslice::init_gpu() { std::abort(); }
void fieldslice::kill_gpu() {}
scalarslice fieldslice::Mag() { std::abort(); }
scalarslice::~scalarslice() {}
void sphere::scalarUsp(bsComplex*, int, int) { std::abort(); }
void sphere::scalarUip(bsComplex*, int, int) { std::abort(); }
void nearfieldStruct::scalarUf() { std::abort(); }
void nearfieldStruct::scalarUfLut() { std::abort(); }
void nearfieldStruct::scalarUpLut() { std::abort(); }
void nearfieldStruct::scalarUs() { std::abort(); }
void nearfieldStruct::sumUf() { std::abort(); }
void nearfieldStruct::vectorUf() { std::abort(); }
void nearfieldStruct::vectorUfLut() { std::abort(); }

extern "C" {

int ref_bessjyv_sph(int N, double x, double* j, double* y) {
    double vm;
    std::vector<double> jp(N + 2), yp(N + 2), jj(N + 2), yy(N + 2);
    bessjyv_sph(N, x, vm, jj.data(), yy.data(), jp.data(), yp.data());
    for (int l = 0; l <= N; l++) {
        j[l] = jj[l];
        y[l] = yy[l];
    }
    return 0;
}

int ref_cbessjyva_sph(int N, double zr, double zi, double* j, double* y, double* jp, double* yp) {
    double vm;
    std::vector<std::complex<double>> a(N + 2), b(N + 2), c(N + 2), d(N + 2);
    cbessjyva_sph(N, std::complex<double>(zr, zi), vm, a.data(), b.data(), c.data(), d.data());
    for (int l = 0; l <= N; l++) {
        j[2 * l] = a[l].real(); j[2 * l + 1] = a[l].imag();
        y[2 * l] = b[l].real(); y[2 * l + 1] = b[l].imag();
        jp[2 * l] = c[l].real(); jp[2 * l + 1] = c[l].imag();
        yp[2 * l] = d[l].real(); yp[2 * l + 1] = d[l].imag();
    }
    return 0;
}

int ref_calc_nl(float a, float lambda) {
    sphere s(0, 0, 0, a);
    s.calcNl(lambda);
    return s.Nl;
}

// sphere::calcCoeff: A and B as the reference stores them (single precision)
int ref_calc_coeff(float a, float lambda, float nre, float nim, double* A, double* B) {
    sphere s(0, 0, 0, a);
    s.calcNl(lambda);
    s.calcCoeff(lambda, bsComplex(nre, nim));
    for (int l = 0; l <= s.Nl; l++) {
        A[2 * l] = s.A[l].r; A[2 * l + 1] = s.A[l].i;
        B[2 * l] = s.B[l].r; B[2 * l + 1] = s.B[l].i;
    }
    return s.Nl;
}

// sphere::calcHankelLut: rR x (Nl+1) complex (j, y) at r in [max(a,dmin), dmax]
int ref_hankel_lut(float a, float k, float dmin, float dmax, int Nl, int rR, double* h) {
    sphere s(0, 0, 0, a);
    s.Nl = Nl;
    s.d_min = dmin;
    s.d_max = dmax;
    std::vector<bsComplex> t((size_t)rR * (Nl + 1));
    s.calcHankelLut(t.data(), k, rR);
    for (size_t i = 0; i < t.size(); i++) {
        h[2 * i] = t[i].r;
        h[2 * i + 1] = t[i].i;
    }
    return 0;
}

// sphere::calcBesselLut: aR x (Nl+1) complex j_l(k n r), r in [0, a]
int ref_bessel_lut(float a, float k, float nre, float nim, int Nl, int aR, double* j) {
    sphere s(0, 0, 0, a);
    s.Nl = Nl;
    std::vector<bsComplex> t((size_t)aR * (Nl + 1));
    s.calcBesselLut(t.data(), k, bsComplex(nre, nim), aR);
    for (size_t i = 0; i < t.size(); i++) {
        j[2 * i] = t[i].r;
        j[2 * i + 1] = t[i].i;
    }
    return 0;
}

// nearfieldStruct::calcBesselLut: dR x (m+1) real table for the incident field
int ref_uf_bessel_lut(float lambda, int m, float dmin, float dmax, int dR, double* j) {
    nearfieldStruct* nf = new nearfieldStruct();
    nf->lambda = lambda;
    nf->m = m;
    std::vector<float> t((size_t)dR * (m + 1));
    nf->calcBesselLut(t.data(), dmin, dmax, dR);
    for (size_t i = 0; i < t.size(); i++) j[i] = t[i];
    delete nf;
    return 0;
}

// nearfieldStruct::calcWaves: srand(NULL) then mcSampleNA (nearfield.cpp:96-108)
int ref_mc_sample(int nk, float kx, float ky, float kz, float na_in, float na_out, double* out) {
    std::vector<bsVector> w(nk);
    srand(0);
    mcSampleNA(&w[0], nk, bsVector(kx, ky, kz), na_in, na_out);
    for (int i = 0; i < nk; i++)
        for (int c = 0; c < 3; c++) out[3 * i + c] = w[i][c];
    return 0;
}

int ref_rand(unsigned seed, int n, int* out) {
    srand(seed);
    for (int i = 0; i < n; i++) out[i] = rand();
    return 0;
}

// rts::quad<float,3>(pMin, pMax, n) * scale, then dist/dist_max to a point
int ref_quad_dist(const float* pmin, const float* pmax, const float* nrm, float scale, const float* pt,
                  float* dmin, float* dmax) {
    rts::quad<float, 3> q(bsPoint(pmin[0], pmin[1], pmin[2]), bsPoint(pmax[0], pmax[1], pmax[2]),
                          bsVector(nrm[0], nrm[1], nrm[2]));
    q = q * scale;
    bsPoint p(pt[0], pt[1], pt[2]);
    *dmin = q.dist(p);
    *dmax = q.dist_max(p);
    return 0;
}

// rts::material<ptype>(filename).getN(lambda) (material.h:470-480, 617-621)
int ref_material_eval(const char* path, int n, const double* lambdas, double* out) {
    rts::material<ptype> m{std::string(path)};
    for (int i = 0; i < n; i++) {
        rts::complex<ptype> c = m.getN((ptype)lambdas[i]);
        out[2 * i] = c.real();
        out[2 * i + 1] = c.imag();
    }
    return 0;
}

// rts::material<double>(filename).computeN(n0, n_samples, pf) (material.h:257-432):
// the returned material's samples (wavelength, n, kappa), increasing in
// wavelength, n_samples of them (0: the file's count).  The double
// instantiation is the one whose arrays match FFTW's double transforms.
int ref_material_kk(const char* path, double n0, int n_samples, double pf, double* lambdas, double* n_out) {
    rts::material<double> m{std::string(path)};
    rts::material<double> kk = m.computeN(n0, (unsigned)n_samples, pf);
    kk.setN0(0.0);  // getF adds n0 to every stored value
    rts::function<double, rts::complex<double>> f = kk.getF();
    for (unsigned i = 0; i < f.getN(); i++) {
        lambdas[i] = f.getX(i);
        n_out[2 * i] = f.getY(i).real();
        n_out[2 * i + 1] = f.getY(i).imag();
    }
    return (int)f.getN();
}

// scalarslice::toEnvi's file handling (scalarslice.cu:146-166)
int ref_envi_add_band(const char* path, const float* band, int samples, int lines, double wavelength, int append) {
    EnviFile f(path, append ? "a" : "w");
    f.addBand((void*)band, samples, lines, wavelength);
    f.close();
    return 0;
}

}  // extern "C"
