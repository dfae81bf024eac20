/*
 * bimsim_oracle.h -- TEST INFRASTRUCTURE, not product code.
 *
 * Double-precision CPU restatement of the reference's near-field-to-detector
 * path (seberisha/bimsim-cuda).  Only tests/, __graft_entry__.smoke() and
 * bench.py (cpu_baseline leg and --impl reference arm) may load it, and only
 * as the checker or the timed CPU baseline.  The CUDA library never links it.
 *
 * Every function follows a reference file:line, cited at its definition.
 */
#ifndef BIMSIM_ORACLE_H
#define BIMSIM_ORACLE_H

#include "../include/bimsim_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Geometry derived from bs_params, as LoadParameters/setNearfield/calcSpheres
 * derive it (arguments.h:340-438, microscope.cu:700-718, sphere.cpp:222-240). */
typedef struct bso_geom {
    int32_t R;               /* near-field pixels per side */
    int32_t det_res;         /* detector pixels per side   */
    int32_t crop_res;        /* res*ss                      */
    int32_t crop_off;        /* padding*res*ss              */
    double A[3], X[3], Y[3]; /* near-field quad nf.pos      */
    double kmag;             /* 2*PI/lambda with PI=3.14159f */
    double sub_amp;          /* subA (nfScalarUpLut.cu:378) */
    double cos_alpha, cos_beta;
} bso_geom;

/* Per-sphere derived sizes (sphere.cpp:222-240, sphere.h:71-74). */
typedef struct bso_sphere_geom {
    int32_t Nl;
    int32_t aR, dR, thetaR;
    double d_min, d_max;
} bso_sphere_geom;

int bso_derive(const bs_params* p, bso_geom* g);
int bso_sphere_derive(const bs_params* p, const bs_sphere* s, bso_sphere_geom* out);

/* Nl = ceil(ka + 4 (ka)^(1/3) + 2) in single precision (sphere.h:71-74). */
int bso_calc_nl(double a, double lambda);

/* Spherical Bessel j_l, y_l (l = 0..N) of a real argument, scaled as the
 * reference's bessjyv_sph returns them (bessjy.cpp:709-728). */
int bso_sbessel_real(int N, double x, double* j, double* y);

/* Complex spherical Bessel j_l, y_l and derivatives as cbessjyva_sph
 * (cbessjy.cpp:718-737) returns them; `typo` reproduces cbessjy.cpp:541. */
int bso_sbessel_complex(int N, double zr, double zi, int typo,
                        double* j, double* y, double* jp, double* yp);

/* Mie coefficients A_l, B_l, l = 0..Nl, interleaved complex (sphere.cpp:21-97). */
int bso_mie(double k, double a, double n_re, double n_im, int Nl, double* A, double* B);

/* glibc rand() sequence after srand(seed), restated (TYPE_3 additive generator). */
int bso_glibc_rand(unsigned seed, int n, int* out);

/* Monte Carlo aperture samples exactly as mcSampleNA after srand(0)
 * (montecarlo.cpp:9-71, nearfield.cpp:96-108), single precision. */
int bso_mc_sample(int nk, const double* kdir, double na_in, double na_out, double* out);

/* Per-sphere tables: Usp (dR x thetaR) and Uip (aR x thetaR) complex,
 * radial-major [r][theta] (values of sphere.cu:4-99). */
int bso_sphere_luts(const bs_params* p, const bs_sphere* s, double* usp, double* uip);

/* Uf Bessel table (dR x (m+1)) of nearfieldStruct::calcBesselLut
 * (nearfield.cpp:222-283), with its d_min/d_max. */
int bso_uf_table(const bs_params* p, double* table, double* d_min, double* d_max);

/* Full path.  U, Uf: R*R interleaved complex near fields after sumUf
 * (before the detector); D, Di: det_res^2 detector images.  Any output may
 * be NULL.  nthreads <= 0 uses all cores. */
int bso_simulate(const bs_params* p, const bs_sphere* s, int ns,
                 const double* waves, int nk, int nthreads,
                 double* U, double* Uf, double* D, double* Di);

/* Near field only, restricted to pixel rows [row0, row1) (bounded CPU
 * samples for the timed baseline).  U receives (row1-row0)*R complex. */
int bso_nearfield_rows(const bs_params* p, const bs_sphere* s, int ns,
                       const double* waves, int nk, int nthreads,
                       int row0, int row1, double* U);

/* Detector chain on given near fields (microscope.cu:608-662, 722-814). */
int bso_detector(const bs_params* p, const double* U, const double* Uf, double* D, double* Di);
/* The band of bso_nearfield_rows with its CPU time split into scene set-up,
 * the complete LUTs and the band itself (times[3], seconds). */
int bso_nearfield_rows_timed(const bs_params* p, const bs_sphere* s, int ns, const double* waves, int nk,
                             int nthreads, int row0, int row1, double* U, double* times);
/* Far field Ud (crop_res^2 complex, interleaved): band-passed U on the crop, scaled by 1/R^2. */
int bso_far_field(const bs_params* p, const double* U, double* out);

/* Ring point sources, mode 1 (detector images rotated, microscope.cu:1004-1093),
 * 2 (radial line of ring samples, :1097-1183) or 3 (near fields rotated,
 * :1189-1253 with nfInterpolate.cu); D, Di: det_res^2 detector images. */
int bso_simulate_rings(const bs_params* p, const bs_sphere* s, int ns, const double* waves, int nk, int nthreads,
                       int mode, int points, int rings, double* D, double* Di);

/* Kramers-Kronig real index from kappa at the resampled wavelengths
 * (material::computeN, rts/optics/material.h:257-432): n_out[N]. */
int bso_kk_transform(int N, int pf, double n0, const double* lambdas, const double* kappas, double* n_out);

/* Detector with applyBackpropagation (microscope.cu:423-470, 592-605) over
 * distance d applied to U before the band-pass. */
int bso_detector_bp(const bs_params* p, const double* U, const double* Uf, double d, double* D, double* Di);

/* Forward (sign=-1) or inverse (sign=+1, unnormalised) 1-D DFT of n complex. */
int bso_fft(int n, int sign, double* data);

/* ENVI band writer restated from rts/envi/envi.h:196-433 and
 * rts/envi/envi_header.h:318-375 (float32 BSQ). */
int bso_envi_add_band(const char* path, const float* band, int samples, int lines,
                      double wavelength, int append);

#ifdef __cplusplus
}
#endif

#endif
