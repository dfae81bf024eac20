// fftw3.h -- TEST INFRASTRUCTURE: a stand-in for the few FFTW 3 calls that the
// reference's Kramers-Kronig routine makes (rts/optics/material.h:257-432,
// material::computeN, compiled only when FFTW_AVAILABLE is defined), so that
// oracle/ref_shim.cpp can run that routine in place; FFTW itself is not in
// this image.  Only the documented semantics of those calls are provided:
// fftw_plan_dft_1d plans an unnormalised one-dimensional complex DFT of n
// points, out[k] = sum_j in[j] exp(sign 2 pi i j k / n) with FFTW_FORWARD = -1
// and FFTW_BACKWARD = +1, and fftw_execute runs it.  The transform here is the
// direct O(n^2) sum in double precision with exact twiddle angles (j k reduced
// modulo n), for the small sizes the checks use.  Never part of the product.
#ifndef BS_REF_FFTW3_H
#define BS_REF_FFTW3_H

#include <cmath>
#include <cstdlib>
#include <vector>

typedef double fftw_complex[2];

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)

struct bs_fftw_plan_s {
    int n, sign;
    fftw_complex *in, *out;
};
typedef bs_fftw_plan_s* fftw_plan;

inline void* fftw_malloc(size_t n) { return std::malloc(n); }
inline void fftw_free(void* p) { std::free(p); }

inline fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned) {
    return new bs_fftw_plan_s{n, sign, in, out};
}

inline void fftw_execute(const fftw_plan p) {
    const int n = p->n;
    std::vector<double> re(n), im(n);
    const double two_pi = 6.283185307179586476925286766559;
    for (int k = 0; k < n; k++) {
        double sr = 0, si = 0;
        for (int j = 0; j < n; j++) {
            const double a = p->sign * two_pi * (double)(((long long)j * k) % n) / n;
            const double c = std::cos(a), s = std::sin(a);
            sr += p->in[j][0] * c - p->in[j][1] * s;
            si += p->in[j][0] * s + p->in[j][1] * c;
        }
        re[k] = sr;
        im[k] = si;
    }
    for (int k = 0; k < n; k++) {
        p->out[k][0] = re[k];
        p->out[k][1] = im[k];
    }
}

inline void fftw_destroy_plan(fftw_plan p) { delete p; }

#endif
