// bs_kernels.h -- launchers of the CUDA kernels (bs_nearfield.cu, bs_detector.cu).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

#include "bs_internal.h"

namespace bs {

// Plane waves are processed in chunks of 64, 32 or 16 (chosen per run from the
// predicted fraction of staged windows) after grouping them by direction; the
// host supplies one bounding cone per chunk.
constexpr int WAVE_CHUNK_MAX = 64;

// Mixed LUT kernel staging: float2 table values a 16 x 16 pixel tile stages
// per wave chunk, and the angle margin (radians) added to its window bounds.
// 64-wave chunks (two pixels per thread, 128 registers): 51 KB, 4 blocks per
// SM (config 2: 99.6 % of windows staged; 43 KB: 98 %, 730 against 721 ms);
// 32- and 16-wave chunks (one pixel per thread, coarser pixel pitches): 72 KB,
// 3 blocks per SM, so that wider windows fit -- config 3 266 against 305 ms
// per band, config 5 at 512^2 9.9 against 11.7 s, both with 32-wave chunks
// where 43 KB windows needed 16.
constexpr int LUT_TILE = 16;
__host__ __device__ constexpr int lut_stage_entries(int chunk) { return chunk >= 64 ? 6400 : 9000; }
constexpr float LUT_STAGE_MARGIN = 2e-3f;
// Shared-memory row stride of a staged window W entries wide: odd, so that
// lanes reading the same column of different rows fall in different banks.
__host__ __device__ constexpr int lut_stage_stride(int W) { return W | 1; }

template <class T>
struct cpx;
using zd = cpx<double>;

// Load every kernel of the library into the current device's context now: with
// CUDA's default lazy loading a kernel is loaded at its first launch, and a load
// while other streams' kernels run waits for them (a served request that was the
// first to use a kernel waited for the long slices on the other workers' streams:
// p50 8.3 s against 1.9 s with every kernel loaded up front).
void preload_nearfield_kernels();
void preload_detector_kernels();

// One bilinear LUT cell at (r, t): {T00, T10 - T00, T01 - T00, T11 - T10 - T01 + T00}
// as (re, im) pairs, so that T(r + a, t + b) = (v0 + a v1) + b (v2 + a v3).
template <class T>
struct alignas(8 * sizeof(T)) Patch {
    T v[8];
};

// ---- near field ----
template <class T>
void launch_uf(const Scene& sc, const double* tab, const double* w, cpx<T>* Uf, cudaStream_t st);
void launch_uf_table(const Scene& sc, double* tab, double* scratch, cudaStream_t st);
void launch_mie(const Sphere* sph, int ns, double k, zd* scratch, int lstride, zd* A, zd* B, cudaStream_t st);
// spheres [s0, s0 + n) in one launch; starts (device): first global row of each
// sphere (n + 1 values, the last = total_rows) then first coefficient (n values)
void launch_coef_rows_batch(const Sphere* sph, int s0, int n, const long long* starts, long long total_rows,
                            double k, const zd* A, const zd* B, zd* tab, double* scratch, cudaStream_t st);
void launch_legendre_table(int thetaR, int Lmax, double* P, cudaStream_t st);
template <class T>
void launch_lut_build(const zd* tab, int rows, int L, const double* P, int Pstride, int thetaR, Patch<T>* out,
                      cudaStream_t st);
template <class T>
void launch_phase(const Scene& sc, const Sphere* sph, const double* waves, cpx<T>* ph, float4* kw4, cudaStream_t st);
void launch_us_lut_f64(const Scene& sc, const Sphere* sph, int s0, int s1, int accumulate, int finalize,
                       const double* waves, const zd* ph, const Patch<double>* lut, const zd* Uf, zd* U,
                       cudaStream_t st);
// mixed path: tex holds, for sphere s0 + j, the texture objects of
// {Usp re, Usp im, Uip re, Uip im} at [4 j .. 4 j + 3]
// lin: linear float2 tables (Sphere::usp_off / uip_off in float2 units, rows
// of Sphere::lin_stride entries);
// cones: one {axis, half-angle} per `chunk` waves; counters[0..1] receive
// the staged and total (sphere, chunk) counts of every block (may be null);
// kcmp (R x R, or null with a single sphere chunk) carries each pixel's Kahan
// compensation from one sphere chunk's launch to the next, so that chunked
// tables give the bits of one launch over all spheres;
// stage = false runs the texture-only variant
void launch_us_lut_tex(const Scene& sc, const Sphere* sph, int s0, int s1, int accumulate, int finalize,
                       const float4* kw4, const float4* cones, const cpx<float>* ph, const unsigned long long* tex,
                       const float2* lin, const cpx<float>* Uf, cpx<float>* U, unsigned long long* counters,
                       float2* kcmp, bool stage, int chunk, cudaStream_t st);
// One table of the mixed path's table build: the rows (one spare) of one
// sphere's Usp or Uip with their coefficient rows at tab + tab_off, written to
// the planes sre/sim and the linear rows at lin + lin_off.
struct LutBuildJob {
    long long tab_off, lin_off;
    int rows, L, thetaR, lin_stride;
    cudaSurfaceObject_t sre, sim;
};
// the tables of `jobs` (device array of njobs <= 65535 entries, at most max_rows
// rows and max_theta angles each) in one launch: the sums of launch_lut_build in
// double, stored as float in the real and imaginary planes (CUDA arrays, through
// surfaces) and in the linear rows used for staging
void launch_lut_build_tex_batch(const LutBuildJob* jobs, int njobs, int max_rows, int max_theta, const zd* tab,
                                const double* P, int Pstride, float2* lin, cudaStream_t st);

// Direct scattered field through the addition theorem of spherical harmonics:
// recurrence factors rec, per-wave tables tab (nk x L(L+1)/2), per-sphere
// coefficients coef (ns x L(L+1)/2 x 2 complex), then the per-pixel sum.
void launch_sh_tables(const Scene& sc, const Sphere* sph, int L, const double* waves, double2* rec, double2* tab,
                      zd* coef, cudaStream_t st);
template <class T>
void launch_us_sh(const Scene& sc, const Sphere* sph, int L, const zd* A, const zd* B, const double2* rec,
                  const zd* coef, const cpx<T>* Uf, cpx<T>* U, cudaStream_t st);
template <class T>
void launch_sum_only(const Scene& sc, const Sphere* sph, const cpx<T>* Uf, cpx<T>* U, cudaStream_t st);
// U and Uf (src: U then Uf, R x R each) rotated about the slice centre into dst;
// c, s: cosine and sine of the angle
template <class T>
void launch_rotate_fields(int R, float c, float s, const cpx<T>* src, cpx<T>* dst, cudaStream_t st);

// ---- detector ----
// twiddles: out[i * ld_i + j * ld_j] = exp(sign 2 pi i ((off_i + i) * freq[j] mod R) / R)
template <class T>
void launch_twiddle(int ni, int nj, const int* freq, int off_i, int R, int sign, int ld_i, int ld_j, cpx<T>* out,
                    cudaStream_t st);

// C[b] (M x N) = A[b] (M x K) * B[b] (K x N), complex, row-major, batch over
// blockIdx.z with element strides sA, sB, sC (0 = shared operand).
// epi 0: store; epi 1: multiply by mask[m*N + n]; epi 2: store |scale * c|^2
// into the real array I[b] (M x N, batch stride sC); epi 3: store scale * c.
// GEMMs with fewer output tiles than SMs split K over more blocks and add the
// parts in a fixed order (deterministic) when `scratch` holds
// cgemm_scratch_elems(M, N, K, batch) elements; else one block per tile.
size_t cgemm_scratch_elems(int M, int N, int K, int batch);
template <class T>
void launch_cgemm(int M, int N, int K, int batch, const cpx<T>* A, int lda, long long sA, const cpx<T>* B, int ldb,
                  long long sB, cpx<T>* C, int ldc, long long sC, int epi, const float* mask, T scale, T* I,
                  cpx<T>* scratch, size_t scratch_elems, cudaStream_t st);

// D[b][iv][iu] (+)= sum over the ss x ss block of I[b] / ss^2 (fieldslice.cu:71-108);
// accumulate adds to D (the detector sums point sources)
template <class T>
void launch_bin(int res, int ss, int batch, int accumulate, const T* I, T* D, cudaStream_t st);

// Ring point sources on the detector (microscope.cu:37-250): dst[b] += src[b]
// rotated by (c, s) about ((int)(res/2), (int)(res/2)), b = 0, 1; line[b][r] +=
// the tree sum of src[b] at radius r, angles with (cos, sin) cs[k], k < points
// (points <= 1023); D[b] = line[b] interpolated at each pixel's radius.
template <class T>
void launch_rotate_add_images(int res, float c, float s, const T* src, T* dst, cudaStream_t st);
template <class T>
void launch_ring_line(int res, int points, int L, const float2* cs, const T* img, T* line, cudaStream_t st);
template <class T>
void launch_line_image(int res, int L, const T* line, T* D, cudaStream_t st);

// Real part of the reference's FFT Hilbert transform of chi2 (N samples zero-padded
// to M) at the first N points, chi1; g is scratch of M doubles.
void launch_kk(int N, int M, const double* chi2, double* g, double* chi1, cudaStream_t st);

// x[i] *= a[i], i < n (complex)
template <class T>
void launch_cmul(int n, const cpx<T>* a, cpx<T>* x, cudaStream_t st);

// image kinds 2, 3: -log10(D/Di), D/Di (microscope.cu:722-775); 0, 1: copies
template <class T>
void launch_image(int n, int kind, const T* D, const T* Di, T* out, cudaStream_t st);

}  // namespace bs
