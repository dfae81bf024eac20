// bs_detector.cu -- the objective band-pass and detector
// (microscope.cu:495-526, 608-662, 722-814; fieldslice.cpp:25-94;
// fieldslice.cu:71-108, 141-150, 319-338).
//
// The reference runs four full R x R cuFFTs per slice, zeroes every frequency
// outside the objective's annulus |f| in [NA_in, NA_out]/lambda, and keeps only
// the central (res*ss)^2 crop of the inverse.  With realistic sampling the
// passband holds a few hundred of R bins per axis, so here the transform is a
// band-limited (pruned) DFT: forward along x for the passband columns only,
// forward along y for the passband rows only, mask, then inverse along x and
// y for the crop only, each stage a small complex GEMM against exact twiddle
// tables.  |.|^2, 1/R^2 scaling and the ss x ss detector integration are fused
// at the end.
#include <cuda_runtime.h>

#include <algorithm>

#include "bs_kernels.h"
#include "bs_math.cuh"

namespace bs {

template <class T>
__global__ void twiddle_kernel(int ni, int nj, const int* __restrict__ freq, int off_i, int R, int sign, int ld_i,
                               int ld_j, cpx<T>* __restrict__ out) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)ni * nj) return;
    int i = (int)(e / nj), j = (int)(e % nj);
    long long m = ((long long)(off_i + i) * (long long)freq[j]) % R;
    double s, c;
    sincospi(2.0 * (double)m / (double)R, &s, &c);
    out[(long long)i * ld_i + (long long)j * ld_j] = mk((T)c, (T)(sign * s));
}

// Tiled complex GEMM.  Block 16 x 16 threads, tile BM x BN = 64 x 32, each
// thread 4 x 2 outputs, BK = 16.  Float accumulation is split into per-tile
// partial sums combined with Kahan compensation.
constexpr int GB_M = 64, GB_N = 32, GB_K = 16;

// Epilogue of one output element c of batch b: epi 0 store, 1 store times the
// band-pass mask, 2 |scale c|^2 into I, 3 store scale c.
template <class T>
__device__ __forceinline__ void cgemm_store(int epi, long long o, int gm, int gn, int N, T vr, T vi,
                                            cpx<T>* __restrict__ C, const float* __restrict__ mask, T scale,
                                            T* __restrict__ I) {
    if (epi == 2) {
        vr *= scale;
        vi *= scale;
        I[o] = vr * vr + vi * vi;
    } else if (epi == 3) {  // scaled field (the far field Ud, Ufd)
        C[o] = mk(vr * scale, vi * scale);
    } else {
        if (epi == 1) {
            T mval = (T)mask[(long long)gm * N + gn];
            vr *= mval;
            vi *= mval;
        }
        C[o] = mk(vr, vi);
    }
}

// ksplit > 1 (few output tiles, long K): block z = b * ksplit + ks sums the
// ks-th of ksplit equal K ranges into part[b][ks][M][N]; cgemm_reduce_kernel
// adds the ranges in order (deterministic) and applies the epilogue.
template <class T>
__global__ void __launch_bounds__(256) cgemm_kernel(int M, int N, int K, const cpx<T>* __restrict__ A, int lda,
                                                    long long sA, const cpx<T>* __restrict__ B, int ldb, long long sB,
                                                    cpx<T>* __restrict__ C, int ldc, long long sC, int epi,
                                                    const float* __restrict__ mask, T scale, T* __restrict__ I,
                                                    int ksplit, cpx<T>* __restrict__ part) {
    __shared__ cpx<T> As[GB_K][GB_M + 1];
    __shared__ cpx<T> Bs[GB_K][GB_N + 1];
    const int b = blockIdx.z / ksplit, ks = blockIdx.z % ksplit;
    A += b * sA;
    B += b * sB;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * GB_M, n0 = blockIdx.x * GB_N;
    const int kc = ((K + ksplit - 1) / ksplit + GB_K - 1) / GB_K * GB_K;  // K range per split, whole tiles
    const int kbeg = ks * kc, kend = min(K, kbeg + kc);
    T accr[4][2], acci[4][2], cr[4][2], ci[4][2];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 2; j++) accr[i][j] = acci[i][j] = cr[i][j] = ci[i][j] = 0;
    for (int k0 = kbeg; k0 < kend; k0 += GB_K) {
        for (int e = threadIdx.x; e < GB_K * GB_M; e += 256) {
            int kk = e % GB_K, mm = e / GB_K;
            int gm = m0 + mm, gk = k0 + kk;
            As[kk][mm] = (gm < M && gk < kend) ? A[(long long)gm * lda + gk] : mk((T)0, (T)0);
        }
        for (int e = threadIdx.x; e < GB_K * GB_N; e += 256) {
            int nn = e % GB_N, kk = e / GB_N;
            int gn = n0 + nn, gk = k0 + kk;
            Bs[kk][nn] = (gn < N && gk < kend) ? B[(long long)gk * ldb + gn] : mk((T)0, (T)0);
        }
        __syncthreads();
        T pr[4][2], pi[4][2];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 2; j++) pr[i][j] = pi[i][j] = 0;
#pragma unroll
        for (int kk = 0; kk < GB_K; kk++) {
            cpx<T> a[4], bb[2];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 2; j++) bb[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 2; j++) {
                    pr[i][j] += a[i].re * bb[j].re - a[i].im * bb[j].im;
                    pi[i][j] += a[i].re * bb[j].im + a[i].im * bb[j].re;
                }
        }
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 2; j++) {  // Kahan step
                T yr = pr[i][j] - cr[i][j], yi = pi[i][j] - ci[i][j];
                T trr = accr[i][j] + yr, tii = acci[i][j] + yi;
                cr[i][j] = (trr - accr[i][j]) - yr;
                ci[i][j] = (tii - acci[i][j]) - yi;
                accr[i][j] = trr;
                acci[i][j] = tii;
            }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 2; j++) {
            int gm = m0 + ty + 16 * i, gn = n0 + tx + 16 * j;
            if (gm >= M || gn >= N) continue;
            if (ksplit > 1)
                part[((long long)blockIdx.z * M + gm) * N + gn] = mk(accr[i][j], acci[i][j]);
            else
                cgemm_store(epi, b * sC + (long long)gm * ldc + gn, gm, gn, N, accr[i][j], acci[i][j], C, mask, scale,
                            I);
        }
}

template <class T>
__global__ void cgemm_reduce_kernel(int M, int N, int batch, int ksplit, const cpx<T>* __restrict__ part,
                                    cpx<T>* __restrict__ C, int ldc, long long sC, int epi,
                                    const float* __restrict__ mask, T scale, T* __restrict__ I) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)batch * M * N) return;
    const int b = (int)(e / ((long long)M * N)), gm = (int)(e / N % M), gn = (int)(e % N);
    T sr = 0, si = 0, cr = 0, ci = 0;  // Kahan over the K ranges, in order
    for (int ks = 0; ks < ksplit; ks++) {
        const cpx<T> v = part[(((long long)b * ksplit + ks) * M + gm) * N + gn];
        const T yr = v.re - cr, yi = v.im - ci;
        const T tr = sr + yr, ti = si + yi;
        cr = (tr - sr) - yr;
        ci = (ti - si) - yi;
        sr = tr;
        si = ti;
    }
    cgemm_store(epi, b * sC + (long long)gm * ldc + gn, gm, gn, N, sr, si, C, mask, scale, I);
}

template <class T>
__global__ void bin_kernel(int res, int ss, int accumulate, const T* __restrict__ I, T* __restrict__ D) {
    int b = blockIdx.y;
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= res * res) return;
    int iu = e % res, iv = e / res;
    int cw = res * ss;
    const T* Ib = I + (long long)b * cw * cw;
    T acc = 0;
    for (int ix = 0; ix < ss; ix++)
        for (int iy = 0; iy < ss; iy++) acc += Ib[(long long)(iv * ss + iy) * cw + iu * ss + ix];
    // accumulate: the detector sums over point sources (IntegrateAndResample adds, fieldslice.cu:71-108)
    T* out = D + (long long)b * res * res + e;
    *out = (accumulate ? *out : (T)0) + acc / (T)(ss * ss);
}

template <class T>
__global__ void image_kernel(int n, int kind, const T* __restrict__ D, const T* __restrict__ Di, T* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (kind == 0) out[i] = D[i];
    else if (kind == 1) out[i] = Di[i];
    else if (kind == 2) out[i] = -log10(D[i] / Di[i]);
    else out[i] = D[i] / Di[i];
}

template <class T>
void launch_twiddle(int ni, int nj, const int* freq, int off_i, int R, int sign, int ld_i, int ld_j, cpx<T>* out,
                    cudaStream_t st) {
    long long n = (long long)ni * nj;
    if (n == 0) return;
    twiddle_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(ni, nj, freq, off_i, R, sign, ld_i, ld_j, out);
}

// Splits of K for a GEMM with few output tiles: enough blocks for about two per
// SM, each split at least 4 K tiles long, at most 64 splits.
int cgemm_ksplit(int M, int N, int K, int batch) {
    int dev = 0, n_sm = 1;  // attribute queries are cheap host calls; no shared cache between threads
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) !=
                                                   cudaSuccess)
        n_sm = 1;
    const long long tiles = (long long)((N + GB_N - 1) / GB_N) * ((M + GB_M - 1) / GB_M) * batch;
    if (tiles <= 0 || tiles >= n_sm) return 1;
    long long ks = (2LL * n_sm + tiles - 1) / tiles;
    ks = std::min<long long>(ks, std::max(1, K / (4 * GB_K)));
    return (int)std::min<long long>(ks, 64);
}

size_t cgemm_scratch_elems(int M, int N, int K, int batch) {
    const int ks = cgemm_ksplit(M, N, K, batch);
    return ks > 1 ? (size_t)batch * ks * M * N : 0;
}

template <class T>
void launch_cgemm(int M, int N, int K, int batch, const cpx<T>* A, int lda, long long sA, const cpx<T>* B, int ldb,
                  long long sB, cpx<T>* C, int ldc, long long sC, int epi, const float* mask, T scale, T* I,
                  cpx<T>* scratch, size_t scratch_elems, cudaStream_t st) {
    int ks = cgemm_ksplit(M, N, K, batch);
    if ((size_t)batch * ks * M * N > scratch_elems || !scratch) ks = 1;
    dim3 grid((N + GB_N - 1) / GB_N, (M + GB_M - 1) / GB_M, batch * ks);
    cgemm_kernel<T><<<grid, 256, 0, st>>>(M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC, epi, mask, scale, I, ks,
                                          scratch);
    if (ks > 1) {
        const long long n = (long long)batch * M * N;
        cgemm_reduce_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(M, N, batch, ks, scratch, C, ldc, sC, epi,
                                                                            mask, scale, I);
    }
}

template <class T>
void launch_bin(int res, int ss, int batch, int accumulate, const T* I, T* D, cudaStream_t st) {
    dim3 grid((res * res + 255) / 256, batch);
    bin_kernel<T><<<grid, 256, 0, st>>>(res, ss, accumulate, I, D);
}

template <class T>
void launch_image(int n, int kind, const T* D, const T* Di, T* out, cudaStream_t st) {
    image_kernel<T><<<(n + 255) / 256, 256, 0, st>>>(n, kind, D, Di, out);
}

// ---------------------------------------------------------------------------
// Ring point sources on the detector (--interpolate 1 and 2).  The reference
// samples the images through linearly filtered float textures with border
// addressing; here coordinates are formed in single precision as its kernels
// form them (each operation rounded on its own, no fused multiply-add) and the
// bilinear weights are exact, zero outside the image.
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T image_bilinear(const T* __restrict__ f, int res, float x, float y) {
    const float fx = floorf(x), fy = floorf(y);
    const int i0 = (int)fx, j0 = (int)fy;
    const T a = (T)(x - fx), e = (T)(y - fy);
    auto at = [&](int i, int j) -> T {
        return (i >= 0 && i < res && j >= 0 && j < res) ? f[(size_t)j * res + i] : (T)0;
    };
    return (1 - a) * (1 - e) * at(i0, j0) + a * (1 - e) * at(i0 + 1, j0) + (1 - a) * e * at(i0, j0 + 1) +
           a * e * at(i0 + 1, j0 + 1);
}

// InterpolateAndIntegrateUd / Ufd (microscope.cu:89-135): dst[b] += src[b]
// rotated by (c, s) about ((int)(res/2), (int)(res/2)); b = 0: D, 1: Di.
template <class T>
__global__ void rotate_add_images_kernel(int res, float c, float s, const T* __restrict__ src, T* __restrict__ dst) {
    const int iu = blockIdx.x * blockDim.x + threadIdx.x, iv = blockIdx.y, b = blockIdx.z;
    if (iu >= res) return;
    const float uc = (float)(int)(res / 2.0);
    const float du = __fsub_rn((float)iu, uc), dv = __fsub_rn((float)iv, uc);
    const float x = __fsub_rn(__fadd_rn(uc, __fmul_rn(du, c)), __fmul_rn(dv, s));
    const float y = __fadd_rn(__fadd_rn(uc, __fmul_rn(du, s)), __fmul_rn(dv, c));
    const size_t plane = (size_t)res * res;
    dst[b * plane + (size_t)iv * res + iu] += image_bilinear(src + b * plane, res, x, y);
}

// simRing_Ud / simRing_Ufd (microscope.cu:138-250): block (r, b) adds to
// line[b][r] the image samples at (uc + r cos t_k, uc - r sin t_k), k < points,
// summed in the reference's shared-memory tree (steps points/2, ..., 1: with a
// count that is not a power of two some samples never reach the sum).
// cs[k] = (cos t_k, sin t_k) rounded to float.
template <class T>
__global__ void ring_line_kernel(int res, int points, int L, const float2* __restrict__ cs, const T* __restrict__ img,
                                 T* __restrict__ line) {
    extern __shared__ __align__(16) unsigned char ring_smem[];
    T* sh = reinterpret_cast<T*>(ring_smem);
    const int r = blockIdx.x, b = blockIdx.y;
    const float uc = (float)(int)(res / 2.0);
    const T* f = img + (size_t)b * res * res;
    for (int k = threadIdx.x; k < points; k += blockDim.x) {
        const float2 t = cs[k];
        const float x = __fadd_rn(uc, __fmul_rn((float)r, t.x)), y = __fsub_rn(uc, __fmul_rn((float)r, t.y));
        sh[k] = image_bilinear(f, res, x, y);
    }
    __syncthreads();
    for (unsigned step = (unsigned)points / 2; step >= 1; step >>= 1) {
        for (unsigned k = threadIdx.x; k < step; k += blockDim.x) sh[k] += sh[k + step];
        __syncthreads();
    }
    if (threadIdx.x == 0) line[(size_t)b * L + r] += sh[0];
}

// InterpolateAndIntegrateUdFromLine / UfdFromLine (microscope.cu:37-85): the
// detector pixel at distance r = sqrt((iu-uc)^2 + (iv-uc)^2) from the centre
// is line[b] linearly interpolated at r, zero beyond its L entries.
template <class T>
__global__ void line_image_kernel(int res, int L, const T* __restrict__ line, T* __restrict__ D) {
    const int iu = blockIdx.x * blockDim.x + threadIdx.x, iv = blockIdx.y, b = blockIdx.z;
    if (iu >= res) return;
    const float uc = (float)(int)(res / 2.0);
    const float du = __fsub_rn((float)iu, uc), dv = __fsub_rn((float)iv, uc);
    const float r = __fsqrt_rn(__fadd_rn(__fmul_rn(du, du), __fmul_rn(dv, dv)));
    const float fr = floorf(r);
    const int i0 = (int)fr;
    const T a = (T)(r - fr);
    const T* l = line + (size_t)b * L;
    const T v0 = i0 < L ? l[i0] : (T)0, v1 = i0 + 1 < L ? l[i0 + 1] : (T)0;
    D[(size_t)b * res * res + (size_t)iv * res + iu] = (1 - a) * v0 + a * v1;
}

template <class T>
void launch_rotate_add_images(int res, float c, float s, const T* src, T* dst, cudaStream_t st) {
    dim3 grid((res + 127) / 128, res, 2);
    rotate_add_images_kernel<T><<<grid, 128, 0, st>>>(res, c, s, src, dst);
}

template <class T>
void launch_ring_line(int res, int points, int L, const float2* cs, const T* img, T* line, cudaStream_t st) {
    const int threads = points >= 1024 ? 1024 : ((points + 31) / 32) * 32;
    ring_line_kernel<T><<<dim3(L, 2), threads, (size_t)points * sizeof(T), st>>>(res, points, L, cs, img, line);
}

template <class T>
void launch_line_image(int res, int L, const T* line, T* D, cudaStream_t st) {
    dim3 grid((res + 127) / 128, res, 2);
    line_image_kernel<T><<<grid, 128, 0, st>>>(res, L, line, D);
}

// ---------------------------------------------------------------------------
// Kramers-Kronig (material::computeN, rts/optics/material.h:257-432): the
// reference multiplies the FFT of the zero-padded chi2 (M points) by i for
// 0 < f < M/2, by -i for f >= M/2 and by 0 at f = 0, transforms back and
// divides by M.  For real chi2 the real part of that is a circular convolution
// with g(m) = (1/M) (sum_{0<f<M/2} -sin(2 pi f m / M) + sum_{f>=M/2} sin(2 pi f m / M)).
// The sines of a whole period add to zero, so g(m) = -(2/M) sum_{f=1}^{K} sin(2 pi f m / M)
// with K = ceil(M/2) - 1, and the finite sum has the closed form
// sin(K t) sin((K+1) t) / sin(t), t = pi m / M (g(0) = 0).  Each sine is reduced in
// integers to sinpi of a ratio in [0, 1/2], so that rounding the ratio costs one ulp
// relative (near a / M = 1 the rounded ratio would lose the small distance to 1,
// and sin(t) for m = M - 1 is the divisor).  Double precision throughout.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double sinpi_ratio(long long a, long long M) {  // sin(pi a / M), a >= 0
    long long r = a % (2 * M);
    double sign = 1.0;
    if (r >= M) {
        r -= M;
        sign = -1.0;
    }
    if (2 * r > M) r = M - r;
    return sign * sinpi((double)r / (double)M);
}

__global__ void kk_kernel_g(int M, double* __restrict__ g) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    if (m == 0) {
        g[0] = 0;
        return;
    }
    const long long K = (M + 1) / 2 - 1;
    const double num = sinpi_ratio(K * m, M) * sinpi_ratio((K + 1) * m, M);
    g[m] = -2.0 * (num / sinpi_ratio(m, M)) / (double)M;
}

__global__ void kk_kernel_conv(int N, int M, const double* __restrict__ chi2, const double* __restrict__ g,
                               double* __restrict__ chi1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double acc = 0;
    for (int j = 0; j < N; j++) acc += chi2[j] * g[(i - j + M) % M];
    chi1[i] = acc;
}

void launch_kk(int N, int M, const double* chi2, double* g, double* chi1, cudaStream_t st) {
    kk_kernel_g<<<(M + 127) / 128, 128, 0, st>>>(M, g);
    kk_kernel_conv<<<(N + 127) / 128, 128, 0, st>>>(N, M, chi2, g, chi1);
}

// x[i] *= a[i] for complex arrays (applyBackpropagation's phase on the passband spectrum)
template <class T>
__global__ void cmul_kernel(int n, const cpx<T>* __restrict__ a, cpx<T>* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const cpx<T> p = a[i], q = x[i];
    x[i] = mk(p.re * q.re - p.im * q.im, p.re * q.im + p.im * q.re);
}

template <class T>
void launch_cmul(int n, const cpx<T>* a, cpx<T>* x, cudaStream_t st) {
    if (n > 0) cmul_kernel<T><<<(n + 255) / 256, 256, 0, st>>>(n, a, x);
}

// Loads every kernel of this file (cudaFuncGetAttributes), see preload_kernels.
template <class T>
static void preload_detector_t() {
    cudaFuncAttributes a;
    cudaFuncGetAttributes(&a, twiddle_kernel<T>);
    cudaFuncGetAttributes(&a, cgemm_kernel<T>);
    cudaFuncGetAttributes(&a, cgemm_reduce_kernel<T>);
    cudaFuncGetAttributes(&a, bin_kernel<T>);
    cudaFuncGetAttributes(&a, image_kernel<T>);
    cudaFuncGetAttributes(&a, rotate_add_images_kernel<T>);
    cudaFuncGetAttributes(&a, ring_line_kernel<T>);
    cudaFuncGetAttributes(&a, line_image_kernel<T>);
    cudaFuncGetAttributes(&a, cmul_kernel<T>);
}
void preload_detector_kernels() {
    preload_detector_t<float>();
    preload_detector_t<double>();
    cudaFuncAttributes a;
    cudaFuncGetAttributes(&a, kk_kernel_g);
    cudaFuncGetAttributes(&a, kk_kernel_conv);
}

#define BS_DET_INST(T)                                                                                          \
    template void launch_twiddle<T>(int, int, const int*, int, int, int, int, int, cpx<T>*, cudaStream_t);      \
    template void launch_cgemm<T>(int, int, int, int, const cpx<T>*, int, long long, const cpx<T>*, int,       \
                                  long long, cpx<T>*, int, long long, int, const float*, T, T*, cpx<T>*,       \
                                  size_t, cudaStream_t);                                                        \
    template void launch_bin<T>(int, int, int, int, const T*, T*, cudaStream_t);                                    \
    template void launch_image<T>(int, int, const T*, const T*, T*, cudaStream_t);                             \
    template void launch_rotate_add_images<T>(int, float, float, const T*, T*, cudaStream_t);                 \
    template void launch_ring_line<T>(int, int, int, const float2*, const T*, T*, cudaStream_t);              \
    template void launch_line_image<T>(int, int, const T*, T*, cudaStream_t);                                \
    template void launch_cmul<T>(int, const cpx<T>*, cpx<T>*, cudaStream_t);
BS_DET_INST(float)
BS_DET_INST(double)

}  // namespace bs
