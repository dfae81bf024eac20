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

template <class T>
__global__ void __launch_bounds__(256) cgemm_kernel(int M, int N, int K, const cpx<T>* __restrict__ A, int lda,
                                                    long long sA, const cpx<T>* __restrict__ B, int ldb, long long sB,
                                                    cpx<T>* __restrict__ C, int ldc, long long sC, int epi,
                                                    const float* __restrict__ mask, T scale, T* __restrict__ I) {
    __shared__ cpx<T> As[GB_K][GB_M + 1];
    __shared__ cpx<T> Bs[GB_K][GB_N + 1];
    const int b = blockIdx.z;
    A += b * sA;
    B += b * sB;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * GB_M, n0 = blockIdx.x * GB_N;
    T accr[4][2], acci[4][2], cr[4][2], ci[4][2];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 2; j++) accr[i][j] = acci[i][j] = cr[i][j] = ci[i][j] = 0;
    for (int k0 = 0; k0 < K; k0 += GB_K) {
        for (int e = threadIdx.x; e < GB_K * GB_M; e += 256) {
            int kk = e % GB_K, mm = e / GB_K;
            int gm = m0 + mm, gk = k0 + kk;
            As[kk][mm] = (gm < M && gk < K) ? A[(long long)gm * lda + gk] : mk((T)0, (T)0);
        }
        for (int e = threadIdx.x; e < GB_K * GB_N; e += 256) {
            int nn = e % GB_N, kk = e / GB_N;
            int gn = n0 + nn, gk = k0 + kk;
            Bs[kk][nn] = (gn < N && gk < K) ? B[(long long)gk * ldb + gn] : mk((T)0, (T)0);
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
            T vr = accr[i][j], vi = acci[i][j];
            long long o = b * sC + (long long)gm * ldc + gn;
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

template <class T>
void launch_cgemm(int M, int N, int K, int batch, const cpx<T>* A, int lda, long long sA, const cpx<T>* B, int ldb,
                  long long sB, cpx<T>* C, int ldc, long long sC, int epi, const float* mask, T scale, T* I,
                  cudaStream_t st) {
    dim3 grid((N + GB_N - 1) / GB_N, (M + GB_M - 1) / GB_M, batch);
    cgemm_kernel<T><<<grid, 256, 0, st>>>(M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC, epi, mask, scale, I);
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

#define BS_DET_INST(T)                                                                                          \
    template void launch_twiddle<T>(int, int, const int*, int, int, int, int, int, cpx<T>*, cudaStream_t);      \
    template void launch_cgemm<T>(int, int, int, int, const cpx<T>*, int, long long, const cpx<T>*, int,       \
                                  long long, cpx<T>*, int, long long, int, const float*, T, T*, cudaStream_t); \
    template void launch_bin<T>(int, int, int, int, const T*, T*, cudaStream_t);                                    \
    template void launch_image<T>(int, int, const T*, const T*, T*, cudaStream_t);
BS_DET_INST(float)
BS_DET_INST(double)

}  // namespace bs
