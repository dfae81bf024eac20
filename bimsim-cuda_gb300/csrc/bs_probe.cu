// bs_probe.cu -- measured single- and double-precision FMA throughput of the
// current GPU, the denominators of the scattered-field kernels' roofline.
#include <cuda_runtime.h>

#include "bimsim_gb300.h"

namespace {

// 8 independent FMA chains per thread; the result is written so the chains
// are not removed.  Every launch is bounded (fixed iteration count).
template <class T>
__global__ void fma_loop(T* out, int iters, T a, T b) {
    T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 16; j++) {
            x0 = x0 * a + b;
            x1 = x1 * a + b;
            x2 = x2 * a + b;
            x3 = x3 * a + b;
            x4 = x4 * a + b;
            x5 = x5 * a + b;
            x6 = x6 * a + b;
            x7 = x7 * a + b;
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// The same chains as packed pairs: Blackwell's fma.rn.f32x2 does two
// single-precision FMAs per instruction, so the FP32 peak is the larger of the
// scalar and the packed loop.
__global__ void fma2_loop(float* out, int iters, float a, float b) {
    unsigned long long x[4], av, bv;
    asm("mov.b64 %0, {%1, %1};" : "=l"(av) : "f"(a));
    asm("mov.b64 %0, {%1, %1};" : "=l"(bv) : "f"(b));
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float u = (float)threadIdx.x + 2 * k, v = u + 1;
        asm("mov.b64 %0, {%1, %2};" : "=l"(x[k]) : "f"(u), "f"(v));
    }
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 16; j++)
#pragma unroll
            for (int k = 0; k < 4; k++) asm("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(x[k]) : "l"(av), "l"(bv));
    }
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float lo, hi;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(x[k]));
        acc += lo + hi;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

template <class T>
void run_loop(T* out, int blocks, int threads, int iters, bool packed) {
    fma_loop<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
}
template <>
void run_loop<float>(float* out, int blocks, int threads, int iters, bool packed) {
    if (packed) fma2_loop<<<blocks, threads>>>(out, iters, 0.999999f, 1e-7f);
    else fma_loop<float><<<blocks, threads>>>(out, iters, 0.999999f, 1e-7f);
}

template <class T>
int measure(double* tflops, int iters, bool packed = false) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 2;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int threads = 256, blocks = sms * 8;
    T* out = nullptr;
    if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(T)) != cudaSuccess) return 3;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    run_loop<T>(out, blocks, threads, iters / 4, packed);  // warm-up
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(e0);
        run_loop<T>(out, blocks, threads, iters, packed);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return 2;
    double flop = 2.0 * 8 * 16 * (double)iters * blocks * threads;
    *tflops = flop / (best * 1e-3) / 1e12;
    return 0;
}

}  // namespace

extern "C" bs_status bs_measure_fma_peak(double* fp32_tflops, double* fp64_tflops) {
    if (!fp32_tflops || !fp64_tflops) return BS_ERR_ARG;
    double packed = 0;
    if (measure<float>(fp32_tflops, 4096) != 0) return BS_ERR_CUDA;
    if (measure<float>(&packed, 4096, true) != 0) return BS_ERR_CUDA;  // 8 FMAs per iteration step either way
    if (packed > *fp32_tflops) *fp32_tflops = packed;
    if (measure<double>(fp64_tflops, 64) != 0) return BS_ERR_CUDA;
    return BS_OK;
}
