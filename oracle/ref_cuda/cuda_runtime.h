// cuda_runtime.h -- TEST INFRASTRUCTURE: a host-only stand-in for the subset of
// the CUDA runtime that the reference's .cu sources call, so that those
// sources compile with g++ and run on the CPU (oracle/Makefile, target
// ref-sim).  "Device" memory is host memory, a kernel launch is a loop over
// blocks and threads (prelude.h), a cudaArray is a host array and a texture
// fetch is bilinear filtering in software (ref_runtime.cpp).  Only the calls
// the reference makes are provided, with the semantics the CUDA programming
// guide documents for them.  It is never part of the product library.
#ifndef BS_REF_CUDA_RUNTIME_H
#define BS_REF_CUDA_RUNTIME_H

#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2, cudaErrorInvalidValue = 11 };
enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3,
    cudaMemcpyDefault = 4
};

struct uint3 { unsigned int x, y, z; };
struct dim3 {
    unsigned int x, y, z;
    dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};
struct float2 { float x, y; };
struct float4 { float x, y, z, w; };
struct double2 { double x, y; };
inline float2 make_float2(float x, float y) { return float2{x, y}; }
inline float4 make_float4(float x, float y, float z, float w) { return float4{x, y, z, w}; }

// launch geometry of the emulated kernel being run (one host thread runs a launch)
extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

const char* cudaGetErrorString(cudaError_t e);
cudaError_t cudaSetDevice(int dev);
cudaError_t cudaDeviceSynchronize();
cudaError_t cudaThreadSynchronize();
cudaError_t cudaGetLastError();
cudaError_t cudaMalloc(void** p, size_t n);
template <class T>
inline cudaError_t cudaMalloc(T** p, size_t n) { return cudaMalloc(reinterpret_cast<void**>(p), n); }
cudaError_t cudaFree(void* p);
cudaError_t cudaMemcpy(void* dst, const void* src, size_t n, cudaMemcpyKind kind);
cudaError_t cudaMemset(void* p, int v, size_t n);

struct cudaDeviceProp { int major, minor, multiProcessorCount; char name[256]; };
cudaError_t cudaGetDeviceProperties(cudaDeviceProp* p, int dev);

// events: wall-clock stand-ins (the reference prints the times with --verbose)
typedef struct bs_ref_event* cudaEvent_t;
typedef void* cudaStream_t;
cudaError_t cudaEventCreate(cudaEvent_t* e);
cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t s = 0);
cudaError_t cudaEventSynchronize(cudaEvent_t e);
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t a, cudaEvent_t b);
cudaError_t cudaEventDestroy(cudaEvent_t e);

// ---- arrays and legacy texture references ----
enum cudaChannelFormatKind { cudaChannelFormatKindSigned, cudaChannelFormatKindUnsigned, cudaChannelFormatKindFloat };
struct cudaChannelFormatDesc { int x, y, z, w; cudaChannelFormatKind f; };
cudaChannelFormatDesc cudaCreateChannelDesc(int x, int y, int z, int w, cudaChannelFormatKind f);

struct cudaArray {
    size_t width, height, elem;  // elements per row, rows, bytes per element
    unsigned char* data;
};
cudaError_t cudaMallocArray(cudaArray** a, const cudaChannelFormatDesc* d, size_t w, size_t h = 0, unsigned flags = 0);
cudaError_t cudaFreeArray(cudaArray* a);
cudaError_t cudaMemcpy2DToArray(cudaArray* dst, size_t wOffset, size_t hOffset, const void* src, size_t spitch,
                                size_t width, size_t height, cudaMemcpyKind kind);
cudaError_t cudaMemcpyToArray(cudaArray* dst, size_t wOffset, size_t hOffset, const void* src, size_t count,
                              cudaMemcpyKind kind);

#define cudaTextureType1D 0x01
#define cudaTextureType2D 0x02
enum cudaTextureReadMode { cudaReadModeElementType = 0, cudaReadModeNormalizedFloat = 1 };
enum cudaTextureAddressMode { cudaAddressModeWrap = 0, cudaAddressModeClamp = 1, cudaAddressModeMirror = 2,
                              cudaAddressModeBorder = 3 };
enum cudaTextureFilterMode { cudaFilterModePoint = 0, cudaFilterModeLinear = 1 };

template <class T, int dim = cudaTextureType1D, int mode = cudaReadModeElementType>
struct texture {
    cudaTextureAddressMode addressMode[3] = {cudaAddressModeClamp, cudaAddressModeClamp, cudaAddressModeClamp};
    cudaTextureFilterMode filterMode = cudaFilterModePoint;
    int normalized = 0;
    const cudaArray* array = nullptr;
};

template <class T, int dim, int mode>
inline cudaError_t cudaBindTextureToArray(texture<T, dim, mode>& t, const cudaArray* a, const cudaChannelFormatDesc&) {
    t.array = a;
    return cudaSuccess;
}
template <class T, int dim, int mode>
inline cudaError_t cudaUnbindTexture(texture<T, dim, mode>& t) {
    t.array = nullptr;
    return cudaSuccess;
}

// One filtered fetch of `ncomp` float components at unnormalised coordinates
// (x, y) of a 1-D (height 1) or 2-D array; see ref_runtime.cpp.
void bs_ref_tex_fetch(const cudaArray* a, int ncomp, const cudaTextureAddressMode* am, int filter, int normalized,
                      float x, float y, float* out);

template <int dim, int mode>
inline float tex2D(const texture<float, dim, mode>& t, float x, float y) {
    float v;
    bs_ref_tex_fetch(t.array, 1, t.addressMode, t.filterMode, t.normalized, x, y, &v);
    return v;
}
template <int dim, int mode>
inline float2 tex2D(const texture<float2, dim, mode>& t, float x, float y) {
    float v[2];
    bs_ref_tex_fetch(t.array, 2, t.addressMode, t.filterMode, t.normalized, x, y, v);
    return float2{v[0], v[1]};
}
template <int dim, int mode>
inline float tex1D(const texture<float, dim, mode>& t, float x) {
    float v;
    bs_ref_tex_fetch(t.array, 1, t.addressMode, t.filterMode, t.normalized, x, 0.5f, &v);
    return v;
}
template <int dim, int mode>
inline float4 tex1D(const texture<float4, dim, mode>& t, float x) {
    float v[4];
    bs_ref_tex_fetch(t.array, 4, t.addressMode, t.filterMode, t.normalized, x, 0.5f, v);
    return float4{v[0], v[1], v[2], v[3]};
}

#endif
