// bs_noalloc.cu -- Mie coefficients for callers that cannot allocate device
// memory.
//
// bs_mie_noalloc computes the same coefficients as the context path (the
// mie_kernel of bs_nearfield.cu, sphere::calcCoeff of the reference) but
// takes every buffer from the caller and allocates nothing: its Bessel work
// space is the file-scope device array below, a fixed 3 MiB that every GPU
// loading this library holds until the process exits.  Callers that cannot
// call cudaMalloc include code running inside CUDA stream capture (where an
// allocation would end the capture), real-time or serving loops that reserve
// all memory up front, and frameworks whose memory belongs to their own pool
// allocator and must not be fragmented by a library.
#include <cuda_runtime.h>

#include <mutex>

#include "bimsim_gb300.h"
#include "bs_math.cuh"

namespace bs {

void set_last_error(const char* msg);

namespace {

constexpr int NOALLOC_MAX_SPHERES = 256;
constexpr int NOALLOC_MAX_ORDER = 127;
constexpr int NOALLOC_L = NOALLOC_MAX_ORDER + 1;
constexpr int NOALLOC_MAX_DEVICES = 64;

// Six complex Bessel arrays of NOALLOC_L orders per sphere:
// j, y, j', y' at k a and j, j' at k n a.  256 * 6 * 128 * 16 B = 3 MiB.
static __device__ __align__(256) zd g_noalloc_bessel[NOALLOC_MAX_SPHERES * 6 * NOALLOC_L];

// The sphere's own order count Nl = ceil(ka + 4 (ka)^(1/3) + 2) in single
// precision, in the order of sphere::calcNl (sphere.h:71-74) and of the host's
// calc_nl, with lambda = 2 PI / k rounded to float.  powf on the GPU may differ
// from the host's by an ulp, which changes Nl only when the sum lies within a
// few ulps of an integer.
__device__ int noalloc_calc_nl(double a_in, double k) {
    const float lam = (float)(2.0 * (double)3.14159f / k);
    const float pif = 3.14159f;
    float ka = __fmul_rn(2.0f, pif);
    ka = __fmul_rn(ka, (float)a_in);
    ka = __fdiv_rn(ka, lam);
    const float third = (float)(1.0 / 3.0);
    float v = __fmul_rn(4.0f, powf(ka, third));
    v = __fadd_rn(ka, v);
    v = __fadd_rn(v, 2.0f);
    return (int)ceilf(v);
}

__global__ void mie_noalloc_kernel(const double* __restrict__ sph, int ns, int nl_cap, double k,
                                   zd* __restrict__ work, zd* __restrict__ A, zd* __restrict__ B) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ns) return;
    const double a = sph[3 * s], n_re = sph[3 * s + 1], n_im = sph[3 * s + 2];
    // Orders above the sphere's own Nl are not part of its series (the context
    // path never computes them); they are returned as zeros.  Evaluating them
    // would divide underflowed Bessel values (0/0, 0 * inf) for small spheres.
    const int nl = min(nl_cap, noalloc_calc_nl(a, k));
    zd* ja = work + (size_t)s * 6 * NOALLOC_L;
    zd* ya = ja + NOALLOC_L;
    zd* jpa = ya + NOALLOC_L;
    zd* ypa = jpa + NOALLOC_L;
    zd* jn = ypa + NOALLOC_L;
    zd* jpn = jn + NOALLOC_L;
    const zd n = mk(n_re, n_im);
    const zd ka = mk(k * a, 0.0);
    const zd kna = (n * k) * a;
    sph_complex(nl, ka, true, ja, ya, jpa, ypa);
    sph_complex(nl, kna, true, jn, nullptr, jpn, nullptr);
    zd* As = A + (size_t)s * (nl_cap + 1);
    zd* Bs = B + (size_t)s * (nl_cap + 1);
    for (int l = nl + 1; l <= nl_cap; l++) As[l] = Bs[l] = mk(0.0, 0.0);
    for (int l = 0; l <= nl; l++) {
        const zd h = mk(ja[l].re - ya[l].im, ja[l].im + ya[l].re);
        const zd hp = mk(jpa[l].re - ypa[l].im, jpa[l].im + ypa[l].re);
        const zd an = ja[l] * hp - jpa[l] * h;
        const zd bn = jn[l] * hp - (h * jpn[l]) * n;
        const zd cn = (ja[l] * jpn[l]) * n - jn[l] * jpa[l];
        const zd f = mk(2.0 * l + 1.0, 0.0) * ipow(l);
        As[l] = f * (an / bn);
        Bs[l] = f * (cn / bn);
    }
}

std::mutex g_mutex;
void* g_work[NOALLOC_MAX_DEVICES] = {};

}  // namespace
}  // namespace bs

extern "C" bs_status bs_mie_noalloc(const double* spheres, int32_t ns, int32_t nl, double k, double* A, double* B,
                                    void* stream) {
    using namespace bs;
    if (ns < 0 || ns > NOALLOC_MAX_SPHERES) {
        set_last_error("bs_mie_noalloc: sphere count outside 0..256 (the fixed work space holds 256 spheres)");
        return BS_ERR_ARG;
    }
    if (nl < 0 || nl > NOALLOC_MAX_ORDER) {
        set_last_error("bs_mie_noalloc: order outside 0..127 (the fixed work space holds 128 orders)");
        return BS_ERR_ARG;
    }
    if (!(k > 0)) {
        set_last_error("bs_mie_noalloc: wavenumber must be > 0");
        return BS_ERR_ARG;
    }
    if (ns > 0 && (!spheres || !A || !B)) {
        set_last_error("bs_mie_noalloc: null buffer");
        return BS_ERR_ARG;
    }
    if (ns == 0) return BS_OK;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        set_last_error("bs_mie_noalloc: no usable current CUDA device");
        return BS_ERR_CUDA;
    }
    void* work = nullptr;
    {
        // First call on a device: resolve the device address of the work
        // space with that device current (the array's name is only a host
        // stand-in).  Make this first call before any stream capture.
        std::lock_guard<std::mutex> lock(g_mutex);
        if (!g_work[dev]) {
            void* ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_noalloc_bessel);
            if (e != cudaSuccess || !ptr) {
                set_last_error("bs_mie_noalloc: cudaGetSymbolAddress of the work space failed");
                return BS_ERR_CUDA;
            }
            g_work[dev] = ptr;
        }
        work = g_work[dev];
    }
    mie_noalloc_kernel<<<(ns + 63) / 64, 64, 0, (cudaStream_t)stream>>>(spheres, ns, nl, k, (zd*)work, (zd*)A, (zd*)B);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        return BS_ERR_CUDA;
    }
    return BS_OK;
}
