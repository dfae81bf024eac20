// ref_runtime.cpp -- TEST INFRASTRUCTURE: definitions behind cuda_runtime.h,
// cufft.h and prelude.h of this directory (the host-run build of the
// reference; see cuda_runtime.h).  Nothing here is product code.
#include <ucontext.h>

#include <chrono>
#include <cmath>
#include <complex>
#include <functional>
#include <map>
#include <memory>
#include <vector>

#include "cufft.h"
#include "cuda_runtime.h"

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

// `extern __shared__ float shared[]` of the reference's ring kernels
// (microscope.cu:142,200) resolves here; their blocks run one after another,
// so one array serves as every block's shared memory.
float shared[1 << 16];

// ---- cooperative blocks ----------------------------------------------------
// The threads of one block as coroutines on the calling host thread.  Each
// round resumes, in thread order, every thread that has not returned; a thread
// runs until it returns or calls __syncthreads().  Threads that returned no
// longer take part in the barrier, as on the GPU.
namespace {
thread_local bool g_coop = false;
thread_local ucontext_t g_sched;
thread_local std::vector<ucontext_t>* g_ctx = nullptr;
thread_local std::vector<char>* g_done = nullptr;
thread_local const std::function<void()>* g_body = nullptr;
thread_local int g_cur = 0;

void coop_trampoline() {
    (*g_body)();
    (*g_done)[g_cur] = 1;  // returns to uc_link, the scheduler
}
}  // namespace

void bs_ref_syncthreads() {
    if (g_coop) swapcontext(&(*g_ctx)[g_cur], &g_sched);
}

namespace bs_ref {
void coop_block(const dim3& block, const std::function<void()>& body) {
    const int n = (int)(block.x * block.y * block.z);
    const size_t stack = 1 << 16;
    std::vector<ucontext_t> ctx(n);
    std::unique_ptr<char[]> stacks(new char[(size_t)n * stack]);
    std::vector<char> done(n, 0);
    g_ctx = &ctx;
    g_done = &done;
    g_body = &body;
    for (int i = 0; i < n; i++) {
        getcontext(&ctx[i]);
        ctx[i].uc_stack.ss_sp = stacks.get() + (size_t)i * stack;
        ctx[i].uc_stack.ss_size = stack;
        ctx[i].uc_link = &g_sched;
        makecontext(&ctx[i], coop_trampoline, 0);
    }
    g_coop = true;
    for (bool pending = true; pending;) {
        pending = false;
        for (int i = 0; i < n; i++) {
            if (done[i]) continue;
            g_cur = i;
            ::threadIdx = uint3{(unsigned)i % block.x, ((unsigned)i / block.x) % block.y,
                                (unsigned)i / (block.x * block.y)};
            swapcontext(&g_sched, &ctx[i]);
            if (!done[i]) pending = true;
        }
    }
    g_coop = false;
}
}  // namespace bs_ref

const char* cudaGetErrorString(cudaError_t e) { return e == cudaSuccess ? "no error" : "host-run CUDA stand-in error"; }
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
cudaError_t cudaThreadSynchronize() { return cudaSuccess; }
cudaError_t cudaGetLastError() { return cudaSuccess; }

// zero-filled, so that results never depend on leftover memory
cudaError_t cudaMalloc(void** p, size_t n) {
    *p = std::calloc(n ? n : 1, 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFree(void* p) {
    std::free(p);
    return cudaSuccess;
}
cudaError_t cudaMemcpy(void* dst, const void* src, size_t n, cudaMemcpyKind) {
    if (n) std::memmove(dst, src, n);
    return cudaSuccess;
}
cudaError_t cudaMemset(void* p, int v, size_t n) {
    if (n) std::memset(p, v, n);
    return cudaSuccess;
}
cudaError_t cudaGetDeviceProperties(cudaDeviceProp* p, int) {
    std::memset(p, 0, sizeof(*p));
    p->major = 10;
    p->multiProcessorCount = 1;
    std::snprintf(p->name, sizeof(p->name), "host-run stand-in");
    return cudaSuccess;
}

struct bs_ref_event { std::chrono::steady_clock::time_point t; };
cudaError_t cudaEventCreate(cudaEvent_t* e) {
    *e = new bs_ref_event();
    return cudaSuccess;
}
cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t) {
    e->t = std::chrono::steady_clock::now();
    return cudaSuccess;
}
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t a, cudaEvent_t b) {
    *ms = std::chrono::duration<float, std::milli>(b->t - a->t).count();
    return cudaSuccess;
}
cudaError_t cudaEventDestroy(cudaEvent_t e) {
    delete e;
    return cudaSuccess;
}

cudaChannelFormatDesc cudaCreateChannelDesc(int x, int y, int z, int w, cudaChannelFormatKind f) {
    return cudaChannelFormatDesc{x, y, z, w, f};
}
cudaError_t cudaMallocArray(cudaArray** a, const cudaChannelFormatDesc* d, size_t w, size_t h, unsigned) {
    cudaArray* r = new cudaArray;
    r->width = w;
    r->height = h ? h : 1;
    r->elem = (size_t)(d->x + d->y + d->z + d->w) / 8;
    r->data = static_cast<unsigned char*>(std::calloc(r->width * r->height * r->elem, 1));
    *a = r;
    return cudaSuccess;
}
cudaError_t cudaFreeArray(cudaArray* a) {
    if (a) {
        std::free(a->data);
        delete a;
    }
    return cudaSuccess;
}
cudaError_t cudaMemcpy2DToArray(cudaArray* dst, size_t wOffset, size_t hOffset, const void* src, size_t spitch,
                                size_t width, size_t height, cudaMemcpyKind) {
    if (wOffset + width > dst->width * dst->elem || hOffset + height > dst->height) return cudaErrorInvalidValue;
    for (size_t r = 0; r < height; r++)
        std::memcpy(dst->data + (hOffset + r) * dst->width * dst->elem + wOffset,
                    static_cast<const unsigned char*>(src) + r * spitch, width);
    return cudaSuccess;
}
cudaError_t cudaMemcpyToArray(cudaArray* dst, size_t wOffset, size_t hOffset, const void* src, size_t count,
                              cudaMemcpyKind) {
    size_t off = hOffset * dst->width * dst->elem + wOffset;
    if (off + count > dst->width * dst->height * dst->elem) return cudaErrorInvalidValue;
    std::memcpy(dst->data + off, src, count);
    return cudaSuccess;
}

// ---- texture fetch --------------------------------------------------------
// Linear filtering as the CUDA programming guide's texture-fetching appendix
// defines it for unnormalised coordinates: xB = x - 0.5, i = floor(xB),
// alpha = xB - i, result = (1 - alpha) T[i] + alpha T[i + 1] (and the same in
// y).  The hardware keeps alpha in 9-bit fixed point (8 fractional bits); the
// weights here are exact unless bs_ref_set_tex_weight_bits(8) asks for that
// rounding.  Wrap and mirror addressing exist only for normalised coordinates,
// so with unnormalised ones they clamp; border reads zero outside.
static int g_weight_bits = 0;
extern "C" void bs_ref_set_tex_weight_bits(int bits) { g_weight_bits = bits; }

static bool address(long i, long n, cudaTextureAddressMode m, int normalized, long* out) {
    if (i >= 0 && i < n) {
        *out = i;
        return true;
    }
    if (m == cudaAddressModeBorder) return false;
    if (normalized && m == cudaAddressModeWrap) {
        *out = ((i % n) + n) % n;
        return true;
    }
    if (normalized && m == cudaAddressModeMirror) {
        long p = ((i % (2 * n)) + 2 * n) % (2 * n);
        *out = p < n ? p : 2 * n - 1 - p;
        return true;
    }
    *out = i < 0 ? 0 : n - 1;
    return true;
}

static double weight(double f) {
    if (g_weight_bits <= 0) return f;
    const double s = std::ldexp(1.0, g_weight_bits);
    return std::nearbyint(f * s) / s;
}

void bs_ref_tex_fetch(const cudaArray* a, int ncomp, const cudaTextureAddressMode* am, int filter, int normalized,
                      float x, float y, float* out) {
    const long W = (long)a->width, H = (long)a->height;
    double xs = x, ys = y;
    if (normalized) {
        xs *= W;
        ys *= H;
    }
    auto texel = [&](long i, long j, int c) -> double {
        long ii, jj;
        if (!address(i, W, am[0], normalized, &ii) || !address(j, H, am[1], normalized, &jj)) return 0.0;
        float v;
        std::memcpy(&v, a->data + ((size_t)jj * W + ii) * a->elem + c * sizeof(float), sizeof(float));
        return v;
    };
    for (int c = 0; c < ncomp; c++) {
        if (filter == cudaFilterModePoint) {
            out[c] = (float)texel((long)std::floor(xs), (long)std::floor(ys), c);
            continue;
        }
        const double xb = xs - 0.5, yb = ys - 0.5;
        const long i = (long)std::floor(xb), j = (long)std::floor(yb);
        const double al = weight(xb - i), be = weight(yb - j);
        const double v = (1 - al) * (1 - be) * texel(i, j, c) + al * (1 - be) * texel(i + 1, j, c) +
                         (1 - al) * be * texel(i, j + 1, c) + al * be * texel(i + 1, j + 1, c);
        out[c] = (float)v;
    }
}

// ---- cuFFT ------------------------------------------------------------------
namespace {
struct Plan {
    int nx, ny;
    cufftType type;
};
std::map<int, Plan> g_plans;
int g_next_plan = 1;

// unnormalised DFT of n points with stride s, exact twiddles exp(sign 2 pi i jk/n)
void dft_line(std::complex<double>* a, int n, size_t s, int sign, std::vector<std::complex<double>>& tmp) {
    tmp.assign(n, 0.0);
    for (int k = 0; k < n; k++) {
        std::complex<double> acc = 0.0;
        for (int j = 0; j < n; j++) {
            const long m = ((long)j * k) % n;
            const double ang = sign * 2.0 * M_PI * (double)m / n;
            acc += a[(size_t)j * s] * std::complex<double>(std::cos(ang), std::sin(ang));
        }
        tmp[k] = acc;
    }
    for (int k = 0; k < n; k++) a[(size_t)k * s] = tmp[k];
}

void dft2(std::vector<std::complex<double>>& d, int nx, int ny, int sign) {
    std::vector<std::complex<double>> tmp;
    for (int r = 0; r < nx; r++) dft_line(d.data() + (size_t)r * ny, ny, 1, sign, tmp);
    for (int c = 0; c < ny; c++) dft_line(d.data() + c, nx, (size_t)ny, sign, tmp);
}
}  // namespace

cufftResult cufftPlan2d(cufftHandle* plan, int nx, int ny, cufftType type) {
    if (nx < 1 || ny < 1) return CUFFT_INVALID_SIZE;
    *plan = g_next_plan++;
    g_plans[*plan] = Plan{nx, ny, type};
    return CUFFT_SUCCESS;
}
cufftResult cufftDestroy(cufftHandle plan) { return g_plans.erase(plan) ? CUFFT_SUCCESS : CUFFT_INVALID_PLAN; }

cufftResult cufftExecC2C(cufftHandle plan, cufftComplex* in, cufftComplex* out, int direction) {
    auto it = g_plans.find(plan);
    if (it == g_plans.end() || it->second.type != CUFFT_C2C) return CUFFT_INVALID_PLAN;
    const int nx = it->second.nx, ny = it->second.ny;
    std::vector<std::complex<double>> d((size_t)nx * ny);
    for (size_t i = 0; i < d.size(); i++) d[i] = {in[i].x, in[i].y};
    dft2(d, nx, ny, direction);
    for (size_t i = 0; i < d.size(); i++) out[i] = float2{(float)d[i].real(), (float)d[i].imag()};
    return CUFFT_SUCCESS;
}
cufftResult cufftExecZ2Z(cufftHandle plan, cufftDoubleComplex* in, cufftDoubleComplex* out, int direction) {
    auto it = g_plans.find(plan);
    if (it == g_plans.end() || it->second.type != CUFFT_Z2Z) return CUFFT_INVALID_PLAN;
    const int nx = it->second.nx, ny = it->second.ny;
    std::vector<std::complex<double>> d((size_t)nx * ny);
    for (size_t i = 0; i < d.size(); i++) d[i] = {in[i].x, in[i].y};
    dft2(d, nx, ny, direction);
    for (size_t i = 0; i < d.size(); i++) out[i] = double2{d[i].real(), d[i].imag()};
    return CUFFT_SUCCESS;
}
