// bs_api.cu -- the C ABI of include/bimsim_gb300.h: context, device memory,
// the per-slice stage pipeline, and result readback.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "bimsim_gb300.h"
#include "bs_internal.h"
#include "bs_kernels.h"
#include "bs_math.cuh"

using namespace bs;

namespace {

thread_local std::string g_err;

bs_status fail(bs_status st, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return st;
}

#define CK(x)                                                                                               \
    do {                                                                                                    \
        cudaError_t e_ = (x);                                                                               \
        if (e_ != cudaSuccess)                                                                              \
            return fail(e_ == cudaErrorMemoryAllocation ? BS_ERR_NOMEM : BS_ERR_CUDA, "%s failed: %s (%s:%d)", \
                        #x, cudaGetErrorString(e_), __FILE__, __LINE__);                                    \
    } while (0)

#define LAUNCHED(ctx)                                                                                   \
    do {                                                                                                \
        (ctx)->launches++;                                                                              \
        cudaError_t e_ = cudaGetLastError();                                                            \
        if (e_ != cudaSuccess)                                                                          \
            return fail(BS_ERR_CUDA, "kernel launch failed: %s (%s:%d)", cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                                      \
    } while (0)

// A context's device buffer.  Allocation and release are stream-ordered on
// the owning context's stream (cudaMallocAsync / cudaFreeAsync): cudaFree
// would wait for every stream of the device, so a context growing a buffer
// would stall behind a long slice running on another context of the server.
struct DevBuf {
    void* p = nullptr;
    size_t n = 0;
    const cudaStream_t* st = nullptr;  // the owning context's stream (set by bs_create)
    cudaError_t ensure(size_t bytes) {
        if (bytes == 0) bytes = 256;
        if (bytes <= n) return cudaSuccess;
        release();
        cudaError_t e = st ? cudaMallocAsync(&p, bytes, *st) : cudaMalloc(&p, bytes);
        if (e == cudaSuccess) n = bytes;
        else p = nullptr;
        return e;
    }
    void release() {
        if (p) {
            if (st) cudaFreeAsync(p, *st);
            else cudaFree(p);
        }
        p = nullptr;
        n = 0;
    }
    template <class X>
    X* as() const {
        return reinterpret_cast<X*>(p);
    }
};

bool valid_params(const bs_params* p, std::string& why) {
    if (!(p->lambda > 0)) { why = "lambda must be > 0"; return false; }
    if (p->resolution <= 0) { why = "resolution must be > 0"; return false; }
    if (p->padding < 0) { why = "padding must be >= 0"; return false; }
    if (p->supersample < 1) { why = "supersample must be >= 1"; return false; }
    if (p->field_order < 0 || p->field_order > MAX_ORDER) { why = "field order out of range"; return false; }
    if (p->condenser[0] < 0 || p->condenser[1] > 1 || p->condenser[0] > p->condenser[1]) {
        why = "condenser NA must satisfy 0 <= NA_in <= NA_out <= 1"; return false;
    }
    long long R = (long long)p->resolution * p->supersample * (2LL * p->padding + 1);
    if (R > 65536) { why = "near-field resolution above 65536"; return false; }
    if (p->us_lut_r == 1 || p->us_lut_theta == 1 || p->uf_lut_r == 1 || p->us_lut_r < 0 || p->us_lut_theta < 0 ||
        p->uf_lut_r < 0) {
        why = "LUT sizes must be 0 (reference default) or >= 2"; return false;
    }
    return true;
}

// One sphere's tables for the mixed path: real and imaginary float planes of
// Usp (thetaR x dR) and Uip (thetaR x aR) in CUDA arrays, with a surface
// object per plane for the build and a texture object per plane for the
// gathers.  Index k: 0 Usp re, 1 Usp im, 2 Uip re, 3 Uip im.
struct TexSlot {
    cudaArray_t arr[4] = {};
    cudaTextureObject_t tex[4] = {};
    cudaSurfaceObject_t surf[4] = {};
    int w = 0, h[4] = {0, 0, 0, 0};

    void release() {
        for (int k = 0; k < 4; k++) {
            if (tex[k]) cudaDestroyTextureObject(tex[k]);
            if (surf[k]) cudaDestroySurfaceObject(surf[k]);
            if (arr[k]) cudaFreeArray(arr[k]);
            tex[k] = surf[k] = 0;
            arr[k] = nullptr;
            h[k] = 0;
        }
        w = 0;
    }

    // (re)allocate plane k with at least `rows` rows of `width` floats
    cudaError_t ensure(int k, int width, int rows) {
        if (arr[k] && w == width && h[k] >= rows) return cudaSuccess;
        if (tex[k]) cudaDestroyTextureObject(tex[k]);
        if (surf[k]) cudaDestroySurfaceObject(surf[k]);
        if (arr[k]) cudaFreeArray(arr[k]);
        tex[k] = surf[k] = 0;
        arr[k] = nullptr;
        cudaChannelFormatDesc fd = cudaCreateChannelDesc<float>();
        // rows rounded up to a multiple of 256 (reads never pass the spare row): fewer
        // reallocations, whose cudaFreeArray waits for the whole device
        rows = (rows + 255) & ~255;
        cudaError_t e = cudaMallocArray(&arr[k], &fd, width, rows, cudaArraySurfaceLoadStore | cudaArrayTextureGather);
        if (e != cudaSuccess) return e;
        cudaResourceDesc rd = {};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = arr[k];
        e = cudaCreateSurfaceObject(&surf[k], &rd);
        if (e != cudaSuccess) return e;
        cudaTextureDesc td = {};
        td.addressMode[0] = cudaAddressModeClamp;
        td.addressMode[1] = cudaAddressModeClamp;
        td.filterMode = cudaFilterModePoint;
        td.readMode = cudaReadModeElementType;
        td.normalizedCoords = 0;
        e = cudaCreateTextureObject(&tex[k], &rd, &td, nullptr);
        if (e != cudaSuccess) return e;
        w = width;
        h[k] = rows;
        return cudaSuccess;
    }
};

}  // namespace

struct bs_ctx {
    bs_params prm{};
    std::vector<bs_sphere> spheres;
    std::vector<double> waves;
    bool waves_set = false;
    int device = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[6] = {};
    size_t budget = 0;  // LUT bytes allowed; 0 = automatic

    // derived per simulate
    Scene sc{};
    std::vector<Sphere> hs;
    int res = 0, ss = 1, crop = 0, off = 0, R = 0, Lmax = 1;
    int prec = -1;
    bool have = false;

    DevBuf d_sph, d_waves, d_kw4, d_ph, d_A, d_B, d_mie, d_tab, d_tabscr, d_legP, d_lut, d_uft, d_uftscr;
    DevBuf d_cones, d_cnt;  // per-chunk wave cones; staged / total counters of the mixed LUT kernel
    DevBuf d_far;           // far fields Ud, Ufd on request (bs_get_far_field)
    DevBuf d_starts;        // row / coefficient offsets of a coefficient batch
    DevBuf d_lbjobs, d_lbjobs2;  // Usp and Uip tables of a coefficient batch for the mixed LUT build
    DevBuf d_kcmp;               // Kahan compensation of the mixed LUT sums between sphere chunks
    DevBuf d_fsave;         // U, Uf of a ring's first source (bs_simulate_ring_interp)
    DevBuf d_dacc;          // detector sum of bs_simulate_ring_detector
    DevBuf d_line, d_ringcs;  // radial lines and ring (cos, sin) of bs_simulate_ring_line
    int det_Nv = 0;         // passband rows of the last detector run (0: no far field)
    DevBuf d_fields;  // [2][R*R] U then Uf
    DevBuf d_su, d_sv, d_mask, d_wx, d_wy, d_wix, d_wiy, d_f1, d_f2, d_g1, d_I, d_D, d_img;
    int legP_theta = 0, legP_L = 0;
    std::vector<TexSlot> slots;  // mixed-path tables, one per sphere of a chunk
    DevBuf d_texobj;
    int64_t launches = 0;
    int64_t interactions = 0;
    bs_stats stats{};
    // table reuse between runs (bs_set_lut_reuse)
    bool reuse = false;
    int stream_prio = 0;  // bs_set_stream_priority (0: the default priority)
    int lut_staging = 0;  // bs_set_lut_staging: 0 model-chosen, 1 staged kernel, 2 texture-only kernel
    int lut_chunk = 0;    // bs_set_lut_wave_chunk: 0 model-chosen, else waves per chunk
    bool bp_on = false;   // bs_set_backpropagation
    double bp_d = 0;
    DevBuf d_bp;          // back-propagation phase on the passband grid
    DevBuf d_shrec, d_shtab, d_shcoef;  // direct method: harmonic recurrences, per-wave and per-sphere tables
    DevBuf d_gscr;        // split-K parts of the detector GEMMs
    DevBuf d_ufw;         // condenser aperture factor per order of the incident field
    bool lut_valid = false;
    std::vector<double> lut_key;
};

// Every linear device buffer of a context.
static std::vector<DevBuf*> ctx_bufs(bs_ctx* c) {
    return {&c->d_sph, &c->d_waves, &c->d_kw4, &c->d_ph, &c->d_A, &c->d_B, &c->d_mie, &c->d_tab,
            &c->d_tabscr, &c->d_legP, &c->d_lut, &c->d_uft, &c->d_uftscr, &c->d_fields, &c->d_su,
            &c->d_sv, &c->d_mask, &c->d_wx, &c->d_wy, &c->d_wix, &c->d_wiy, &c->d_f1, &c->d_f2,
            &c->d_g1, &c->d_I, &c->d_D, &c->d_img, &c->d_cones, &c->d_cnt, &c->d_far,
            &c->d_starts, &c->d_lbjobs, &c->d_lbjobs2, &c->d_kcmp, &c->d_fsave, &c->d_dacc, &c->d_line, &c->d_ringcs, &c->d_bp, &c->d_shrec, &c->d_shtab, &c->d_shcoef, &c->d_gscr, &c->d_ufw};
}

static void release_all(bs_ctx* c) {
    for (DevBuf* b : ctx_bufs(c)) b->release();
    for (auto& sl : c->slots) sl.release();
    c->d_texobj.release();
    c->legP_theta = c->legP_L = 0;
    c->lut_valid = false;
    c->have = false;
}

static size_t elem_r(int prec) { return prec == BS_PREC_FP64 ? sizeof(double) : sizeof(float); }

extern "C" {

const char* bs_version(void) { return "bimsim-gb300 0.1 (sm_103a)"; }

const char* bs_last_error(void) { return g_err.c_str(); }

}  // extern "C"

// Lets other translation units of the library report through bs_last_error().
namespace bs {
void set_last_error(const char* msg) { g_err = msg; }
}  // namespace bs

extern "C" {

// Every kernel loaded on the context's device before its first run (once per
// device and process; see preload_nearfield_kernels).
static void preload_kernels(int device) {
    static std::mutex mu;
    static std::vector<int> done;
    std::lock_guard<std::mutex> lock(mu);
    if (std::find(done.begin(), done.end(), device) != done.end()) return;
    preload_nearfield_kernels();
    preload_detector_kernels();
    cudaGetLastError();  // a kernel this device cannot load reports at its launch instead
    done.push_back(device);
}

bs_status bs_create(const bs_params* params, bs_ctx** out) {
    if (!params || !out) return fail(BS_ERR_ARG, "bs_create: null argument");
    std::string why;
    if (!valid_params(params, why)) return fail(BS_ERR_ARG, "bs_create: %s", why.c_str());
    bs_ctx* c = new bs_ctx();
    c->prm = *params;
    cudaError_t e = cudaGetDevice(&c->device);
    if (e == cudaSuccess) preload_kernels(c->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
    for (int i = 0; i < 6 && e == cudaSuccess; i++) e = cudaEventCreate(&c->ev[i]);
    for (DevBuf* b : ctx_bufs(c)) b->st = &c->st;
    c->d_texobj.st = &c->st;
    if (e != cudaSuccess) {
        delete c;
        return fail(BS_ERR_CUDA, "bs_create: %s", cudaGetErrorString(e));
    }
    *out = c;
    return BS_OK;
}

bs_status bs_destroy(bs_ctx* c) {
    if (!c) return BS_OK;
    if (c->st) cudaStreamSynchronize(c->st);
    release_all(c);
    if (c->st) cudaStreamSynchronize(c->st);  // the stream-ordered frees
    for (int i = 0; i < 6; i++)
        if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    if (c->st) cudaStreamDestroy(c->st);
    delete c;
    return BS_OK;
}

bs_status bs_set_params(bs_ctx* c, const bs_params* params) {
    if (!c || !params) return fail(BS_ERR_ARG, "bs_set_params: null argument");
    std::string why;
    if (!valid_params(params, why)) return fail(BS_ERR_ARG, "bs_set_params: %s", why.c_str());
    c->prm = *params;
    c->have = false;
    return BS_OK;
}

bs_status bs_set_spheres(bs_ctx* c, const bs_sphere* s, int32_t n) {
    if (!c || n < 0 || (n > 0 && !s)) return fail(BS_ERR_ARG, "bs_set_spheres: bad arguments");
    for (int i = 0; i < n; i++)
        if (!(s[i].a > 0) || !std::isfinite(s[i].x) || !std::isfinite(s[i].y) || !std::isfinite(s[i].z))
            return fail(BS_ERR_ARG, "bs_set_spheres: sphere %d has a non-positive radius or bad centre", i + 1);
    c->spheres.assign(s, s + n);
    c->have = false;
    return BS_OK;
}

bs_status bs_set_waves(bs_ctx* c, const double* dirs, int32_t nk) {
    if (!c || nk < 1 || !dirs) return fail(BS_ERR_ARG, "bs_set_waves: need at least one direction");
    c->waves.assign(dirs, dirs + 3 * (size_t)nk);
    c->waves_set = true;
    c->have = false;
    return BS_OK;
}

bs_status bs_sample_waves_compat(bs_ctx* c, int32_t nk) {
    if (!c || nk < 1) return fail(BS_ERR_ARG, "bs_sample_waves_compat: nk must be >= 1");
    c->waves.resize(3 * (size_t)nk);
    mc_sample_compat(nk, c->prm.k_dir, c->prm.condenser[0], c->prm.condenser[1], c->waves.data());
    c->waves_set = true;
    c->have = false;
    return BS_OK;
}

bs_status bs_set_lut_budget(bs_ctx* c, size_t bytes) {
    if (!c) return fail(BS_ERR_ARG, "bs_set_lut_budget: null context");
    c->budget = bytes;
    return BS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Derivation of the slice and sphere parameters (arguments.h:340-438,
// microscope.cu:700-718, sphere.cpp:222-240, nfScalarUpLut.cu:365-379)
// ---------------------------------------------------------------------------
static bs_status derive(bs_ctx* c) {
    const bs_params& p = c->prm;
    Quad det = quad_from(p.plane_min, p.plane_max, p.plane_normal);
    Quad nf = quad_scale(det, (double)(2 * p.padding + 1));
    c->res = p.resolution;
    c->ss = p.supersample;
    c->crop = c->res * c->ss;
    c->off = p.padding * c->crop;
    c->R = c->crop * (2 * p.padding + 1);
    Scene& sc = c->sc;
    sc = Scene{};
    const V3* v[3] = {&nf.A, &nf.X, &nf.Y};
    double* d[3] = {sc.A, sc.X, sc.Y};
    for (int i = 0; i < 3; i++) {
        d[i][0] = v[i]->x;
        d[i][1] = v[i]->y;
        d[i][2] = v[i]->z;
    }
    for (int i = 0; i < 3; i++) {
        sc.focus[i] = p.focus[i];
        sc.kdir[i] = p.k_dir[i];
    }
    sc.kmag = 2 * PI_REF / p.lambda;
    sc.amp = p.amplitude;
    sc.cos_a = std::cos(std::asin(p.condenser[0]));
    sc.cos_b = std::cos(std::asin(p.condenser[1]));
    sc.R = c->R;
    sc.m = p.field_order;
    sc.plane_wave = p.plane_wave;
    sc.lut_uf = p.lut_uf;
    sc.lut_us = p.lut_us;
    sc.scalar = p.scalar;
    if (p.plane_wave) {
        sc.nk = 1;
        sc.wave_amp = p.amplitude;
    } else {
        if (!c->waves_set)
            return fail(BS_ERR_STATE, "bs_simulate: no plane-wave directions (call bs_set_waves or bs_sample_waves_compat)");
        sc.nk = (int)(c->waves.size() / 3);
        double sub = 2 * PI_REF * p.amplitude * ((1 - sc.cos_b) - (1 - sc.cos_a));
        // the Monte Carlo weight is the reference's single-precision quotient 1.0f/nk
        // (nfScalarUs.cu:457, nfScalarUpLut.cu:83,89), kept in every precision
        sc.wave_amp = (double)(1.0f / (float)sc.nk) * sub;
    }
    V3 f{p.focus[0], p.focus[1], p.focus[2]};
    sc.uf_dmin = quad_dist(nf, f);
    sc.uf_dmax = quad_dist_max(nf, f);
    sc.uf_dR = p.uf_lut_r > 0 ? p.uf_lut_r : 2 * c->R;
    sc.ns = (int)c->spheres.size();
    c->hs.resize(sc.ns);
    double diag = v3_len(V3{nf.X.x + nf.Y.x, nf.X.y + nf.Y.y, nf.X.z + nf.Y.z});
    int coef = 0;
    c->Lmax = std::max(2, sc.m + 1);
    for (int i = 0; i < sc.ns; i++) {
        const bs_sphere& in = c->spheres[i];
        Sphere& S = c->hs[i];
        S = Sphere{};
        S.p[0] = in.x;
        S.p[1] = in.y;
        S.p[2] = in.z;
        S.a = in.a;
        S.n_re = in.n_re;
        S.n_im = in.n_im;
        S.Nl = calc_nl(in.a, p.lambda);
        if (S.Nl < 1 || S.Nl > MAX_ORDER) return fail(BS_ERR_ARG, "sphere %d: order %d out of range", i + 1, S.Nl);
        V3 ctr{in.x, in.y, in.z};
        S.dmin = quad_dist(nf, ctr);
        S.dmax = quad_dist_max(nf, ctr);
        double a_inter = (S.dmin < in.a) ? std::sqrt(in.a - S.dmin) : 0.0;  // sphere.cpp:231-233 (sic)
        S.aR = (int)(1 + 2.0 * c->R * a_inter / diag);
        S.dR = p.us_lut_r > 0 ? p.us_lut_r : 2 * c->R;
        S.thetaR = p.us_lut_theta > 0 ? p.us_lut_theta : 1000;
        S.r0 = std::max(in.a, S.dmin);
        S.xs_usp = (S.dR - 1) / (S.dmax - S.r0);
        S.xs_uip = (S.aR - 1) / (S.a - S.dmin);
        S.coef_off = coef;
        coef += S.Nl + 1;
        c->Lmax = std::max(c->Lmax, S.Nl + 1);
    }
    return BS_OK;
}

// ---------------------------------------------------------------------------
// The band-limited detector (microscope.cu:495-526, 608-662)
// ---------------------------------------------------------------------------
// Frequency of FFT bin i as the reference's bandpass kernel assigns it (note
// -(R-1-i) rather than -(R-i) on the negative side).
static double bin_freq(int i, int R, double step) { return (i <= R / 2) ? i * step : -(double)(R - 1 - i) * step; }

// applyBackpropagation's factor -exp(i kz d) at spectrum bin (iu, iv) of an R x R near field, in the
// reference kernel's own arithmetic (microscope.cu:423-488): the momentum-space width Kx, its step
// dkx, kx, k and kz are single-precision variables, du, dv and lambda double, and the phase kz d a
// single-precision product; zero where kx^2 + ky^2 >= k^2, compared in single precision.
static void backprop_factor(int iu, int iv, int R, double du, double dv, double lambda, float d, double* re,
                            double* im) {
    const float two_pi = 2.0f * (float)PI_REF;  // 2*PI, PI = 3.14159f
    const float dkx = (float)((double)(two_pi * (float)R) * du) / (float)R;
    const float dky = (float)((double)(two_pi * (float)R) * dv) / (float)R;
    const float kx = (float)(iu <= R / 2 ? (double)iu * (double)dkx : -(double)(R - 1 - iu) * (double)dkx);
    const float ky = (float)(iv <= R / 2 ? (double)iv * (double)dky : -(double)(R - 1 - iv) * (double)dky);
    const float k = (float)((double)two_pi / lambda);
    const float kx_sq = kx * kx, ky_sq = ky * ky, k_sq = k * k;
    if (!(kx_sq + ky_sq < k_sq)) {
        *re = *im = 0.0;
        return;
    }
    const float kk = k * k, q = kk - kx_sq;
    const float kz = std::sqrt(q - ky_sq);
    const double ph = (double)(kz * d);
    *re = -std::cos(ph);
    *im = -std::sin(ph);
}

// Bins along u and v inside the objective's outer NA (the only ones the
// band-pass keeps), with the frequency steps.
static void passbands(const bs_ctx* c, std::vector<int>& su, std::vector<int>& sv, double& du, double& dv) {
    const int R = c->R;
    du = 1.0 / std::sqrt(c->sc.X[0] * c->sc.X[0] + c->sc.X[1] * c->sc.X[1] + c->sc.X[2] * c->sc.X[2]);
    dv = 1.0 / std::sqrt(c->sc.Y[0] * c->sc.Y[0] + c->sc.Y[1] * c->sc.Y[1] + c->sc.Y[2] * c->sc.Y[2]);
    const double hi = c->prm.objective[1] / c->prm.lambda;
    su.clear();
    sv.clear();
    for (int i = 0; i < R; i++) {
        if (std::fabs(bin_freq(i, R, du)) <= hi) su.push_back(i);
        if (std::fabs(bin_freq(i, R, dv)) <= hi) sv.push_back(i);
    }
}

template <class T>
static bs_status run_detector(bs_ctx* c, bool accumulate) {
    const bs_params& p = c->prm;
    const int R = c->R;
    double du, dv;
    std::vector<int> su, sv;
    passbands(c, su, sv, du, dv);
    double lo = p.objective[0] / p.lambda, hi = p.objective[1] / p.lambda;
    auto freq = [R](int i, double step) { return bin_freq(i, R, step); };
    const int Nu = (int)su.size(), Nv = (int)sv.size(), C = c->crop, res = c->res;
    c->det_Nv = (Nu == 0) ? 0 : Nv;
    CK(c->d_D.ensure(2 * (size_t)res * res * sizeof(T)));
    if (Nu == 0 || Nv == 0) {
        if (!accumulate) CK(cudaMemsetAsync(c->d_D.p, 0, 2 * (size_t)res * res * sizeof(T), c->st));
        return BS_OK;
    }
    std::vector<float> mask((size_t)Nv * Nu);
    for (int j = 0; j < Nv; j++)
        for (int k = 0; k < Nu; k++) {
            double u = freq(su[k], du), v = freq(sv[j], dv);
            double fm = std::sqrt(u * u + v * v);
            mask[(size_t)j * Nu + k] = (fm < lo || fm > hi) ? 0.f : 1.f;
        }
    size_t ce = sizeof(cpx<T>);
    CK(c->d_su.ensure(Nu * sizeof(int)));
    CK(c->d_sv.ensure(Nv * sizeof(int)));
    CK(c->d_mask.ensure(mask.size() * sizeof(float)));
    CK(c->d_wx.ensure((size_t)R * Nu * ce));
    CK(c->d_wy.ensure((size_t)Nv * R * ce));
    CK(c->d_wix.ensure((size_t)Nu * C * ce));
    CK(c->d_wiy.ensure((size_t)C * Nv * ce));
    CK(c->d_f1.ensure(2 * (size_t)R * Nu * ce));
    CK(c->d_f2.ensure(2 * (size_t)Nv * Nu * ce));
    CK(c->d_g1.ensure(2 * (size_t)Nv * C * ce));
    CK(c->d_I.ensure(2 * (size_t)C * C * sizeof(T)));
    CK(cudaMemcpyAsync(c->d_su.p, su.data(), Nu * sizeof(int), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->d_sv.p, sv.data(), Nv * sizeof(int), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->d_mask.p, mask.data(), mask.size() * sizeof(float), cudaMemcpyHostToDevice, c->st));
    cpx<T>* wx = c->d_wx.as<cpx<T>>();
    cpx<T>* wy = c->d_wy.as<cpx<T>>();
    cpx<T>* wix = c->d_wix.as<cpx<T>>();
    cpx<T>* wiy = c->d_wiy.as<cpx<T>>();
    // forward x: Wx[x][k] = e^{-2 pi i x su_k / R}; forward y: Wy[j][y] = e^{-2 pi i y sv_j / R}
    launch_twiddle<T>(R, Nu, c->d_su.as<int>(), 0, R, -1, Nu, 1, wx, c->st);
    LAUNCHED(c);
    launch_twiddle<T>(R, Nv, c->d_sv.as<int>(), 0, R, -1, 1, R, wy, c->st);
    LAUNCHED(c);
    // inverse on the crop only: Wix[k][x] = e^{+2 pi i (off+x) su_k / R}, Wiy[y][j] likewise
    launch_twiddle<T>(C, Nu, c->d_su.as<int>(), c->off, R, +1, 1, C, wix, c->st);
    LAUNCHED(c);
    launch_twiddle<T>(C, Nv, c->d_sv.as<int>(), c->off, R, +1, Nv, 1, wiy, c->st);
    LAUNCHED(c);
    const cpx<T>* fields = c->d_fields.as<cpx<T>>();
    cpx<T>* f1 = c->d_f1.as<cpx<T>>();
    cpx<T>* f2 = c->d_f2.as<cpx<T>>();
    cpx<T>* g1 = c->d_g1.as<cpx<T>>();
    T* I = c->d_I.as<T>();
    long long RR = (long long)R * R;
    // split-K scratch for the GEMMs with few output tiles
    const size_t scr = std::max(std::max(cgemm_scratch_elems(R, Nu, R, 2), cgemm_scratch_elems(Nv, Nu, R, 2)),
                                std::max(cgemm_scratch_elems(Nv, C, Nu, 2), cgemm_scratch_elems(C, C, Nv, 2)));
    CK(c->d_gscr.ensure(std::max<size_t>(scr, 1) * ce));
    cpx<T>* gs = c->d_gscr.as<cpx<T>>();
    launch_cgemm<T>(R, Nu, R, 2, fields, R, RR, wx, Nu, 0, f1, Nu, (long long)R * Nu, 0, nullptr, (T)1, nullptr, gs,
                    scr, c->st);
    LAUNCHED(c);
    launch_cgemm<T>(Nv, Nu, R, 2, wy, R, 0, f1, Nu, (long long)R * Nu, f2, Nu, (long long)Nv * Nu, 1,
                    c->d_mask.as<float>(), (T)1, nullptr, gs, scr, c->st);
    LAUNCHED(c);
    if (c->bp_on) {
        // applyBackpropagation (microscope.cu:423-488, 592-605) on U only: -exp(i kz d) with
        // kz = sqrt(k^2 - kx^2 - ky^2), k = 2 PI / lambda, kx = 2 PI u; zero where kx^2 + ky^2 >= k^2
        std::vector<cpx<T>> bp((size_t)Nv * Nu);
        for (int j = 0; j < Nv; j++)
            for (int kk = 0; kk < Nu; kk++) {
                double re, im;
                backprop_factor(su[kk], sv[j], R, du, dv, p.lambda, (float)c->bp_d, &re, &im);
                bp[(size_t)j * Nu + kk] = mk((T)re, (T)im);
            }
        CK(c->d_bp.ensure(bp.size() * sizeof(cpx<T>)));
        CK(cudaMemcpyAsync(c->d_bp.p, bp.data(), bp.size() * sizeof(cpx<T>), cudaMemcpyHostToDevice, c->st));
        launch_cmul<T>(Nv * Nu, c->d_bp.as<cpx<T>>(), f2, c->st);  // batch 0: U
        LAUNCHED(c);
        CK(cudaStreamSynchronize(c->st));  // bp is a host vector of this scope
    }
    launch_cgemm<T>(Nv, C, Nu, 2, f2, Nu, (long long)Nv * Nu, wix, C, 0, g1, C, (long long)Nv * C, 0, nullptr, (T)1,
                    nullptr, gs, scr, c->st);
    LAUNCHED(c);
    T scale = (T)(1.0 / ((double)R * (double)R));
    launch_cgemm<T>(C, C, Nv, 2, wiy, Nv, 0, g1, C, (long long)Nv * C, nullptr, C, (long long)C * C, 2, nullptr,
                    scale, I, gs, scr, c->st);
    LAUNCHED(c);
    launch_bin<T>(res, c->ss, 2, accumulate ? 1 : 0, I, c->d_D.as<T>(), c->st);
    LAUNCHED(c);
    return BS_OK;
}

// Place each sphere's Usp and Uip patches in the LUT pool; spheres whose
// tables together exceed the budget go to later chunks (each chunk is built
// and applied before the next one overwrites the pool).  FP64: one
// Patch<double> per entry.  Mixed: one float2 per entry in linear rows of
// thetaR + 1 entries (the last column repeated, rounded up to an even count
// for 16-byte rows), and a second copy of every entry in the texture planes,
// which also counts against the budget.
static bs_status plan_tables(std::vector<Sphere>& hs, bool mixed, size_t budget, std::vector<int>& chunk_start,
                             size_t& pool, size_t& maxrows, size_t& maxL) {
    const size_t patch = mixed ? sizeof(float2) : sizeof(Patch<double>);
    const size_t copies = mixed ? 2 : 1;
    const int ns = (int)hs.size();
    chunk_start.clear();
    size_t acc = 0;
    pool = 0;
    maxrows = 0;
    maxL = 0;
    for (int i = 0; i < ns; i++) {
        Sphere& S = hs[i];
        S.lin_stride = mixed ? ((S.thetaR + 2) & ~1) : S.thetaR;
        size_t need = (size_t)(S.dR + S.aR) * S.lin_stride * patch;
        if (need * copies > budget)
            return fail(BS_ERR_NOMEM, "LUT of sphere %d needs %zu bytes, over the budget of %zu", i + 1,
                        need * copies, budget);
        if (i == 0 || (acc + need) * copies > budget) {
            chunk_start.push_back(i);
            acc = 0;
        }
        S.usp_off = (int64_t)(acc / patch);
        S.uip_off = S.usp_off + (int64_t)S.dR * S.lin_stride;
        acc += need;
        pool = std::max(pool, acc);
        maxrows = std::max(maxrows, (size_t)(S.dR + S.aR));
        maxL = std::max(maxL, (size_t)(S.Nl + 1));
    }
    chunk_start.push_back(ns);
    return BS_OK;
}

// Spheres whose coefficient rows are computed in one launch: consecutive
// spheres of a table chunk, at most COEF_BATCH_ROWS rows together (a single
// larger sphere forms its own batch).  starts: first global row of each sphere
// and the total, then the first coefficient of each sphere.
constexpr long long COEF_BATCH_ROWS = 1 << 19;

struct CoefBatch {
    int b0, b1;
    long long rows, coefs;
    std::vector<long long> starts;
};

static std::vector<CoefBatch> coef_batches(const std::vector<Sphere>& hs, const std::vector<int>& chunk_start) {
    std::vector<CoefBatch> out;
    for (size_t ci = 0; ci + 1 < chunk_start.size(); ci++) {
        int b0 = chunk_start[ci];
        const int s1 = chunk_start[ci + 1];
        while (b0 < s1) {
            CoefBatch b{b0, b0, 0, 0, {}};
            std::vector<long long> cs;
            while (b.b1 < s1) {
                const Sphere& S = hs[b.b1];
                const long long r = S.dR + S.aR;
                if (b.b1 > b0 && b.rows + r > COEF_BATCH_ROWS) break;
                b.starts.push_back(b.rows);
                cs.push_back(b.coefs);
                b.rows += r;
                b.coefs += r * (S.Nl + 1);
                b.b1++;
            }
            b.starts.push_back(b.rows);
            b.starts.insert(b.starts.end(), cs.begin(), cs.end());
            out.push_back(std::move(b));
            b0 = out.back().b1;
        }
    }
    return out;
}

static bs_status plan_luts(bs_ctx* c, bool mixed, std::vector<int>& chunk_start, size_t& pool, size_t& maxrows,
                           size_t& maxL) {
    size_t budget = c->budget;
    if (!budget) {
        size_t free_b = 0, total_b = 0;
        CK(cudaMemGetInfo(&free_b, &total_b));
        budget = (size_t)(0.80 * (double)(free_b + c->d_lut.n * (mixed ? 2 : 1)));
    }
    return plan_tables(c->hs, mixed, budget, chunk_start, pool, maxrows, maxL);
}

// Order plane waves in compact groups of `chunk`: their projections on the
// plane perpendicular to the mean direction are split recursively at a
// multiple of `chunk` along the wider axis (a median split when the count
// allows), so every group but one holds `chunk` waves and the one short
// group goes last.  The sum over waves does not depend on the order (up to
// rounding); compact groups have narrow bounding cones, so each tile's table
// window per group stays small enough for shared memory (on the config-2 scene
// 98-99.7 % of windows fit, against 60-86 % for chunks cut from a Hilbert
// curve order, whose chunks can straddle the curve's jumps).
static void group_split(std::vector<size_t>& idx, size_t lo, size_t hi, const std::vector<double>& px,
                        const std::vector<double>& py, size_t chunk, std::vector<std::pair<size_t, size_t>>& groups) {
    const size_t n = hi - lo;
    if (n <= chunk) {
        groups.push_back({lo, hi});
        return;
    }
    double x0 = px[idx[lo]], x1 = x0, y0 = py[idx[lo]], y1 = y0;
    for (size_t i = lo; i < hi; i++) {
        x0 = std::min(x0, px[idx[i]]);
        x1 = std::max(x1, px[idx[i]]);
        y0 = std::min(y0, py[idx[i]]);
        y1 = std::max(y1, py[idx[i]]);
    }
    const std::vector<double>& key = (x1 - x0 >= y1 - y0) ? px : py;
    std::stable_sort(idx.begin() + lo, idx.begin() + hi, [&key](size_t a, size_t b) { return key[a] < key[b]; });
    const size_t half = (size_t)std::llround((double)n / (2.0 * (double)chunk));
    const size_t k = chunk * std::max<size_t>(1, half);
    group_split(idx, lo, lo + k, px, py, chunk, groups);
    group_split(idx, lo + k, hi, px, py, chunk, groups);
}

static void sort_waves(std::vector<double>& w, int chunk) {
    size_t nk = w.size() / 3;
    if (nk < 3) return;
    double m[3] = {0, 0, 0};
    for (size_t i = 0; i < nk; i++)
        for (int c = 0; c < 3; c++) m[c] += w[3 * i + c];
    double ml = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
    if (!(ml > 0)) return;
    for (int c = 0; c < 3; c++) m[c] /= ml;
    double a[3] = {1, 0, 0};
    if (std::fabs(m[0]) > 0.9) a[0] = 0, a[1] = 1;
    double e1[3] = {a[1] * m[2] - a[2] * m[1], a[2] * m[0] - a[0] * m[2], a[0] * m[1] - a[1] * m[0]};
    double l1 = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    for (int c = 0; c < 3; c++) e1[c] /= l1;
    double e2[3] = {m[1] * e1[2] - m[2] * e1[1], m[2] * e1[0] - m[0] * e1[2], m[0] * e1[1] - m[1] * e1[0]};
    std::vector<double> px(nk), py(nk);
    std::vector<size_t> idx(nk);
    for (size_t i = 0; i < nk; i++) {
        const double* k = &w[3 * i];
        px[i] = k[0] * e1[0] + k[1] * e1[1] + k[2] * e1[2];
        py[i] = k[0] * e2[0] + k[1] * e2[1] + k[2] * e2[2];
        idx[i] = i;
    }
    std::vector<std::pair<size_t, size_t>> groups;
    group_split(idx, 0, nk, px, py, (size_t)chunk, groups);
    std::stable_partition(groups.begin(), groups.end(),
                          [chunk](const std::pair<size_t, size_t>& g) { return g.second - g.first == (size_t)chunk; });
    std::vector<double> out;
    out.reserve(w.size());
    for (const auto& g : groups)
        for (size_t i = g.first; i < g.second; i++)
            for (int c = 0; c < 3; c++) out.push_back(w[3 * idx[i] + c]);
    w.swap(out);
}

// Bounding cone (unit axis, half-angle in radians) of every `chunk`
// consecutive waves, with a small margin for single-precision rounding.  A
// chunk holding a direction that is not a unit vector gets half-angle pi,
// which turns the angular window off for it.
static std::vector<float4> wave_cones(const std::vector<double>& w, int chunk) {
    size_t nk = w.size() / 3;
    size_t nch = (nk + chunk - 1) / chunk;
    std::vector<float4> out(nch);
    for (size_t ch = 0; ch < nch; ch++) {
        size_t a = ch * chunk, b = std::min(nk, a + chunk);
        double m[3] = {0, 0, 0};
        bool unit = true;
        for (size_t i = a; i < b; i++) {
            const double* k = &w[3 * i];
            double kl = std::sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
            if (!(std::fabs(kl - 1.0) <= 1e-6)) unit = false;
            for (int c = 0; c < 3; c++) m[c] += k[c];
        }
        double ml = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
        double beta = 0;
        if (ml > 1e-3 && unit) {
            for (int c = 0; c < 3; c++) m[c] /= ml;
            for (size_t i = a; i < b; i++) {
                const double* k = &w[3 * i];
                double cth = k[0] * m[0] + k[1] * m[1] + k[2] * m[2];
                beta = std::max(beta, std::acos(std::min(1.0, std::max(-1.0, cth))));
            }
        } else {
            m[0] = 0, m[1] = 0, m[2] = 1;
            beta = TRUE_PI;
        }
        out[ch] = make_float4((float)m[0], (float)m[1], (float)m[2], (float)(beta + 1e-4));
    }
    return out;
}

// Predicted fraction of (tile, sphere, wave chunk) units whose table window
// the staged mixed kernel can hold in shared memory, from the kernel's own
// bounds evaluated on a sample of tiles, spheres and chunks: the tile's
// distance range (nearest point of the tile rectangle, farthest corner) gives
// the rows, the corners' angles from the tile-centre direction give gamma.
// When few windows fit, the texture-only kernel is faster (no shared memory
// taken from the texture cache).
// Measured on the config-2 scene at 1536^2 near-field pixels (texture-only
// kernel 383 ms): staged kernel with 23 % of windows staged 395 ms, 41 %
// 360 ms, 85 % 329 ms; at 3072^2, 98 % staged 772 ms against 1510 ms.
// The fraction of windows the staged kernel must fit to beat the texture-only
// one: its texture fallback runs with the L1 that its shared-memory stage
// leaves -- 64-wave chunks (51 KB x 4 blocks per SM): 0.3; smaller chunks
// (72 KB x 3 blocks): 0.7 (served 256^2 - 512^2 requests with 48-62 % of
// windows staged took 169-320 ms staged against 123-273 ms texture-only;
// config 3 at 71 % 326 against 383 ms).
static double staged_min_fraction(int chunk) { return chunk >= WAVE_CHUNK_MAX ? 0.3 : 0.7; }
static double predict_staged_fraction(const bs_ctx* c, const std::vector<float4>& cones, int s0, int s1, int chunk) {
    const int cap = lut_stage_entries(chunk);
    const Scene& sc = c->sc;
    const int R = sc.R, tiles = (R + LUT_TILE - 1) / LUT_TILE;
    const int ts = std::max(1, tiles / 16), ss = std::max(1, (s1 - s0) / 32);
    const int cs = std::max(1, (int)cones.size() / 16);
    auto pos = [&](double u, double v, double* q) {
        for (int k = 0; k < 3; k++) q[k] = sc.A[k] + sc.X[k] * (u / R) + sc.Y[k] * (v / R);
    };
    const double X2 = sc.X[0] * sc.X[0] + sc.X[1] * sc.X[1] + sc.X[2] * sc.X[2];
    const double Y2 = sc.Y[0] * sc.Y[0] + sc.Y[1] * sc.Y[1] + sc.Y[2] * sc.Y[2];
    long long staged = 0, total = 0;
    for (int ty = 0; ty < tiles; ty += ts)
        for (int tx = 0; tx < tiles; tx += ts) {
            const double u0 = tx * LUT_TILE, v0 = ty * LUT_TILE;
            const double u1 = std::min(u0 + LUT_TILE - 1, (double)R - 1), v1 = std::min(v0 + LUT_TILE - 1, (double)R - 1);
            for (int si = s0; si < s1; si += ss) {
                const Sphere& S = c->hs[si];
                double e[3];
                for (int k = 0; k < 3; k++) e[k] = S.p[k] - sc.A[k];
                // nearest point of the tile rectangle (X and Y span the plane at right angles)
                const double un = std::min(std::max((e[0] * sc.X[0] + e[1] * sc.X[1] + e[2] * sc.X[2]) / X2 * R, u0), u1);
                const double vn = std::min(std::max((e[0] * sc.Y[0] + e[1] * sc.Y[1] + e[2] * sc.Y[2]) / Y2 * R, v0), v1);
                double q[3], ctr[3];
                pos(un, vn, q);
                const double dmin = std::sqrt((q[0] - S.p[0]) * (q[0] - S.p[0]) + (q[1] - S.p[1]) * (q[1] - S.p[1]) +
                                              (q[2] - S.p[2]) * (q[2] - S.p[2]));
                const int nch = (int)((cones.size() + cs - 1) / cs);
                total += nch;
                if (!(dmin >= S.a) || dmin == 0) continue;
                pos(u0 + 7.5, v0 + 7.5, ctr);
                double cl = 0;
                for (int k = 0; k < 3; k++) {
                    ctr[k] -= S.p[k];
                    cl += ctr[k] * ctr[k];
                }
                cl = std::sqrt(cl);
                double dmax = 0, gam = 0;
                const double cu[4] = {u0, u1, u0, u1}, cv[4] = {v0, v0, v1, v1};
                for (int k = 0; k < 4; k++) {
                    pos(cu[k], cv[k], q);
                    double r[3] = {q[0] - S.p[0], q[1] - S.p[1], q[2] - S.p[2]};
                    const double d = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
                    dmax = std::max(dmax, d);
                    const double cosg = (r[0] * ctr[0] + r[1] * ctr[1] + r[2] * ctr[2]) / (d * cl);
                    gam = std::max(gam, std::acos(std::min(1.0, std::max(-1.0, cosg))));
                }
                gam += LUT_STAGE_MARGIN;
                auto row = [&](double d) {
                    double x = (d - S.r0) / (S.dmax - S.r0) * (S.dR - 1);
                    return (int)std::floor(std::min(std::max(x, 0.0), (double)(S.dR - 1)));
                };
                const int rlo = row(dmin), nrows = std::min(row(dmax) + 1, S.dR - 1) - rlo + 1;
                const double tsc = (S.thetaR - 1) / PI_REF;
                for (size_t ch = 0; ch < cones.size(); ch += cs) {
                    const float4 k = cones[ch];
                    const double thc =
                        std::acos(std::min(1.0, std::max(-1.0, (k.x * ctr[0] + k.y * ctr[1] + k.z * ctr[2]) / cl)));
                    const int t_lo = std::max(0, (int)std::floor((thc - k.w - gam) * tsc) - 1);
                    const int t_hi = std::min(S.thetaR, (int)std::floor((thc + k.w + gam) * tsc) + 2);
                    const int W = t_hi - t_lo + 1;
                    if (W >= 2 && (long long)nrows * lut_stage_stride(W) <= cap) staged++;
                }
            }
        }
    return total ? (double)staged / (double)total : 0.0;
}

// Waves per chunk for the mixed LUT kernel, with the matching wave order and
// cones: the largest of 64, 32 and 16 whose predicted staged fraction reaches
// 0.8, else the one with the largest fraction if that reaches its
// staged_min_fraction, else the largest fraction among those that reach
// theirs.  Smaller chunks have narrower cones, so more windows fit, but each
// chunk pays a window copy, two barriers and a Kahan step.  64 whenever the
// texture-only kernel will run; bs_set_lut_wave_chunk fixes the chunk instead.
struct ChunkPlan {
    int chunk = WAVE_CHUNK_MAX;
    std::vector<double> w;
    std::vector<float4> cones;
    double predicted = 0;
};

static ChunkPlan choose_chunk(const bs_ctx* c, const std::vector<double>& waves, int ns) {
    ChunkPlan first, best, viable;  // viable: the best that the staged kernel would run to advantage
    best.predicted = viable.predicted = -1;
    if (c->lut_chunk) {
        best.chunk = c->lut_chunk;
        best.w = waves;
        sort_waves(best.w, best.chunk);
        best.cones = wave_cones(best.w, best.chunk);
        best.predicted = predict_staged_fraction(c, best.cones, 0, ns, best.chunk);
        return best;
    }
    for (int cand : {WAVE_CHUNK_MAX, WAVE_CHUNK_MAX / 2, WAVE_CHUNK_MAX / 4}) {
        ChunkPlan cp;
        cp.chunk = cand;
        cp.w = waves;
        sort_waves(cp.w, cand);
        cp.cones = wave_cones(cp.w, cand);
        cp.predicted = predict_staged_fraction(c, cp.cones, 0, ns, cand);
        if (cand == WAVE_CHUNK_MAX) {
            first = cp;
            if (c->lut_staging == 2) return first;
        }
        const bool enough = cp.predicted >= 0.8;
        if (cp.predicted >= staged_min_fraction(cand) && cp.predicted > viable.predicted) viable = cp;
        if (cp.predicted > best.predicted || enough) best = std::move(cp);
        if (enough) break;
    }
    if (c->lut_staging == 0 && best.predicted < staged_min_fraction(best.chunk)) {
        if (viable.predicted >= 0) return viable;
        return first;  // 64-wave chunks below their threshold too: the texture-only kernel runs
    }
    return best;
}

// ---------------------------------------------------------------------------
// The near field
// ---------------------------------------------------------------------------
template <class T>
static bs_status run_nearfield(bs_ctx* c) {
    Scene& sc = c->sc;
    const bs_params& p = c->prm;
    const int R = c->R, ns = sc.ns, nk = sc.nk;
    const bool fp64 = std::is_same<T, double>::value;
    CK(c->d_fields.ensure(2 * (size_t)R * R * sizeof(cpx<T>)));
    cpx<T>* U = c->d_fields.as<cpx<T>>();
    cpx<T>* Uf = U + (size_t)R * R;
    // upload spheres and waves
    CK(c->d_sph.ensure(std::max(1, ns) * sizeof(Sphere)));
    std::vector<double> w(c->waves);
    std::vector<float4> cones;
    int chunk = WAVE_CHUNK_MAX;
    double predicted = 0;
    if (p.plane_wave) {
        w.assign(p.k_dir, p.k_dir + 3);
    } else if (!fp64 && p.scalar && p.lut_us && ns > 0) {
        ChunkPlan cp = choose_chunk(c, w, ns);
        chunk = cp.chunk;
        w.swap(cp.w);
        cones.swap(cp.cones);
        predicted = cp.predicted;
    } else {
        sort_waves(w, chunk);
    }
    c->stats.lut_wave_chunk = chunk;
    CK(c->d_waves.ensure(w.size() * sizeof(double)));
    CK(cudaMemcpyAsync(c->d_waves.p, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, c->st));

    // ---- incident field ----
    cudaEventRecord(c->ev[0], c->st);
    if (p.lut_uf && !p.plane_wave && p.scalar) {
        CK(c->d_uft.ensure((size_t)sc.uf_dR * (sc.m + 1) * sizeof(double)));
        CK(c->d_uftscr.ensure((size_t)sc.uf_dR * (sc.m + 1) * sizeof(double)));
        launch_uf_table(sc, c->d_uft.as<double>(), c->d_uftscr.as<double>(), c->st);
        LAUNCHED(c);
    }
    {
        // condenser aperture factor of each order, the same for every pixel (nfScalarUf.cu:46-175)
        std::vector<double> w(sc.m + 1);
        double a0 = 1, a1 = sc.cos_a, a2 = 1, b0 = 1, b1 = sc.cos_b, b2 = 1;
        auto step = [](int n, double x, double& q0, double& q1) {  // rts/math/legendre.h:17-25
            const double qn = ((2 * n - 1) * x * q1 - (n - 1) * q0) / n;
            q0 = q1;
            q1 = qn;
        };
        for (int l = 0; l <= sc.m; l++) {
            if (l > 0) {
                a2 = a0;
                step(l + 1, sc.cos_a, a0, a1);
                b2 = b0;
                step(l + 1, sc.cos_b, b0, b1);
            }
            w[l] = a1 - a2 - b1 + b2;
        }
        CK(c->d_ufw.ensure(w.size() * sizeof(double)));
        CK(cudaMemcpyAsync(c->d_ufw.p, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, c->st));
        launch_uf<T>(sc, c->d_uft.as<double>(), c->d_ufw.as<double>(), Uf, c->st);
        LAUNCHED(c);
        CK(cudaStreamSynchronize(c->st));  // w is a host vector of this scope
    }
    cudaEventRecord(c->ev[1], c->st);

    // ---- LUT placement (before the sphere table goes to the device) ----
    std::vector<int> chunk_start;
    std::vector<CoefBatch> batches;
    size_t pool = 0, maxrows = 0, maxL = 0;
    if (p.scalar && p.lut_us && ns > 0) {
        bs_status pst = plan_luts(c, !fp64, chunk_start, pool, maxrows, maxL);
        if (pst != BS_OK) return pst;
        batches = coef_batches(c->hs, chunk_start);
    }

    // ---- Mie coefficients ----
    int ncoef = 0;
    for (auto& S : c->hs) ncoef += S.Nl + 1;
    const bool scatter = p.scalar && ns > 0;
    if (scatter) {
        CK(c->d_A.ensure(ncoef * sizeof(zd)));
        CK(c->d_B.ensure(ncoef * sizeof(zd)));
        CK(c->d_mie.ensure((size_t)ns * 6 * c->Lmax * sizeof(zd)));
        CK(cudaMemcpyAsync(c->d_sph.p, c->hs.data(), ns * sizeof(Sphere), cudaMemcpyHostToDevice, c->st));
        launch_mie(c->d_sph.as<Sphere>(), ns, sc.kmag, c->d_mie.as<zd>(), c->Lmax, c->d_A.as<zd>(),
                   c->d_B.as<zd>(), c->st);
        LAUNCHED(c);
        if (p.lut_us) {  // the LUT kernels' phases and float directions (the direct method forms its own)
            CK(c->d_ph.ensure((size_t)ns * nk * sizeof(cpx<T>)));
            CK(c->d_kw4.ensure((size_t)nk * sizeof(float4)));
            launch_phase<T>(sc, c->d_sph.as<Sphere>(), c->d_waves.as<double>(), c->d_ph.as<cpx<T>>(),
                            c->d_kw4.as<float4>(), c->st);
            LAUNCHED(c);
        }
    } else if (ns > 0) {
        CK(cudaMemcpyAsync(c->d_sph.p, c->hs.data(), ns * sizeof(Sphere), cudaMemcpyHostToDevice, c->st));
    }
    cudaEventRecord(c->ev[2], c->st);
    c->interactions = 0;

    if (!p.scalar) {
        launch_sum_only<T>(sc, c->d_sph.as<Sphere>(), Uf, U, c->st);
        LAUNCHED(c);
        cudaEventRecord(c->ev[3], c->st);
    } else if (!p.lut_us) {
        cudaEventRecord(c->ev[3], c->st);
        if (ns == 0) {
            CK(cudaMemcpyAsync(U, Uf, (size_t)R * R * sizeof(cpx<T>), cudaMemcpyDeviceToDevice, c->st));
        } else {
            // the addition theorem turns the per-wave Legendre sums into per-sphere coefficients
            const int L = c->Lmax, nlm = L * (L + 1) / 2;
            CK(c->d_shrec.ensure((size_t)nlm * sizeof(double2)));
            CK(c->d_shtab.ensure((size_t)nk * nlm * sizeof(double2)));
            CK(c->d_shcoef.ensure((size_t)ns * nlm * 2 * sizeof(zd)));
            launch_sh_tables(sc, c->d_sph.as<Sphere>(), L, c->d_waves.as<double>(), c->d_shrec.as<double2>(),
                             c->d_shtab.as<double2>(), c->d_shcoef.as<zd>(), c->st);
            c->launches += 3;
            launch_us_sh<T>(sc, c->d_sph.as<Sphere>(), L, c->d_A.as<zd>(), c->d_B.as<zd>(), c->d_shrec.as<double2>(),
                            c->d_shcoef.as<zd>(), Uf, U, c->st);
            LAUNCHED(c);
        }
        c->interactions = (long long)R * R * ns * nk;
    } else {
        int thetaR = ns > 0 ? c->hs[0].thetaR : 1000;
        if (ns > 0) {
            CK(c->d_lut.ensure(pool));
            long long maxcoef = 0, maxstarts = 0;
            for (const CoefBatch& b : batches) {
                maxcoef = std::max(maxcoef, b.coefs);
                maxstarts = std::max(maxstarts, (long long)b.starts.size());
            }
            CK(c->d_tab.ensure((size_t)maxcoef * sizeof(zd)));
            CK(c->d_tabscr.ensure((size_t)maxcoef * 2 * sizeof(double)));
            CK(c->d_starts.ensure((size_t)maxstarts * sizeof(long long)));
            if (c->legP_theta != thetaR || c->legP_L < c->Lmax) {
                CK(c->d_legP.ensure((size_t)thetaR * c->Lmax * sizeof(double)));
                launch_legendre_table(thetaR, c->Lmax, c->d_legP.as<double>(), c->st);
                LAUNCHED(c);
                c->legP_theta = thetaR;
                c->legP_L = c->Lmax;
            }
        }
        const int nchunks = (int)chunk_start.size() - 1;
        if (!fp64 && nchunks > 1) CK(c->d_kcmp.ensure((size_t)R * R * sizeof(float2)));
        bool use_stage = false;
        int max_chunk = 0;
        for (int ci = 0; ci < nchunks; ci++) max_chunk = std::max(max_chunk, chunk_start[ci + 1] - chunk_start[ci]);
        // tables of the previous run still in the pool and in the texture slots?
        std::vector<double> key;
        if (c->reuse && nchunks == 1) {
            key = {fp64 ? 1.0 : 0.0, sc.kmag, (double)c->Lmax, (double)ns};
            for (const Sphere& S : c->hs) {
                const double v[] = {S.p[0], S.p[1], S.p[2], S.a, S.n_re, S.n_im, S.dmin, S.dmax, S.r0,
                                    (double)S.Nl, (double)S.aR, (double)S.dR, (double)S.thetaR,
                                    (double)S.lin_stride, (double)S.usp_off, (double)S.uip_off};
                key.insert(key.end(), v, v + sizeof(v) / sizeof(v[0]));
            }
        }
        const bool reuse_now = !key.empty() && c->lut_valid && key == c->lut_key;
        c->lut_valid = false;  // set again below once this run's tables are complete
        c->stats.lut_tables_built = reuse_now ? 0 : ns;
        if (!fp64 && ns > 0) {
            // the texture planes are gather-capable 2D CUDA arrays (thetaR wide, rows + 1 high)
            int maxw = 0, maxh = 0;
            CK(cudaDeviceGetAttribute(&maxw, cudaDevAttrMaxTexture2DGatherWidth, c->device));
            CK(cudaDeviceGetAttribute(&maxh, cudaDevAttrMaxTexture2DGatherHeight, c->device));
            for (const Sphere& S : c->hs)
                if (S.thetaR > maxw || std::max(S.dR, S.aR) + 1 > maxh)
                    return fail(BS_ERR_UNSUPPORTED,
                                "mixed precision: a %d x %d lookup table exceeds the %d x %d texture limit of this GPU "
                                "(use BS_PREC_FP64 or fewer table samples)",
                                std::max(S.dR, S.aR), S.thetaR, maxh - 1, maxw);
            if ((int)c->slots.size() < max_chunk) c->slots.resize(max_chunk);
            CK(c->d_texobj.ensure((size_t)4 * max_chunk * sizeof(unsigned long long)));
            if (cones.empty()) {
                cones = wave_cones(w, chunk);
                predicted = predict_staged_fraction(c, cones, 0, ns, chunk);
            }
            c->stats.lut_staged_predicted = predicted;
            use_stage = c->lut_staging == 1 ||
                        (c->lut_staging == 0 && c->stats.lut_staged_predicted >= staged_min_fraction(chunk));
            CK(c->d_cones.ensure(cones.size() * sizeof(float4)));
            CK(cudaMemcpyAsync(c->d_cones.p, cones.data(), cones.size() * sizeof(float4), cudaMemcpyHostToDevice,
                               c->st));
            CK(c->d_cnt.ensure(2 * sizeof(unsigned long long)));
            CK(cudaMemsetAsync(c->d_cnt.p, 0, 2 * sizeof(unsigned long long), c->st));
        }
        bool first_build = true;
        for (int ci = 0; ci < std::max(1, nchunks); ci++) {
            int s0 = ns > 0 ? chunk_start[ci] : 0, s1 = ns > 0 ? chunk_start[ci + 1] : 0;
            std::vector<unsigned long long> handles;
            for (const CoefBatch& b : batches) {
                if (reuse_now || b.b0 < s0 || b.b1 > s1) continue;
                CK(cudaMemcpyAsync(c->d_starts.p, b.starts.data(), b.starts.size() * sizeof(long long),
                                   cudaMemcpyHostToDevice, c->st));
                launch_coef_rows_batch(c->d_sph.as<Sphere>(), b.b0, b.b1 - b.b0, c->d_starts.as<long long>(), b.rows,
                                       sc.kmag, c->d_A.as<zd>(), c->d_B.as<zd>(), c->d_tab.as<zd>(),
                                       c->d_tabscr.as<double>(), c->st);
                LAUNCHED(c);
                // mixed path: the tables of every sphere of the batch in two launches (the
                // dR-row Usp tables, then the shorter Uip tables)
                for (int t = 0; t < 2 && !fp64; t++) {
                    std::vector<LutBuildJob> jobs;
                    int max_rows = 0, max_theta = 1;
                    for (int i = b.b0; i < b.b1; i++) {
                        const Sphere& S = c->hs[i];
                        const int L = S.Nl + 1;
                        TexSlot& sl = c->slots[i - s0];
                        if (t == 0) {
                            // one spare row repeats the last, so a gather at the last row clamps as the texture would
                            const int rows[4] = {S.dR, S.dR, S.aR, S.aR};
                            for (int k = 0; k < 4; k++) CK(sl.ensure(k, S.thetaR, rows[k] + 1));
                        }
                        LutBuildJob j{};
                        j.tab_off = b.starts[(size_t)(b.b1 - b.b0) + 1 + (i - b.b0)] + (t ? (long long)S.dR * L : 0);
                        j.lin_off = t ? S.uip_off : S.usp_off;
                        j.rows = (t ? S.aR : S.dR) + 1;
                        j.L = L;
                        j.thetaR = S.thetaR;
                        j.lin_stride = S.lin_stride;
                        j.sre = sl.surf[2 * t];
                        j.sim = sl.surf[2 * t + 1];
                        max_rows = std::max(max_rows, j.rows);
                        max_theta = std::max(max_theta, S.thetaR);
                        jobs.push_back(j);
                    }
                    if (jobs.empty()) continue;
                    DevBuf& jb = t ? c->d_lbjobs2 : c->d_lbjobs;
                    CK(jb.ensure(jobs.size() * sizeof(LutBuildJob)));
                    CK(cudaMemcpyAsync(jb.p, jobs.data(), jobs.size() * sizeof(LutBuildJob), cudaMemcpyHostToDevice,
                                       c->st));
                    for (size_t j0 = 0; j0 < jobs.size(); j0 += 65535) {  // the grid's z extent
                        launch_lut_build_tex_batch(jb.as<LutBuildJob>() + j0,
                                                   (int)std::min<size_t>(65535, jobs.size() - j0), max_rows, max_theta,
                                                   c->d_tab.as<zd>(), c->d_legP.as<double>(), c->legP_L,
                                                   c->d_lut.as<float2>(), c->st);
                        LAUNCHED(c);
                    }
                }
                for (int i = b.b0; i < b.b1 && fp64; i++) {
                    const Sphere& S = c->hs[i];
                    const int L = S.Nl + 1;
                    const zd* tab = c->d_tab.as<zd>() + b.starts[(size_t)(b.b1 - b.b0) + 1 + (i - b.b0)];
                    Patch<double>* lut = c->d_lut.as<Patch<double>>();
                    launch_lut_build<double>(tab, S.dR, L, c->d_legP.as<double>(), c->legP_L, S.thetaR,
                                             lut + S.usp_off, c->st);
                    LAUNCHED(c);
                    launch_lut_build<double>(tab + (size_t)S.dR * L, S.aR, L, c->d_legP.as<double>(), c->legP_L,
                                             S.thetaR, lut + S.uip_off, c->st);
                    LAUNCHED(c);
                }
            }
            if (!fp64)
                for (int i = s0; i < s1; i++)
                    for (int k = 0; k < 4; k++) handles.push_back(c->slots[i - s0].tex[k]);
            if (!fp64 && !handles.empty())
                CK(cudaMemcpyAsync(c->d_texobj.p, handles.data(), handles.size() * sizeof(unsigned long long),
                                   cudaMemcpyHostToDevice, c->st));
            if (first_build) {
                cudaEventRecord(c->ev[3], c->st);
                first_build = false;
            }
            int finalize = (ci == std::max(1, nchunks) - 1);
            if (fp64) {
                launch_us_lut_f64(sc, c->d_sph.as<Sphere>(), s0, s1, ci > 0, finalize, c->d_waves.as<double>(),
                                  c->d_ph.as<zd>(), c->d_lut.as<Patch<double>>(), (const zd*)Uf, (zd*)U, c->st);
            } else {
                launch_us_lut_tex(sc, c->d_sph.as<Sphere>(), s0, s1, ci > 0, finalize, c->d_kw4.as<float4>(),
                                  c->d_cones.as<float4>(), c->d_ph.as<cpx<float>>(),
                                  c->d_texobj.as<unsigned long long>(), c->d_lut.as<float2>(), (const cpx<float>*)Uf,
                                  (cpx<float>*)U, ns > 0 ? c->d_cnt.as<unsigned long long>() : nullptr,
                                  nchunks > 1 ? c->d_kcmp.as<float2>() : nullptr, use_stage, chunk, c->st);
            }
            LAUNCHED(c);
            // the handle list and the table slots are reused by the next chunk
            if (!fp64 && ci + 1 < std::max(1, nchunks)) CK(cudaStreamSynchronize(c->st));
        }
        if (!key.empty()) {
            c->lut_key.swap(key);
            c->lut_valid = true;
        }
        c->interactions = (long long)R * R * ns * nk;
    }
    cudaEventRecord(c->ev[4], c->st);
    return BS_OK;
}

// Device bytes the buffers of run_nearfield and run_detector reach for the
// derived scene of `c` (each DevBuf at least 256 bytes; texture planes as
// width x height floats, as bs_get_info counts them).  0 if the tables do not
// fit lut_budget.
static size_t estimate_bytes(bs_ctx* c, bool fp64, size_t lut_budget) {
    const bs_params& p = c->prm;
    const Scene& sc = c->sc;
    const size_t R = c->R, ns = sc.ns, nk = sc.nk, C = c->crop, res = c->res;
    const size_t cT = fp64 ? sizeof(cpx<double>) : sizeof(cpx<float>), rT = fp64 ? sizeof(double) : sizeof(float);
    auto B = [](size_t n) { return std::max<size_t>(n, 256); };
    size_t b = 0;
    b += B(2 * R * R * cT);                                   // U, Uf
    b += B(std::max<size_t>(1, ns) * sizeof(Sphere));
    b += B((p.plane_wave ? 1 : nk) * 3 * sizeof(double));     // directions
    if (p.lut_uf && !p.plane_wave && p.scalar) b += 2 * B((size_t)sc.uf_dR * (sc.m + 1) * sizeof(double));
    b += B((size_t)(sc.m + 1) * sizeof(double));               // incident-field aperture factors
    if (p.scalar && ns > 0) {
        size_t ncoef = 0;
        for (const Sphere& S : c->hs) ncoef += S.Nl + 1;
        b += 2 * B(ncoef * sizeof(zd)) + B(ns * 6 * (size_t)c->Lmax * sizeof(zd));
        if (p.lut_us) b += B(ns * nk * cT) + B(nk * sizeof(float4));  // phases, float directions
        if (!p.lut_us) {  // direct method: harmonic recurrences, per-wave and per-sphere tables
            const size_t nlm = (size_t)c->Lmax * (c->Lmax + 1) / 2;
            b += B(nlm * sizeof(double2)) + B(nk * nlm * sizeof(double2)) + B(ns * nlm * 2 * sizeof(zd));
        }
    }
    if (p.scalar && p.lut_us && ns > 0) {
        std::vector<Sphere> hs = c->hs;
        std::vector<int> cs;
        size_t pool = 0, maxrows = 0, maxL = 0;
        if (plan_tables(hs, !fp64, lut_budget ? lut_budget : SIZE_MAX / 4, cs, pool, maxrows, maxL) != BS_OK)
            return 0;
        const size_t thetaR = hs[0].thetaR;
        long long maxcoef = 0, maxstarts = 0;
        for (const CoefBatch& cb : coef_batches(hs, cs)) {
            maxcoef = std::max(maxcoef, cb.coefs);
            maxstarts = std::max(maxstarts, (long long)cb.starts.size());
        }
        b += B(pool) + B((size_t)maxcoef * sizeof(zd)) + B((size_t)maxcoef * 2 * sizeof(double)) +
             B((size_t)maxstarts * sizeof(long long));
        b += B(thetaR * (size_t)c->Lmax * sizeof(double));    // Legendre table
        if (!fp64) {
            if (cs.size() > 2) b += B(R * R * sizeof(float2));  // Kahan carry between chunks
            // slot k holds the k-th sphere of every chunk: the largest of those tables, plus a spare row each
            size_t max_chunk = 0;
            for (size_t ci = 0; ci + 1 < cs.size(); ci++) max_chunk = std::max(max_chunk, (size_t)(cs[ci + 1] - cs[ci]));
            for (size_t k = 0; k < max_chunk; k++) {
                size_t hd = 0, ha = 0;
                for (size_t ci = 0; ci + 1 < cs.size(); ci++) {
                    const size_t i = cs[ci] + k;
                    if (i < (size_t)cs[ci + 1]) {
                        hd = std::max(hd, (size_t)hs[i].dR + 1);
                        ha = std::max(ha, (size_t)hs[i].aR + 1);
                    }
                }
                // the planes' rows are allocated in multiples of 256 (TexSlot::ensure)
                b += 2 * thetaR * (((hd + 255) & ~(size_t)255) + ((ha + 255) & ~(size_t)255)) * sizeof(float);
            }
            b += B(4 * max_chunk * sizeof(unsigned long long)) + B((nk + 15) / 16 * sizeof(float4)) +
                 B(2 * sizeof(unsigned long long));
        }
    }
    std::vector<int> su, sv;
    double du, dv;
    passbands(c, su, sv, du, dv);
    const size_t Nu = su.size(), Nv = sv.size();
    b += B(2 * res * res * rT);                               // D, Di
    if (Nu && Nv) {
        b += B(Nu * sizeof(int)) + B(Nv * sizeof(int)) + B(Nv * Nu * sizeof(float));
        b += B(R * Nu * cT) + B(Nv * R * cT) + B(Nu * C * cT) + B(C * Nv * cT);
        b += B(2 * R * Nu * cT) + B(2 * Nv * Nu * cT) + B(2 * Nv * C * cT) + B(2 * C * C * rT);
        const int Ri = (int)R, Ui = (int)Nu, Vi = (int)Nv, Ci = (int)C;
        const size_t scr = std::max(std::max(cgemm_scratch_elems(Ri, Ui, Ri, 2), cgemm_scratch_elems(Vi, Ui, Ri, 2)),
                                    std::max(cgemm_scratch_elems(Vi, Ci, Ui, 2), cgemm_scratch_elems(Ci, Ci, Vi, 2)));
        b += B(std::max<size_t>(scr, 1) * cT);  // split-K parts
    }
    b += B(res * res * rT);                                   // image staging
    return b;
}

extern "C" {

bs_status bs_set_backpropagation(bs_ctx* c, int32_t enable, double d) {
    if (!c || !std::isfinite(d)) return fail(BS_ERR_ARG, "bs_set_backpropagation: bad arguments");
    c->bp_on = enable != 0;
    c->bp_d = d;
    return BS_OK;
}

bs_status bs_set_lut_wave_chunk(bs_ctx* c, int32_t chunk) {
    if (!c || (chunk != 0 && chunk != 16 && chunk != 32 && chunk != 64))
        return fail(BS_ERR_ARG, "bs_set_lut_wave_chunk: chunk must be 0, 16, 32 or 64");
    c->lut_chunk = chunk;
    return BS_OK;
}

bs_status bs_set_lut_staging(bs_ctx* c, int32_t mode) {
    if (!c || mode < 0 || mode > 2) return fail(BS_ERR_ARG, "bs_set_lut_staging: mode must be 0, 1 or 2");
    c->lut_staging = mode;
    return BS_OK;
}

bs_status bs_set_stream_priority(bs_ctx* c, int32_t priority) {
    if (!c) return fail(BS_ERR_ARG, "bs_set_stream_priority: null context");
    int least = 0, greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e != cudaSuccess) return fail(BS_ERR_CUDA, "bs_set_stream_priority: %s", cudaGetErrorString(e));
    const int prio = std::min(least, std::max(greatest, (int)priority));
    if (prio == c->stream_prio) return BS_OK;
    // the context's work so far finishes on the old stream; later work goes to the new one
    e = cudaStreamSynchronize(c->st);
    cudaStream_t st = nullptr;
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, prio);
    if (e != cudaSuccess) return fail(BS_ERR_CUDA, "bs_set_stream_priority: %s", cudaGetErrorString(e));
    cudaStreamDestroy(c->st);
    c->st = st;
    c->stream_prio = prio;
    return BS_OK;
}

bs_status bs_set_lut_reuse(bs_ctx* c, int32_t enable) {
    if (!c) return fail(BS_ERR_ARG, "bs_set_lut_reuse: null context");
    c->reuse = enable != 0;
    if (!c->reuse) c->lut_valid = false;
    return BS_OK;
}

bs_status bs_release_buffers(bs_ctx* c) {
    if (!c) return fail(BS_ERR_ARG, "bs_release_buffers: null context");
    CK(cudaStreamSynchronize(c->st));
    release_all(c);
    return BS_OK;
}

bs_status bs_estimate_bytes(const bs_params* params, const bs_sphere* spheres, int32_t ns, int32_t nk,
                            bs_precision prec, uint64_t lut_budget, uint64_t* bytes) {
    if (!params || !bytes || ns < 0 || nk < 0 || (ns > 0 && !spheres))
        return fail(BS_ERR_ARG, "bs_estimate_bytes: bad arguments");
    if (prec != BS_PREC_FP64 && prec != BS_PREC_MIXED) return fail(BS_ERR_ARG, "bs_estimate_bytes: unknown precision");
    std::string why;
    if (!valid_params(params, why)) return fail(BS_ERR_ARG, "bs_estimate_bytes: %s", why.c_str());
    std::unique_ptr<bs_ctx> c(new bs_ctx());  // host state only: no stream, no device memory
    c->prm = *params;
    c->spheres.assign(spheres, spheres + ns);
    c->waves.assign(3 * (size_t)std::max(nk, 1), 0.0);
    c->waves_set = true;
    bs_status st = derive(c.get());
    if (st != BS_OK) return st;
    size_t b = estimate_bytes(c.get(), prec == BS_PREC_FP64, (size_t)lut_budget);
    if (!b) return fail(BS_ERR_NOMEM, "bs_estimate_bytes: a sphere's tables exceed the LUT budget of %llu bytes",
                        (unsigned long long)lut_budget);
    *bytes = b;
    return BS_OK;
}

}  // extern "C"

// One slice; with accumulate the detector images add to those of the previous
// slice on this context (same precision and detector size).
static bs_status simulate_impl(bs_ctx* c, bs_precision prec, bool accumulate) {
    c->have = false;
    bs_status st = derive(c);
    if (st != BS_OK) return st;
    c->prec = prec;
    c->stats.lut_tables_built = 0;
    c->stats.lut_staged_predicted = 0;
    int64_t l0 = c->launches;
    st = (prec == BS_PREC_FP64) ? run_nearfield<double>(c) : run_nearfield<float>(c);
    if (st != BS_OK) return st;
    st = (prec == BS_PREC_FP64) ? run_detector<double>(c, accumulate) : run_detector<float>(c, accumulate);
    if (st != BS_OK) return st;
    cudaEventRecord(c->ev[5], c->st);
    CK(cudaStreamSynchronize(c->st));
    CK(cudaGetLastError());
    float t[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < 5; i++) cudaEventElapsedTime(&t[i], c->ev[i], c->ev[i + 1]);
    c->stats.ms_uf = t[0];
    c->stats.ms_mie = t[1];
    c->stats.ms_lut = t[2];
    c->stats.ms_us = t[3];
    c->stats.ms_detector = t[4];
    float tot = 0;
    cudaEventElapsedTime(&tot, c->ev[0], c->ev[5]);
    c->stats.ms_total = tot;
    c->stats.kernel_launches = c->launches - l0;
    c->stats.us_interactions = c->interactions;
    c->stats.lut_chunks_staged = c->stats.lut_chunks_total = 0;
    if (prec == BS_PREC_MIXED && c->prm.scalar && c->prm.lut_us && !c->hs.empty()) {
        unsigned long long cnt[2] = {0, 0};
        CK(cudaMemcpy(cnt, c->d_cnt.p, sizeof(cnt), cudaMemcpyDeviceToHost));
        c->stats.lut_chunks_staged = (int64_t)cnt[0];
        c->stats.lut_chunks_total = (int64_t)cnt[1];
    }
    c->have = true;
    return BS_OK;
}

extern "C" {

bs_status bs_simulate(bs_ctx* c, bs_precision prec) {
    if (!c) return fail(BS_ERR_ARG, "bs_simulate: null context");
    if (prec != BS_PREC_FP64 && prec != BS_PREC_MIXED) return fail(BS_ERR_ARG, "bs_simulate: unknown precision");
    return simulate_impl(c, prec, false);
}

bs_status bs_simulate_sources(bs_ctx* c, const double* sources, int32_t n, bs_precision prec) {
    if (!c || !sources || n < 1) return fail(BS_ERR_ARG, "bs_simulate_sources: need at least one source");
    if (prec != BS_PREC_FP64 && prec != BS_PREC_MIXED)
        return fail(BS_ERR_ARG, "bs_simulate_sources: unknown precision");
    for (int32_t i = 0; i < n; i++)
        for (int k = 0; k < 4; k++)
            if (!std::isfinite(sources[4 * i + k]))
                return fail(BS_ERR_ARG, "bs_simulate_sources: source %d is not finite", i + 1);
    const bs_params saved = c->prm;
    const bool saved_reuse = c->reuse;
    c->reuse = true;  // the sphere tables do not depend on the focus or the amplitude
    bs_stats sum{};
    bs_status st = BS_OK;
    for (int32_t i = 0; i < n && st == BS_OK; i++) {
        for (int k = 0; k < 3; k++) c->prm.focus[k] = sources[4 * i + k];
        c->prm.amplitude = sources[4 * i + 3];
        st = simulate_impl(c, prec, i > 0);
        if (st != BS_OK) break;
        const bs_stats& s = c->stats;
        sum.ms_total += s.ms_total;
        sum.ms_uf += s.ms_uf;
        sum.ms_mie += s.ms_mie;
        sum.ms_lut += s.ms_lut;
        sum.ms_us += s.ms_us;
        sum.ms_detector += s.ms_detector;
        sum.kernel_launches += s.kernel_launches;
        sum.us_interactions += s.us_interactions;
        sum.lut_chunks_staged += s.lut_chunks_staged;
        sum.lut_chunks_total += s.lut_chunks_total;
        sum.lut_tables_built += s.lut_tables_built;
        sum.lut_staged_predicted = s.lut_staged_predicted;
        sum.lut_wave_chunk = s.lut_wave_chunk;
    }
    c->reuse = saved_reuse;
    if (!saved_reuse) c->lut_valid = false;
    const bool have = c->have;
    c->prm = saved;
    c->have = have && st == BS_OK;  // images stay valid: they do not depend on prm after the run
    if (st == BS_OK) c->stats = sum;
    return st;
}

}  // extern "C"

template <class T>
static bs_status far_field(bs_ctx* c, int which, double* host) {
    const int C = c->crop, Nv = c->det_Nv;
    const size_t n = (size_t)C * C;
    if (Nv == 0) {  // nothing passes the objective: the far field is zero
        std::fill(host, host + 2 * n, 0.0);
        return BS_OK;
    }
    CK(c->d_far.ensure(n * sizeof(cpx<T>)));
    const T scale = (T)(1.0 / ((double)c->R * (double)c->R));
    const cpx<T>* g1 = c->d_g1.as<cpx<T>>() + (size_t)which * Nv * C;
    launch_cgemm<T>(C, C, Nv, 1, c->d_wiy.as<cpx<T>>(), Nv, 0, g1, C, 0, c->d_far.as<cpx<T>>(), C, 0, 3, nullptr,
                    scale, nullptr, c->d_gscr.as<cpx<T>>(), c->d_gscr.n / sizeof(cpx<T>), c->st);
    LAUNCHED(c);
    std::vector<cpx<T>> t(n);
    CK(cudaMemcpyAsync(t.data(), c->d_far.p, n * sizeof(cpx<T>), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    for (size_t i = 0; i < n; i++) {
        host[2 * i] = (double)t[i].re;
        host[2 * i + 1] = (double)t[i].im;
    }
    return BS_OK;
}

extern "C" {

bs_status bs_get_far_field(bs_ctx* c, bs_field_kind kind, double* host, size_t count) {
    if (!c || !host) return fail(BS_ERR_ARG, "bs_get_far_field: null argument");
    if (!c->have) return fail(BS_ERR_STATE, "bs_get_far_field: no simulation result");
    if (kind != BS_FIELD_TOTAL && kind != BS_FIELD_INCIDENT) return fail(BS_ERR_ARG, "bs_get_far_field: unknown field");
    if (count < (size_t)c->crop * c->crop)
        return fail(BS_ERR_ARG, "bs_get_far_field: need %zu complex values", (size_t)c->crop * c->crop);
    const int which = kind == BS_FIELD_TOTAL ? 0 : 1;
    return c->prec == BS_PREC_FP64 ? far_field<double>(c, which, host) : far_field<float>(c, which, host);
}

bs_status bs_material_eval(const char* path, const double* lambdas, int32_t n, double* out) {
    if (!path || n < 0 || (n > 0 && (!lambdas || !out))) return fail(BS_ERR_ARG, "bs_material_eval: bad arguments");
    std::ifstream f(path);
    if (!f) return fail(BS_ERR_IO, "Material Error -- file not found: %s", path);
    std::string text((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    std::vector<float> lam, re, im;
    std::string err;
    if (!material_load(text, lam, re, im, err)) return fail(BS_ERR_IO, "%s: %s", path, err.c_str());
    for (int32_t i = 0; i < n; i++) {
        float r, k;
        material_eval(lam, re, im, (float)lambdas[i], r, k);
        out[2 * i] = r;
        out[2 * i + 1] = k;
    }
    return BS_OK;
}

bs_status bs_material_kk(const char* path, double n0, int32_t n_samples, int32_t pf, double* lambdas, double* n_out) {
    if (!path || !lambdas || !n_out || n_samples < 0 || pf < 1 || !(n0 > 0))
        return fail(BS_ERR_ARG, "bs_material_kk: bad arguments");
    std::ifstream f(path);
    if (!f) return fail(BS_ERR_IO, "Material Error -- file not found: %s", path);
    std::string text((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    // rts::material<double>: the instantiation whose arrays match FFTW's double transforms
    std::vector<double> lam, re, im;
    std::string err;
    if (!material_load(text, lam, re, im, err)) return fail(BS_ERR_IO, "%s: %s", path, err.c_str());
    const int N = n_samples ? n_samples : (int)lam.size();
    if (N < 2 || N > BS_KK_MAX_SAMPLES)
        return fail(BS_ERR_ARG, "bs_material_kk: %d samples (2 to %d)", N, BS_KK_MAX_SAMPLES);
    if (pf > 16) return fail(BS_ERR_ARG, "bs_material_kk: padding factor %d above 16", pf);
    const int M = N * pf;
    // resample kappa at evenly spaced wavenumbers, from the shortest wavelength up (material.h:294-316)
    const double nu_min = 10000.0 / lam.back(), nu_max = 10000.0 / lam.front();
    const double dnu = (nu_max - nu_min) / (N - 1);
    std::vector<double> chi2(N), kap(N);
    for (int i = 0; i < N; i++) {
        const double l = 10000.0 / (nu_max - i * dnu);
        double nr, ni;
        material_eval(lam, re, im, l, nr, ni);
        kap[i] = ni;
        const float k = (float)(2 * (float)PI_REF / l);      // float k, alpha as in the reference
        const float alpha = (float)(ni * (double)(2 * k));
        chi2[i] = -(double)alpha * (n0 / (double)k);
        lambdas[i] = l;
    }
    double *d_chi2 = nullptr, *d_g = nullptr, *d_chi1 = nullptr;
    cudaStream_t st = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&d_chi2, N * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d_g, (size_t)M * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d_chi1, N * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_chi2, chi2.data(), N * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        launch_kk(N, M, d_chi2, d_g, d_chi1, st);
        e = cudaGetLastError();
    }
    std::vector<double> chi1(N);
    if (e == cudaSuccess) e = cudaMemcpyAsync(chi1.data(), d_chi1, N * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_chi2);
    cudaFree(d_g);
    cudaFree(d_chi1);
    if (st) cudaStreamDestroy(st);
    if (e != cudaSuccess) return fail(BS_ERR_CUDA, "bs_material_kk: %s", cudaGetErrorString(e));
    for (int i = 0; i < N; i++) {
        n_out[2 * i] = chi1[i] / (2 * n0) + n0;
        n_out[2 * i + 1] = kap[i];
    }
    return BS_OK;
}

}  // extern "C"

// Ring point sources (--interpolate 1, 2, 3; microscope.cu:1004-1253).  Ring
// r = 1, 2, ... has radius r um; its sources sit at the angles of
// generatePointSources (microscope.cu:1298-1325): t_0 = 2 pi / points in float,
// each next one the float sum of the previous and that step; cosines and sines
// are double values rounded to float (the reference used float ones).
static std::vector<float> ring_angles(int points) {
    const float step = 2 * (float)PI_REF / (float)points;
    std::vector<float> t(points);
    float th = step;
    for (int i = 0; i < points; i++) {
        t[i] = th;
        th += step;
    }
    return t;
}

static void stats_add(bs_stats& sum, const bs_stats& s) {
    sum.ms_total += s.ms_total;
    sum.ms_uf += s.ms_uf;
    sum.ms_mie += s.ms_mie;
    sum.ms_lut += s.ms_lut;
    sum.ms_us += s.ms_us;
    sum.ms_detector += s.ms_detector;
    sum.kernel_launches += s.kernel_launches;
    sum.us_interactions += s.us_interactions;
    sum.lut_chunks_staged += s.lut_chunks_staged;
    sum.lut_chunks_total += s.lut_chunks_total;
    sum.lut_tables_built += s.lut_tables_built;
    sum.lut_staged_predicted = s.lut_staged_predicted;
    sum.lut_wave_chunk = s.lut_wave_chunk;
}

// One source of a ring driver at (x, y, z) with amplitude a; its stats are
// added to sum.  The sphere tables are built by the first source and reused.
static bs_status ring_source(bs_ctx* c, bs_precision prec, const double* xyz, double a, bool accumulate,
                             bs_stats& sum) {
    if (xyz)
        for (int k = 0; k < 3; k++) c->prm.focus[k] = xyz[k];
    c->prm.amplitude = a;
    bs_status st = simulate_impl(c, prec, accumulate);
    if (st == BS_OK) stats_add(sum, c->stats);
    return st;
}

// The detector images of the near field in d_fields rotated by each angle,
// added to the detector (nearfieldStruct::Interpolate + SimulateImaging,
// microscope.cu:834-846); d_fields itself is kept in d_fsave and overwritten.
template <class T>
static bs_status field_rotations(bs_ctx* c, const std::vector<float>& angles) {
    const size_t n = 2 * (size_t)c->R * c->R;
    CK(c->d_fsave.ensure(n * sizeof(cpx<T>)));
    CK(cudaMemcpyAsync(c->d_fsave.p, c->d_fields.p, n * sizeof(cpx<T>), cudaMemcpyDeviceToDevice, c->st));
    for (float a : angles) {
        launch_rotate_fields<T>(c->R, (float)std::cos((double)a), (float)std::sin((double)a), c->d_fsave.as<cpx<T>>(),
                                c->d_fields.as<cpx<T>>(), c->st);
        LAUNCHED(c);
        bs_status st = run_detector<T>(c, true);
        if (st != BS_OK) return st;
    }
    CK(cudaStreamSynchronize(c->st));
    CK(cudaGetLastError());
    return BS_OK;
}

// Mode 1 (InterpAtDetector, microscope.cu:312-321): the sum so far is in
// d_dacc, the ring's first source alone in d_D; both are added to d_dacc, then
// that image rotated by each angle.
template <class T>
static bs_status image_rotations(bs_ctx* c, const std::vector<float>& angles) {
    const T* one = c->d_D.as<T>();
    T* acc = c->d_dacc.as<T>();
    launch_rotate_add_images<T>(c->res, 1.f, 0.f, one, acc, c->st);  // angle 0: the image itself
    LAUNCHED(c);
    for (float a : angles) {
        launch_rotate_add_images<T>(c->res, (float)std::cos((double)a), (float)std::sin((double)a), one, acc, c->st);
        LAUNCHED(c);
    }
    CK(cudaStreamSynchronize(c->st));
    CK(cudaGetLastError());
    return BS_OK;
}

// Mode 2 (InterpLineForAllPointSources, microscope.cu:336-354): the current
// source's D and Di feed their radial lines.
template <class T>
static bs_status line_samples(bs_ctx* c, int points, int L) {
    launch_ring_line<T>(c->res, points, L, c->d_ringcs.as<float2>(), c->d_D.as<T>(), c->d_line.as<T>(), c->st);
    LAUNCHED(c);
    CK(cudaGetLastError());
    return BS_OK;
}

// Shared frame of the ring drivers: tables reused across the sources, the
// context's focus, amplitude and reuse setting restored afterwards.
template <class F>
static bs_status ring_driver(bs_ctx* c, bs_precision prec, int32_t points, int32_t rings, const char* name, F&& body) {
    if (!c || points < 1 || rings < 1) return fail(BS_ERR_ARG, "%s: points and rings must be >= 1", name);
    if (prec != BS_PREC_FP64 && prec != BS_PREC_MIXED) return fail(BS_ERR_ARG, "%s: unknown precision", name);
    const bs_params saved = c->prm;
    const bool saved_reuse = c->reuse;
    c->reuse = true;  // the sphere tables do not depend on the focus or the amplitude
    bs_stats sum{};
    bs_status st = body(sum);
    c->prm = saved;
    c->reuse = saved_reuse;
    if (!saved_reuse) c->lut_valid = false;
    if (st != BS_OK) {
        c->have = false;
        return st;
    }
    c->stats = sum;
    c->have = true;
    return BS_OK;
}

static void ring_focus(float t0, int ring, double* xyz) {
    xyz[0] = (float)std::cos((double)t0) * (float)ring;
    xyz[1] = (float)std::sin((double)t0) * (float)ring;
    xyz[2] = 0;
}

extern "C" {

bs_status bs_simulate_ring_interp(bs_ctx* c, int32_t points, int32_t rings, bs_precision prec) {
    return ring_driver(c, prec, points, rings, "bs_simulate_ring_interp", [&](bs_stats& sum) {
        // the source at the context's own focus (SimulateExtendedSourceWithInterpolation, microscope.cu:1189-1253)
        bs_status st = ring_source(c, prec, nullptr, c->prm.amplitude, false, sum);
        const std::vector<float> th = ring_angles(points);
        const std::vector<float> rest(th.begin() + 1, th.end());
        for (int ring = 1; ring < rings && st == BS_OK; ring++) {
            double f[3];
            ring_focus(th[0], ring, f);
            // only a ring's first source is simulated; source i's near field is that one rotated by its angle
            st = ring_source(c, prec, f, 1.0, true, sum);
            if (st == BS_OK && !rest.empty())
                st = prec == BS_PREC_FP64 ? field_rotations<double>(c, rest) : field_rotations<float>(c, rest);
        }
        return st;
    });
}

bs_status bs_simulate_ring_detector(bs_ctx* c, int32_t points, int32_t rings, bs_precision prec) {
    return ring_driver(c, prec, points, rings, "bs_simulate_ring_detector", [&](bs_stats& sum) {
        // SimulateExtendedSourceInterpAtDetector (microscope.cu:1004-1093)
        bs_status st = ring_source(c, prec, nullptr, c->prm.amplitude, false, sum);
        if (st != BS_OK) return st;
        const size_t bytes = 2 * (size_t)c->res * c->res * elem_r(prec);
        CK(c->d_dacc.ensure(bytes));
        CK(cudaMemcpyAsync(c->d_dacc.p, c->d_D.p, bytes, cudaMemcpyDeviceToDevice, c->st));
        const std::vector<float> th = ring_angles(points);
        const std::vector<float> rest(th.begin() + 1, th.end());
        for (int ring = 1; ring < rings && st == BS_OK; ring++) {
            double f[3];
            ring_focus(th[0], ring, f);
            st = ring_source(c, prec, f, 1.0, false, sum);  // d_D: this source alone (saveDetectorForOnePs)
            if (st == BS_OK)
                st = prec == BS_PREC_FP64 ? image_rotations<double>(c, rest) : image_rotations<float>(c, rest);
        }
        if (st != BS_OK) return st;
        CK(cudaMemcpyAsync(c->d_D.p, c->d_dacc.p, bytes, cudaMemcpyDeviceToDevice, c->st));
        CK(cudaStreamSynchronize(c->st));
        return BS_OK;
    });
}

bs_status bs_simulate_ring_line(bs_ctx* c, int32_t points, int32_t rings, bs_precision prec) {
    if (points > BS_RING_LINE_MAX_POINTS)
        return fail(BS_ERR_ARG, "bs_simulate_ring_line: at most %d points per ring (one thread block per ring)",
                    BS_RING_LINE_MAX_POINTS);
    return ring_driver(c, prec, points, rings, "bs_simulate_ring_line", [&](bs_stats& sum) {
        // SimulateExtendedSourceInterpLineAtDetector (microscope.cu:1097-1183): the context's focus, then
        // (j, 0, 0) for j = 1 .. rings-1, all with amplitude 1; every source's image feeds the radial lines
        // of `rings` entries, which then replace the detector images.
        const size_t er = elem_r(prec), L = (size_t)rings;
        CK(c->d_line.ensure(2 * L * er));
        CK(cudaMemsetAsync(c->d_line.p, 0, 2 * L * er, c->st));
        std::vector<float2> cs(points);
        for (int k = 0; k < points; k++) {
            const float t = (float)((2.0 * PI_REF / points) * (k + 1));
            cs[k] = make_float2((float)std::cos((double)t), (float)std::sin((double)t));
        }
        CK(c->d_ringcs.ensure(cs.size() * sizeof(float2)));
        CK(cudaMemcpyAsync(c->d_ringcs.p, cs.data(), cs.size() * sizeof(float2), cudaMemcpyHostToDevice, c->st));
        bs_status st = BS_OK;
        for (int j = 0; j < rings && st == BS_OK; j++) {
            const double f[3] = {(double)j, 0, 0};
            st = ring_source(c, prec, j == 0 ? nullptr : f, 1.0, false, sum);
            if (st == BS_OK) st = prec == BS_PREC_FP64 ? line_samples<double>(c, points, rings)
                                                       : line_samples<float>(c, points, rings);
        }
        if (st != BS_OK) return st;
        if (prec == BS_PREC_FP64)
            launch_line_image<double>(c->res, rings, c->d_line.as<double>(), c->d_D.as<double>(), c->st);
        else
            launch_line_image<float>(c->res, rings, c->d_line.as<float>(), c->d_D.as<float>(), c->st);
        LAUNCHED(c);
        CK(cudaStreamSynchronize(c->st));
        CK(cudaGetLastError());
        return BS_OK;
    });
}

bs_status bs_plane_point(const bs_params* params, double u, double v, double* xyz) {
    if (!params || !xyz) return fail(BS_ERR_ARG, "bs_plane_point: null argument");
    Quad q = quad_from(params->plane_min, params->plane_max, params->plane_normal);
    xyz[0] = q.A.x + q.X.x * u + q.Y.x * v;
    xyz[1] = q.A.y + q.X.y * u + q.Y.y * v;
    xyz[2] = q.A.z + q.X.z * u + q.Y.z * v;
    return BS_OK;
}

static bs_status image_to_host(bs_ctx* c, bs_image_kind kind, std::vector<double>& out) {
    if (!c) return fail(BS_ERR_ARG, "null context");
    if (!c->have) return fail(BS_ERR_STATE, "no simulation result (call bs_simulate first)");
    if (kind < BS_IMG_INTENSITY || kind > BS_IMG_TRANSMITTANCE) return fail(BS_ERR_ARG, "unknown image kind");
    int n = c->res * c->res;
    size_t es = elem_r(c->prec);
    CK(c->d_img.ensure((size_t)n * es));
    if (c->prec == BS_PREC_FP64) {
        const double* D = c->d_D.as<double>();
        launch_image<double>(n, kind, D, D + n, c->d_img.as<double>(), c->st);
    } else {
        const float* D = c->d_D.as<float>();
        launch_image<float>(n, kind, D, D + n, c->d_img.as<float>(), c->st);
    }
    LAUNCHED(c);
    out.resize(n);
    if (c->prec == BS_PREC_FP64) {
        CK(cudaMemcpyAsync(out.data(), c->d_img.p, n * sizeof(double), cudaMemcpyDeviceToHost, c->st));
        CK(cudaStreamSynchronize(c->st));
    } else {
        std::vector<float> tmp(n);
        CK(cudaMemcpyAsync(tmp.data(), c->d_img.p, n * sizeof(float), cudaMemcpyDeviceToHost, c->st));
        CK(cudaStreamSynchronize(c->st));
        for (int i = 0; i < n; i++) out[i] = tmp[i];
    }
    return BS_OK;
}

bs_status bs_get_image(bs_ctx* c, bs_image_kind kind, float* host, size_t count) {
    if (!host) return fail(BS_ERR_ARG, "bs_get_image: null buffer");
    if (c && count < (size_t)c->res * c->res) return fail(BS_ERR_ARG, "bs_get_image: buffer holds %zu of %d values", count, c->res * c->res);
    std::vector<double> v;
    bs_status st = image_to_host(c, kind, v);
    if (st != BS_OK) return st;
    for (size_t i = 0; i < v.size(); i++) host[i] = (float)v[i];
    return BS_OK;
}

bs_status bs_get_image_f64(bs_ctx* c, bs_image_kind kind, double* host, size_t count) {
    if (!host) return fail(BS_ERR_ARG, "bs_get_image_f64: null buffer");
    if (c && count < (size_t)c->res * c->res) return fail(BS_ERR_ARG, "bs_get_image_f64: buffer too small");
    std::vector<double> v;
    bs_status st = image_to_host(c, kind, v);
    if (st != BS_OK) return st;
    std::memcpy(host, v.data(), v.size() * sizeof(double));
    return BS_OK;
}

bs_status bs_get_field(bs_ctx* c, bs_field_kind kind, double* host, size_t count) {
    if (!c || !host) return fail(BS_ERR_ARG, "bs_get_field: null argument");
    if (!c->have) return fail(BS_ERR_STATE, "bs_get_field: no simulation result");
    size_t n = (size_t)c->R * c->R;
    if (count < n) return fail(BS_ERR_ARG, "bs_get_field: buffer holds %zu of %zu complex values", count, n);
    size_t off = (kind == BS_FIELD_INCIDENT) ? n : 0;
    if (c->prec == BS_PREC_FP64) {
        CK(cudaMemcpy(host, c->d_fields.as<zd>() + off, n * sizeof(zd), cudaMemcpyDeviceToHost));
    } else {
        std::vector<cpx<float>> tmp(n);
        CK(cudaMemcpy(tmp.data(), c->d_fields.as<cpx<float>>() + off, n * sizeof(cpx<float>), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; i++) {
            host[2 * i] = tmp[i].re;
            host[2 * i + 1] = tmp[i].im;
        }
    }
    return BS_OK;
}

bs_status bs_write_envi(bs_ctx* c, bs_image_kind kind, const char* path, int32_t append, double band_value) {
    if (!path) return fail(BS_ERR_ARG, "bs_write_envi: null path");
    std::vector<double> v;
    bs_status st = image_to_host(c, kind, v);
    if (st != BS_OK) return st;
    std::vector<float> f(v.begin(), v.end());
    char err[512] = {0};
    if (envi_add_band(path, f.data(), c->res, c->res, band_value, append, err, sizeof(err)) != 0)
        return fail(BS_ERR_IO, "%s", err);
    return BS_OK;
}

bs_status bs_envi_add_band(const char* path, const float* band, int32_t samples, int32_t lines, double band_value,
                           int32_t append) {
    if (!path || !band || samples < 1 || lines < 1) return fail(BS_ERR_ARG, "bs_envi_add_band: bad argument");
    char err[512] = {0};
    if (envi_add_band(path, band, samples, lines, band_value, append, err, sizeof(err)) != 0)
        return fail(BS_ERR_IO, "%s", err);
    return BS_OK;
}

bs_status bs_sweep(bs_ctx* c, const double* lambdas, int32_t nl, const double* n_table, bs_precision prec,
                   bs_image_kind kind, float* images, const char* envi_path, int32_t band_as_nu) {
    if (!c || !lambdas || nl < 1) return fail(BS_ERR_ARG, "bs_sweep: need at least one wavelength");
    const size_t ns = c->spheres.size();
    if (ns > 0 && !n_table) return fail(BS_ERR_ARG, "bs_sweep: need the refractive-index table");
    for (int32_t l = 0; l < nl; l++)
        if (!(lambdas[l] > 0)) return fail(BS_ERR_ARG, "bs_sweep: wavelength %d is not positive", l + 1);
    const bs_params saved_p = c->prm;
    const std::vector<bs_sphere> saved_s = c->spheres;
    const int saved_staging = c->lut_staging;
    const size_t npix = (size_t)c->prm.resolution * c->prm.resolution;
    // Empirical tuning of the mixed LUT kernel: with the choice left to the model
    // and at least 4 bands, band 0 runs the staged kernel and band 1 the
    // texture-only one; the faster serves the rest.  Both give the same bits, so
    // the images do not depend on the choice.
    const bool tune = saved_staging == 0 && prec == BS_PREC_MIXED && nl >= 4 && c->prm.scalar && c->prm.lut_us &&
                      ns > 0;
    float ms_stage = 0, ms_tex = 0;
    bs_status st = BS_OK;
    // Both trial kernels run at the chunk a single auto-chosen run of this scene uses (the choice
    // depends on the tile and table geometry, which is the same for every band), so every band has
    // the bits of a single run.
    const int saved_chunk = c->lut_chunk;
    if (tune && saved_chunk == 0) {
        c->prm.lambda = lambdas[0];
        for (size_t i = 0; i < ns; i++) {
            c->spheres[i].n_re = n_table[2 * i];
            c->spheres[i].n_im = n_table[2 * i + 1];
        }
        st = derive(c);
        if (st == BS_OK) c->lut_chunk = choose_chunk(c, c->waves, (int)ns).chunk;
    }
    for (int32_t l = 0; l < nl && st == BS_OK; l++) {
        c->prm.lambda = lambdas[l];
        for (size_t i = 0; i < ns; i++) {
            c->spheres[i].n_re = n_table[2 * ((size_t)l * ns + i)];
            c->spheres[i].n_im = n_table[2 * ((size_t)l * ns + i) + 1];
        }
        if (tune) c->lut_staging = l == 0 ? 1 : (l == 1 ? 2 : (ms_stage <= ms_tex ? 1 : 2));
        st = bs_simulate(c, prec);
        if (tune && l == 0) ms_stage = c->stats.ms_us;
        if (tune && l == 1) ms_tex = c->stats.ms_us;
        if (st == BS_OK && images) st = bs_get_image(c, kind, images + (size_t)l * npix, npix);
        if (st == BS_OK && envi_path)
            st = bs_write_envi(c, kind, envi_path, l > 0, band_as_nu ? 1e4 / lambdas[l] : lambdas[l]);
    }
    c->prm = saved_p;
    c->spheres = saved_s;
    c->lut_staging = saved_staging;
    c->lut_chunk = saved_chunk;
    c->have = false;
    return st;
}

bs_status bs_get_info(bs_ctx* c, bs_info* out) {
    if (!c || !out) return fail(BS_ERR_ARG, "bs_get_info: null argument");
    const bs_params& p = c->prm;
    int R = p.resolution * p.supersample * (2 * p.padding + 1);
    out->nf_res = R;
    out->det_res = p.resolution;
    out->n_spheres = (int)c->spheres.size();
    out->n_waves = p.plane_wave ? 1 : (int)(c->waves.size() / 3);
    out->uf_lut_r = p.uf_lut_r > 0 ? p.uf_lut_r : 2 * R;
    out->us_lut_theta = p.us_lut_theta > 0 ? p.us_lut_theta : 1000;
    int64_t tot = 0;
    for (const DevBuf* b : ctx_bufs(c)) tot += (int64_t)b->n;
    for (const auto& sl : c->slots)
        for (int k = 0; k < 4; k++) tot += (int64_t)sl.w * sl.h[k] * (int64_t)sizeof(float);
    out->device_bytes = tot;
    return BS_OK;
}

bs_status bs_get_stats(bs_ctx* c, bs_stats* out) {
    if (!c || !out) return fail(BS_ERR_ARG, "bs_get_stats: null argument");
    *out = c->stats;
    return BS_OK;
}

bs_status bs_get_mie(bs_ctx* c, int32_t sphere, double* A, double* B, int32_t count) {
    if (!c || !A || !B) return fail(BS_ERR_ARG, "bs_get_mie: null argument");
    if (!c->have || sphere < 0 || sphere >= (int)c->hs.size() || !c->prm.scalar)
        return fail(BS_ERR_STATE, "bs_get_mie: no coefficients for sphere %d", sphere);
    const Sphere& S = c->hs[sphere];
    if (count < S.Nl + 1) return fail(BS_ERR_ARG, "bs_get_mie: need %d orders", S.Nl + 1);
    CK(cudaMemcpy(A, c->d_A.as<zd>() + S.coef_off, (S.Nl + 1) * sizeof(zd), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(B, c->d_B.as<zd>() + S.coef_off, (S.Nl + 1) * sizeof(zd), cudaMemcpyDeviceToHost));
    return BS_OK;
}

bs_status bs_get_lut(bs_ctx* c, int32_t sphere, int32_t which, double* host, size_t count) {
    if (!c || !host) return fail(BS_ERR_ARG, "bs_get_lut: null argument");
    if (!c->have || !c->prm.lut_us || !c->prm.scalar || sphere < 0 || sphere >= (int)c->hs.size())
        return fail(BS_ERR_STATE, "bs_get_lut: no table for sphere %d", sphere);
    const Sphere& S = c->hs[sphere];
    size_t rows = which == 0 ? S.dR : S.aR;
    size_t n = rows * S.thetaR;
    if (count < n) return fail(BS_ERR_ARG, "bs_get_lut: need %zu complex values", n);
    int64_t off = which == 0 ? S.usp_off : S.uip_off;
    if (c->prec == BS_PREC_FP64) {
        std::vector<Patch<double>> t(n);
        CK(cudaMemcpy(t.data(), c->d_lut.as<Patch<double>>() + off, n * sizeof(Patch<double>), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; i++) {
            host[2 * i] = t[i].v[0];
            host[2 * i + 1] = t[i].v[1];
        }
    } else {
        int slot = sphere;  // valid when the last run held every sphere in one chunk
        if (slot >= (int)c->slots.size() || !c->slots[slot].arr[which * 2])
            return fail(BS_ERR_STATE, "bs_get_lut: table of sphere %d not resident", sphere);
        std::vector<float> re(n), im(n);
        CK(cudaMemcpy2DFromArray(re.data(), S.thetaR * sizeof(float), c->slots[slot].arr[which * 2], 0, 0,
                                 S.thetaR * sizeof(float), rows, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy2DFromArray(im.data(), S.thetaR * sizeof(float), c->slots[slot].arr[which * 2 + 1], 0, 0,
                                 S.thetaR * sizeof(float), rows, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; i++) {
            host[2 * i] = re[i];
            host[2 * i + 1] = im[i];
        }
    }
    return BS_OK;
}

}  // extern "C"
