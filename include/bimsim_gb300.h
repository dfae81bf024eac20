/*
 * bimsim_gb300.h -- C ABI of the GB300 near-field-to-detector library.
 *
 * The reference (seberisha/bimsim-cuda) has no plugin or FFI interface: its
 * boundary is the `bimsim` executable, whose flags fill the global
 * `microscopeStruct* SCOPE` (arguments.h:564-593) and whose fileoutStruct
 * writes the detector images (fileout.cu:47-159).  Internally the path is
 *     microscopeStruct::init()      microscope.cu:537
 *     microscopeStruct::Simulate()  microscope.cu:849
 *     microscopeStruct::get*()      microscope.cu:722-814
 *     scalarslice::toEnvi()         scalarslice.cu:146-166
 * This header replaces that object with an opaque context and plain C entry
 * points (pointers, sizes, status codes).  Every call returns a bs_status;
 * the reference instead printed CUDA errors and carried on
 * (rts/cuda/error.h:12-21) or called exit(1) (arguments.h:175,249,292).
 *
 * Units follow the reference: lengths in micrometres, wavelength in
 * micrometres, numerical apertures as plain numbers.
 */
#ifndef BIMSIM_GB300_H
#define BIMSIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bs_status {
    BS_OK = 0,
    BS_ERR_ARG = 1,          /* invalid argument (reference: exit(1) in arguments.h) */
    BS_ERR_CUDA = 2,         /* CUDA runtime error (reference: printed and ignored) */
    BS_ERR_NOMEM = 3,        /* device allocation failed or over the HBM budget */
    BS_ERR_STATE = 4,        /* call out of order (e.g. image before simulate) */
    BS_ERR_IO = 5,           /* file could not be opened or written */
    BS_ERR_TIMEOUT = 6,      /* a bounded wait ran out */
    BS_ERR_UNSUPPORTED = 7,  /* feature not built */
    BS_ERR_NOTREADY = 8      /* serving: result not finished yet */
} bs_status;

/* Arithmetic of the per-pixel work.  FP64 keeps every stage in double; MIXED
 * keeps Mie coefficients, Bessel tables, the LUT build, the incident field
 * and per-(pixel, sphere) geometry in double and runs the per-sample sums and
 * the detector transform in float with compensated accumulation. */
typedef enum bs_precision { BS_PREC_FP64 = 0, BS_PREC_MIXED = 1 } bs_precision;

/* Detector images (microscope.cu:722-814). */
typedef enum bs_image_kind {
    BS_IMG_INTENSITY = 0,     /* getIntensity():          D             */
    BS_IMG_INCIDENT = 1,      /* getIncidentFieldImage(): Di            */
    BS_IMG_ABSORBANCE = 2,    /* getAbsorbance():         -log10(D/Di)  */
    BS_IMG_TRANSMITTANCE = 3  /* getTransmittance():      D/Di          */
} bs_image_kind;

/* Near-field planes (nearfieldStruct::U and ::Uf, nearfield.h:38-42). */
typedef enum bs_field_kind { BS_FIELD_TOTAL = 0, BS_FIELD_INCIDENT = 1 } bs_field_kind;

/*
 * Simulation state after the reference's LoadParameters (arguments.h:564-593):
 * the fields of nearfieldStruct (nearfield.h:14-120) and microscopeStruct
 * (microscope.h:23-142) that the single-source path reads.  The `bimsim` CLI
 * of this project fills it from the reference's flags.
 */
typedef struct bs_params {
    double lambda;            /* nf.lambda, um (arguments.h:115-132)                  */
    double amplitude;         /* nf.A (arguments.h:455)                                */
    double k_dir[3];          /* nf.k, unit incident direction (arguments.h:484-493)   */
    double focus[3];          /* nf.focus (arguments.h:479-481)                        */
    double condenser[2];      /* nf.condenser NA inner/outer (arguments.h:459-468)     */
    double objective[2];      /* SCOPE->objective NA inner/outer (arguments.h:322-338) */
    double plane_min[3];      /* detector plane corners and normal given to            */
    double plane_max[3];      /*   microscopeStruct::setPos (arguments.h:340-407)      */
    double plane_normal[3];
    int32_t resolution;       /* detector pixels per side (--resolution)               */
    int32_t padding;          /* --padding, FFT padding factor p                       */
    int32_t supersample;      /* ss (arguments.h:411-418)                              */
    int32_t field_order;      /* nf.m, incident-field order (--field-order)            */
    int32_t scalar;           /* 1 = scalar, 0 = the reference's vector stub           */
    int32_t plane_wave;       /* --plane-wave                                          */
    int32_t lut_uf;           /* nf.lut_uf (arguments.h:92-113)                        */
    int32_t lut_us;           /* nf.lut_us                                             */
    int32_t us_lut_r;         /* Usp radial samples; 0 = reference 2*R (sphere.cpp:238)*/
    int32_t us_lut_theta;     /* Usp/Uip angular samples; 0 = 1000 (defaults.h:83)     */
    int32_t uf_lut_r;         /* Uf LUT radial samples; 0 = 2*R (nfScalarUfLut.cu:134) */
    int32_t reserved;
} bs_params;

/* One sphere with its refractive index already evaluated at lambda
 * (sphere.h:14-92; the material lookup is nearfield.cpp:119-124). */
typedef struct bs_sphere {
    double x, y, z;           /* centre, um  */
    double a;                 /* radius, um  */
    double n_re, n_im;        /* n + i k     */
} bs_sphere;

/* Derived sizes of a context (read back for tests and callers). */
typedef struct bs_info {
    int32_t nf_res;           /* near-field pixels per side R = res*ss*(2p+1) */
    int32_t det_res;          /* detector pixels per side                      */
    int32_t n_spheres;
    int32_t n_waves;
    int32_t uf_lut_r;
    int32_t us_lut_theta;
    int64_t device_bytes;     /* HBM held by the context                       */
} bs_info;

/* Per-stage device timings (ms) and launch count of the last bs_simulate. */
typedef struct bs_stats {
    double ms_total;
    double ms_uf;
    double ms_mie;
    double ms_lut;
    double ms_us;
    double ms_detector;
    int64_t kernel_launches;
    int64_t us_interactions;  /* (pixel, sphere, wave) triples evaluated */
    /* Mixed-precision LUT path: (pixel tile, sphere, wave chunk) units whose
     * table window was staged in shared memory, and all such units. */
    int64_t lut_chunks_staged;
    int64_t lut_chunks_total;
    int64_t lut_tables_built;  /* sphere tables (Usp + Uip) built; 0 when reused */
    double lut_staged_predicted;  /* the kernel choice's model of lut_chunks_staged / total */
    int64_t lut_wave_chunk;       /* waves per chunk of the mixed LUT kernel (64, 32 or 16) */
} bs_stats;

typedef struct bs_ctx bs_ctx;

/* Library version string. */
const char* bs_version(void);

/* Last error message of this host thread (empty string if none). */
const char* bs_last_error(void);

/* Allocate a context on the current CUDA device (microscopeStruct::init,
 * microscope.cu:537; nearfieldStruct::init, nearfield.cpp:25).  The context
 * owns all device memory and one CUDA stream.  The first context of a device
 * in a process loads every kernel of the library there: CUDA otherwise loads
 * a kernel at its first launch, and such a load waits for the kernels that
 * other streams are running. */
bs_status bs_create(const bs_params* params, bs_ctx** out);

/* Free everything the context holds (microscopeStruct::destroy). */
bs_status bs_destroy(bs_ctx* ctx);

/* Replace the parameters of an existing context (a new LoadParameters pass,
 * arguments.h:564-593, without reallocating); results of the last run are
 * dropped. */
bs_status bs_set_params(bs_ctx* ctx, const bs_params* params);

/* Sphere list (lSpheres arguments.h:193-320, with the material resolved). */
bs_status bs_set_spheres(bs_ctx* ctx, const bs_sphere* spheres, int32_t n);

/* Monte Carlo plane-wave directions, 3*nk doubles (x,y,z per wave).
 * Replaces nearfieldStruct::calcWaves (nearfield.cpp:96-108) so that results
 * do not depend on a random generator. */
bs_status bs_set_waves(bs_ctx* ctx, const double* dirs, int32_t nk);

/* The reference's own sampler: glibc rand() from seed 0 (nearfield.cpp:102,
 * montecarlo.cpp:9-71), restated bit-for-bit in single precision. */
bs_status bs_sample_waves_compat(bs_ctx* ctx, int32_t nk);

/* Run the near field and the detector (microscopeStruct::Simulate,
 * microscope.cu:849-857).  Synchronous. */
bs_status bs_simulate(bs_ctx* ctx, bs_precision precision);

/* Copy a detector image to host memory (float32, row-major, det_res^2). */
bs_status bs_get_image(bs_ctx* ctx, bs_image_kind kind, float* host, size_t count);

/* Same image in double precision (FP64 runs keep double images). */
bs_status bs_get_image_f64(bs_ctx* ctx, bs_image_kind kind, double* host, size_t count);

/* Copy a near-field plane to host memory as interleaved (re, im) doubles,
 * nf_res^2 complex values. */
bs_status bs_get_field(bs_ctx* ctx, bs_field_kind kind, double* host, size_t count);

/* Far field at the detector (microscopeStruct::Ud / Ufd after the objective
 * band-pass and crop, microscope.cu:608-655, scaled by 1/R^2 like ScaleField):
 * (res*ss)^2 interleaved (re, im) doubles of the last run (the last point
 * source after bs_simulate_sources). */
bs_status bs_get_far_field(bs_ctx* ctx, bs_field_kind kind, double* host, size_t count);

/* Append or write one band to an ENVI file (scalarslice::toEnvi,
 * scalarslice.cu:146-166; rts/envi/envi.h:196-433).  band_value is the
 * header's wavelength entry (lambda, or 1e4/lambda for --nu). */
bs_status bs_write_envi(bs_ctx* ctx, bs_image_kind kind, const char* path,
                        int32_t append, double band_value);

/* The same ENVI writer for a caller's host image (samples x lines float32,
 * row-major): EnviFile(path, append ? "a" : "w").addBand(...) then close()
 * (rts/envi/envi.h:196-233, 325-343, 423-433; header envi_header.h:318-375).
 * A band of another size than the file's bands is refused, as the reference's
 * EnviFile refuses it. */
bs_status bs_envi_add_band(const char* path, const float* band, int32_t samples, int32_t lines,
                           double band_value, int32_t append);

/* Upper bound on the bytes of per-sphere lookup tables held at once; spheres
 * beyond it are processed in successive chunks.  0 (default) = 80% of free HBM.
 * No reference counterpart: the reference allocated one cudaArray per sphere
 * (nfScalarUpLut.cu:388-399). */
bs_status bs_set_lut_budget(bs_ctx* ctx, size_t bytes);

bs_status bs_get_info(bs_ctx* ctx, bs_info* out);
bs_status bs_get_stats(bs_ctx* ctx, bs_stats* out);

/* Mie coefficients A_l, B_l (l = 0..Nl) of one sphere from the last run, as
 * interleaved complex doubles; sphere::A / sphere::B (sphere.h:39-43). */
bs_status bs_get_mie(bs_ctx* ctx, int32_t sphere, double* A, double* B, int32_t count);

/* Lookup table of one sphere from the last run (which = 0: Usp, dR x thetaR;
 * 1: Uip, aR x thetaR), radial-major interleaved complex doubles; the values
 * of sphere::Usp / sphere::Uip (sphere.cpp:222-272, sphere.cu:4-99).  Valid
 * for spheres of the last table chunk. */
bs_status bs_get_lut(bs_ctx* ctx, int32_t sphere, int32_t which, double* host, size_t count);

/* Measured FMA throughput (TFLOP/s, 2 flop per FMA) of the current GPU in
 * single and double precision, from bounded FMA-chain kernels timed with
 * CUDA events (single precision: the larger of scalar FMAs and packed
 * fma.rn.f32x2 pairs).  The denominator of the scattered-field kernels' roofline.
 * No reference counterpart. */
bs_status bs_measure_fma_peak(double* fp32_tflops, double* fp64_tflops);

/* Extended (point-source) illumination: microscopeStruct::SimulateExtendedSource
 * (microscope.cu:873-913) over the point sources LoadExtendedSource makes from
 * a source image (microscope.cu:1257-1296).  Source i has focus
 * sources[4i .. 4i+2] and amplitude sources[4i+3]; each is simulated like
 * bs_simulate and the detector images add up (D = sum D_i, Di = sum Di_i, as
 * IntegrateAndResample accumulates, fieldslice.cu:71-108); absorbance and
 * transmittance come from the sums.  The sphere tables do not depend on the
 * focus or amplitude and are built once per call.  The context's own focus
 * and amplitude are kept; bs_get_stats sums the per-source timings. */
bs_status bs_simulate_sources(bs_ctx* ctx, const double* sources, int32_t n, bs_precision prec);

/* Refractive index n + ik at each wavelength (um) from a material file
 * (rts::material<float>(filename).getN(lambda), material.h:434-621): rows of
 * "lambda n k" (default) or the columns named by a first comment line
 * "# ... [wavenumber,n,k]" (also microns, A = absorbance); rows sorted by
 * wavelength; linear interpolation between rows with the reference's swapped
 * weights (rts/math/function.h:44-75), clamped at the ends; single precision.
 * Blank lines are skipped (the reference's parser never returns on one). */
bs_status bs_material_eval(const char* path, const double* lambdas, int32_t n, double* n_out);

/* Kramers-Kronig real index of a material file (material::computeN,
 * rts/optics/material.h:257-432, which the reference never calls and which
 * needs FFTW).  The file is read and kappa interpolated in double precision,
 * as rts::material<double> does (the instantiation whose arrays match FFTW's
 * double transforms).  kappa is resampled at n_samples (0: the file's entry count,
 * at most BS_KK_MAX_SAMPLES) wavenumbers evenly spaced from 1e4 / lambda_min
 * down to 1e4 / lambda_max; chi2 = -alpha n0 / k with k = 2 pi / lambda and
 * alpha = 2 k kappa in single precision (the reference's float k and alpha);
 * chi2 zero-padded to pf * n_samples points (pf 1 to 16) goes through the reference's FFT
 * Hilbert transform (x i for 0 < f < M/2, x -i for f >= M/2, DC removed,
 * inverse / M), here as the equivalent circular convolution on the GPU in
 * double precision; n = Re(chi1) / (2 n0) + n0.  Outputs: the sample
 * wavelengths (increasing, um) and (n, kappa) pairs.  The reference's routine
 * hands complex<float> arrays to FFTW's double transforms in the float
 * instantiation; this is its double instantiation. */
#define BS_KK_MAX_SAMPLES 16384
bs_status bs_material_kk(const char* path, double n0, int32_t n_samples, int32_t pf, double* lambdas,
                         double* n_out);

/* Ring point sources by near-field rotation: the reference's --interpolate 3
 * (SimulateExtendedSourceWithInterpolation, microscope.cu:1185-1253, with
 * nfInterpolate.cu:13-115).  The detector sums the slice of the context's own
 * source and, for rings r = 1 .. rings-1 of radius r um, `points` sources at
 * angles 2 pi (i + 1) / points (z = 0, amplitude 1): each ring's first source
 * is simulated, and source i's near field is that one rotated about the slice
 * centre by source i's own angle (bilinear, zero outside the slice), as the
 * reference does.  The context's focus and amplitude are kept. */
bs_status bs_simulate_ring_interp(bs_ctx* ctx, int32_t points, int32_t rings, bs_precision prec);

/* Ring point sources by detector-image rotation: the reference's --interpolate 1
 * (SimulateExtendedSourceInterpAtDetector, microscope.cu:1004-1093, with
 * InterpolateAndIntegrateUd/Ufd, microscope.cu:89-135).  The same sources as
 * bs_simulate_ring_interp; each ring's first source is simulated and source i's
 * detector images are that source's images rotated about the detector centre
 * ((int)(res/2), both axes) by source i's angle (bilinear, zero outside). */
bs_status bs_simulate_ring_detector(bs_ctx* ctx, int32_t points, int32_t rings, bs_precision prec);

/* Radial-line ring sources: the reference's --interpolate 2
 * (SimulateExtendedSourceInterpLineAtDetector, microscope.cu:1097-1183, with
 * simRing_Ud/Ufd :138-250 and InterpolateAndIntegrateUdFromLine :37-85).
 * Sources at the context's focus and at (j, 0, 0) um, j = 1 .. rings-1, all with
 * amplitude 1.  For each source and each radius r < rings (pixels), the
 * source's detector image is sampled at `points` angles 2 pi (k + 1) / points
 * around the detector centre and the samples are added in the reference's
 * shared-memory tree (for a count that is not a power of two some samples are
 * left out, as there); the per-radius sums over all sources form a line of
 * `rings` entries, and each detector pixel is that line interpolated at its
 * distance from the centre (zero beyond the line).  points <= 1023 (the
 * reference runs one thread block of at most 1024 threads per ring). */
#define BS_RING_LINE_MAX_POINTS 1023
bs_status bs_simulate_ring_line(bs_ctx* ctx, int32_t points, int32_t rings, bs_precision prec);

/* Point pos(u, v) = A + u X + v Y of the detector plane quad (microscopeStruct::pos;
 * the quad of arguments.h:340-407 built by rts/math/quad.h:55-84), e.g. for
 * placing point sources at image pixels (u = x / width, v = y / height). */
bs_status bs_plane_point(const bs_params* params, double u, double v, double* xyz);

/* Spectral sweep: the reference's per-wavelength runs (one `bimsim --lambda
 * ... --append` process per band, runBimSim.py:80-86 and specimage.py) in one
 * call.  For wavelength l of nl, every sphere s takes the index
 * n_table[2*(l*ns + s)] + i n_table[2*(l*ns + s) + 1]; the slice is computed
 * as bs_simulate would and image `kind` goes to images + l*res*res (float32,
 * may be NULL) and, when envi_path is given, to band l of that ENVI file
 * (band value lambda, or 1e4/lambda when band_as_nu).  The context's own
 * wavelength and indices are restored afterwards; results of the last
 * band are dropped.  With bs_set_lut_staging left at 0 and at least 4 mixed
 * bands, bands 0 and 1 time the staged and texture-only LUT kernels and the
 * faster runs the rest (identical bits either way). */
bs_status bs_sweep(bs_ctx* ctx, const double* lambdas, int32_t nl, const double* n_table, bs_precision prec,
                   bs_image_kind kind, float* images, const char* envi_path, int32_t band_as_nu);

/* Back-propagation of the total near field U over distance d (um) before the
 * objective band-pass: the reference's applyBackpropagation
 * (microscope.cu:423-470, 592-605), which its Simulate() has commented out
 * (microscope.cu:853), with d the plane position z_d (arguments.h:409).  The
 * spectrum is multiplied by -exp(i kz d), kz = sqrt(k^2 - kx^2 - ky^2),
 * k = 2 pi / lambda, on the band-pass frequency grid (zero where kx^2 + ky^2
 * >= k^2).  The incident field Uf is not propagated.  Off by default. */
bs_status bs_set_backpropagation(bs_ctx* ctx, int32_t enable, double d);

/* Waves per chunk of the mixed LUT kernel: 0 (default) picks 64, 32 or 16 per
 * run from the predicted fraction of staged windows; 16, 32 or 64 fixes it.
 * The staged and texture-only kernels give the same bits at the same chunk. */
bs_status bs_set_lut_wave_chunk(bs_ctx* ctx, int32_t chunk);

/* Kernel of the mixed-precision LUT stage: 0 (default) chooses from a model
 * of how many table windows fit in shared memory, 1 always stages windows in
 * shared memory (texture gathers where a window does not fit), 2 uses texture
 * gathers only.  All three give the same bits.  No reference counterpart. */
bs_status bs_set_lut_staging(bs_ctx* ctx, int32_t mode);

/* Keep the lookup tables of the last run and skip rebuilding them when the
 * next bs_simulate on this context has the same tables: same spheres (centre,
 * radius, index), wavelength, plane, table sizes and precision, and all
 * tables fitting the LUT budget at once.  Off by default (every simulate then
 * does the whole path, as the reference does); the serving front end turns it
 * on for its contexts.  No reference counterpart. */
bs_status bs_set_lut_reuse(bs_ctx* ctx, int32_t enable);

/* Priority of the context's stream, as cudaStreamCreateWithPriority takes it:
 * lower numbers are scheduled first when blocks of several streams wait for
 * the GPU; clamped to the device's range (cudaDeviceGetStreamPriorityRange),
 * default 0.  The context finishes its queued work, then continues on a new
 * stream of that priority.  Results do not depend on it.  The serving front
 * end gives cheap requests the higher priorities, so that their kernels are
 * not queued behind the blocks of a long slice.  No reference counterpart. */
bs_status bs_set_stream_priority(bs_ctx* ctx, int32_t priority);

/* Return every device buffer of the context to the CUDA allocator (results of
 * the last run are dropped).  No reference counterpart. */
bs_status bs_release_buffers(bs_ctx* ctx);

/* Device bytes a context would hold after bs_simulate of this scene: near
 * fields, detector transform, tables (capped by lut_budget when it is > 0, as
 * bs_set_lut_budget does) and the per-sphere and per-wave arrays.  Host-only;
 * the serving front end admits requests with it.  No reference counterpart. */
bs_status bs_estimate_bytes(const bs_params* params, const bs_sphere* spheres, int32_t n_spheres, int32_t n_waves,
                            bs_precision prec, uint64_t lut_budget, uint64_t* bytes);

/* ------------------------------------------------------------------------
 * Serving front end.  The reference runs one simulation per process; this
 * queue runs many slices on one GPU: requests wait in arrival order, a pool
 * of contexts (one CUDA stream each) runs as many as fit the device-memory
 * budget at once (smaller requests may pass a head request that does not fit
 * yet, each at most 8 times), a context keeps its tables for the next
 * request with the same scene (requests are steered to it), and every result
 * is what bs_simulate on a fresh context gives for the same inputs.
 * ------------------------------------------------------------------------ */
typedef struct bs_server bs_server;

typedef struct bs_server_config {
    int32_t workers;          /* requests in flight at once; 0 = 4                        */
    int32_t dry_run;          /* 1: schedule without a GPU (capacity planning, tests):     */
                              /*    a request "runs" for 1 ms and returns an image of      */
                              /*    its ticket number                                      */
    uint64_t hbm_budget;      /* device bytes for all contexts; 0 = 80 % of free memory    */
} bs_server_config;

typedef struct bs_request {
    bs_params params;
    const bs_sphere* spheres; /* copied at submit */
    int32_t n_spheres;
    int32_t n_waves;          /* directions in `waves`, or the count for the compat sampler */
    const double* waves;      /* n_waves x 3 unit vectors, copied; NULL = bs_sample_waves_compat */
    int32_t precision;        /* bs_precision                                             */
    int32_t image;            /* bs_image_kind returned by bs_fetch                        */
} bs_request;

typedef struct bs_result_info {
    double ms_queued;         /* submit -> start */
    double ms_total;          /* submit -> done  */
    double ms_gpu;            /* device time of the slice (bs_stats.ms_total)             */
    int32_t status;           /* bs_status of the run                                      */
    int32_t lut_reused;       /* 1 if the tables came from the previous request            */
    int32_t worker;
    int32_t reserved;
} bs_result_info;

typedef struct bs_server_stats {
    int64_t submitted, completed, failed, queued, running;
    int64_t lut_reuses;
    double p50_ms, p99_ms, mean_ms, max_ms;  /* submit -> done, completed requests */
    uint64_t bytes_in_use, bytes_peak, hbm_budget;
} bs_server_stats;

bs_status bs_server_create(const bs_server_config* cfg, bs_server** out);
/* Stops accepting work, finishes what is running, drops what waits. */
bs_status bs_server_destroy(bs_server* srv);
/* BS_ERR_NOMEM when the request alone does not fit the budget. */
bs_status bs_submit(bs_server* srv, const bs_request* req, uint64_t* ticket);
/* *done = 1 once the request finished (successfully or not). */
bs_status bs_poll(bs_server* srv, uint64_t ticket, int32_t* done);
/* Blocks up to timeout_s seconds (< 0: no limit); BS_ERR_TIMEOUT if unfinished. */
bs_status bs_wait(bs_server* srv, uint64_t ticket, double timeout_s);
/* Copies the image (res x res float32) and releases the ticket.  Returns the
 * run's own status if it failed (message in bs_last_error()), BS_ERR_NOTREADY
 * if it has not finished. */
bs_status bs_fetch(bs_server* srv, uint64_t ticket, float* host, size_t count, bs_result_info* info);
bs_status bs_server_get_stats(bs_server* srv, bs_server_stats* out);

/* Mie coefficients without any device allocation, for callers that cannot
 * call cudaMalloc (code inside CUDA stream capture, serving loops that reserve
 * all memory up front, frameworks that own device memory through their own
 * pool).  No counterpart in the reference; it computes what
 * bs_simulate/bs_get_mie compute per sphere.
 *   spheres  device array, ns x {a, n_re, n_im} (radius um, complex index)
 *   ns       0..256;  nl: highest order, 0..127;  k: wavenumber 2*PI/lambda
 *   A, B     device arrays, ns x (nl + 1) interleaved complex doubles; sphere
 *            s fills orders 0..min(nl, Nl_s), Nl_s its own order count
 *            (sphere::calcNl, sphere.h:71-74, with lambda = 2*PI/k), and
 *            zeros above, as the context path computes no order beyond Nl_s
 *   stream   cudaStream_t to run on (NULL = legacy default stream); the call is
 *            asynchronous on it.
 * The Bessel work space is a fixed 3 MiB device array inside this library,
 * held by every GPU that loads it; it is fully rewritten before being read,
 * so nothing needs clearing, but every call shares it: calls whose kernels
 * overlap on the GPU (different streams, or threads sharing a device) race.
 * The first call on a device resolves the array's device address, so make it
 * before any stream capture.  That address is kept for the process: do not
 * call cudaDeviceReset on the device after the first call.  Sizes beyond the
 * limits return BS_ERR_ARG. */
bs_status bs_mie_noalloc(const double* spheres, int32_t ns, int32_t nl, double k, double* A, double* B,
                         void* stream);

#ifdef __cplusplus
}
#endif

#endif /* BIMSIM_GB300_H */
