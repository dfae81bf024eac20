// ref_run.cpp -- TEST INFRASTRUCTURE.  Entry points of the host-run build of
// the reference (oracle/_ref/libref_sim_f32.so and libref_sim_f64.so, made by
// `make -C oracle ref-sim` from the reference's own sources, compiled in place
// with the CUDA stand-ins of oracle/ref_cuda).  One call runs the reference's
// CLI path for a list of its own flags:
//     SetArguments, arglist::parse, LoadParameters   (arguments.h:27-90,564-593)
//     microscopeStruct::init                         (microscope.cu:537)
//     nearfieldStruct::Simulate, step by step         (nearfield.cpp:194-218)
//     microscopeStruct::SimulateImaging              (microscope.cu:840)
//     getIntensity / getIncidentFieldImage / getAbsorbance (microscope.cu:722-814)
// (stop = 3: with microscopeStruct::applyBackpropagation, microscope.cu:592-605,
// between them, where Simulate has it commented out, microscope.cu:853),
// or, with stop = 2 and the reference's --interpolate 1, 2 or 3 (or 0 with no
// rings), the ring-source
// driver that its Save dispatches to for that mode (fileout.cu:219-243):
//     SimulateExtendedSourceInterpAtDetector         (microscope.cu:1004-1093)
//     SimulateExtendedSourceInterpLineAtDetector     (microscope.cu:1097-1183)
//     SimulateExtendedSourceWithInterpolation        (microscope.cu:1189-1253)
// or, with stop = 4 and --extended-source, the point-source driver Save runs
// for the sources LoadParameters loaded from the image (fileout.cu:197-207):
//     LoadExtendedSource                             (microscope.cu:1258-1296)
//     SimulateExtendedSource                         (microscope.cu:873-913)
// and keeps its Monte Carlo directions, Mie coefficients, per-sphere tables,
// near fields and detector images for the accessors below.  Simulate is taken
// step by step only so that the tables can be read after calcSpheres; the
// steps and their order are the reference's.  Only tests/golden/make_golden.py
// loads this library, to record golden vectors.
#include <cstring>
#include <map>
#include <string>
#include <vector>

// the reference's main.cpp includes these before arguments.h, which relies on
// the `using namespace std` that rts/cuda/error.h (via fileout.h) brings in
#include "sphere.h"
#include "rts/optics/material.h"
#include "nearfield.h"
#include "microscope.h"
#include "fieldslice.h"
#include "fileout.h"
#include "arguments.h"

microscopeStruct* SCOPE = nullptr;
// `extern __shared__ bsComplex sh_scaledPhase[]` of the reference's unused
// optPc_gpuScalarUpLut (nfScalarUpLut.cu:220) resolves here; it never runs.
bsComplex sh_scaledPhase[1 << 12];
fileoutStruct gFileOut;
bool verbose = false;
bool gui = false;

namespace {
std::map<std::string, std::vector<double>> g_out;

template <class T>
void put_complex(const std::string& key, const rts::complex<T>* p, size_t n) {
    std::vector<double>& v = g_out[key];
    v.resize(2 * n);
    for (size_t i = 0; i < n; i++) {
        v[2 * i] = (double)p[i].r;
        v[2 * i + 1] = (double)p[i].i;
    }
}

template <class T>
void put_real(const std::string& key, const T* p, size_t n) {
    std::vector<double>& v = g_out[key];
    v.assign(p, p + n);
}

// the inputs as the reference holds them after parsing (single-precision flag values)
void put_scene() {
    const nearfieldStruct& nf = SCOPE->nf;
    g_out["scene"] = {(double)nf.lambda, (double)nf.A, (double)nf.k[0], (double)nf.k[1], (double)nf.k[2],
                      (double)nf.focus[0], (double)nf.focus[1], (double)nf.focus[2], (double)nf.condenser[0],
                      (double)nf.condenser[1], (double)SCOPE->objective[0], (double)SCOPE->objective[1],
                      (double)SCOPE->padding, (double)SCOPE->ss, (double)nf.m, (double)nf.lut_us,
                      (double)nf.lut_uf, (double)nf.planeWave, (double)nf.nWaves};
    g_out["nf_quad"] = {(double)nf.pos.A[0], (double)nf.pos.A[1], (double)nf.pos.A[2], (double)nf.pos.X[0],
                        (double)nf.pos.X[1], (double)nf.pos.X[2], (double)nf.pos.Y[0], (double)nf.pos.Y[1],
                        (double)nf.pos.Y[2]};
}

// Monte Carlo directions, sizes, per-sphere inputs and Mie coefficients after
// calcWaves / calcSpheres
void put_waves_and_spheres() {
    const nearfieldStruct& nf = SCOPE->nf;
    std::vector<double> w;
    for (const bsVector& k : nf.inWaves)
        for (int c = 0; c < 3; c++) w.push_back((double)k[c]);
    g_out["waves"] = w;
    g_out["dims"] = {(double)nf.U.R[0], (double)nf.U.R[1], (double)SCOPE->Ud.R[0] / SCOPE->ss,
                     (double)SCOPE->ss, (double)nf.sVector.size(), (double)nf.inWaves.size()};
    for (size_t s = 0; s < nf.sVector.size(); s++) {
        const sphere& S = nf.sVector[s];
        const std::string p = "sphere" + std::to_string(s) + ".";
        // d_min and d_max are set only when the tables are built (the direct mode leaves them unset)
        const double dmin = nf.lut_us ? (double)S.d_min : 0.0, dmax = nf.lut_us ? (double)S.d_max : 0.0;
        g_out[p + "geom"] = {(double)S.Nl, dmin, dmax, (double)S.Usp.R[0], (double)S.Usp.R[1], (double)S.Uip.R[0],
                             (double)S.Uip.R[1]};
        g_out[p + "in"] = {(double)S.p[0], (double)S.p[1], (double)S.p[2], (double)S.a, (double)S.n.real(),
                           (double)S.n.imag()};
        put_complex(p + "A", S.A.data(), S.A.size());
        put_complex(p + "B", S.B.data(), S.B.size());
    }
}

void put_detector() {
    scalarslice I = SCOPE->getIntensity();
    scalarslice Ii = SCOPE->getIncidentFieldImage();
    scalarslice Ab = SCOPE->getAbsorbance();
    const size_t nd = (size_t)I.R[0] * I.R[1];
    put_real("D", I.S, nd);
    put_real("Di", Ii.S, nd);
    put_real("Absorbance", Ab.S, nd);
}

// The ring-source driver for SCOPE->interpolate, called as fileout.cu:219-243
// calls it, then the detector images it leaves.
int run_rings() {
    put_scene();  // before the drivers move the focus and amplitude
    microscopeStruct* scope = SCOPE;
    if (scope->interpolate == 1)
        scope->SimulateExtendedSourceInterpAtDetector(scope->nf.extSource);
    else if (scope->interpolate == 2)
        scope->SimulateExtendedSourceInterpLineAtDetector(scope->nf.extSource);
    else if (scope->interpolate == 3)
        scope->SimulateExtendedSourceWithInterpolation(0, scope->nf.extSource);
    else if (scope->interpolate == 0 && scope->nf.extSource[1] == 0)
        // SimulateExtendedGausssianSourceNoInterp (microscope.cu:1327-1409) with no rings: the central
        // source only.  With one ring or more its loop `for (int j = spacing; ...; j += spacing)`,
        // spacing = 0.5, never advances, so it is not run.
        scope->SimulateExtendedGausssianSourceNoInterp(scope->nf.extSource);
    else
        return 2;
    put_waves_and_spheres();
    put_detector();
    g_out["rings"] = {(double)scope->interpolate, (double)scope->nf.extSource[0], (double)scope->nf.extSource[1]};
    return 0;
}

// The state after LoadParameters and init, nothing simulated: the scene, the
// near-field plane, the sizes and each sphere with the index its material gives
// at the wavelength (mVector[iMaterial](lambda), as calcSpheres takes it,
// nearfield.cpp:126-129).
int run_parse() {
    put_scene();
    const nearfieldStruct& nf = SCOPE->nf;
    g_out["dims"] = {(double)nf.U.R[0], (double)nf.U.R[1], (double)SCOPE->Ud.R[0] / SCOPE->ss, (double)SCOPE->ss,
                     (double)nf.sVector.size(), (double)nf.nWaves};
    for (size_t s = 0; s < nf.sVector.size(); s++) {
        const sphere& S = nf.sVector[s];
        rts::material<ptype> m = SCOPE->nf.mVector[S.iMaterial];
        const rts::complex<ptype> n = m(nf.lambda);
        g_out["sphere" + std::to_string(s) + ".in"] = {(double)S.p[0], (double)S.p[1], (double)S.p[2], (double)S.a,
                                                        (double)n.real(), (double)n.imag()};
    }
    return 0;
}

// The extended source LoadParameters loaded, and SimulateExtendedSource over it.
int run_sources() {
    put_scene();
    microscopeStruct* scope = SCOPE;
    if (scope->focalPoints.empty()) return 3;
    std::vector<double> pts;
    for (const sourcePoint& p : scope->focalPoints)
        for (double v : {(double)p.f[0], (double)p.f[1], (double)p.f[2], (double)p.A}) pts.push_back(v);
    g_out["sources"] = pts;
    scope->SimulateExtendedSource();
    put_waves_and_spheres();
    put_detector();
    return 0;
}
}  // namespace

extern "C" {

// Run the reference on `argv` (argv[0] is the program name).  stop = 1 ends
// after calcSpheres (tables only); 0 runs the whole single-source path; 2 runs
// the ring-source driver of the parsed --interpolate mode (1, 2 or 3) and keeps
// the detector images; 3 is 0 with the near field back-propagated over the
// plane position before the band-pass (U and Uf are kept as sumUf left them);
// 4 runs SimulateExtendedSource over the sources of --extended-source and keeps
// them (x, y, z, amplitude) and the detector images; 6 keeps the parsed state
// only (run_parse); 5 ends after sumUf (the
// near fields only: with --vector the reference's getFarField copies the y and z
// components into a crop slice allocated without them, fieldslice.cu:340-361).
int ref_sim_run(int argc, const char** argv, int stop) {
    g_out.clear();
    std::vector<std::string> keep(argv, argv + argc);
    std::vector<char*> av;
    for (std::string& s : keep) av.push_back(&s[0]);
    rts::arglist args;
    SetArguments(args);
    args.parse(argc, av.data());
    SCOPE = new microscopeStruct();
    LoadParameters(args);
    SCOPE->init();
    nearfieldStruct& nf = SCOPE->nf;
    if (stop == 2) return run_rings();
    if (stop == 4) return run_sources();
    if (stop == 6) return run_parse();

    nf.t_Uf = 0;
    nf.t_Us = 0;
    nf.calcWaves();
    nf.calcUf();
    nf.calcSpheres();

    put_scene();
    put_waves_and_spheres();
    for (size_t s = 0; s < nf.sVector.size(); s++) {
        const sphere& S = nf.sVector[s];
        const std::string p = "sphere" + std::to_string(s) + ".";
        if (nf.lut_us) {
            put_complex(p + "Usp", S.Usp.x_hat, (size_t)S.Usp.R[0] * S.Usp.R[1]);
            put_complex(p + "Uip", S.Uip.x_hat, (size_t)S.Uip.R[0] * S.Uip.R[1]);
        }
    }
    if (stop == 1) return 0;

    nf.calcUs();
    nf.sumUf();
    const size_t nnf = (size_t)nf.U.R[0] * nf.U.R[1];
    put_complex("U", nf.U.x_hat, nnf);
    put_complex("Uf", nf.Uf.x_hat, nnf);
    if (stop == 5) return 0;

    if (stop == 3) SCOPE->applyBackpropagation();
    SCOPE->SimulateImaging();
    put_detector();
    put_complex("Ud", SCOPE->Ud.x_hat, (size_t)SCOPE->Ud.R[0] * SCOPE->Ud.R[1]);
    return 0;
}

// The reference's executable on `argv` as its main() runs it (main.cpp:42-78):
// SetArguments, parse, LoadParameters, microscopeStruct::init, then
// fileoutStruct::Save (fileout.cu:189-265), which simulates and writes the
// output files the flags name (ENVI through rts/envi; colour images go to the
// STIM stand-in, which writes nothing).  The output settings are reset first,
// as a fresh process would have them.
int ref_sim_save(int argc, const char** argv) {
    g_out.clear();
    std::vector<std::string> keep(argv, argv + argc);
    std::vector<char*> av;
    for (std::string& s : keep) av.push_back(&s[0]);
    rts::arglist args;
    SetArguments(args);
    args.parse(argc, av.data());
    gFileOut = fileoutStruct();
    SCOPE = new microscopeStruct();
    LoadParameters(args);
    SCOPE->init();
    gFileOut.Save(SCOPE);
    return 0;
}

// Number of values stored under `key` (-1 if none).
long ref_sim_size(const char* key) {
    auto it = g_out.find(key);
    return it == g_out.end() ? -1 : (long)it->second.size();
}

// Copy the values stored under `key` into out (ref_sim_size(key) doubles).
int ref_sim_get(const char* key, double* out) {
    auto it = g_out.find(key);
    if (it == g_out.end()) return 1;
    std::memcpy(out, it->second.data(), it->second.size() * sizeof(double));
    return 0;
}

void bs_ref_set_tex_weight_bits(int bits);
int ref_sim_set_tex_weight_bits(int bits) {
    bs_ref_set_tex_weight_bits(bits);
    return 0;
}

}  // extern "C"
