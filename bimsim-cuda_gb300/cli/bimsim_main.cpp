// bimsim_main.cpp -- the `bimsim` command line, a drop-in for the reference's
// executable on the single-source near-field-to-detector path.
//
// Flag names, defaults, arity rules and their order of evaluation follow the
// reference (SetArguments arguments.h:27-90, defaults.h, LoadParameters
// arguments.h:564-593); outputs follow fileoutStruct::saveDetector
// (fileout.cu:47-159).  The simulation itself runs through the C ABI of
// libbimsim_gb300.so.  Added flags (absent from the reference):
//   --precision mixed|fp64   arithmetic of the per-pixel work (default mixed)
//   --lut-res R T            scattered-field LUT radial x angular samples
//   --uf-lut-res R           incident-field LUT radial samples
//   --waves-file FILE        plane-wave directions, "x y z" per line
//   --dry-run                print the derived parameters as JSON and stop
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "bimsim_gb300.h"
#include "image_io.h"

namespace {

// ---------------------------------------------------------------------------
// Argument list with the reference's grammar (rts/tools/arguments.h:18-413):
// "--name v1 v2 ..." sets a flag and its space-separated values; a default
// value makes the flag count as set.
// ---------------------------------------------------------------------------
struct Arg {
    std::string name, desc, range;
    std::vector<std::string> vals;
    bool set = false;
};

class ArgList {
public:
    void section(const std::string& s) { sections_.push_back({s, (int)args_.size()}); }
    void add(const std::string& name, const std::string& desc, const std::string& def = "",
             const std::string& range = "") {
        Arg a;
        a.name = name;
        a.desc = desc;
        a.range = range;
        a.vals = split(def);
        a.set = !def.empty();
        args_.push_back(a);
    }
    void parse(int argc, char** argv) {
        if (argc <= 1) return;
        std::string name, params;
        for (int i = 1; i < argc; i++) {
            if (argv[i][0] == '-' && argv[i][1] == '-') {
                if (!name.empty()) set(name, params);
                name = argv[i] + 2;
                params.clear();
            } else {
                if (!params.empty()) params += " ";
                params += argv[i];
            }
        }
        set(name, params);
    }
    bool operator()(const std::string& n) const {
        const Arg* a = find(n);
        return a && a->set;
    }
    int nargs(const std::string& n) const { return (int)get(n).vals.size(); }
    float f(const std::string& n, int i = 0) const {
        const Arg& a = get(n);
        if ((int)a.vals.size() <= i) return 0;
        float r;
        std::istringstream is(a.vals[i]);
        if (!(is >> r)) r = 0;
        return r;
    }
    int i(const std::string& n, int k = 0) const {
        const Arg& a = get(n);
        if ((int)a.vals.size() <= k) return 0;
        int r;
        std::istringstream is(a.vals[k]);
        if (!(is >> r)) r = 0;
        return r;
    }
    std::string text(const std::string& n, int k = 0) const {
        const Arg& a = get(n);
        return (int)a.vals.size() > k ? a.vals[k] : "";
    }
    std::string help() const {
        std::ostringstream os;
        size_t si = 0;
        for (size_t k = 0; k < args_.size(); k++) {
            while (si < sections_.size() && sections_[si].second == (int)k) os << "\n" << sections_[si++].first << "\n";
            std::string left = " --" + args_[k].name;
            if (!args_[k].vals.empty()) {
                left += " ( = ";
                for (auto& v : args_[k].vals) left += v + " ";
                left += ")";
            }
            os << left;
            for (size_t pad = left.size(); pad < 40; pad++) os << ' ';
            os << args_[k].desc;
            if (!args_[k].range.empty()) os << "\n" << std::string(44, ' ') << args_[k].range;
            os << "\n";
        }
        return os.str();
    }

private:
    static std::vector<std::string> split(const std::string& s) {
        std::vector<std::string> v;
        std::stringstream ss(s);
        std::string item;
        while (std::getline(ss, item, ' ')) v.push_back(item);
        return v;
    }
    void set(const std::string& n, const std::string& params) {
        Arg* a = find(n);
        if (!a) {
            std::cout << "ERROR - Argument not recognized: " << n << std::endl;
            return;
        }
        a->vals = split(params);
        a->set = true;
    }
    Arg* find(const std::string& n) {
        for (auto& a : args_)
            if (a.name == n) return &a;
        return nullptr;
    }
    const Arg* find(const std::string& n) const {
        for (auto& a : args_)
            if (a.name == n) return &a;
        return nullptr;
    }
    const Arg& get(const std::string& n) const {
        const Arg* a = find(n);
        if (!a) {
            std::cout << "ERROR - Unspecified parameter name: " << n << std::endl;
            std::exit(1);
        }
        if (!a->set) {
            std::cout << "ERROR - Argument requested without being set: " << n << std::endl;
            std::exit(1);
        }
        return *a;
    }
    std::vector<Arg> args_;
    std::vector<std::pair<std::string, int>> sections_;
};

// SetArguments, arguments.h:27-90 (defaults from defaults.h)
void define(ArgList& a) {
    a.section("Interface Flags");
    a.add("help", "prints this help");
    a.add("verbose", "verbose output");
    a.section("Output Parameters");
    a.add("vector", "run a vector field simulation");
    a.add("intensity", "output measured intensity (filename)", "out_i.bmp");
    a.add("incident", "output measured incident field (filename)", "out_inc.bmp");
    a.add("absorbance", "output measured absorbance (filename)", "out_a.bmp");
    a.add("absorbance-spec", "output measured absorbance spectrum (filename)", "out_as.bmp");
    a.add("transmittance", "output measured transmittance (filename)", "");
    a.add("far-field", "output far-field at detector (filename)", "out_f.bmp");
    a.add("near-field", "output field at focal plane (filename)", "out_n.bmp");
    a.add("extended-source", "image of source at focus (filename)", "");
    a.add("interpolate", "option to interpolate the point sources", "-1");
    a.add("output-type", "output field value", "magnitude", "magnitude, polarization, real, imaginary");
    a.add("colormap", "colormap", "brewer", "gray, brewer");
    a.add("append", "append result to an existing (binary) file");
    a.section("Sphere Parameters");
    a.add("spheres", "sphere position", "", "--spheres x y z a m");
    a.add("sphere-file", "sphere file:", "", "[x y z radius material]");
    a.add("materials", "refractive indices as n, k pairs", "1.4 0.05", "--materials n0 k0 n1 k1 n2 k2");
    a.add("material-file", "material file", "", "[lambda n k]");
    a.section("Optics");
    a.add("lambda", "incident wavelength (micrometers)", "1");
    a.add("nu", "incident frequency (in cm^-1) (if specified, lambda is ignored)");
    a.add("k", "k-vector direction in spherical coordinates", "", "--k theta phi; theta = [0 2*pi], phi = [0 pi]");
    a.add("amplitude", "incident field amplitude", "1");
    a.add("condenser", "condenser numerical aperature (a pair of values specify an inner obscuration)", "0 1");
    a.add("objective", "objective numerical aperature (a pair of values specify an inner obscuration)", "0 1");
    a.add("focus", "focal position for the incident point source", "0 0 0");
    a.add("plane-wave", "simulates an incident plane wave");
    a.add("points-rings", "pair of values specying the number of rings and the number of point sources per ring", "1 1");
    a.section("Imaging Parameters");
    a.add("resolution", "resolution of the detector", "256");
    a.add("plane-lower-left", "lower-left position of the image plane", "-5 0 -5");
    a.add("plane-upper-right", "upper-right position of the image plane", "5 0 5");
    a.add("plane-normal", "normal for the image plane", "0 1 0");
    a.add("xy", "specify an x-y axis-aligned image (standard microscope)");
    a.add("xz", "specify a x-z axis-aligned image");
    a.add("yz", "specify a y-z axis-aligned image");
    a.section("Sampling Parameters");
    a.add("samples", "Monte-Carlo samples used to compute Us", "400");
    a.add("padding", "FFT padding for the objective bandpass", "1");
    a.add("supersample", "super-sampling rate for the detector field", "1");
    a.add("field-order", "order of the incident field", "10");
    a.add("seed", "seed for the Monte-Carlo random number generator");
    a.add("recursive", "evaluate all Bessel functions recursively");
    a.add("recursive-us", "evaluate scattered-field Bessel functions recursively");
    a.add("lut-uf", "evaluate the focused-field using a look-up table");
    a.section("GB300 build");
    a.add("precision", "arithmetic of the per-pixel work", "mixed", "mixed, fp64");
    a.add("lut-res", "scattered-field LUT samples (radial angular); default 2*R 1000");
    a.add("uf-lut-res", "incident-field LUT radial samples; default 2*R");
    a.add("waves-file", "plane-wave directions, one 'x y z' per line (replaces the Monte Carlo sampler)");
    a.add("dry-run", "print the derived parameters and stop");
}

bool is_binary(const std::string& f) {  // fileout.cu:161-183
    size_t i = f.find_last_of('.');
    if (i == std::string::npos) return true;
    std::string ext = f.substr(i + 1);
    return !(ext == "bmp" || ext == "jpg" || ext == "tif" || ext == "gif" || ext == "png");
}

struct Material {
    float n, k;
};

struct RawSphere {
    float x, y, z, a;
    unsigned m;
};

// lSpheres(string), arguments.h:193-228: "x y z a [m]" per line
void parse_spheres(const std::string& text, std::vector<RawSphere>& out) {
    std::stringstream ss(text);
    while (!ss.eof()) {
        RawSphere s{0, 0, 0, 0, 0};
        ss >> s.x >> s.y >> s.z >> s.a;
        if (ss.peek() != '\n') ss >> s.m;
        out.push_back(s);
        ss.ignore(1000, '\n');
        ss.peek();
    }
}

int fail(const std::string& msg) {
    std::cout << msg << std::endl;
    return 1;
}

int check(bs_status st) {
    if (st != BS_OK) {
        std::cout << "BIMSim Error: " << bs_last_error() << std::endl;
        return 1;
    }
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    ArgList args;
    define(args);
    args.parse(argc, argv);
    if (args("help")) {
        std::cout << args.help() << std::endl;
        return 1;  // the reference exits with 1 after --help (main.cpp:63-67)
    }
    bool verbose = args("verbose");
    bs_params p{};

    // lFlags (arguments.h:92-113)
    p.lut_us = 1;
    p.lut_uf = 0;
    if (args("recursive")) {
        p.lut_us = 0;
        p.lut_uf = 0;
    } else if (args("recursive-us")) {
        p.lut_us = 0;
    } else if (args("lut-uf")) {
        p.lut_uf = 1;
    }

    // lWavelength (arguments.h:115-132)
    bool wavenumber = false;
    float lambda;
    if (args("nu")) {
        lambda = 10000 / args.f("nu");
        wavenumber = true;
    } else {
        lambda = args.f("lambda");
    }
    p.lambda = lambda;

    // lMaterials (arguments.h:134-191)
    std::vector<Material> mats;
    if (args("material-file")) {
        // one material per file, evaluated at lambda (rts::material<float>(file).getN, nearfield.cpp:119-124)
        for (int i = 0; i < args.nargs("material-file"); i++) {
            double l = lambda, n[2];
            if (check(bs_material_eval(args.text("material-file", i).c_str(), &l, 1, n))) return 1;
            mats.push_back({(float)n[0], (float)n[1]});
        }
    } else {
        int nm = args.nargs("materials");
        if (nm == 1) {
            mats.push_back({args.f("materials"), 0});
        } else if (nm % 2 != 0) {
            return fail("BIMSim Error: materials must be specified in n, k pairs");
        } else {
            for (int i = 0; i < nm; i += 2) mats.push_back({args.f("materials", i), args.f("materials", i + 1)});
        }
    }

    // lSpheres (arguments.h:230-320)
    std::vector<RawSphere> raw;
    if (args("spheres")) {
        int na = args.nargs("spheres");
        unsigned nS;
        if (na <= 5) {
            nS = 1;
        } else if (na % 5 == 0) {
            nS = na / 5;
        } else {
            return fail("BIMSIM Error: Invalid number of sphere parameters.");
        }
        std::stringstream ss;
        for (unsigned s = 0; s < nS; s++) {
            unsigned nP = (nS == 1) ? na : 5;
            for (unsigned i = 0; i < nP; i++) ss << args.f("spheres", s * 5 + i) << " ";
            ss << std::endl;
        }
        parse_spheres(ss.str(), raw);
    }
    if (args("sphere-file")) {
        for (int f = 0; f < args.nargs("sphere-file"); f++) {
            std::ifstream ifs(args.text("sphere-file", f));
            if (!ifs) return fail("Error loading sphere file.");
            std::string text((std::istreambuf_iterator<char>(ifs)), std::istreambuf_iterator<char>());
            parse_spheres(text, raw);
        }
    }
    for (size_t s = 0; s < raw.size(); s++) {
        if (raw[s].m + 1 > mats.size()) {
            std::cout << "BIMSIM Error - A material is not loaded for sphere " << s + 1 << "." << std::endl;
            std::cout << "Material requested: " << raw[s].m + 1 << std::endl;
            std::cout << "Number of materials: " << mats.size() << std::endl;
            return 1;
        }
    }

    // lOptics (arguments.h:322-338)
    p.objective[0] = 0;
    p.objective[1] = 1;
    if (args("objective")) {
        if (args.nargs("objective") == 1) {
            p.objective[0] = 0.0;
            p.objective[1] = args.f("objective");
        } else {
            p.objective[0] = args.f("objective", 0);
            p.objective[1] = args.f("objective", 1);
        }
    }

    // lImagePlane (arguments.h:340-438)
    float pmin[3] = {-5, 0, -5}, pmax[3] = {5, 0, 5}, nrm[3] = {0, 1, 0};
    float s = 40, pos = 0;
    if (args("xy")) {
        if (args.nargs("xy") >= 1) s = args.f("xy", 0);
        if (args.nargs("xy") == 2) pos = args.f("xy", 1);
        float a[3] = {-s / 2, -s / 2, pos}, b[3] = {s / 2, s / 2, pos}, n[3] = {0, 0, 1};
        for (int c = 0; c < 3; c++) pmin[c] = a[c], pmax[c] = b[c], nrm[c] = n[c];
    } else if (args("xz")) {
        float size = 40;
        if (args.nargs("xz") >= 1) size = args.f("xz", 0);
        if (args.nargs("xz") >= 2) pos = args.f("xz", 1);
        float a[3] = {-size / 2, pos, -size / 2}, b[3] = {size / 2, pos, size / 2}, n[3] = {0, -1, 0};
        for (int c = 0; c < 3; c++) pmin[c] = a[c], pmax[c] = b[c], nrm[c] = n[c];
    } else if (args("yz")) {
        float size = 40;
        if (args.nargs("yz") >= 1) size = args.f("yz", 0);
        if (args.nargs("yz") >= 2) pos = args.f("yz", 1);
        float a[3] = {pos, -size / 2, -size / 2}, b[3] = {pos, size / 2, size / 2}, n[3] = {1, 0, 0};
        for (int c = 0; c < 3; c++) pmin[c] = a[c], pmax[c] = b[c], nrm[c] = n[c];
    } else {
        for (int c = 0; c < 3; c++) {
            pmin[c] = args.f("plane-lower-left", c);
            pmax[c] = args.f("plane-upper-right", c);
            nrm[c] = args.f("plane-normal", c);
        }
    }
    for (int c = 0; c < 3; c++) {
        p.plane_min[c] = pmin[c];
        p.plane_max[c] = pmax[c];
        p.plane_normal[c] = nrm[c];
    }
    // supersampling from the plane size s (only --xy changes s, arguments.h:347-418)
    float res = args.f("resolution");
    float dx = s / res;
    int ss = 1;
    if (dx > lambda / 2.0) ss = (int)std::ceil(2 * s / (res * lambda));
    p.resolution = (int)res;
    p.padding = (int)args.f("padding");
    p.supersample = ss;

    // lNearfield (arguments.h:440-505)
    p.scalar = args("vector") ? 0 : 1;
    p.plane_wave = args("plane-wave") ? 1 : 0;
    p.amplitude = args.f("amplitude");
    if (args.nargs("condenser") == 1) {
        p.condenser[0] = 0;
        p.condenser[1] = args.f("condenser", 0);
    } else {
        p.condenser[0] = args.f("condenser", 0);
        p.condenser[1] = args.f("condenser", 1);
    }
    for (int c = 0; c < 3; c++) p.focus[c] = args.f("focus", c);
    float sph_r = 1, sph_t = 0, sph_p = 0;  // spherical (1, theta, phi) -> cartesian (rts/math/vector.h:73-84)
    if (args("k")) {
        sph_t = args.f("k", 0);
        sph_p = args.f("k", 1);
    }
    p.k_dir[0] = sph_r * std::cos(sph_t) * std::sin(sph_p);
    p.k_dir[1] = sph_r * std::sin(sph_t) * std::sin(sph_p);
    p.k_dir[2] = sph_r * std::cos(sph_p);
    p.field_order = args.i("field-order");
    int nk = args.i("samples");
    // --seed is read but has no effect in the reference: calcWaves re-seeds
    // with srand(NULL) (nearfield.cpp:102); the same holds here.

    // extensions of this build
    if (args("lut-res")) {
        p.us_lut_r = args.i("lut-res", 0);
        p.us_lut_theta = args.i("lut-res", 1);
    }
    if (args("uf-lut-res")) p.uf_lut_r = args.i("uf-lut-res", 0);
    std::string prec = args.text("precision");
    bs_precision precision = (prec == "fp64") ? BS_PREC_FP64 : BS_PREC_MIXED;
    // extended source (LoadExtendedSource, microscope.cu:1257-1296): one point
    // source per non-zero pixel at pos(x/width, y/height) of the detector plane,
    // amplitude pixel/255; x outer, y inner
    std::vector<double> sources;
    if (args("extended-source")) {
        int w = 0, h = 0;
        std::vector<unsigned char> px;
        std::string err;
        if (!bsio::read_channel0(args.text("extended-source"), w, h, px, err)) return fail("BIMSim Error: " + err);
        for (int x = 0; x < w; x++)
            for (int y = 0; y < h; y++) {
                unsigned char v = px[(size_t)y * w + x];
                if (v == 0) continue;
                float u = (float)x / (float)w, vv = (float)y / (float)h;
                double f[3];
                if (check(bs_plane_point(&p, u, vv, f))) return 1;
                sources.insert(sources.end(), {f[0], f[1], f[2], (double)((float)v / 255)});
            }
        if (verbose) std::cout << "Number of point sources: " << sources.size() / 4 << std::endl;
    }
    const int interp = sources.empty() ? args.i("interpolate") : -1;
    // --points-rings: sources per ring, then rings (nf.extSource, arguments.h:471-474)
    int ring_points = args.i("points-rings", 0), ring_count = args.i("points-rings", 1);
    if (interp < -1 || interp > 3)
        return fail("BIMSim Error: --interpolate " + std::to_string(interp) + " is not a mode (-1, 0, 1, 2, 3)");
    // Mode 0 (SimulateExtendedGausssianSourceNoInterp, microscope.cu:1327-1409) steps its ring loop
    // `for (int j = spacing; j < numRings; j += spacing)` by spacing = 0.5, which never advances an int:
    // with one ring or more the reference never finishes; with none it simulates the central source.
    if (interp == 0 && ring_count >= 1)
        return fail("BIMSim Error: --interpolate 0 with " + std::to_string(ring_count) +
                    " rings does not terminate in the reference (its ring loop never advances)");
    // Modes 1 and 3 with fewer than two rings simulate the central source only, whatever the points.
    if ((interp == 1 || interp == 3) && ring_count < 2) {
        ring_count = 1;
        ring_points = ring_points < 1 ? 1 : ring_points;
    }

    // spheres with their refractive index at lambda (material n + i k, rts/optics/material.h:434-446)
    std::vector<bs_sphere> spheres;
    for (auto& r : raw) spheres.push_back({r.x, r.y, r.z, r.a, mats[r.m].n, mats[r.m].k});

    // lOutputParams (arguments.h:507-562)
    bool append = args("append");
    std::string intFile = args.text("intensity"), incFile = args.text("incident"), absFile = args.text("absorbance"),
                absSpecFile = args.text("absorbance-spec"), transFile;
    if (args("transmittance")) transFile = args.text("transmittance");
    std::string nearFile = args.text("near-field"), farFile = args.text("far-field");
    std::string fieldStr = args.text("output-type");
    bsio::Colormap cmap = bsio::CM_BREWER;
    {
        std::string cm = args.text("colormap");
        if (cm == "gray")
            cmap = bsio::CM_GRAY;
        else if (cm != "brewer")
            std::cout << "color-map value not recognized (using default): " << cm << std::endl;
    }

    if (args("dry-run")) {
        std::printf("{\"lambda\": %.9g, \"amplitude\": %.9g, \"k\": [%.9g, %.9g, %.9g], \"focus\": [%.9g, %.9g, %.9g], "
                    "\"condenser\": [%.9g, %.9g], \"objective\": [%.9g, %.9g], \"plane_min\": [%.9g, %.9g, %.9g], "
                    "\"plane_max\": [%.9g, %.9g, %.9g], \"normal\": [%.9g, %.9g, %.9g], \"resolution\": %d, "
                    "\"padding\": %d, \"supersample\": %d, \"field_order\": %d, \"samples\": %d, \"scalar\": %d, "
                    "\"plane_wave\": %d, \"lut_uf\": %d, \"lut_us\": %d, \"us_lut\": [%d, %d], \"uf_lut\": %d, "
                    "\"precision\": \"%s\", \"wavenumber\": %d, \"append\": %d, \"point_sources\": %zu, "
                    "\"interpolate\": %d, \"points_rings\": [%d, %d], \"spheres\": [",
                    p.lambda, p.amplitude, p.k_dir[0], p.k_dir[1], p.k_dir[2], p.focus[0], p.focus[1], p.focus[2],
                    p.condenser[0], p.condenser[1], p.objective[0], p.objective[1], p.plane_min[0], p.plane_min[1],
                    p.plane_min[2], p.plane_max[0], p.plane_max[1], p.plane_max[2], p.plane_normal[0],
                    p.plane_normal[1], p.plane_normal[2], p.resolution, p.padding, p.supersample, p.field_order, nk,
                    p.scalar, p.plane_wave, p.lut_uf, p.lut_us, p.us_lut_r, p.us_lut_theta, p.uf_lut_r,
                    precision == BS_PREC_FP64 ? "fp64" : "mixed", wavenumber ? 1 : 0, append ? 1 : 0,
                    sources.size() / 4, interp, ring_points, ring_count);
        for (size_t i = 0; i < spheres.size(); i++)
            std::printf("%s[%.9g, %.9g, %.9g, %.9g, %.9g, %.9g]", i ? ", " : "", spheres[i].x, spheres[i].y,
                        spheres[i].z, spheres[i].a, spheres[i].n_re, spheres[i].n_im);
        std::printf("], \"outputs\": {\"intensity\": \"%s\", \"incident\": \"%s\", \"absorbance\": \"%s\", "
                    "\"absorbance_spec\": \"%s\", \"transmittance\": \"%s\"}}\n",
                    intFile.c_str(), incFile.c_str(), absFile.c_str(), absSpecFile.c_str(), transFile.c_str());
        return 0;
    }

    // ---- simulate (microscopeStruct::init + fileoutStruct::Save, fileout.cu:189-265) ----
    bs_ctx* ctx = nullptr;
    if (check(bs_create(&p, &ctx))) return 1;
    if (check(bs_set_spheres(ctx, spheres.data(), (int)spheres.size()))) return 1;
    if (!p.plane_wave) {
        if (args("waves-file")) {
            std::ifstream wf(args.text("waves-file"));
            if (!wf) return fail("BIMSim Error: cannot read " + args.text("waves-file"));
            std::vector<double> w;
            double v;
            while (wf >> v) w.push_back(v);
            if (w.size() < 3 || w.size() % 3) return fail("BIMSim Error: waves file needs x y z per line");
            if (check(bs_set_waves(ctx, w.data(), (int)(w.size() / 3)))) return 1;
        } else {
            if (check(bs_sample_waves_compat(ctx, nk))) return 1;
        }
    }
    if (interp >= 1) {
        // fileout.cu:218-243: mode 3 SimulateExtendedSourceWithInterpolation, 1
        // SimulateExtendedSourceInterpAtDetector, 2 SimulateExtendedSourceInterpLineAtDetector; then saveDetector
        bs_status st = interp == 3   ? bs_simulate_ring_interp(ctx, ring_points, ring_count, precision)
                       : interp == 1 ? bs_simulate_ring_detector(ctx, ring_points, ring_count, precision)
                                     : bs_simulate_ring_line(ctx, ring_points, ring_count, precision);
        if (check(st)) return 1;
    } else if (sources.empty()) {
        if (check(bs_simulate(ctx, precision))) return 1;
        // fileoutStruct::saveNearField / saveFarField (fileout.cu:3-45): field images of
        // the last source in the single-source path
        auto field_image = [&](const std::string& file, bool far) -> int {
            if (file.empty()) return 0;
            bool mag = fieldStr == "magnitude", re = fieldStr == "real", im = fieldStr == "imaginary";
            if (!mag && !re && !im) return 0;  // other output types write nothing here
            if (is_binary(file)) {
                std::cout << "\t\t field images need an image file name (.bmp or .png): " << file << std::endl;
                return 0;
            }
            int n = 0;
            std::vector<double> f;
            if (far) {
                n = p.resolution * p.supersample;
                f.resize(2 * (size_t)n * n);
                if (check(bs_get_far_field(ctx, BS_FIELD_TOTAL, f.data(), (size_t)n * n))) return 1;
            } else {
                bs_info inf{};
                bs_get_info(ctx, &inf);
                n = inf.nf_res;
                f.resize(2 * (size_t)n * n);
                if (check(bs_get_field(ctx, BS_FIELD_TOTAL, f.data(), (size_t)n * n))) return 1;
            }
            std::vector<double> v((size_t)n * n);
            for (size_t i = 0; i < v.size(); i++)
                v[i] = mag ? std::sqrt(f[2 * i] * f[2 * i] + f[2 * i + 1] * f[2 * i + 1]) : (re ? f[2 * i] : f[2 * i + 1]);
            std::string err;
            if (!bsio::write_scalar_image(file, n, n, v, mag, cmap, err)) return fail("BIMSim Error: " + err);
            return 0;
        };
        // mode 0 with no rings saves the detector only (fileout.cu:230-236)
        if (interp == -1 && (field_image(nearFile, false) || field_image(farFile, true))) return 1;
    } else {
        // SimulateExtendedSource (microscope.cu:873-913): the detector sums the point sources
        if (check(bs_simulate_sources(ctx, sources.data(), (int)(sources.size() / 4), precision))) return 1;
    }

    // ---- fileoutStruct::saveDetector (fileout.cu:47-159) ----
    double band = wavenumber ? (double)(10000.0f / lambda) : (double)lambda;
    struct Out {
        const std::string& file;
        bs_image_kind kind;
    } outs[] = {{intFile, BS_IMG_INTENSITY}, {incFile, BS_IMG_INCIDENT}, {absFile, BS_IMG_ABSORBANCE}};
    auto save = [&](const std::string& file, bs_image_kind kind) -> int {
        if (file.empty()) return 0;
        std::cout << "\t\t saving: " << file << std::endl;
        if (!is_binary(file)) {
            // scalarslice::toImage(file) with its defaults: range [0, max], Brewer map
            // (the --colormap flag reaches only the field images, fileout.cu:3-45)
            std::vector<double> v((size_t)p.resolution * p.resolution);
            if (check(bs_get_image_f64(ctx, kind, v.data(), v.size()))) return 1;
            std::string err;
            if (!bsio::write_scalar_image(file, p.resolution, p.resolution, v, true, bsio::CM_BREWER, err))
                return fail("BIMSim Error: " + err);
            return 0;
        }
        return check(bs_write_envi(ctx, kind, file.c_str(), append ? 1 : 0, band));
    };
    for (auto& o : outs)
        if (save(o.file, o.kind)) return 1;
    if (!absSpecFile.empty()) {
        std::cout << "\t\t saving: " << absSpecFile << std::endl;
        if (is_binary(absSpecFile)) {  // getAbsorbanceSpectrum() is a stub returning 0 (microscope.cu:749-762)
            std::ofstream f(absSpecFile, std::ios::app);
            if (wavenumber)
                f << 10000.0f / lambda << "," << 0.0f << std::endl;
            else
                f << lambda << "," << 0.0f << std::endl;
        }
    }
    if (save(transFile, BS_IMG_TRANSMITTANCE)) return 1;
    if (verbose) {
        bs_stats st{};
        bs_info inf{};
        bs_get_stats(ctx, &st);
        bs_get_info(ctx, &inf);
        std::cout << "---------Timings-------------" << std::endl
                  << "Uf = " << st.ms_uf << "ms" << std::endl
                  << "Us = " << st.ms_lut + st.ms_us << "ms" << std::endl
                  << "detector = " << st.ms_detector << "ms" << std::endl
                  << "near field " << inf.nf_res << "^2, " << inf.n_spheres << " spheres, " << inf.n_waves
                  << " waves, " << st.kernel_launches << " kernel launches" << std::endl;
    }
    bs_destroy(ctx);
    return 0;
}
