// bs_host.cpp -- host-side geometry, the reference-compatible Monte Carlo
// sampler and the ENVI writer.  Compiled with -ffp-contract=off so that the
// single-precision sampler gives the same bits as the reference's host code.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "bs_internal.h"

namespace bs {

static inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 mul(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
static inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
double v3_len(V3 a) { return std::sqrt(dot(a, a)); }

// rts::quad(pMin, pMax, normal) (rts/math/quad.h:55-84): X and Y span the
// square whose diagonal is pMax - pMin, in the plane with the given normal.
Quad quad_from(const double* pmin, const double* pmax, const double* n) {
    V3 a{pmin[0], pmin[1], pmin[2]}, b{pmax[0], pmax[1], pmax[2]}, nn{n[0], n[1], n[2]};
    V3 diag = sub(b, a);
    V3 side{diag.y * nn.z - diag.z * nn.y, diag.z * nn.x - diag.x * nn.z, diag.x * nn.y - diag.y * nn.x};
    V3 B = add(add(a, mul(diag, 0.5)), mul(side, 0.5));
    V3 C = sub(add(a, mul(diag, 0.5)), mul(side, 0.5));
    return {a, sub(B, a), sub(C, a)};
}

// Scale about the centre (rts/math/quad.h:162-177).
Quad quad_scale(const Quad& q, double s) {
    V3 c = add(add(q.A, mul(q.X, 0.5)), mul(q.Y, 0.5));
    Quad r;
    r.X = mul(q.X, s);
    r.Y = mul(q.Y, s);
    r.A = sub(sub(c, mul(r.X, 0.5)), mul(r.Y, 0.5));
    return r;
}

// Closest point of triangle (A, B, C) to p by the barycentric region test
// of rts/math/triangle.h:62-177; like the reference, regions 2, 4 and 6 snap
// to a vertex instead of searching the two adjacent edges.
static V3 triangle_closest(V3 A, V3 B, V3 C, V3 p) {
    V3 e0 = sub(B, A), e1 = sub(C, A), w = sub(A, p);
    double a = dot(e0, e0), b = dot(e0, e1), c = dot(e1, e1), d = dot(e0, w), e = dot(e1, w);
    double det = a * c - b * b, s = b * e - c * d, t = b * d - a * e;
    if (s + t <= det) {
        if (s < 0) {
            if (t < 0) {
                s = 0;
                t = 0;
            } else {
                s = 0;
                t = (e >= 0) ? 0 : ((-e >= c) ? 1 : -e / c);
            }
        } else if (t < 0) {
            s = (d >= 0) ? 0 : ((-d >= a) ? 1 : -d / a);
            t = 0;
        } else {
            double inv = 1.0 / det;
            s *= inv;
            t *= inv;
        }
    } else if (s < 0) {
        s = 0;
        t = 1;
    } else if (t < 0) {
        s = 1;
        t = 0;
    } else {
        double num = c + e - b - d;
        if (num <= 0) {
            s = 0;
        } else {
            double den = a - 2 * b + c;
            s = (num >= den) ? 1 : num / den;
        }
        t = 1 - s;
    }
    return add(add(A, mul(e0, s)), mul(e1, t));
}

double quad_dist(const Quad& q, V3 p) {  // rts/math/quad.h:179-195
    V3 AX = add(q.A, q.X), AY = add(q.A, q.Y), AXY = add(AX, q.Y);
    double d0 = v3_len(sub(p, triangle_closest(q.A, AX, AY, p)));
    double d1 = v3_len(sub(p, triangle_closest(AXY, AX, AY, p)));
    return d0 < d1 ? d0 : d1;
}

double quad_dist_max(const Quad& q, V3 p) {  // rts/math/quad.h:197-205
    V3 AX = add(q.A, q.X), AY = add(q.A, q.Y), AXY = add(AX, q.Y);
    return std::max(std::max(v3_len(sub(q.A, p)), v3_len(sub(AX, p))),
                    std::max(v3_len(sub(AY, p)), v3_len(sub(AXY, p))));
}

// Nl = ceil(ka + 4 (ka)^(1/3) + 2) evaluated in single precision, the way
// sphere::calcNl (sphere.h:71-74) evaluates it.
int calc_nl(double a_in, double lambda_in) {
    volatile float a = (float)a_in, lam = (float)lambda_in, pif = 3.14159f;
    volatile float ka = 2.0f * pif;
    ka = ka * a;
    ka = ka / lam;
    volatile float third = (float)(1.0 / 3.0);
    volatile float root = std::pow((float)ka, (float)third);
    volatile float v = 4.0f * root;
    v = ka + v;
    v = v + 2.0f;
    return (int)std::ceil((float)v);
}

// glibc's rand() (TYPE_3 state): x_i = x_{i-3} + x_{i-31} (mod 2^32) after a
// Lehmer (16807) seeding of 31 words and 310 discarded draws; seed 0 acts as 1.
namespace {
class LegacyRand {
public:
    explicit LegacyRand(unsigned seed) {
        if (seed == 0) seed = 1;
        x_.resize(344);
        int64_t w = seed;
        x_[0] = (uint32_t)w;
        for (int i = 1; i < 31; i++) {
            w = (16807LL * w) % 2147483647LL;
            x_[i] = (uint32_t)w;
        }
        for (int i = 31; i < 34; i++) x_[i] = x_[i - 31];
        for (int i = 34; i < 344; i++) x_[i] = x_[i - 31] + x_[i - 3];
    }
    int next() {
        size_t i = x_.size();
        uint32_t v = x_[i - 31] + x_[i - 3];
        x_.push_back(v);
        return (int)(v >> 1);
    }

private:
    std::vector<uint32_t> x_;
};
}  // namespace

// mcSampleNA (montecarlo.cpp:9-71) after the srand(0) of nearfield.cpp:102:
// z uniform between cos(asin NA_out) and cos(asin NA_in), azimuth uniform,
// rotated from +z onto k by the quaternion matrix of rts/math/quaternion.h.
// Every step is single precision in the reference's order.
void mc_sample_compat(int nk, const double* kdir, double na_in, double na_out, double* out) {
    LegacyRand rng(0);
    volatile float kx = (float)kdir[0], ky = (float)kdir[1], kz = (float)kdir[2];
    float M[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};  // M[row][col]
    volatile float cz = 0.0f;
    cz = cz + kx * 0.0f;
    cz = cz + ky * 0.0f;
    cz = cz + kz * 1.0f;
    if (cz != 1.0f) {
        volatile float ax = 0.0f * kz - 1.0f * ky, ay = 1.0f * kx - 0.0f * kz, az = 0.0f * ky - 0.0f * kx;
        volatile float n2 = 0.0f;
        n2 = n2 + ax * ax;
        n2 = n2 + ay * ay;
        n2 = n2 + az * az;
        volatile float nl = std::sqrt((float)n2);
        ax = ax / nl;
        ay = ay / nl;
        az = az / nl;
        volatile float ang = std::acos((float)cz);
        volatile float qw = (float)std::cos((double)ang / 2.0);
        volatile float sh = (float)std::sin((double)ang / 2.0);
        volatile float qx = ax * sh, qy = ay * sh, qz = az * sh;
        volatile float x2 = qx + qx, y2 = qy + qy, z2 = qz + qz;
        volatile float xx = qx * x2, xy = qx * y2, xz = qx * z2, yy = qy * y2, yz = qy * z2, zz = qz * z2;
        volatile float wx = qw * x2, wy = qw * y2, wz = qw * z2;
        M[0][0] = 1.0f - (yy + zz);
        M[0][1] = xy - wz;
        M[0][2] = xz + wy;
        M[1][0] = xy + wz;
        M[1][1] = 1.0f - (xx + zz);
        M[1][2] = yz - wx;
        M[2][0] = xz - wy;
        M[2][1] = yz + wx;
        M[2][2] = 1.0f - (xx + yy);
    }
    volatile float zin = std::cos(std::asin((float)na_in)), zout = std::cos(std::asin((float)na_out));
    volatile float zrange = zin - zout;
    const float rmax = (float)2147483647;
    const float pif = 3.14159f;
    for (int i = 0; i < nk; i++) {
        volatile float z = ((float)rng.next() / rmax) * zrange;
        z = z + zout;
        volatile float az = ((float)rng.next() / rmax) * 2.0f;
        az = az * pif;
        volatile float polar = std::acos((float)z);
        volatile float v0 = 1.0f * std::cos((float)az);
        v0 = v0 * std::sin((float)polar);
        volatile float v1 = 1.0f * std::sin((float)az);
        v1 = v1 * std::sin((float)polar);
        volatile float v2 = 1.0f * std::cos((float)polar);
        float v[3] = {v0, v1, v2};
        for (int r = 0; r < 3; r++) {
            volatile float acc = 0.0f;
            for (int c = 0; c < 3; c++) {
                volatile float t = M[r][c] * v[c];
                acc = acc + t;
            }
            out[3 * i + r] = acc;
        }
    }
}

// ---------------------------------------------------------------------------
// ENVI (rts/envi/envi.h:196-433, rts/envi/envi_header.h:318-375): float32,
// band sequential, little endian, one wavelength entry per band; in append
// mode the existing header is read back and the band count grows.
// ---------------------------------------------------------------------------
namespace {
std::string num(double v) {
    std::ostringstream os;
    os << v;  // default stream formatting (6 significant digits), as the reference
    return os.str();
}

std::string strip(const std::string& s) {
    size_t a = s.find_first_not_of(' ');
    if (a == std::string::npos) return "";
    size_t b = s.find_last_not_of(' ');
    return s.substr(a, b - a + 1);
}

std::vector<std::string> comma_list(const std::string& s) {
    std::vector<std::string> v;
    size_t st = 0;
    while (true) {
        size_t c = s.find(',', st);
        v.push_back(strip(s.substr(st, c == std::string::npos ? std::string::npos : c - st)));
        if (c == std::string::npos) break;
        st = c + 1;
    }
    return v;
}

struct Header {
    std::string description, file_type = "ENVI Standard", interleave = "bsq", sensor = "Unknown",
                units = "Unknown", zt0 = "Unknown", zt1 = "Unknown";
    unsigned samples = 0, lines = 0, bands = 0, offset = 0;
    int data_type = 4, byte_order = 0;
    double xs = 0, ys = 0, px = 1, py = 1;
    std::vector<std::string> names;
    std::vector<double> wl;
};

bool read_header(const std::string& path, Header& h) {
    std::ifstream in(path);
    if (!in) return false;
    std::string tag, line;
    in >> tag;
    if (tag != "ENVI") return false;
    std::getline(in, line);
    while (std::getline(in, line)) {
        size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        std::string key = strip(line.substr(0, eq));
        std::string val = strip(line.substr(eq + 1));
        size_t ob = val.find('{');
        if (ob != std::string::npos) {
            std::string body = val.substr(ob + 1);
            while (body.find('}') == std::string::npos && std::getline(in, line)) body += line;
            body = strip(body.substr(0, body.find('}')));
            if (key == "description") {
                h.description = body;
            } else if (key == "band names") {
                h.names = comma_list(body);
            } else if (key == "wavelength") {
                h.wl.clear();
                for (auto& s : comma_list(body)) h.wl.push_back(std::atof(s.c_str()));
            } else if (key == "pixel size") {
                auto v = comma_list(body);
                if (v.size() >= 2) {
                    h.px = std::atof(v[0].c_str());
                    h.py = std::atof(v[1].c_str());
                }
            } else if (key == "z plot titles") {
                auto v = comma_list(body);
                if (v.size() >= 2) {
                    h.zt0 = v[0];
                    h.zt1 = v[1];
                }
            }
            continue;
        }
        if (key == "samples") h.samples = (unsigned)std::atoi(val.c_str());
        else if (key == "lines") h.lines = (unsigned)std::atoi(val.c_str());
        else if (key == "bands") h.bands = (unsigned)std::atoi(val.c_str());
        else if (key == "header offset") h.offset = (unsigned)std::atoi(val.c_str());
        else if (key == "file type") h.file_type = val;
        else if (key == "data type") h.data_type = std::atoi(val.c_str());
        else if (key == "interleave") h.interleave = val;
        else if (key == "sensor type") h.sensor = val;
        else if (key == "byte order") h.byte_order = std::atoi(val.c_str());
        else if (key == "x start") h.xs = std::atof(val.c_str());
        else if (key == "y start") h.ys = std::atof(val.c_str());
        else if (key == "wavelength units") h.units = val;
    }
    return true;
}

bool write_header(const std::string& path, const Header& h) {
    std::ofstream o(path);
    if (!o) return false;
    o << "ENVI\n"
      << "description = {\n"
      << "  " << h.description << "}\n"
      << "samples = " << h.samples << "\n"
      << "lines = " << h.lines << "\n"
      << "bands = " << h.bands << "\n"
      << "header offset = " << h.offset << "\n"
      << "file type = " << h.file_type << "\n"
      << "data type = " << h.data_type << "\n"
      << "interleave = " << h.interleave << "\n"
      << "sensor type = " << h.sensor << "\n"
      << "byte order = " << h.byte_order << "\n"
      << "x start = " << num(h.xs) << "\n"
      << "y start = " << num(h.ys) << "\n"
      << "wavelength units = " << h.units << "\n"
      << "z plot titles = {" << h.zt0 << ", " << h.zt1 << "}\n"
      << "pixel size = {" << num(h.px) << ", " << num(h.py) << ", units=Meters}\n";
    if (!h.names.empty()) {
        o << "band names = {\n";
        for (size_t i = 0; i < h.names.size(); i++) o << h.names[i] << (i + 1 < h.names.size() ? ", " : "");
        o << "}\n";
    }
    o << "wavelength = {\n";
    for (size_t i = 0; i < h.wl.size(); i++) o << num(h.wl[i]) << (i + 1 < h.wl.size() ? ", " : "");
    o << "}\n";
    return (bool)o;
}
}  // namespace

int envi_add_band(const char* path, const float* band, int samples, int lines, double wavelength, int append,
                  char* err, size_t errlen) {
    std::string dat(path), hdr = dat + ".hdr";
    Header h;
    bool has_data = false;
    if (append) {
        read_header(hdr, h);
        if (FILE* t = std::fopen(path, "rb")) {
            std::fseek(t, 0, SEEK_END);
            has_data = std::ftell(t) > 0;
            std::fclose(t);
        }
    }
    if (has_data && (h.lines != (unsigned)lines || h.samples != (unsigned)samples)) {
        std::snprintf(err, errlen, "ENVI Error: cannot change the image size of a locked BSQ file (%s)", path);
        return 1;
    }
    FILE* f = std::fopen(path, append ? "ab" : "wb");
    if (!f) {
        std::snprintf(err, errlen, "ENVI Error: unable to open binary file: %s", path);
        return 2;
    }
    size_t n = (size_t)samples * lines;
    size_t wrote = std::fwrite(band, sizeof(float), n, f);
    std::fclose(f);
    if (wrote != n) {
        std::snprintf(err, errlen, "ENVI Error: short write to %s", path);
        return 2;
    }
    h.bands++;
    h.samples = samples;
    h.lines = lines;
    h.wl.push_back(wavelength);
    if (!write_header(hdr, h)) {
        std::snprintf(err, errlen, "ENVI Error: unable to write header %s", hdr.c_str());
        return 2;
    }
    return 0;
}

}  // namespace bs

// ---------------------------------------------------------------------------
// Material files (rts/optics/material.h:57-160, 434-540; rts/math/function.h).
// Single precision throughout, as the reference's material<ptype = float>.
// ---------------------------------------------------------------------------
namespace bs {

namespace {

enum MatField { MF_MICRONS, MF_WAVENUMBER, MF_N, MF_K, MF_A, MF_IGNORE };

template <class T>
struct MatPoint {
    T lambda;
    T n_re, n_im;
};

// one value as `stream >> T` reads it (strtof / strtod), the number of characters used in *used
template <class T>
T read_value(const std::string& s, size_t* used);
template <>
float read_value<float>(const std::string& s, size_t* used) { return std::stof(s, used); }
template <>
double read_value<double>(const std::string& s, size_t* used) { return std::stod(s, used); }

// "microns,n,k"-style column list (entryType, material.h:62-95)
std::vector<MatField> parse_format(std::string f) {
    std::vector<MatField> out;
    for (;;) {
        size_t e = f.find(',');
        std::string t = f.substr(0, e);
        out.push_back(t == "microns" ? MF_MICRONS
                      : t == "wavenumber" ? MF_WAVENUMBER
                      : t == "n" ? MF_N
                      : t == "k" ? MF_K
                      : t == "A" ? MF_A
                      : MF_IGNORE);
        if (e == std::string::npos) break;
        f = f.substr(e + 1);
    }
    return out;
}

}  // namespace

template <class T>
bool material_load(const std::string& text, std::vector<T>& lam, std::vector<T>& re, std::vector<T>& im,
                   std::string& err) {
    std::stringstream ss(text);
    std::string line, format = "microns,n,k";
    // an optional first comment line names the columns: "# ... [wavenumber,n,k]" (material.h:490-510)
    if (ss.peek() == '#') {
        std::getline(ss, line);
        size_t a = line.find('['), b = line.find(']');
        if (a != std::string::npos && b != std::string::npos) format = line.substr(a + 1, b - a - 1);
    }
    const std::vector<MatField> cols = parse_format(format);
    std::vector<MatPoint<T>> pts;
    int lineno = 0;
    while (std::getline(ss, line)) {
        lineno++;
        if (!line.empty() && line[0] == '#') continue;
        if (line.find_first_not_of(" \t\r") == std::string::npos) continue;  // the reference loops forever here
        // inputEntry (material.h:105-160): before each value skip every character
        // that is not a digit (so signs are dropped: "-0.5" reads 0.5), then read a T
        MatPoint<T> p{0, 0, 0};
        size_t pos = 0;
        for (MatField c : cols) {
            while (pos < line.size() && (line[pos] < '0' || line[pos] > '9')) pos++;
            if (pos >= line.size()) {
                err = "material line " + std::to_string(lineno) + " has fewer values than the format [" + format +
                      "]";
                return false;
            }
            size_t used = 0;
            const T v = read_value<T>(line.substr(pos), &used);
            pos += used;
            switch (c) {
                case MF_MICRONS: p.lambda = v; break;
                case MF_WAVENUMBER: p.lambda = (T)10000.0 / v; break;
                case MF_N: p.n_re = v; break;
                case MF_K: p.n_im = v; break;
                case MF_A: p.n_im = (v * p.lambda) / (4 * (float)PI_REF); break;  // _A(), material.h:37-40
                default: break;
            }
        }
        // function::insert: before the first point with a larger wavelength (function.h:80-98)
        auto it = std::upper_bound(pts.begin(), pts.end(), p,
                                   [](const MatPoint<T>& a, const MatPoint<T>& b) { return a.lambda < b.lambda; });
        pts.insert(it, p);
    }
    if (pts.empty()) {
        err = "material file has no entries";
        return false;
    }
    lam.clear();
    re.clear();
    im.clear();
    for (auto& q : pts) {
        lam.push_back(q.lambda);
        re.push_back(q.n_re);
        im.push_back(q.n_im);
    }
    return true;
}

// material::getN = function::linear(lambda) + n0 with n0 = 0 for files
// (material.h:617-621, function.h:44-75): the first point with a larger
// wavelength bounds the interval, ends clamp, and the weights are swapped as in
// the reference: value = y_lo * a + y_hi * (1 - a), a = (l - l_lo) / (l_hi - l_lo).
template <class T>
void material_eval(const std::vector<T>& lam, const std::vector<T>& re, const std::vector<T>& im, T l, T& n_re,
                   T& n_im) {
    size_t i = std::upper_bound(lam.begin(), lam.end(), l) - lam.begin();
    if (i == lam.size()) {
        n_re = re.back();
        n_im = im.back();
    } else if (i == 0) {
        n_re = re.front();
        n_im = im.front();
    } else {
        const T a = (l - lam[i - 1]) / (lam[i] - lam[i - 1]);
        n_re = re[i - 1] * a + re[i] * ((T)1 - a);
        n_im = im[i - 1] * a + im[i] * ((T)1 - a);
    }
}

template bool material_load<float>(const std::string&, std::vector<float>&, std::vector<float>&,
                                   std::vector<float>&, std::string&);
template bool material_load<double>(const std::string&, std::vector<double>&, std::vector<double>&,
                                    std::vector<double>&, std::string&);
template void material_eval<float>(const std::vector<float>&, const std::vector<float>&, const std::vector<float>&,
                                   float, float&, float&);
template void material_eval<double>(const std::vector<double>&, const std::vector<double>&,
                                    const std::vector<double>&, double, double&, double&);

}  // namespace bs
