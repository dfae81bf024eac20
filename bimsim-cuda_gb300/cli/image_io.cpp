// Image readers and writers of the `bimsim` command line (see image_io.h).
#include "image_io.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>

namespace bsio {
namespace {

bool ends_with(const std::string& s, const std::string& e) {
    if (s.size() < e.size()) return false;
    std::string t = s.substr(s.size() - e.size());
    for (auto& ch : t) ch = (char)std::tolower((unsigned char)ch);
    return t == e;
}

uint32_t le32(const unsigned char* p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
uint16_t le16(const unsigned char* p) { return (uint16_t)(p[0] | (p[1] << 8)); }

void put32le(std::vector<unsigned char>& b, uint32_t v) {
    for (int i = 0; i < 4; i++) b.push_back((unsigned char)(v >> (8 * i)));
}
void put16le(std::vector<unsigned char>& b, uint16_t v) {
    b.push_back((unsigned char)v);
    b.push_back((unsigned char)(v >> 8));
}
void put32be(std::vector<unsigned char>& b, uint32_t v) {
    for (int i = 3; i >= 0; i--) b.push_back((unsigned char)(v >> (8 * i)));
}

// PNG checksums: CRC-32 (ISO 3309 polynomial 0xEDB88320, bitwise) and Adler-32 (RFC 1950)
uint32_t crc32(const unsigned char* d, size_t n, uint32_t c = 0xFFFFFFFFu) {
    for (size_t i = 0; i < n; i++) {
        c ^= d[i];
        for (int k = 0; k < 8; k++) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1u)));
    }
    return c;
}

uint32_t adler32(const std::vector<unsigned char>& d) {
    uint32_t a = 1, b = 0;
    for (unsigned char x : d) {
        a = (a + x) % 65521u;
        b = (b + a) % 65521u;
    }
    return (b << 16) | a;
}

bool read_pgm(const std::vector<unsigned char>& f, int& w, int& h, std::vector<unsigned char>& out,
              std::string& err) {
    const bool binary = f[1] == '5';
    size_t pos = 2;
    auto next_int = [&](int& v) -> bool {
        for (;;) {
            while (pos < f.size() && std::isspace(f[pos])) pos++;
            if (pos < f.size() && f[pos] == '#') {
                while (pos < f.size() && f[pos] != '\n') pos++;
                continue;
            }
            break;
        }
        if (pos >= f.size() || !std::isdigit(f[pos])) return false;
        v = 0;
        while (pos < f.size() && std::isdigit(f[pos])) v = v * 10 + (f[pos++] - '0');
        return true;
    };
    int maxv = 0;
    if (!next_int(w) || !next_int(h) || !next_int(maxv) || w <= 0 || h <= 0 || maxv <= 0 || maxv > 255) {
        err = "unsupported PGM header (8-bit P5/P2 only)";
        return false;
    }
    out.resize((size_t)w * h);
    if (binary) {
        pos++;  // the single whitespace after maxval
        if (f.size() < pos + out.size()) {
            err = "truncated PGM";
            return false;
        }
        std::memcpy(out.data(), f.data() + pos, out.size());
    } else {
        for (auto& px : out) {
            int v = 0;
            if (!next_int(v)) {
                err = "truncated PGM";
                return false;
            }
            px = (unsigned char)v;
        }
    }
    return true;
}

bool read_bmp(const std::vector<unsigned char>& f, int& w, int& h, std::vector<unsigned char>& out,
              std::string& err) {
    if (f.size() < 54) {
        err = "truncated BMP";
        return false;
    }
    const uint32_t data = le32(&f[10]), hsize = le32(&f[14]);
    const int32_t bw = (int32_t)le32(&f[18]), bh = (int32_t)le32(&f[22]);
    const uint16_t bpp = le16(&f[28]);
    const uint32_t comp = le32(&f[30]);
    if (comp != 0 || (bpp != 8 && bpp != 24 && bpp != 32) || bw <= 0 || bh == 0) {
        err = "unsupported BMP (uncompressed 8-, 24- or 32-bit only)";
        return false;
    }
    w = bw;
    h = bh < 0 ? -bh : bh;
    const bool top_down = bh < 0;
    const size_t stride = ((size_t)w * bpp / 8 + 3) & ~(size_t)3;
    if (f.size() < data + stride * h) {
        err = "truncated BMP";
        return false;
    }
    uint32_t ncol = bpp == 8 ? le32(&f[46]) : 0;
    if (bpp == 8 && ncol == 0) ncol = 256;
    const unsigned char* pal = &f[14 + hsize];
    out.resize((size_t)w * h);
    for (int y = 0; y < h; y++) {
        const unsigned char* row = &f[data + stride * (size_t)(top_down ? y : h - 1 - y)];
        for (int x = 0; x < w; x++) {
            unsigned char r;
            if (bpp == 8) {
                const unsigned idx = row[x];
                r = idx < ncol ? pal[4 * idx + 2] : 0;  // palette entries are B, G, R, 0
            } else {
                r = row[x * (bpp / 8) + 2];  // pixels are B, G, R(, A)
            }
            out[(size_t)y * w + x] = r;
        }
    }
    return true;
}

}  // namespace

bool read_channel0(const std::string& path, int& width, int& height, std::vector<unsigned char>& out,
                   std::string& err) {
    std::ifstream in(path, std::ios::binary);
    if (!in) {
        err = "cannot open " + path;
        return false;
    }
    std::vector<unsigned char> f((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    if (f.size() >= 2 && f[0] == 'P' && (f[1] == '5' || f[1] == '2')) return read_pgm(f, width, height, out, err);
    if (f.size() >= 2 && f[0] == 'B' && f[1] == 'M') return read_bmp(f, width, height, out, err);
    err = path + ": not a PGM or BMP image";
    return false;
}

std::vector<unsigned char> colormap(const std::vector<double>& v, double vmin, double vmax, Colormap cm) {
    // ColorBrewer RdYlBu, 11 classes, from blue to red: the control points of
    // the reference's Brewer map (rts/visualization/colormap.h), which stores
    // them as 8-bit levels / 255 written with six decimals (so 255 * c can
    // fall just below the level, e.g. 69 -> 68.99994 -> 68 after truncation)
    static const unsigned char brewer8[11][3] = {{49, 54, 149},   {69, 117, 180},  {116, 173, 209}, {171, 217, 233},
                                                 {224, 243, 248}, {255, 255, 191}, {254, 224, 144}, {253, 174, 97},
                                                 {244, 109, 67},  {215, 48, 39},   {165, 0, 38}};
    float brewer[11][3];
    for (int i = 0; i < 11; i++)
        for (int c = 0; c < 3; c++) brewer[i][c] = (float)(std::round(brewer8[i][c] / 255.0 * 1e6) / 1e6);
    std::vector<unsigned char> rgb(v.size() * 3);
    const float lo = (float)vmin, span = (float)vmax - lo;  // the reference maps single-precision images
    for (size_t i = 0; i < v.size(); i++) {
        const float a = ((float)v[i] - lo) / span;
        unsigned char* px = &rgb[3 * i];
        if (!(a == a)) {  // NaN (also vmin == vmax): black
            px[0] = px[1] = px[2] = 0;
            continue;
        }
        if (cm == CM_GRAY) {
            const float g = a > 1.f ? 1.f : (a < 0.f ? 0.f : a);
            px[0] = px[1] = px[2] = (unsigned char)(255.f * g);
        } else {
            // applyBrewer (rts/visualization/colormap.h:92-110): tex1D at the normalised
            // coordinate a + 1/22 (a float sum), linear filtering, clamp: texel coordinate
            // 11 t - 0.5 between control points floor of it and the next, with exact weights
            // (the texture unit's are 8-bit)
            const float t = a + (float)(1.0 / 22);
            const double xb = (double)t * 11 - 0.5;
            const double fl = std::floor(xb);
            const double fr = xb - fl;
            int i0 = (int)fl, i1 = i0 + 1;
            i0 = i0 < 0 ? 0 : (i0 > 10 ? 10 : i0);
            i1 = i1 < 0 ? 0 : (i1 > 10 ? 10 : i1);
            for (int c = 0; c < 3; c++)
                px[c] = (unsigned char)(255.f * (float)((1 - fr) * brewer[i0][c] + fr * brewer[i1][c]));
        }
    }
    return rgb;
}

bool write_rgb(const std::string& path, int w, int h, const std::vector<unsigned char>& rgb, std::string& err) {
    std::vector<unsigned char> b;
    if (ends_with(path, ".bmp")) {
        const size_t stride = ((size_t)w * 3 + 3) & ~(size_t)3;
        const uint32_t size = (uint32_t)(54 + stride * h);
        b.push_back('B');
        b.push_back('M');
        put32le(b, size);
        put32le(b, 0);
        put32le(b, 54);
        put32le(b, 40);
        put32le(b, (uint32_t)w);
        put32le(b, (uint32_t)h);  // bottom-up rows
        put16le(b, 1);
        put16le(b, 24);
        put32le(b, 0);
        put32le(b, (uint32_t)(stride * h));
        put32le(b, 2835);
        put32le(b, 2835);
        put32le(b, 0);
        put32le(b, 0);
        for (int y = h - 1; y >= 0; y--) {
            const size_t start = b.size();
            for (int x = 0; x < w; x++) {
                const unsigned char* px = &rgb[3 * ((size_t)y * w + x)];
                b.push_back(px[2]);
                b.push_back(px[1]);
                b.push_back(px[0]);
            }
            while (b.size() - start < stride) b.push_back(0);
        }
    } else if (ends_with(path, ".png")) {
        static const unsigned char sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
        b.assign(sig, sig + 8);
        auto chunk = [&b](const char* type, const std::vector<unsigned char>& data) {
            put32be(b, (uint32_t)data.size());
            const size_t t0 = b.size();
            b.insert(b.end(), type, type + 4);
            b.insert(b.end(), data.begin(), data.end());
            put32be(b, crc32(&b[t0], b.size() - t0) ^ 0xFFFFFFFFu);
        };
        std::vector<unsigned char> ihdr;
        put32be(ihdr, (uint32_t)w);
        put32be(ihdr, (uint32_t)h);
        ihdr.push_back(8);  // bit depth
        ihdr.push_back(2);  // RGB
        ihdr.push_back(0);
        ihdr.push_back(0);
        ihdr.push_back(0);
        chunk("IHDR", ihdr);
        std::vector<unsigned char> raw;  // filter byte 0 + row
        raw.reserve((size_t)h * (3 * w + 1));
        for (int y = 0; y < h; y++) {
            raw.push_back(0);
            raw.insert(raw.end(), rgb.begin() + 3 * (size_t)y * w, rgb.begin() + 3 * (size_t)(y + 1) * w);
        }
        std::vector<unsigned char> z = {0x78, 0x01};  // zlib header, stored blocks
        for (size_t off = 0; off < raw.size() || off == 0;) {
            const size_t n = std::min<size_t>(65535, raw.size() - off);
            const bool last = off + n >= raw.size();
            z.push_back(last ? 1 : 0);
            put16le(z, (uint16_t)n);
            put16le(z, (uint16_t)~n);
            z.insert(z.end(), raw.begin() + off, raw.begin() + off + n);
            off += n;
            if (last) break;
        }
        put32be(z, adler32(raw));
        chunk("IDAT", z);
        chunk("IEND", {});
    } else {
        err = path + ": image format not supported (use .bmp or .png, or no extension for ENVI)";
        return false;
    }
    std::ofstream o(path, std::ios::binary);
    if (!o || !o.write((const char*)b.data(), (std::streamsize)b.size())) {
        err = "cannot write " + path;
        return false;
    }
    return true;
}

bool write_scalar_image(const std::string& path, int w, int h, const std::vector<double>& v, bool positive,
                        Colormap cm, std::string& err) {
    // value of largest magnitude (first one on ties, like cublasIsamax)
    double m = 0;
    for (double x : v)
        if (std::fabs(x) > std::fabs(m)) m = x;
    const double vmin = positive ? 0.0 : -std::fabs(m), vmax = positive ? m : std::fabs(m);
    return write_rgb(path, w, h, colormap(v, vmin, vmax, cm), err);
}

}  // namespace bsio
