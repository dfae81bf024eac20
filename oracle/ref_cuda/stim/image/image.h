// TEST INFRASTRUCTURE: stand-in for the absent STIM library's image class, as
// far as the reference's microscope.cu uses it (LoadExtendedSource,
// microscope.cu:1258-1296: width(), height() and the value of channel 0 at
// column x, row y).  It reads 8-bit binary PGM (P5) files, rows from the top,
// which is what the checks write; any other file gives an empty image.
#ifndef BS_REF_STIM_IMAGE_H
#define BS_REF_STIM_IMAGE_H
#include <cctype>
#include <fstream>
#include <iterator>
#include <vector>

namespace stim {
template <class T>
class image {
    int w_ = 0, h_ = 0;
    std::vector<unsigned char> px_;

public:
    explicit image(const char* path) {
        std::ifstream in(path, std::ios::binary);
        std::vector<unsigned char> f((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
        if (f.size() < 2 || f[0] != 'P' || f[1] != '5') return;
        size_t pos = 2;
        int v[3];
        for (int k = 0; k < 3; k++) {
            while (pos < f.size() && std::isspace(f[pos])) pos++;
            if (pos >= f.size() || !std::isdigit(f[pos])) return;
            v[k] = 0;
            while (pos < f.size() && std::isdigit(f[pos])) v[k] = v[k] * 10 + (f[pos++] - '0');
        }
        pos++;  // the whitespace after maxval
        if (v[2] > 255 || f.size() < pos + (size_t)v[0] * v[1]) return;
        w_ = v[0];
        h_ = v[1];
        px_.assign(f.begin() + pos, f.begin() + pos + (size_t)w_ * h_);
    }
    int width() const { return w_; }
    int height() const { return h_; }
    T operator()(int x, int y, int) const { return (T)px_[(size_t)y * w_ + x]; }
};
}  // namespace stim
#endif
