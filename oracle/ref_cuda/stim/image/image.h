// TEST INFRASTRUCTURE: stand-in for the absent STIM library's image class,
// enough for the reference's microscope.cu (LoadExtendedSource) to compile;
// the oracle checks never load an extended-source image through it.
#ifndef BS_REF_STIM_IMAGE_H
#define BS_REF_STIM_IMAGE_H
namespace stim {
template <class T>
class image {
public:
    explicit image(const char*) {}
    int width() const { return 0; }
    int height() const { return 0; }
    T operator()(int, int, int) const { return T(); }
};
}  // namespace stim
#endif
