// TEST INFRASTRUCTURE: stand-in for the absent external STIM header that the reference's
// scalarslice.h includes; the enum names compile the reference's host sources
// for the oracle checks, and gpu2image / cpu2image (its image writers) write
// nothing in the host-run build, whose checks record no image files.
#ifndef BIMSIM_REF_STUB_STIM_COLORMAP_H
#define BIMSIM_REF_STUB_STIM_COLORMAP_H
#include <string>
namespace stim {
enum colormapType { cmBrewer, cmGrayscale };
template <class T>
void gpu2image(T*, std::string, int, int, T, T, colormapType = cmBrewer) {}
template <class T>
void cpu2image(T*, std::string, int, int, T, T, colormapType = cmBrewer) {}
}  // namespace stim
#endif
