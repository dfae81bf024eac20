// Stand-in for the absent external STIM header that the reference's
// scalarslice.h includes; the enum names compile the reference's host sources
// for the oracle checks, and gpu2image (image output, never called by those
// checks) lets scalarslice.cu compile for the host-run build.
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
