// Stand-in for the absent external STIM header that the reference's
// scalarslice.h includes; only the enum names are needed to compile the
// reference's host sources for the oracle checks.
#ifndef BIMSIM_REF_STUB_STIM_COLORMAP_H
#define BIMSIM_REF_STUB_STIM_COLORMAP_H
namespace stim { enum colormapType { cmBrewer, cmGrayscale }; }
#endif
