// ref_colormap.cpp -- TEST INFRASTRUCTURE.  Part of the host-run build of the
// reference (oracle/_ref/libref_sim_*.so, `make -C oracle ref-sim`): runs the
// reference's own colour-map path rts::gpu2cpu of rts/visualization/colormap.h
// (its kernels applyBrewer, with the Brewer texture bound by initBrewer: 11
// control points, normalised coordinates, linear filtering, clamp; and
// applyGrayscale) on the CUDA stand-ins of oracle/ref_cuda.  The recipe
// compiles this file as the tail of that header, which it pipes through the
// launch-syntax sed with __CUDACC__ defined over the header (its CUDA part);
// no copy of the header is written.  The reference's detector images go
// through STIM's gpu2image, which this image does not have; this header is
// the colour map the reference tree itself carries.  Only
// tests/golden/make_ref_sim_golden.py loads it.

// declared by colormap.h for its image writer, which the checks never call
void qt_buffer2image(unsigned char*, std::string, unsigned int, unsigned int) {}

extern "C" {

// The colour-mapped RGB bytes of n values on [vmin, vmax]: cm 0 Brewer, 1 grayscale
// (rts::gpu2cpu, as gpu2image calls it before writing the file).
int ref_colormap(float* v, int n, float vmin, float vmax, int cm, unsigned char* rgb) {
    rts::gpu2cpu<float>(v, rgb, (unsigned)n, vmin, vmax, cm == 0 ? rts::cmBrewer : rts::cmGrayscale);
    return 0;
}

}  // extern "C"
