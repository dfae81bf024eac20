// Image files of the `bimsim` command line: source images for --extended-source
// and colour-mapped outputs for file names with an image extension.
//
// The reference reads and writes images through the STIM library (OpenCV
// underneath), which this build does not have; these are self-written readers
// and writers for uncompressed formats.
#pragma once

#include <string>
#include <vector>

namespace bsio {

// First channel of an 8-bit image, row 0 at the top (what
// stim::image<unsigned char>(x, y, 0) returns in LoadExtendedSource,
// microscope.cu:1257-1296).  Reads binary or ASCII PGM (P5/P2, 8-bit) and
// uncompressed BMP (8-bit palette, 24- or 32-bit).  For colour pixels the
// first channel is red.
bool read_channel0(const std::string& path, int& width, int& height, std::vector<unsigned char>& out,
                   std::string& err);

enum Colormap { CM_BREWER = 0, CM_GRAY = 1 };

// Colour-map values v[y * width + x] on [vmin, vmax] (rts/visualization/colormap.h,
// applyGrayscale / applyBrewer) into 8-bit RGB, row 0 at the top.
std::vector<unsigned char> colormap(const std::vector<double>& v, double vmin, double vmax, Colormap cm);

// Write 8-bit RGB pixels as .bmp (24-bit, uncompressed) or .png (8-bit RGB,
// stored deflate blocks); the extension decides.  Other extensions fail.
bool write_rgb(const std::string& path, int width, int height, const std::vector<unsigned char>& rgb,
               std::string& err);

// scalarslice::toImage(filename, positive, cmap) (scalarslice.cu:94-144): the
// range is [0, m] (positive) or [-|m|, |m|], m the value of largest magnitude.
bool write_scalar_image(const std::string& path, int width, int height, const std::vector<double>& v, bool positive,
                        Colormap cm, std::string& err);

}  // namespace bsio
