// Volume file IO of the terminal programs: MetaImage (.mha with the voxels after
// the header, or .mhd with a separate data file), uncompressed, and headerless
// raw float32.  The reference reads and writes through ITK (ITKImage::read /
// write); these formats are the ones its scripts exchange with it.
#ifndef TGVDCT_METAIMAGE_HPP
#define TGVDCT_METAIMAGE_HPP

#include <cstdint>
#include <string>
#include <vector>

namespace tgvdct_io {

struct Volume {
    uint32_t width = 0, height = 0, depth = 0;
    double spacing[3] = {1.0, 1.0, 1.0};
    double origin[3] = {0.0, 0.0, 0.0};
    std::vector<float> voxels;  // x fastest: z*width*height + y*width + x
    size_t count() const { return (size_t)width * height * depth; }
};

// Reads a .mha / .mhd file (element types MET_UCHAR, MET_CHAR, MET_USHORT,
// MET_SHORT, MET_UINT, MET_INT, MET_FLOAT, MET_DOUBLE; 2 or 3 dimensions; either
// byte order; no compression) and converts the voxels to float.  Throws
// std::runtime_error with the reason on failure.
Volume read_metaimage(const std::string& path);

// Writes float voxels: a .mhd path gets its data in a .raw file beside it, any
// other path a single .mha file.
void write_metaimage(const std::string& path, const Volume& v);

// Headerless little-endian float32, x fastest.
Volume read_raw(const std::string& path, uint32_t width, uint32_t height, uint32_t depth);
void write_raw(const std::string& path, const Volume& v);

// read_raw when raw_dims is "WxHxD" (or "WxH"), else read_metaimage.
Volume read_volume(const std::string& path, const std::string& raw_dims);
// write_raw for a path ending in .raw, else write_metaimage.
void write_volume(const std::string& path, const Volume& v);

}  // namespace tgvdct_io

#endif
