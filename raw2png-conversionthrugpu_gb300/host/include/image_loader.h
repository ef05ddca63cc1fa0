#pragma once
// Decoded-image description shared by every image source (the reference's
// ImageInfo, include/image_loader.h:7-13), and the TIFF reader.  Sources
// deliver samples in PNG byte order (16-bit big-endian) unless they carry
// DICOM parameters, whose 16-bit samples are little-endian as stored in the
// file.  Camera-RAW decoding (LibRaw in the reference) is not part of this
// build.
#include <cstdint>

struct ImageInfo {
    uint32_t width           = 0;
    uint32_t height          = 0;
    int      channels        = 0;   // 1 gray, 3 RGB, 4 RGBA
    int      bits_per_sample = 0;   // 8 or 16
    int      bpp             = 0;   // bytes per pixel = channels * bits_per_sample / 8
};

// TIFF reader with the reference's interface (include/image_loader.h:15-24):
// open, then read strips top to bottom; 16-bit samples come out big-endian
// and MINISWHITE images inverted, as the reference's loader delivers them
// (src/image_loader.cpp:122-214).  This reader handles uncompressed,
// strip-organised, interleaved (chunky) TIFF in either byte order with 8- or
// 16-bit samples, 1, 3 or 4 per pixel; tiled, planar or compressed files
// (libtiff's job in the reference) are refused with a message.
struct TiffReader;
TiffReader* tiff_open(const char* path, ImageInfo& info_out);
int         tiff_read_strip(TiffReader* r, uint8_t* out, int strip_height);
void        tiff_close(TiffReader* r);
