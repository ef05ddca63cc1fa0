#pragma once
// Decoded-image description shared by every image source (the reference's
// ImageInfo, include/image_loader.h:7-13).  TIFF and camera-RAW decoders are
// not part of this build; sources deliver samples in PNG byte order
// (16-bit big-endian) unless they carry DICOM parameters, whose 16-bit
// samples are little-endian as stored in the file.
#include <cstdint>

struct ImageInfo {
    uint32_t width           = 0;
    uint32_t height          = 0;
    int      channels        = 0;   // 1 gray, 3 RGB, 4 RGBA
    int      bits_per_sample = 0;   // 8 or 16
    int      bpp             = 0;   // bytes per pixel = channels * bits_per_sample / 8
};
