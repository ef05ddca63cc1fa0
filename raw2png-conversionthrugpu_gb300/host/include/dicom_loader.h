#pragma once
// Minimal DICOM Part-10 reader for uncompressed pixel data (Implicit VR Little
// Endian, Explicit VR Little Endian) with the reference's DicomSource
// interface (include/dicom_loader.h:23-44).  The reference decodes through
// DCMTK and OpenJPEG, which also cover JPEG, JPEG-LS, RLE and JPEG 2000
// transfer syntaxes; this reader refuses those with a message.
#include <cstdint>
#include <string>
#include <vector>

#include "image_source.h"

struct DicomSource : ImageSource {
    ImageInfo            info_;
    DicomPixelParams     params_;
    std::vector<uint8_t> pixel_data_;     // current frame (16-bit samples little-endian)
    int                  next_row_   = 0;
    int                  num_frames_ = 1;
    int                  cur_frame_  = -1;
    std::string          transfer_syntax_;
    std::string          photometric_;

    DicomSource() = default;
    ~DicomSource() override = default;

    // Parse the header and locate the pixel data; no pixel copy yet.
    bool open(const char* path);
    // Copy frame `index` (0-based) into pixel_data_ and rewind the strip cursor.
    bool load_frame(int index);

    const ImageInfo& info() const override { return info_; }
    const DicomPixelParams* dicom_params() const override { return &params_; }
    int num_frames() const override { return num_frames_; }
    int read_strip(uint8_t* out, int max_rows) override;

private:
    std::vector<uint8_t> file_;
    size_t               px_off_ = 0, px_len_ = 0;
};
