#pragma once
// Strip-by-strip image source (the reference's ImageSource,
// include/image_source.h:7-17): the pipeline's injection point.
#include <cstdint>

#include "dicom_params.h"
#include "image_loader.h"

struct ImageSource {
    virtual ~ImageSource() = default;
    virtual const ImageInfo& info() const = 0;
    // Read up to max_rows rows into out; returns rows read, 0 at the end, < 0 on error.
    virtual int read_strip(uint8_t* out, int max_rows) = 0;
    // Non-null only for DICOM sources: selects the DICOM window transform.
    virtual const DicomPixelParams* dicom_params() const { return nullptr; }
    virtual int num_frames() const { return 1; }
};

// An image already in host memory (rows of info.width * info.bpp bytes).
// The buffer is borrowed and must outlive the source.
struct MemorySource : ImageSource {
    ImageInfo        info_;
    DicomPixelParams params_;
    bool             has_params_ = false;
    const uint8_t*   pixels_     = nullptr;
    int              next_row_   = 0;

    MemorySource() = default;
    MemorySource(const ImageInfo& info, const uint8_t* pixels, const DicomPixelParams* params = nullptr)
        : info_(info), pixels_(pixels)
    {
        if (params) {
            params_ = *params;
            has_params_ = true;
        }
    }
    const ImageInfo& info() const override { return info_; }
    const DicomPixelParams* dicom_params() const override { return has_params_ ? &params_ : nullptr; }
    int read_strip(uint8_t* out, int max_rows) override;
};

// A TIFF file as a strip source (the reference's TiffSource, src/pipeline.cpp).
struct TiffSource : ImageSource {
    TiffSource() = default;
    ~TiffSource() override;
    TiffSource(const TiffSource&) = delete;
    TiffSource& operator=(const TiffSource&) = delete;
    bool open(const char* path);
    const ImageInfo& info() const override { return info_; }
    int read_strip(uint8_t* out, int max_rows) override;

private:
    struct TiffReader* r_ = nullptr;
    ImageInfo info_;
};
