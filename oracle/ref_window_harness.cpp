// ref_window_harness.cpp -- TEST INFRASTRUCTURE.
//
// Compiles the reference's own batch translation unit (src/batch_processor.cpp,
// included unchanged from the reference tree through the include path that
// oracle/build_oracle.py sets) and exports its three static 16->8-bit
// windowing functions with C linkage so the tests can generate golden vectors
// from the reference itself:
//   try_apply_linear_window  src/batch_processor.cpp:202-266 (Q15 fast path)
//   build_dicom16_lut        src/batch_processor.cpp:100-147 (FP32 LUT)
//   apply_dicom16_lut        src/batch_processor.cpp:157-185
// The decoder, loader and pipeline entry points that the translation unit
// references are stubbed below; none of them is ever called.
#include "batch_processor.cpp"

struct DicomFileImpl {};
DicomSource::DicomSource() {}
DicomSource::~DicomSource() {}
bool DicomSource::open(const char*) { return false; }
bool DicomSource::load_frame(int) { return false; }
int  DicomSource::read_strip(uint8_t*, int) { return 0; }

bool ends_with_ci(const char*, const char*) { return false; }
bool is_tiff_file(const char*) { return false; }
bool is_raw_file(const char*) { return false; }
bool is_dicom_file(const char*) { return false; }

TiffReader* tiff_open(const char*, ImageInfo&) { return nullptr; }
int         tiff_read_strip(TiffReader*, uint8_t*, int) { return 0; }
void        tiff_close(TiffReader*) {}
RawReader*  raw_open(const char*, ImageInfo&) { return nullptr; }
int         raw_read_strip(RawReader*, uint8_t*, int) { return 0; }
void        raw_close(RawReader*) {}

bool encode_tiff_to_png(const char*, const char*, const PipelineConfig&) { return false; }
bool encode_raw_to_png(const char*, const char*, const PipelineConfig&) { return false; }
bool encode_dicom_to_png(const char*, const char*, const PipelineConfig&) { return false; }
bool encode_dicom_all_frames_to_png(const char*, const char*, const PipelineConfig&) { return false; }
bool encode_dicom_to_bmp(const char*, const char*, const PipelineConfig&) { return false; }
bool encode_tiff_to_bmp(const char*, const char*, const PipelineConfig&) { return false; }
bool encode_raw_to_bmp(const char*, const char*, const PipelineConfig&) { return false; }
bool encode_source_to_png(ImageSource&, const char*, const PipelineConfig&) { return false; }
bool encode_source_to_bmp(ImageSource&, const char*) { return false; }
void pipeline_reset_gpu_batch_stats() {}
void pipeline_record_file_times(long long, long long) {}
void pipeline_print_gpu_batch_summary(int, int, double, long long, int) {}

extern "C" {

int ref_try_apply_linear_window(const uint8_t* src_le, uint8_t* dst8, int n,
                                const DicomPixelParams* p)
{
    return try_apply_linear_window(src_le, dst8, n, *p) ? 1 : 0;
}

void ref_build_dicom16_lut(uint8_t* lut, const DicomPixelParams* p, int lut_size)
{
    build_dicom16_lut(lut, *p, lut_size);
}

void ref_apply_dicom16_lut(const uint8_t* src_le, uint8_t* dst8, size_t n,
                           const uint8_t* lut, int shift, uint16_t mask16)
{
    apply_dicom16_lut(src_le, dst8, n, lut, shift, mask16);
}

// The dispatch of src/batch_processor.cpp:397-409, built from the reference's
// own functions (LUT cache bypassed: it only memoises the same table).
int ref_window8(const uint8_t* src_le, uint8_t* dst8, int n, const DicomPixelParams* p)
{
    if (try_apply_linear_window(src_le, dst8, n, *p)) return 1;
    const int lut_size = 1 << p->bits_stored;
    std::vector<uint8_t> lut((size_t)lut_size);
    build_dicom16_lut(lut.data(), *p, lut_size);
    apply_dicom16_lut(src_le, dst8, (size_t)n, lut.data(),
                      p->high_bit - p->bits_stored + 1, (uint16_t)(lut_size - 1));
    return 2;
}

}  // extern "C"
