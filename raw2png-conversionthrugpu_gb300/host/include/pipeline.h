#pragma once
// Encode entry points with the reference's interface (include/pipeline.h:8-122).
// A whole image is encoded by one r2p_encode_png call (window, filter, DEFLATE,
// checksums and PNG container on the GPU); with strip_pipeline set, or for
// images beyond one call's limit, strips run through gpu_filter_* and
// GpuDeflateBackend into a PngWriter, as the reference's pipeline does.
// BMP export (encode_*_to_bmp) writes the whole file on the GPU through
// r2p_encode_bmp, in the reference's BMP layout and pixel rules.  Camera-RAW
// input is not part of this build and reports an error.
#include <cstdint>

struct ImageSource;

enum class ExportFormat { PNG, BMP };

struct PipelineConfig {
    int  strip_height    = 0;      // rows per strip; 0 = auto (1024)
    int  deflate_threads = 6;      // accepted for compatibility; DEFLATE runs on the GPU
    int  deflate_level   = 3;      // 0 = stored, 1 = LZ77 + fixed Huffman, 2..9 = dynamic Huffman
    int  frame           = -1;     // DICOM frame, -1 = first
    bool verbose         = false;
    int  gpu_streams     = 0;      // frames in flight for multi-frame export; 0 = auto (4)
    bool use_gpu_deflate = true;   // always on: DEFLATE has no CPU path here
    bool use_gpu_lz77    = true;   // level >= 1 uses the GPU LZ77 match finder
    bool gpu_lz77_debug  = false;
    ExportFormat format  = ExportFormat::PNG;
    // not in the reference
    bool strip_pipeline  = false;  // force the strip-wise path
    int  idat_chunk      = 0;      // IDAT chunk payload bytes (0 = one IDAT for the whole stream)
    int  device          = 0;      // GPU ordinal
};

bool encode_tiff_to_png(const char* input_path, const char* output_path, const PipelineConfig& cfg);
bool encode_raw_to_png(const char* input_path, const char* output_path, const PipelineConfig& cfg);
bool encode_dicom_to_png(const char* input_path, const char* output_path, const PipelineConfig& cfg);
bool encode_dicom_all_frames_to_png(const char* input_path, const char* output_dir, const PipelineConfig& cfg);

void pipeline_reset_gpu_batch_stats();
void pipeline_record_file_times(long long dicom_ms, long long total_ms);
void pipeline_print_gpu_batch_summary(int total_files, int succeeded, double total_wall_s,
                                      long long sum_file_batch_ms, int num_workers);

bool encode_dicom_to_bmp(const char* input_path, const char* output_path, const PipelineConfig& cfg);
bool encode_tiff_to_bmp(const char* input_path, const char* output_path, const PipelineConfig& cfg);
bool encode_raw_to_bmp(const char* input_path, const char* output_path, const PipelineConfig& cfg);

bool encode_source_to_png(ImageSource& src, const char* output_path, const PipelineConfig& cfg);
bool encode_source_to_bmp(ImageSource& src, const char* output_path);
