#pragma once
// Strip-wise window + adaptive PNG filter on the GPU, with the reference's
// interface (include/gpu_filter.h:10-90) so its callers link unchanged.
// No CUDA types appear here; the work runs through r2p_window_filter_device_ex
// (fused window + filter kernel) of the r2p C ABI.
//
// Behaviour kept from the reference (src/gpu_filter.cu:313-520):
//  - the context owns its device input, prior-row and output buffers, its
//    pinned host output (unless device_output_only) and its stream;
//  - the prior row of each strip is the windowed last row of the strip this
//    context processed before (zeros after create/reset), unless the caller
//    passes one;
//  - the returned host pointer belongs to the context and stays valid until
//    the next call.
// Differences: errors are reported on stderr and as a null return (the
// reference exits the process); bpp must be 1, 2, 3, 4, 6 or 8.
#include <cstddef>
#include <cstdint>

#include "dicom_params.h"

struct GpuFilterContext;

// Per-call GPU timing (milliseconds, CUDA events), filled when non-null.
struct GpuTimings {
    float h2d_ms    = 0.f;
    float kernel_ms = 0.f;
    float d2h_ms    = 0.f;
};

GpuFilterContext* gpu_filter_create(int width, int bpp, int strip_height, bool device_output_only = false);
void              gpu_filter_destroy(GpuFilterContext* ctx);

uint8_t* gpu_filter_alloc_pinned(size_t bytes);
void     gpu_filter_free_pinned(uint8_t* ptr);

// Zero the prior row: the next strip is the first row band of a new image.
void gpu_filter_reset(GpuFilterContext* ctx);

// Filter actual_rows rows already in device memory.  dicom != null applies the
// DICOM transform (16-bit samples little-endian in, big-endian out).
const uint8_t* gpu_filter_process_from_device(GpuFilterContext* ctx, const uint8_t* d_input,
                                              const uint8_t* d_prior_row, int actual_rows,
                                              GpuTimings* timings = nullptr,
                                              const DicomPixelParams* dicom = nullptr);

// Same, uploading h_input (and h_prior_row if given) from host memory.  With
// device_output_only the result stays on the device (gpu_filter_device_output)
// and nullptr is returned; gpu_filter_copy_prior_row_to_host then serves as
// the synchronisation point, as in the reference.
const uint8_t* gpu_filter_process_from_host(GpuFilterContext* ctx, const uint8_t* h_input,
                                            const uint8_t* h_prior_row, int actual_rows,
                                            GpuTimings* timings = nullptr,
                                            const DicomPixelParams* dicom = nullptr,
                                            bool device_output_only = false);

// actual_rows * (width * bpp + 1): one filter-type byte per row.
size_t gpu_filter_output_size(const GpuFilterContext* ctx, int actual_rows);

// Device copy of the most recent strip's filtered bytes.
const uint8_t* gpu_filter_device_output(const GpuFilterContext* ctx);

// Copy the carried prior row (windowed last row of the last strip, width*bpp
// bytes) to host memory; waits for the context's stream.
void gpu_filter_copy_prior_row_to_host(const GpuFilterContext* ctx, uint8_t* h_dst);

// Not in the reference: the context's stream (a cudaStream_t), for callers
// that order their own device work after the filter without a host wait.
void* gpu_filter_stream(const GpuFilterContext* ctx);
