#pragma once
// "Compress one filtered strip into raw DEFLATE plus its Adler-32": the
// reference's CompressionBackend interface (include/compression_backend.h:33-78).
// GpuDeflateBackend keeps its contract -- the concatenation of all strips is
// one valid DEFLATE stream with BFINAL only on the last strip -- by emitting
// byte-aligned, independently coded blocks (r2p_deflate_raw_device): a
// non-final strip ends on an empty stored block, the final strip sets BFINAL.
#include <cstddef>
#include <cstdint>
#include <memory>

#include "parallel_deflate.h"

class CompressionBackend {
public:
    virtual ~CompressionBackend() = default;
    virtual DeflateResult compress_strip(const uint8_t* input, size_t input_size, bool is_last) = 0;
    virtual const char* name() const = 0;
};

struct GpuDeflateBackendImpl;

class GpuDeflateBackend : public CompressionBackend {
public:
    explicit GpuDeflateBackend(const ParallelDeflateConfig& cfg, int device = 0);
    ~GpuDeflateBackend() override;
    GpuDeflateBackend(const GpuDeflateBackend&) = delete;
    GpuDeflateBackend& operator=(const GpuDeflateBackend&) = delete;

    // Host input (pageable or pinned).
    DeflateResult compress_strip(const uint8_t* input, size_t input_size, bool is_last) override;
    // Device-resident input (e.g. gpu_filter_device_output), ordered after
    // work already queued on `stream` (a cudaStream_t; null = the backend's own).
    DeflateResult compress_strip_device(const uint8_t* d_input, size_t input_size, bool is_last,
                                        void* stream = nullptr);
    const char* name() const override { return "r2p LZ77 + fixed Huffman (GPU)"; }
    bool ok() const;   // false if the GPU engine could not be created

private:
    std::unique_ptr<GpuDeflateBackendImpl> impl_;
};

// Every configuration gets the GPU backend: there is no CPU fallback.
std::unique_ptr<CompressionBackend> make_compression_backend(const ParallelDeflateConfig& cfg, int num_threads);
