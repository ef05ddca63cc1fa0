#pragma once
// Strip DEFLATE results and the zlib framing helpers of the reference's
// include/parallel_deflate.h:18-80.  In this build the DEFLATE itself runs on
// the GPU (GpuDeflateBackend in compression_backend.h); deflate_strip, the
// reference's CPU zlib path, is not provided.
#include <cstddef>
#include <cstdint>
#include <vector>

struct ParallelDeflateConfig {
    int num_threads = 6;   // kept for source compatibility; the GPU backend ignores it
    int zlib_level  = 3;   // 0 = stored blocks, 1..9 = LZ77 + fixed Huffman (FLEVEL in the header)
};

struct DeflateResult {
    std::vector<uint8_t> data;           // raw DEFLATE bytes, no zlib header or trailer
    unsigned long        strip_adler;    // Adler-32 of the strip's input bytes
    size_t               input_size;     // input bytes
    long long            init_us     = 0;
    long long            compress_us = 0;
};

struct ParallelDeflateState {
    unsigned long running_adler = 1;
    bool          started       = false;
};

// Fold one strip's Adler-32 into the running value (strips in order).
void accum_adler(ParallelDeflateState& state, const DeflateResult& dr);

// 2-byte zlib header for a level (FLEVEL as zlib sets it) and the 4-byte
// big-endian Adler-32 trailer.
void zlib_header(int level, uint8_t out[2]);
void zlib_trailer(const ParallelDeflateState& state, uint8_t out[4]);

// Host checksums of small buffers (chunk headers and the like).
unsigned long adler32_of(const uint8_t* data, size_t len);
unsigned long crc32_of(const uint8_t* data, size_t len);
unsigned long crc32_update(unsigned long crc, const uint8_t* data, size_t len);

// GPU DEFLATE throughput on strip_bytes of synthetic filtered data at levels
// 0 and 1 (the reference's --bench-deflate, parallel_deflate.h:72-80).
void bench_deflate(size_t strip_bytes, int num_threads);
