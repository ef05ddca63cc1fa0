#pragma once
// PNG file writer for a caller-supplied zlib stream, with the reference's
// interface (include/png_writer.h:7-57): IHDR on open, IDAT bytes split into
// chunks of at most 32 KiB (or another size), IEND on close.
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <vector>

enum class PngColorType : uint8_t { Gray = 0, RGB = 2, GrayA = 4, RGBA = 6 };

class PngWriter {
public:
    PngWriter() = default;
    ~PngWriter();
    bool open(const char* path, uint32_t width, uint32_t height, uint8_t bit_depth, PngColorType color_type);
    void begin_idat();
    void write_idat_bytes(const uint8_t* data, size_t size);
    void end_idat();
    void close();
    bool is_open() const { return file_ != nullptr; }
    bool failed() const { return failed_; }
    // IDAT chunk payload size (default 32768, the reference's); call before begin_idat.
    void set_idat_chunk(size_t bytes) { chunk_ = bytes ? bytes : 32768; }

private:
    void write_chunk(const char type[4], const uint8_t* data, uint32_t len);
    void flush_idat_buf();
    FILE*                file_   = nullptr;
    std::vector<uint8_t> buf_;
    size_t               chunk_  = 32768;
    bool                 failed_ = false;
};

// Split a finished single-IDAT PNG (as r2p_encode_png writes it) into IDAT
// chunks of at most chunk_bytes and write it to path.
bool write_png_rechunked(const char* path, const uint8_t* png, size_t len, size_t chunk_bytes);
