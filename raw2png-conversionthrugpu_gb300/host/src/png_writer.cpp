// png_writer.cpp -- PNG chunk writer (the reference's src/png_writer.cpp:33-125
// interface): signature, IHDR, IDAT chunks of at most chunk_ bytes, IEND.
#include "png_writer.h"

#include <algorithm>
#include <cstring>

#include "parallel_deflate.h"

static void be32(uint8_t* p, uint32_t v)
{
    p[0] = (uint8_t)(v >> 24); p[1] = (uint8_t)(v >> 16); p[2] = (uint8_t)(v >> 8); p[3] = (uint8_t)v;
}

PngWriter::~PngWriter()
{
    close();
}

bool PngWriter::open(const char* path, uint32_t width, uint32_t height, uint8_t bit_depth, PngColorType color_type)
{
    close();
    failed_ = false;
    file_ = std::fopen(path, "wb");
    if (!file_) {
        std::fprintf(stderr, "PngWriter: cannot create '%s'\n", path);
        return false;
    }
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (std::fwrite(sig, 1, 8, file_) != 8) failed_ = true;
    uint8_t ihdr[13];
    be32(ihdr, width);
    be32(ihdr + 4, height);
    ihdr[8] = bit_depth;
    ihdr[9] = (uint8_t)color_type;
    ihdr[10] = ihdr[11] = ihdr[12] = 0;   // deflate, adaptive filtering, no interlace
    write_chunk("IHDR", ihdr, 13);
    return !failed_;
}

void PngWriter::begin_idat()
{
    buf_.clear();
    buf_.reserve(chunk_);
}

void PngWriter::write_idat_bytes(const uint8_t* data, size_t size)
{
    while (size) {
        const size_t n = std::min(size, chunk_ - buf_.size());
        buf_.insert(buf_.end(), data, data + n);
        data += n;
        size -= n;
        if (buf_.size() == chunk_) flush_idat_buf();
    }
}

void PngWriter::flush_idat_buf()
{
    if (buf_.empty()) return;
    write_chunk("IDAT", buf_.data(), (uint32_t)buf_.size());
    buf_.clear();
}

void PngWriter::end_idat()
{
    flush_idat_buf();
}

void PngWriter::close()
{
    if (!file_) return;
    flush_idat_buf();
    write_chunk("IEND", nullptr, 0);
    if (std::fclose(file_) != 0) failed_ = true;
    file_ = nullptr;
}

void PngWriter::write_chunk(const char type[4], const uint8_t* data, uint32_t len)
{
    uint8_t h[8];
    be32(h, len);
    std::memcpy(h + 4, type, 4);
    unsigned long crc = crc32_update(0, h + 4, 4);
    if (len) crc = crc32_update(crc, data, len);
    uint8_t t[4];
    be32(t, (uint32_t)crc);
    if (std::fwrite(h, 1, 8, file_) != 8 || (len && std::fwrite(data, 1, len, file_) != len) ||
        std::fwrite(t, 1, 4, file_) != 4)
        failed_ = true;
}

bool write_png_rechunked(const char* path, const uint8_t* png, size_t len, size_t chunk_bytes)
{
    if (len < 8 + 25 + 12) return false;
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        std::fprintf(stderr, "cannot create '%s'\n", path);
        return false;
    }
    bool good = std::fwrite(png, 1, 8, f) == 8;
    size_t pos = 8;
    auto put_chunk = [&](const char* type, const uint8_t* d, uint32_t n) {
        uint8_t h[8], t[4];
        be32(h, n);
        std::memcpy(h + 4, type, 4);
        unsigned long crc = crc32_update(0, h + 4, 4);
        if (n) crc = crc32_update(crc, d, n);
        be32(t, (uint32_t)crc);
        good = good && std::fwrite(h, 1, 8, f) == 8 && (!n || std::fwrite(d, 1, n, f) == n) &&
               std::fwrite(t, 1, 4, f) == 4;
    };
    while (good && pos + 12 <= len) {
        const uint32_t n = ((uint32_t)png[pos] << 24) | ((uint32_t)png[pos + 1] << 16) | ((uint32_t)png[pos + 2] << 8) |
                           png[pos + 3];
        if (pos + 12 + (size_t)n > len) {
            good = false;
            break;
        }
        const uint8_t* type = png + pos + 4;
        const uint8_t* d = png + pos + 8;
        if (std::memcmp(type, "IDAT", 4) == 0) {
            for (size_t o = 0; o < n; o += chunk_bytes)
                put_chunk("IDAT", d + o, (uint32_t)std::min<size_t>(chunk_bytes, n - o));
        } else {
            good = std::fwrite(png + pos, 1, 12 + (size_t)n, f) == 12 + (size_t)n;
        }
        pos += 12 + (size_t)n;
    }
    if (std::fclose(f) != 0) good = false;
    return good && pos == len;
}
