// bmp_writer.cpp -- streaming BMP writer (the reference's BmpWriter
// interface, include/bmp_writer.h; file layout src/bmp_writer.cpp:36-131).
#include "bmp_writer.h"

#include <algorithm>
#include <cstring>
#include <vector>

namespace {

void le16(uint8_t* p, uint32_t v)
{
    p[0] = (uint8_t)v;
    p[1] = (uint8_t)(v >> 8);
}

void le32(uint8_t* p, uint32_t v)
{
    le16(p, v & 0xFFFFu);
    le16(p + 2, v >> 16);
}

}  // namespace

bool bmp_open(BmpWriter& w, const char* path, int width, int height, int channels)
{
    if ((channels != 1 && channels != 3) || width < 1 || height < 1) return false;
    w = BmpWriter{};
    w.width = width;
    w.height = height;
    w.channels = channels;
    w.stride = (width * channels + 3) & ~3;
    const uint32_t pix_off = 54u + (channels == 1 ? 1024u : 0u);
    const uint64_t size = pix_off + (uint64_t)w.stride * (uint64_t)height;
    if (size >= (1ull << 32)) return false;
    w.fp = std::fopen(path, "wb");
    if (!w.fp) return false;
    std::setvbuf(w.fp, nullptr, _IOFBF, (size_t)std::min<uint64_t>(std::max<uint64_t>(size, 65536), 4u << 20));
    uint8_t h[54] = {};
    h[0] = 'B';
    h[1] = 'M';
    le32(h + 2, (uint32_t)size);
    le32(h + 10, pix_off);
    le32(h + 14, 40u);                                  // BITMAPINFOHEADER
    le32(h + 18, (uint32_t)width);
    le32(h + 22, (uint32_t)(-height));                 // rows top to bottom
    le16(h + 26, 1u);
    le16(h + 28, channels == 1 ? 8u : 24u);
    le32(h + 46, channels == 1 ? 256u : 0u);
    bool good = std::fwrite(h, 1, sizeof(h), w.fp) == sizeof(h);
    if (good && channels == 1) {
        uint8_t pal[1024];
        for (int i = 0; i < 256; i++) {
            pal[4 * i] = pal[4 * i + 1] = pal[4 * i + 2] = (uint8_t)i;
            pal[4 * i + 3] = 0;
        }
        good = std::fwrite(pal, 1, sizeof(pal), w.fp) == sizeof(pal);
    }
    if (!good) bmp_close(w);
    return good;
}

bool bmp_write_row(BmpWriter& w, const uint8_t* src)
{
    if (!w.fp || w.written >= w.height) return false;
    thread_local std::vector<uint8_t> row;
    row.assign((size_t)w.stride, 0);
    if (w.channels == 1) {
        std::memcpy(row.data(), src, (size_t)w.width);
    } else {
        for (int x = 0; x < w.width; x++) {
            row[3 * x] = src[3 * x + 2];
            row[3 * x + 1] = src[3 * x + 1];
            row[3 * x + 2] = src[3 * x];
        }
    }
    if (std::fwrite(row.data(), 1, row.size(), w.fp) != row.size()) return false;
    w.written++;
    return true;
}

void bmp_close(BmpWriter& w)
{
    if (w.fp) std::fclose(w.fp);
    w.fp = nullptr;
}
