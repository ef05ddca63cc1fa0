// image_loader.cpp -- minimal TIFF reader (TIFF 6.0 baseline: header, first
// IFD, uncompressed strips) with the output conventions of the reference's
// libtiff-based loader (src/image_loader.cpp:122-214): 16-bit samples
// big-endian (PNG order), MINISWHITE inverted.
#include "image_loader.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "image_source.h"

struct TiffReader {
    std::vector<uint8_t> file;
    ImageInfo info;
    bool be = false;                 // file byte order "MM"
    bool invert = false;             // PhotometricInterpretation 0 (MINISWHITE)
    uint32_t rows_per_strip = 0;
    std::vector<uint64_t> strip_off, strip_len;
    uint32_t next_row = 0;
};

namespace {

uint32_t rd(const TiffReader& r, size_t off, int bytes)
{
    uint32_t v = 0;
    for (int i = 0; i < bytes; i++) {
        const uint32_t b = r.file[off + i];
        v |= r.be ? b << (8 * (bytes - 1 - i)) : b << (8 * i);
    }
    return v;
}

// Values of one IFD entry (SHORT or LONG), read from the entry or its offset.
bool entry_values(const TiffReader& r, size_t e, std::vector<uint32_t>& out)
{
    const uint32_t type = rd(r, e + 2, 2), count = rd(r, e + 4, 4);
    const int sz = type == 3 ? 2 : type == 4 ? 4 : 0;
    if (!sz || count == 0 || count > (1u << 24)) return false;
    size_t at = e + 8;
    if ((uint64_t)sz * count > 4) {
        at = rd(r, e + 8, 4);
        if (at + (uint64_t)sz * count > r.file.size()) return false;
    }
    out.resize(count);
    for (uint32_t i = 0; i < count; i++) out[i] = rd(r, at + (size_t)i * sz, sz);
    return true;
}

}  // namespace

TiffReader* tiff_open(const char* path, ImageInfo& info_out)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        std::fprintf(stderr, "TIFF: cannot open '%s'\n", path);
        return nullptr;
    }
    TiffReader* r = new TiffReader();
    std::fseek(f, 0, SEEK_END);
    const long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    r->file.resize(sz > 0 ? (size_t)sz : 0);
    const bool got = sz > 8 && std::fread(r->file.data(), 1, r->file.size(), f) == r->file.size();
    std::fclose(f);
    auto fail = [&](const char* why) -> TiffReader* {
        std::fprintf(stderr, "TIFF: %s in '%s'\n", why, path);
        delete r;
        return nullptr;
    };
    if (!got) return fail("cannot read the file");
    if (std::memcmp(r->file.data(), "II*\0", 4) == 0) r->be = false;
    else if (std::memcmp(r->file.data(), "MM\0*", 4) == 0) r->be = true;
    else return fail("not a TIFF header (BigTIFF is not supported)");
    const size_t ifd = rd(*r, 4, 4);
    if (ifd + 2 > r->file.size()) return fail("IFD offset out of range");
    const uint32_t n = rd(*r, ifd, 2);
    if (ifd + 2 + 12ull * n > r->file.size()) return fail("IFD runs past the end");
    uint32_t w = 0, h = 0, spp = 1, comp = 1, photo = 1, planar = 1;
    std::vector<uint32_t> bps{1}, offs, lens;
    bool tiled = false;
    r->rows_per_strip = 0xFFFFFFFFu;
    for (uint32_t i = 0; i < n; i++) {
        const size_t e = ifd + 2 + 12 * (size_t)i;
        const uint32_t tag = rd(*r, e, 2);
        std::vector<uint32_t> v;
        switch (tag) {
            case 256: if (entry_values(*r, e, v)) w = v[0]; break;
            case 257: if (entry_values(*r, e, v)) h = v[0]; break;
            case 258: if (entry_values(*r, e, v)) bps = v; break;
            case 259: if (entry_values(*r, e, v)) comp = v[0]; break;
            case 262: if (entry_values(*r, e, v)) photo = v[0]; break;
            case 273: entry_values(*r, e, offs); break;
            case 277: if (entry_values(*r, e, v)) spp = v[0]; break;
            case 278: if (entry_values(*r, e, v)) r->rows_per_strip = v[0]; break;
            case 279: entry_values(*r, e, lens); break;
            case 284: if (entry_values(*r, e, v)) planar = v[0]; break;
            case 322: case 323: case 324: case 325: tiled = true; break;
            default: break;
        }
    }
    if (w == 0 || h == 0) return fail("missing image size");
    if (tiled) return fail("tiled TIFF is not supported by this reader");
    if (comp != 1) return fail("compressed TIFF is not supported by this reader");
    if (planar != 1 && spp > 1) return fail("planar TIFF is not supported by this reader");
    if (spp != 1 && spp != 3 && spp != 4) return fail("samples per pixel must be 1, 3 or 4");
    const uint32_t b = bps[0];
    for (uint32_t x : bps)
        if (x != b) return fail("mixed bits per sample");
    if (b != 8 && b != 16) return fail("bits per sample must be 8 or 16");
    if (offs.empty() || offs.size() != lens.size()) return fail("missing strip offsets");
    r->rows_per_strip = std::min(r->rows_per_strip, h);
    const uint64_t row_b = (uint64_t)w * spp * (b / 8);
    const uint64_t nstrips = (h + r->rows_per_strip - 1) / r->rows_per_strip;
    if (offs.size() < nstrips) return fail("too few strips");
    for (uint64_t k = 0; k < nstrips; k++) {
        const uint64_t rows = std::min<uint64_t>(r->rows_per_strip, h - k * r->rows_per_strip);
        if (lens[k] < rows * row_b || (uint64_t)offs[k] + rows * row_b > r->file.size())
            return fail("strip data runs past the end");
        r->strip_off.push_back(offs[k]);
        r->strip_len.push_back(lens[k]);
    }
    r->invert = (photo == 0);
    r->info.width = w;
    r->info.height = h;
    r->info.channels = (int)spp;
    r->info.bits_per_sample = (int)b;
    r->info.bpp = (int)(spp * (b / 8));
    info_out = r->info;
    return r;
}

int tiff_read_strip(TiffReader* r, uint8_t* out, int strip_height)
{
    if (!r || r->next_row >= r->info.height) return 0;
    const int n = std::min(strip_height, (int)(r->info.height - r->next_row));
    const size_t row_b = (size_t)r->info.width * r->info.bpp;
    for (int i = 0; i < n; i++) {
        const uint32_t y = r->next_row + (uint32_t)i;
        const uint32_t k = y / r->rows_per_strip, in = y % r->rows_per_strip;
        std::memcpy(out + (size_t)i * row_b, r->file.data() + r->strip_off[k] + (size_t)in * row_b, row_b);
    }
    const size_t total = (size_t)n * row_b;
    if (r->info.bits_per_sample == 16 && !r->be)
        for (size_t k = 0; k + 1 < total; k += 2) std::swap(out[k], out[k + 1]);   // to PNG (big-endian) order
    if (r->invert)
        for (size_t k = 0; k < total; k++) out[k] ^= 0xFF;
    r->next_row += (uint32_t)n;
    return n;
}

void tiff_close(TiffReader* r)
{
    delete r;
}

TiffSource::~TiffSource()
{
    tiff_close(r_);
}

bool TiffSource::open(const char* path)
{
    tiff_close(r_);
    r_ = tiff_open(path, info_);
    return r_ != nullptr;
}

int TiffSource::read_strip(uint8_t* out, int max_rows)
{
    return r_ ? tiff_read_strip(r_, out, max_rows) : -1;
}
