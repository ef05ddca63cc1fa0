// dicom_loader.cpp -- minimal DICOM Part-10 reader for uncompressed pixel data.
//
// Header semantics follow the reference's DicomSource::open
// (src/dicom_loader.cpp:317-397) and frame extraction its load_frame
// (:511-531):
//   Rows, Columns, BitsAllocated (8|16), BitsStored, PixelRepresentation,
//   SamplesPerPixel (1..4), HighBit (default BitsStored-1 when absent),
//   NumberOfFrames (IS; absent or < 1 = 1 frame);
//   rescale applied only if a slope or intercept is present and differs from
//   the identity (|m-1| > 1e-9 or |b| > 1e-9);
//   window applied only if both centre and width are present and width > 0
//   (first value of a multi-valued DS);
//   frame i = bytes [i*F, (i+1)*F) of PixelData, F = rows*cols*samples*BitsAllocated/8.
// The file layout (preamble, "DICM", group 0002 in Explicit VR Little Endian,
// then the data set in the transfer syntax of (0002,0010)) is DICOM PS3.10
// section 7; element encodings are PS3.5 section 7.1.
#include "dicom_loader.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace {

constexpr const char* kImplicitLE = "1.2.840.10008.1.2";
constexpr const char* kExplicitLE = "1.2.840.10008.1.2.1";
constexpr uint32_t kUndefined = 0xFFFFFFFFu;

uint16_t le16(const uint8_t* p) { return (uint16_t)(p[0] | (p[1] << 8)); }
uint32_t le32(const uint8_t* p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24); }

// VRs whose explicit encoding has 2 reserved bytes and a 32-bit length (PS3.5 7.1.2)
bool long_form_vr(const uint8_t* vr)
{
    static const char* L[] = {"OB", "OD", "OF", "OL", "OV", "OW", "SQ", "UC", "UR", "UT", "UN", "SV", "UV"};
    for (const char* v : L)
        if (vr[0] == (uint8_t)v[0] && vr[1] == (uint8_t)v[1]) return true;
    return false;
}

struct Element {
    uint16_t group = 0, elem = 0;
    char vr[3] = {0, 0, 0};
    uint32_t len = 0;
    size_t value = 0;      // offset of the value
};

struct Parser {
    const uint8_t* p;
    size_t n;
    const char* err = nullptr;

    // Read one element header at pos (explicit or implicit VR); false at the end or on error.
    bool header(size_t& pos, bool explicit_vr, Element& e)
    {
        if (pos + 8 > n) return false;
        e.group = le16(p + pos);
        e.elem = le16(p + pos + 2);
        e.vr[0] = e.vr[1] = 0;
        // item and delimiter tags never carry a VR
        if (e.group == 0xFFFE) {
            e.len = le32(p + pos + 4);
            e.value = pos + 8;
            return true;
        }
        if (explicit_vr) {
            e.vr[0] = (char)p[pos + 4];
            e.vr[1] = (char)p[pos + 5];
            if (long_form_vr(p + pos + 4)) {
                if (pos + 12 > n) { err = "truncated element header"; return false; }
                e.len = le32(p + pos + 8);
                e.value = pos + 12;
            } else {
                e.len = le16(p + pos + 6);
                e.value = pos + 8;
            }
        } else {
            e.len = le32(p + pos + 4);
            e.value = pos + 8;
        }
        return true;
    }

    // Skip a value of undefined length (a sequence of items) starting at pos;
    // leaves pos after its sequence delimiter.
    bool skip_undefined(size_t& pos, bool explicit_vr, int depth)
    {
        if (depth > 64) { err = "sequences nested too deeply"; return false; }
        for (;;) {
            Element it;
            if (!header(pos, explicit_vr, it)) { err = err ? err : "unterminated sequence"; return false; }
            if (it.group == 0xFFFE && it.elem == 0xE0DD) {          // sequence delimiter
                pos = it.value;
                return true;
            }
            if (it.group != 0xFFFE || it.elem != 0xE000) { err = "malformed sequence"; return false; }
            if (it.len != kUndefined) {                              // item of known length
                if (it.value + (size_t)it.len > n) { err = "truncated item"; return false; }
                pos = it.value + it.len;
                continue;
            }
            pos = it.value;                                          // item of undefined length
            for (;;) {
                Element e;
                if (!header(pos, explicit_vr, e)) { err = err ? err : "unterminated item"; return false; }
                if (e.group == 0xFFFE && e.elem == 0xE00D) { pos = e.value; break; }
                if (e.len == kUndefined) {
                    pos = e.value;
                    if (!skip_undefined(pos, explicit_vr, depth + 1)) return false;
                } else {
                    if (e.value + (size_t)e.len > n) { err = "truncated element"; return false; }
                    pos = e.value + e.len;
                }
            }
        }
    }
};

std::string trimmed(const uint8_t* p, size_t len)
{
    size_t a = 0, b = len;
    while (a < b && (p[a] == ' ' || p[a] == 0)) a++;
    while (b > a && (p[b - 1] == ' ' || p[b - 1] == 0)) b--;
    return std::string(reinterpret_cast<const char*>(p + a), b - a);
}

// First value of a decimal/integer string (DS, IS); false if empty or not a number.
bool first_number(const uint8_t* p, size_t len, double& out)
{
    std::string s = trimmed(p, len);
    const size_t bs = s.find('\\');
    if (bs != std::string::npos) s = trimmed(reinterpret_cast<const uint8_t*>(s.data()), bs);
    if (s.empty()) return false;
    char* end = nullptr;
    const double v = std::strtod(s.c_str(), &end);
    if (end == s.c_str()) return false;
    out = v;
    return true;
}

}  // namespace

bool DicomSource::open(const char* path)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        std::fprintf(stderr, "DICOM: cannot open '%s'\n", path);
        return false;
    }
    std::fseek(f, 0, SEEK_END);
    const long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    file_.assign(sz > 0 ? (size_t)sz : 0, 0);
    const bool got = sz > 0 && std::fread(file_.data(), 1, file_.size(), f) == file_.size();
    std::fclose(f);
    if (!got) {
        std::fprintf(stderr, "DICOM: cannot read '%s'\n", path);
        return false;
    }
    Parser P{file_.data(), file_.size()};
    size_t pos = 0;
    transfer_syntax_.clear();
    if (file_.size() >= 132 && std::memcmp(file_.data() + 128, "DICM", 4) == 0) {
        pos = 132;
        // file meta information: group 0002, always Explicit VR Little Endian
        for (;;) {
            if (pos + 8 > file_.size() || le16(file_.data() + pos) != 0x0002) break;
            Element e;
            if (!P.header(pos, true, e) || e.len == kUndefined || e.value + (size_t)e.len > file_.size()) {
                std::fprintf(stderr, "DICOM: bad file meta information in '%s'\n", path);
                return false;
            }
            if (e.elem == 0x0010) transfer_syntax_ = trimmed(file_.data() + e.value, e.len);
            pos = e.value + e.len;
        }
    }
    bool explicit_vr;
    if (transfer_syntax_.empty()) {
        // no meta header: Implicit VR Little Endian unless the first element carries a VR
        const uint8_t* q = file_.data() + pos;
        explicit_vr = pos + 8 <= file_.size() && std::isupper(q[4]) && std::isupper(q[5]);
        transfer_syntax_ = explicit_vr ? kExplicitLE : kImplicitLE;
    } else if (transfer_syntax_ == kImplicitLE) {
        explicit_vr = false;
    } else if (transfer_syntax_ == kExplicitLE) {
        explicit_vr = true;
    } else {
        std::fprintf(stderr,
                     "DICOM: transfer syntax %s of '%s' is not supported by this reader "
                     "(uncompressed Implicit/Explicit VR Little Endian only)\n",
                     transfer_syntax_.c_str(), path);
        return false;
    }

    bool have_rows = false, have_cols = false, have_hb = false, have_slope = false, have_icpt = false;
    bool have_wc = false, have_ww = false;
    uint16_t rows = 0, cols = 0, bits_alloc = 16, bits_stored = 16, pixel_rep = 0, samples = 1, high_bit = 0;
    double slope = 1.0, intercept = 0.0, wc = 0.0, ww = 0.0, nf = 0.0;
    bool have_nf = false;
    photometric_.clear();
    px_off_ = px_len_ = 0;
    bool have_px = false;
    while (pos < file_.size()) {
        Element e;
        if (!P.header(pos, explicit_vr, e)) {
            if (P.err) {
                std::fprintf(stderr, "DICOM: %s in '%s'\n", P.err, path);
                return false;
            }
            break;
        }
        if (e.len == kUndefined) {
            if (e.group == 0x7FE0 && e.elem == 0x0010) {
                std::fprintf(stderr, "DICOM: encapsulated (compressed) pixel data in '%s' is not supported\n", path);
                return false;
            }
            pos = e.value;
            if (!P.skip_undefined(pos, explicit_vr, 0)) {
                std::fprintf(stderr, "DICOM: %s in '%s'\n", P.err, path);
                return false;
            }
            continue;
        }
        if (e.value + (size_t)e.len > file_.size()) {
            std::fprintf(stderr, "DICOM: element (%04X,%04X) runs past the end of '%s'\n", e.group, e.elem, path);
            return false;
        }
        const uint8_t* v = file_.data() + e.value;
        if (e.group == 0x0028) {
            const bool us = e.len >= 2;
            switch (e.elem) {
                case 0x0002: if (us) samples = le16(v); break;
                case 0x0004: photometric_ = trimmed(v, e.len); break;
                case 0x0008: have_nf = first_number(v, e.len, nf); break;
                case 0x0010: if (us) { rows = le16(v); have_rows = true; } break;
                case 0x0011: if (us) { cols = le16(v); have_cols = true; } break;
                case 0x0100: if (us) bits_alloc = le16(v); break;
                case 0x0101: if (us) bits_stored = le16(v); break;
                case 0x0102: if (us) { high_bit = le16(v); have_hb = true; } break;
                case 0x0103: if (us) pixel_rep = le16(v); break;
                case 0x1050: have_wc = first_number(v, e.len, wc); break;
                case 0x1051: have_ww = first_number(v, e.len, ww); break;
                case 0x1052: have_icpt = first_number(v, e.len, intercept); break;
                case 0x1053: have_slope = first_number(v, e.len, slope); break;
                default: break;
            }
        } else if (e.group == 0x7FE0 && e.elem == 0x0010) {
            px_off_ = e.value;
            px_len_ = e.len;
            have_px = true;
        }
        pos = e.value + e.len;
    }
    if (!have_hb) high_bit = (uint16_t)(bits_stored - 1);
    num_frames_ = 1;
    if (have_nf && nf >= 1.0) num_frames_ = (int)nf;
    if (!have_rows || !have_cols || rows == 0 || cols == 0) {
        std::fprintf(stderr, "DICOM: invalid dimensions %ux%u in '%s'\n", (unsigned)cols, (unsigned)rows, path);
        return false;
    }
    if (bits_alloc != 8 && bits_alloc != 16) {
        std::fprintf(stderr, "DICOM: unsupported BitsAllocated=%u in '%s'\n", (unsigned)bits_alloc, path);
        return false;
    }
    if (samples < 1 || samples > 4) {
        std::fprintf(stderr, "DICOM: unsupported SamplesPerPixel=%u in '%s'\n", (unsigned)samples, path);
        return false;
    }
    if (!have_px) {
        std::fprintf(stderr, "DICOM: pixel data element not found in '%s'\n", path);
        return false;
    }
    info_ = ImageInfo();
    info_.width = cols;
    info_.height = rows;
    info_.channels = samples;
    info_.bits_per_sample = bits_alloc;
    info_.bpp = samples * (bits_alloc / 8);
    params_ = DicomPixelParams();
    params_.bits_allocated = bits_alloc;
    params_.bits_stored = bits_stored;
    params_.high_bit = high_bit;
    params_.pixel_rep = pixel_rep;
    if ((have_slope || have_icpt) && (std::fabs(slope - 1.0) > 1e-9 || std::fabs(intercept) > 1e-9)) {
        params_.apply_rescale = 1;
        params_.rescale_slope = (float)slope;
        params_.rescale_intercept = (float)intercept;
    }
    if (have_wc && have_ww && ww > 0.0) {
        params_.apply_window = 1;
        params_.window_center = (float)wc;
        params_.window_width = (float)ww;
    }
    cur_frame_ = -1;
    next_row_ = 0;
    pixel_data_.clear();
    return true;
}

bool DicomSource::load_frame(int index)
{
    if (index < 0 || index >= num_frames_) {
        std::fprintf(stderr, "DICOM: frame index %d out of range [0,%d)\n", index, num_frames_);
        return false;
    }
    const size_t frame_bytes = (size_t)info_.height * info_.width * info_.channels * (size_t)(info_.bits_per_sample / 8);
    const size_t off = (size_t)index * frame_bytes;
    if (off + frame_bytes > px_len_) {
        std::fprintf(stderr, "DICOM: frame %d out of range -- need %zu bytes, pixel data has %zu\n", index,
                     off + frame_bytes, px_len_);
        return false;
    }
    pixel_data_.assign(file_.begin() + (ptrdiff_t)(px_off_ + off), file_.begin() + (ptrdiff_t)(px_off_ + off + frame_bytes));
    cur_frame_ = index;
    next_row_ = 0;
    return true;
}

int DicomSource::read_strip(uint8_t* out, int max_rows)
{
    const int h = (int)info_.height;
    if (cur_frame_ < 0) return -1;
    if (next_row_ >= h) return 0;
    const int rows = std::min(max_rows, h - next_row_);
    const size_t rb = (size_t)info_.width * info_.bpp;
    std::memcpy(out, pixel_data_.data() + (size_t)next_row_ * rb, (size_t)rows * rb);
    next_row_ += rows;
    return rows;
}
