#pragma once
// Streaming BMP writer with the reference's interface (include/bmp_writer.h):
// one row at a time, top to bottom (negative height in the info header), an
// 8-bit palette file for one channel or a 24-bit file for RGB rows (written
// as BGR), rows zero-padded to 4 bytes.  Whole images exported through
// encode_*_to_bmp are written on the GPU by r2p_encode_bmp in the same layout.
#include <cstdint>
#include <cstdio>

struct BmpWriter {
    FILE* fp       = nullptr;
    int   width    = 0;
    int   stride   = 0;   // padded row bytes (multiple of 4)
    int   height   = 0;
    int   channels = 0;   // 1 or 3
    int   written  = 0;   // rows written so far
};

// Create/truncate `path` and write the headers (and the gray palette).
bool bmp_open(BmpWriter& w, const char* path, int width, int height, int channels);

// One row: `width` gray bytes, or `width * 3` RGB bytes.
bool bmp_write_row(BmpWriter& w, const uint8_t* src);

void bmp_close(BmpWriter& w);
