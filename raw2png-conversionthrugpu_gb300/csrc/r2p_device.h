// r2p_device.h -- device-resident work descriptors shared by the kernels and
// the host engine.  One DevImage per image in HBM; kernels pull work items
// (row bands, DEFLATE blocks) that point back at their image.
#pragma once
#include <stdint.h>

#include "../../include/r2p.h"

namespace r2p {

// Resolved windowing transform applied while loading a row.
enum WinMode : int {
    W_COPY = 0,      // PNG-ordered bytes in, same bytes out
    W_SWAP16 = 1,    // LE 16-bit in, BE 16-bit out, no value change
    W_A2_LUT = 2,    // DICOM PS3.3 window via a per-image table (out depth = in depth)
    W_A2_DIRECT = 3, // same formula evaluated per sample (tables too large)
    W_Q15 = 4,       // 16-bit LE in, 8-bit out, Q15 linear map
    W_LUT8 = 5,      // 16-bit LE in, 8-bit out, FP32-built table
};

// Internal window request of the BMP export: the 16-bit DICOM to 8-bit gray
// formula of the reference's BMP path, resolved to a W_LUT8 table.
constexpr int kReqBmp8 = 0x100;

// Source of a BMP output byte.
enum BmpKind : int {
    BMP_BYTE = 0,     // 8-bit sample as is
    BMP_TAKE = 1,     // one byte of a 16-bit sample (bmp_off: 0 or 1)
    BMP_WINDOW = 2,   // 16-bit sample through the resolved 8-bit window (W_Q15 / W_LUT8)
};

// Largest table kept in shared memory by the filter kernel (bytes).
constexpr int kMaxSmemLut = 32768;

// Window+filter kernel an image's rows go to (DevImage::fpath).
enum FiltPath : int {
    kFiltSmem = 0,    // k_window_filter: TMA-staged tiles in shared memory
    kFiltReg = 1,     // k_window_filter_reg: a row across a group of warps' registers
    kFiltRows = 2,    // k_filter_rows: one warp per row, table built by k_window_lut
};

struct DevImage {
    // geometry
    uint32_t width, height;
    int32_t channels, ib, ob;       // input / output bytes per sample
    int32_t rb, bpp;                // filtered row bytes (without type byte), bytes per pixel
    int32_t in_pitch;               // raw bytes per row
    int32_t fpath;                  // FiltPath: the kernel that filters this image's rows
    uint64_t filt_bytes;            // height * (rb + 1)
    // window request and its resolution (filled on the device)
    int32_t req_mode;               // R2P_WINDOW_*
    int32_t in_be;                  // 16-bit input already big-endian (PNG order)
    r2p_dicom_params dp;
    int32_t mode;                   // WinMode
    int32_t qa, qb;                 // Q15 coefficients
    int32_t lut_shift;
    uint32_t lut_mask;
    int32_t lut_entries, lut_esize; // entries, bytes per entry (1 or 2)
    uint8_t* lut;                   // device table space (lut_cap bytes)
    // buffers
    const uint8_t* raw;
    uint8_t* filt;
    const uint8_t* prior;           // windowed row above row 0 (rb bytes) or null
    uint8_t* last_row;              // receives the windowed last row (rb bytes) or null
    // DEFLATE / PNG
    int32_t level;
    int32_t block_size;             // filtered bytes per DEFLATE block
    int32_t hash_bits;              // LZ77 hash table bits (9 or 10; other values mean 10)
    int32_t nblocks;
    uint32_t blk0;                  // first global block index of this image
    int32_t out_kind;               // 0 = PNG file, 1 = bare zlib stream, 2 = raw DEFLATE
    int32_t open_end;               // 1: no BFINAL; the last block ends with an empty stored block
    int32_t prefix;                 // bytes before the DEFLATE stream (kPngPrefix or 2)
    uint8_t* png;                   // output buffer
    uint64_t png_cap;
    uint64_t* png_len;              // device word receiving the PNG size (or error bit)
    uint32_t idat_crc_partial;      // scratch
    int32_t status;                 // device-side error code (0 = ok)
    // BMP export (png = the file buffer)
    int32_t bmp_kind, bmp_off;      // BmpKind, byte of a 16-bit sample taken by BMP_TAKE
    int32_t bmp_oc, bmp_stride;     // output channels (1 or 3), padded row bytes
    uint32_t bmp_pix_off, bmp_size; // pixel array offset, file bytes
};

// A band of consecutive rows of one image, filtered by one CTA.
struct BandItem {
    uint32_t img;
    uint32_t r0, r1;
};

// Per-DEFLATE-block results written by the block kernels.
struct BlockOut {
    uint32_t img;          // image index
    uint32_t in_off;       // offset of the block in the filtered stream
    uint32_t in_len;       // filtered bytes in the block
    uint32_t out_len;      // compressed bytes (byte aligned)
    uint32_t crc;          // crc32 of the compressed bytes
    uint32_t s1;           // sum of input bytes
    uint64_t s2;           // sum of (in_len - i) * d_i over the block
    uint64_t out_off;      // offset of the block in the DEFLATE stream (set by k_finish)
};

// PNG prefix: signature (8) + IHDR chunk (25) + IDAT length/type (8) + zlib header (2)
constexpr int kPngPrefix = 8 + 25 + 8 + 2;
// PNG suffix: Adler-32 (4) + IDAT CRC (4) + IEND chunk (12)
constexpr int kPngSuffix = 4 + 4 + 12;
// Stored-block header bytes (BFINAL/BTYPE byte, LEN, NLEN)
constexpr int kStoredHdr = 5;
// Default DEFLATE block payload: 64 KiB minus 16 so a block fits one stored
// block (<= 65535 bytes) and every block starts 16-byte aligned.
constexpr int kBlock64 = 65520;
constexpr int kBlock32 = 32752;
// levels of the x^(8n) power table (1024 entries each)
constexpr int kXpowLevels = 4;

}  // namespace r2p
