// host_common.h -- shared helpers of the C++ host layer (not installed).
#pragma once
#include <cstdio>

#include "../../../include/r2p.h"

namespace r2p_host {

// Report a failed r2p call on stderr; true when rc is R2P_OK.
inline bool ok(int rc, const char* what)
{
    if (rc == R2P_OK) return true;
    std::fprintf(stderr, "%s failed: %s (%s)\n", what, r2p_status_string(rc), r2p_last_error());
    return false;
}

// (channels, bytes per sample) for a pixel size: filtering only depends on
// the bytes per pixel, windowing also on the sample size.
inline bool split_bpp(int bpp, int bytes_per_sample, int& channels, int& bps)
{
    if (bytes_per_sample == 1 || bytes_per_sample == 2) {
        if (bpp % bytes_per_sample) return false;
        channels = bpp / bytes_per_sample;
        bps = bytes_per_sample;
        return channels == 1 || channels == 3 || channels == 4;
    }
    switch (bpp) {
        case 1: channels = 1; bps = 1; return true;
        case 2: channels = 1; bps = 2; return true;
        case 3: channels = 3; bps = 1; return true;
        case 4: channels = 4; bps = 1; return true;
        case 6: channels = 3; bps = 2; return true;
        case 8: channels = 4; bps = 2; return true;
        default: return false;
    }
}

// The calling thread's engine on a device (created on first use, kept for
// the thread's lifetime -- the reference's per-thread context cache,
// src/pipeline.cpp:1522-1560).
r2p_engine* thread_engine(int device);

// BMP file of host pixels through r2p_encode_bmp on the calling thread's
// engine, written to `out`.
bool write_bmp(const r2p_image& img, const void* pixels, const char* out, int device);

}  // namespace r2p_host
