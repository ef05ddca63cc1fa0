// ref_cpu_harness.cpp -- TEST INFRASTRUCTURE.
//
// Drives the reference's own CPU codec (src/parallel_deflate.cpp and
// src/png_writer.cpp, compiled unchanged from the reference tree by
// oracle/build_oracle.py) the way its legacy pipeline does
// (src/pipeline.cpp:217-284: deflate_strip per strip, accum_adler, zlib
// header/trailer, PngWriter), so the tests can check that oracle/port_cpu.cpp
// produces the same PNG bytes.
#include "parallel_deflate.h"
#include "png_writer.h"
#include "thread_pool.h"

#include <algorithm>

extern "C" int ref_cpu_png_from_filtered(const uint8_t* filtered, uint32_t width,
                                         uint32_t height, int row_bytes, int bit_depth,
                                         int channels, int level, int strip_height,
                                         int threads, const char* path)
{
    PngColorType ct = channels == 1 ? PngColorType::Gray
                    : channels == 4 ? PngColorType::RGBA : PngColorType::RGB;
    PngWriter w;
    if (!w.open(path, width, height, (uint8_t)bit_depth, ct)) return 0;
    w.begin_idat();
    uint8_t zh[2];
    zlib_header(level, zh);
    w.write_idat_bytes(zh, 2);
    ParallelDeflateConfig cfg;
    cfg.num_threads = threads;
    cfg.zlib_level = level;
    ThreadPool pool(threads);
    ParallelDeflateState st;
    const size_t frb = (size_t)row_bytes + 1;
    const int nstrips = ((int)height + strip_height - 1) / strip_height;
    for (int s = 0; s < nstrips; s++) {
        const int r0 = s * strip_height;
        const int rows = std::min(strip_height, (int)height - r0);
        DeflateResult dr = deflate_strip(filtered + (size_t)r0 * frb, (size_t)rows * frb, cfg,
                                         pool, s == nstrips - 1);
        accum_adler(st, dr);
        if (!dr.data.empty()) w.write_idat_bytes(dr.data.data(), dr.data.size());
    }
    uint8_t tr[4];
    zlib_trailer(st, tr);
    w.write_idat_bytes(tr, 4);
    w.end_idat();
    w.close();
    return 1;
}
