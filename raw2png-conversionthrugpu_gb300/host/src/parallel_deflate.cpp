// parallel_deflate.cpp -- zlib framing and host checksums for strip streams
// (include/parallel_deflate.h of the reference, :60-80; src/parallel_deflate.cpp:197-246),
// plus a GPU DEFLATE benchmark in place of the CPU one.
#include "parallel_deflate.h"

#include <chrono>
#include <cstdio>
#include <vector>

#include "host_common.h"

void accum_adler(ParallelDeflateState& state, const DeflateResult& dr)
{
    // Adler-32 of A||B from adler(A), adler(B) and |B|; adler("") = 1 keeps
    // the first strip's value.
    state.running_adler = r2p_adler32_combine((uint32_t)state.running_adler, (uint32_t)dr.strip_adler,
                                              (uint64_t)dr.input_size);
    state.started = true;
}

void zlib_header(int level, uint8_t out[2])
{
    // CMF 0x78 (deflate, 32 KiB window); FLG carries FLEVEL the way zlib sets
    // it for each level, with FCHECK making CMF*256+FLG a multiple of 31.
    out[0] = 0x78;
    out[1] = level == 1 ? 0x01 : (level >= 2 && level <= 5) ? 0x5E : (level >= 6 && level <= 7) ? 0x9C : 0xDA;
}

void zlib_trailer(const ParallelDeflateState& state, uint8_t out[4])
{
    const uint32_t a = (uint32_t)state.running_adler;
    out[0] = (uint8_t)(a >> 24);
    out[1] = (uint8_t)(a >> 16);
    out[2] = (uint8_t)(a >> 8);
    out[3] = (uint8_t)a;
}

unsigned long adler32_of(const uint8_t* data, size_t len)
{
    // RFC 1950: s1 = 1 + sum d, s2 = sum of the running s1, both mod 65521;
    // 5552 bytes is the longest run that cannot overflow 32 bits.
    uint32_t s1 = 1, s2 = 0;
    while (len) {
        size_t n = len < 5552 ? len : 5552;
        len -= n;
        while (n--) {
            s1 += *data++;
            s2 += s1;
        }
        s1 %= 65521u;
        s2 %= 65521u;
    }
    return ((unsigned long)s2 << 16) | s1;
}

static const uint32_t* crc_table()
{
    static uint32_t t[256];
    static bool init = [] {
        for (uint32_t n = 0; n < 256; n++) {
            uint32_t c = n;
            for (int k = 0; k < 8; k++) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[n] = c;
        }
        return true;
    }();
    (void)init;
    return t;
}

unsigned long crc32_update(unsigned long crc, const uint8_t* data, size_t len)
{
    const uint32_t* t = crc_table();
    uint32_t c = (uint32_t)crc ^ 0xFFFFFFFFu;
    for (size_t i = 0; i < len; i++) c = t[(c ^ data[i]) & 0xFF] ^ (c >> 8);
    return c ^ 0xFFFFFFFFu;
}

unsigned long crc32_of(const uint8_t* data, size_t len)
{
    return crc32_update(0, data, len);
}

void bench_deflate(size_t strip_bytes, int num_threads)
{
    (void)num_threads;
    if (strip_bytes == 0) return;
    r2p_engine* eng = r2p_host::thread_engine(0);
    if (!eng) return;
    // synthetic filtered rows: a filter-type byte, then small residuals with
    // runs, as adaptive filtering leaves them
    std::vector<uint8_t> h(strip_bytes);
    uint32_t x = 12345u;
    for (size_t i = 0; i < strip_bytes; i++) {
        x = x * 1664525u + 1013904223u;
        const uint32_t r = x >> 24;
        h[i] = (i % 4097 == 0) ? 4 : (r < 160 ? 0 : (uint8_t)(r & 7));
    }
    void *d_in = nullptr, *d_out = nullptr, *d_len = nullptr, *s = nullptr, *e0 = nullptr, *e1 = nullptr;
    const size_t cap = r2p_zlib_bound(strip_bytes, 0, 0);
    if (!r2p_host::ok(r2p_device_alloc(strip_bytes, &d_in), "alloc") ||
        !r2p_host::ok(r2p_device_alloc(cap, &d_out), "alloc") || !r2p_host::ok(r2p_device_alloc(8, &d_len), "alloc") ||
        !r2p_host::ok(r2p_stream_create(&s), "stream") || !r2p_host::ok(r2p_event_create(&e0), "event") ||
        !r2p_host::ok(r2p_event_create(&e1), "event"))
        return;
    r2p_memcpy(d_in, h.data(), strip_bytes, s);
    std::printf("GPU DEFLATE benchmark: %zu bytes of synthetic filtered data\n", strip_bytes);
    std::printf("  level   MB/s      ratio\n");
    for (int level : {0, 1}) {
        const int reps = 20;
        for (int i = 0; i < 3; i++)
            r2p_zlib_compress_device(eng, d_in, strip_bytes, level, 0, d_out, cap, (uint64_t*)d_len, s);
        r2p_event_record(e0, s);
        for (int i = 0; i < reps; i++)
            r2p_zlib_compress_device(eng, d_in, strip_bytes, level, 0, d_out, cap, (uint64_t*)d_len, s);
        r2p_event_record(e1, s);
        uint64_t len = 0;
        r2p_memcpy(&len, d_len, 8, s);
        r2p_stream_synchronize(s);
        float ms = 0.f;
        r2p_event_elapsed_ms(e0, e1, &ms);
        const double mbs = (double)strip_bytes * reps / (ms * 1e-3) / 1e6;
        std::printf("  %5d  %8.1f  %8.3f\n", level, mbs, (double)len / (double)strip_bytes);
    }
    r2p_event_destroy(e0);
    r2p_event_destroy(e1);
    r2p_stream_destroy(s);
    r2p_device_free(d_in);
    r2p_device_free(d_out);
    r2p_device_free(d_len);
}
