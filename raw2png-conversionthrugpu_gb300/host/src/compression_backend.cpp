// compression_backend.cpp -- GpuDeflateBackend: the reference's
// CompressionBackend contract (include/compression_backend.h:33-78) on
// r2p_deflate_raw_device.
#include "compression_backend.h"

#include <chrono>
#include <cstring>

#include "host_common.h"

struct GpuDeflateBackendImpl {
    ParallelDeflateConfig cfg;
    r2p_engine* eng = nullptr;
    void* stream = nullptr;
    uint8_t* d_in = nullptr;
    size_t d_in_cap = 0;
    uint8_t* d_out = nullptr;       // stream bytes, then the 4-byte Adler-32
    size_t d_out_cap = 0;
    uint64_t* d_len = nullptr;
    uint8_t* h_out = nullptr;       // pinned download buffer
    size_t h_out_cap = 0;
    bool ok = false;

    ~GpuDeflateBackendImpl()
    {
        if (stream) r2p_stream_synchronize(stream);
        if (d_in) r2p_device_free(d_in);
        if (d_out) r2p_device_free(d_out);
        if (d_len) r2p_device_free(d_len);
        if (h_out) r2p_host_free_pinned(h_out);
        if (stream) r2p_stream_destroy(stream);
        if (eng) r2p_engine_destroy(eng);
    }

    static bool grow_device(uint8_t*& p, size_t& cap, size_t need)
    {
        if (need <= cap) return true;
        if (p) r2p_device_free(p);
        p = nullptr;
        cap = 0;
        void* q = nullptr;
        const size_t n = need + need / 4 + 4096;
        if (!r2p_host::ok(r2p_device_alloc(n, &q), "device alloc")) return false;
        p = static_cast<uint8_t*>(q);
        cap = n;
        return true;
    }

    bool grow_host(size_t need)
    {
        if (need <= h_out_cap) return true;
        if (h_out) r2p_host_free_pinned(h_out);
        h_out = nullptr;
        h_out_cap = 0;
        void* q = nullptr;
        const size_t n = need + need / 4 + 4096;
        if (!r2p_host::ok(r2p_host_alloc_pinned(n, &q), "pinned alloc")) return false;
        h_out = static_cast<uint8_t*>(q);
        h_out_cap = n;
        return true;
    }

    DeflateResult run(const uint8_t* d_src, size_t n, bool is_last, void* s)
    {
        DeflateResult r;
        r.strip_adler = 1;
        r.input_size = n;
        if (!ok || n == 0) {
            if (n) std::fprintf(stderr, "GpuDeflateBackend: engine unavailable\n");
            return r;
        }
        const auto t0 = std::chrono::steady_clock::now();
        const int level = cfg.zlib_level < 0 ? 0 : cfg.zlib_level > 9 ? 9 : cfg.zlib_level;
        const size_t cap = r2p_zlib_bound(n, level, 0);
        if (!grow_device(d_out, d_out_cap, cap) || !grow_host(cap)) return r;
        if (!r2p_host::ok(r2p_deflate_raw_device(eng, d_src, n, level, 0, is_last ? 1 : 0, d_out, d_out_cap, d_len, s),
                          "r2p_deflate_raw_device"))
            return r;
        uint64_t len = 0;
        if (!r2p_host::ok(r2p_memcpy(h_out, d_len, 8, s), "length download") ||
            !r2p_host::ok(r2p_stream_synchronize(s), "sync"))
            return r;
        std::memcpy(&len, h_out, 8);
        if (len >> 63) {
            std::fprintf(stderr, "GpuDeflateBackend: device error %s\n", r2p_status_string((int)(len & 0xFF)));
            return r;
        }
        if (!r2p_host::ok(r2p_memcpy(h_out, d_out, (size_t)len + 4, s), "stream download") ||
            !r2p_host::ok(r2p_stream_synchronize(s), "sync"))
            return r;
        r.data.assign(h_out, h_out + len);
        const uint8_t* a = h_out + len;
        r.strip_adler = ((unsigned long)a[0] << 24) | ((unsigned long)a[1] << 16) | ((unsigned long)a[2] << 8) | a[3];
        r.compress_us =
            std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::steady_clock::now() - t0).count();
        return r;
    }
};

GpuDeflateBackend::GpuDeflateBackend(const ParallelDeflateConfig& cfg, int device) : impl_(new GpuDeflateBackendImpl())
{
    impl_->cfg = cfg;
    void* q = nullptr;
    const auto t0 = std::chrono::steady_clock::now();
    impl_->ok = r2p_host::ok(r2p_engine_create(device, 0, &impl_->eng), "r2p_engine_create") &&
                r2p_host::ok(r2p_stream_create(&impl_->stream), "r2p_stream_create") &&
                r2p_host::ok(r2p_device_alloc(8, &q), "device alloc");
    impl_->d_len = static_cast<uint64_t*>(q);
    (void)t0;
}

GpuDeflateBackend::~GpuDeflateBackend() = default;

bool GpuDeflateBackend::ok() const
{
    return impl_->ok;
}

DeflateResult GpuDeflateBackend::compress_strip(const uint8_t* input, size_t input_size, bool is_last)
{
    GpuDeflateBackendImpl& I = *impl_;
    if (!I.ok || input_size == 0) return I.run(nullptr, input_size, is_last, I.stream);
    const auto t0 = std::chrono::steady_clock::now();
    if (!GpuDeflateBackendImpl::grow_device(I.d_in, I.d_in_cap, input_size) ||
        !r2p_host::ok(r2p_memcpy(I.d_in, input, input_size, I.stream), "strip upload")) {
        DeflateResult r;
        r.strip_adler = 1;
        r.input_size = input_size;
        return r;
    }
    DeflateResult r = I.run(I.d_in, input_size, is_last, I.stream);
    r.init_us = 0;
    r.compress_us =
        std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::steady_clock::now() - t0).count();
    return r;
}

DeflateResult GpuDeflateBackend::compress_strip_device(const uint8_t* d_input, size_t input_size, bool is_last,
                                                       void* stream)
{
    return impl_->run(d_input, input_size, is_last, stream ? stream : impl_->stream);
}

std::unique_ptr<CompressionBackend> make_compression_backend(const ParallelDeflateConfig& cfg, int num_threads)
{
    (void)num_threads;
    return std::unique_ptr<CompressionBackend>(new GpuDeflateBackend(cfg));
}
