// compat_check.cpp -- drives the reference-facing C++ interfaces the way the
// reference's pipeline does (src/pipeline.cpp run_one and its filter pool):
// strips go round-robin to two GpuFilterContexts, the true previous row is
// threaded through gpu_filter_copy_prior_row_to_host, even strips use the
// host entry point and odd strips the device one; the filtered strips are
// then compressed by make_compression_backend()->compress_strip into one zlib
// stream.  Writes the filtered bytes and the zlib stream for the test to check.
//
// usage: compat_check raw.bin width height bpp strip level dicom(0|1) filtered.out zlib.out
//   dicom=1: 16-bit LE CT samples, 12 bits stored, rescale -1024, window 40/400
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "compression_backend.h"
#include "gpu_filter.h"
#include "r2p.h"

static std::vector<uint8_t> slurp(const char* p)
{
    std::vector<uint8_t> v;
    FILE* f = std::fopen(p, "rb");
    if (!f) return v;
    std::fseek(f, 0, SEEK_END);
    v.resize((size_t)std::ftell(f));
    std::fseek(f, 0, SEEK_SET);
    if (std::fread(v.data(), 1, v.size(), f) != v.size()) v.clear();
    std::fclose(f);
    return v;
}

int main(int argc, char** argv)
{
    if (argc != 10) return 2;
    const int W = std::atoi(argv[2]), H = std::atoi(argv[3]), bpp = std::atoi(argv[4]);
    const int strip = std::atoi(argv[5]), level = std::atoi(argv[6]), dicom = std::atoi(argv[7]);
    std::vector<uint8_t> raw = slurp(argv[1]);
    const size_t rb = (size_t)W * bpp;
    if (raw.size() != rb * H) return 3;
    DicomPixelParams p;
    p.bits_allocated = 16; p.bits_stored = 12; p.high_bit = 11; p.pixel_rep = 0;
    p.apply_rescale = 1; p.rescale_slope = 1.f; p.rescale_intercept = -1024.f;
    p.apply_window = 1; p.window_center = 40.f; p.window_width = 400.f;
    const DicomPixelParams* dp = dicom ? &p : nullptr;

    GpuFilterContext* ctx[2] = {gpu_filter_create(W, bpp, strip), gpu_filter_create(W, bpp, strip)};
    if (!ctx[0] || !ctx[1]) return 4;
    void* d_strip = nullptr;
    if (r2p_device_alloc(rb * strip, &d_strip) != R2P_OK) return 5;
    uint8_t* prior = gpu_filter_alloc_pinned(rb);
    std::vector<uint8_t> filtered;
    std::vector<size_t> strip_sizes;
    for (int s = 0, r = 0; r < H; s++, r += strip) {
        const int n = H - r < strip ? H - r : strip;
        GpuFilterContext* c = ctx[s & 1];
        const uint8_t* h_prior = s == 0 ? nullptr : prior;   // the row above, from the other context
        const uint8_t* out;
        if (s == 0) gpu_filter_reset(c);
        GpuTimings t;
        if ((s & 1) == 0) {
            out = gpu_filter_process_from_host(c, raw.data() + (size_t)r * rb, h_prior, n, &t, dp);
        } else {
            void* d_prior = nullptr;
            r2p_device_alloc(rb, &d_prior);
            r2p_memcpy(d_prior, prior, rb, nullptr);
            r2p_memcpy(d_strip, raw.data() + (size_t)r * rb, (size_t)n * rb, nullptr);
            r2p_stream_synchronize(nullptr);
            out = gpu_filter_process_from_device(c, static_cast<uint8_t*>(d_strip), static_cast<uint8_t*>(d_prior), n,
                                                 &t, dp);
            r2p_device_free(d_prior);
        }
        if (!out) return 6;
        if (t.kernel_ms < 0.f) return 7;
        const size_t sz = gpu_filter_output_size(c, n);
        filtered.insert(filtered.end(), out, out + sz);
        strip_sizes.push_back(sz);
        gpu_filter_copy_prior_row_to_host(c, prior);
    }
    ParallelDeflateConfig cfg;
    cfg.zlib_level = level;
    std::unique_ptr<CompressionBackend> be = make_compression_backend(cfg, 4);
    std::vector<uint8_t> z(2);
    zlib_header(level, z.data());
    ParallelDeflateState st;
    size_t off = 0;
    for (size_t i = 0; i < strip_sizes.size(); i++) {
        DeflateResult dr = be->compress_strip(filtered.data() + off, strip_sizes[i], i + 1 == strip_sizes.size());
        if (dr.data.empty() || dr.input_size != strip_sizes[i]) return 8;
        if (dr.strip_adler != adler32_of(filtered.data() + off, strip_sizes[i])) return 9;
        accum_adler(st, dr);
        z.insert(z.end(), dr.data.begin(), dr.data.end());
        off += strip_sizes[i];
    }
    uint8_t trl[4];
    zlib_trailer(st, trl);
    z.insert(z.end(), trl, trl + 4);
    FILE* f = std::fopen(argv[8], "wb");
    std::fwrite(filtered.data(), 1, filtered.size(), f);
    std::fclose(f);
    f = std::fopen(argv[9], "wb");
    std::fwrite(z.data(), 1, z.size(), f);
    std::fclose(f);
    std::printf("%s: %zu strips, %zu filtered bytes -> %zu zlib bytes\n", be->name(), strip_sizes.size(),
                filtered.size(), z.size());
    gpu_filter_free_pinned(prior);
    r2p_device_free(d_strip);
    gpu_filter_destroy(ctx[0]);
    gpu_filter_destroy(ctx[1]);
    return 0;
}
