// pipeline.cpp -- encode entry points (the reference's include/pipeline.h and
// src/pipeline.cpp:1571-1760, 2058-2061) on the r2p C ABI.
//
// Whole-image path: the source's strips are read into one pinned buffer and a
// single r2p_encode_png call windows, filters, compresses, checksums and
// assembles the PNG on the GPU; the host writes the file.
// Strip path (PipelineConfig::strip_pipeline, or an image past one call's
// limit): per strip, gpu_filter_process_from_host (window + filter, prior row
// carried on the device) then GpuDeflateBackend::compress_strip_device on the
// same stream, into a PngWriter -- the structure of the reference's run_one.
#include "pipeline.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <mutex>
#include <thread>
#include <vector>

#include "bounded_queue.h"
#include "compression_backend.h"
#include "dicom_loader.h"
#include "gpu_filter.h"
#include "host_common.h"
#include "image_source.h"
#include "png_writer.h"

namespace r2p_host {

r2p_engine* thread_engine(int device)
{
    struct Holder {
        r2p_engine* e = nullptr;
        int dev = -1;
        ~Holder()
        {
            if (e) r2p_engine_destroy(e);
        }
    };
    thread_local Holder h;
    if (h.e && h.dev == device) return h.e;
    if (h.e) r2p_engine_destroy(h.e);
    h.e = nullptr;
    if (!ok(r2p_engine_create(device, 0, &h.e), "r2p_engine_create")) return nullptr;
    h.dev = device;
    return h.e;
}

// Grow-only pinned buffer owned by the calling thread.
struct PinnedScratch {
    void* p = nullptr;
    size_t cap = 0;
    ~PinnedScratch()
    {
        if (p) r2p_host_free_pinned(p);
    }
    uint8_t* get(size_t n)
    {
        if (n > cap) {
            if (p) r2p_host_free_pinned(p);
            p = nullptr;
            cap = 0;
            if (!ok(r2p_host_alloc_pinned(n, &p), "pinned alloc")) return nullptr;
            cap = n;
        }
        return static_cast<uint8_t*>(p);
    }
};

bool write_bmp(const r2p_image& img, const void* pixels, const char* out, int device)
{
    thread_local PinnedScratch bmp_buf;
    const size_t size = r2p_bmp_bound(&img);
    if (size == 0) {
        std::fprintf(stderr, "BMP: unsupported image %ux%u, %d channel(s), %d byte(s) per sample\n", img.width,
                     img.height, img.channels, img.bytes_per_sample);
        return false;
    }
    uint8_t* bmp = bmp_buf.get(size);
    r2p_engine* eng = thread_engine(device);
    if (!bmp || !eng) return false;
    size_t len = 0;
    if (!ok(r2p_encode_bmp(eng, &img, pixels, bmp, size, &len), "r2p_encode_bmp")) return false;
    FILE* f = std::fopen(out, "wb");
    if (!f) {
        std::fprintf(stderr, "Cannot create BMP: %s\n", out);
        return false;
    }
    const bool good = std::fwrite(bmp, 1, len, f) == len;
    return (std::fclose(f) == 0) && good;
}

}  // namespace r2p_host

using namespace r2p_host;

int MemorySource::read_strip(uint8_t* out, int max_rows)
{
    const int h = (int)info_.height;
    if (!pixels_) return -1;
    if (next_row_ >= h) return 0;
    const int rows = std::min(max_rows, h - next_row_);
    const size_t rb = (size_t)info_.width * info_.bpp;
    std::memcpy(out, pixels_ + (size_t)next_row_ * rb, (size_t)rows * rb);
    next_row_ += rows;
    return rows;
}

namespace {

int strip_rows(const PipelineConfig& cfg)
{
    return cfg.strip_height > 0 ? cfg.strip_height : 1024;
}

int clamp_level(int l)
{
    return l < 0 ? 0 : l > 9 ? 9 : l;
}

// r2p_image for a source: DICOM sources get the DICOM transform at their own
// depth (src/gpu_filter.cu:71-162), others are taken as PNG-ordered samples.
bool describe(const ImageSource& src, const PipelineConfig& cfg, r2p_image& img)
{
    const ImageInfo& info = src.info();
    std::memset(&img, 0, sizeof(img));
    if (info.width == 0 || info.height == 0 || (info.bits_per_sample != 8 && info.bits_per_sample != 16) ||
        (info.channels != 1 && info.channels != 3 && info.channels != 4) ||
        info.bpp != info.channels * info.bits_per_sample / 8) {
        std::fprintf(stderr, "encode: unsupported image %ux%u, %d channel(s), %d bits\n", info.width, info.height,
                     info.channels, info.bits_per_sample);
        return false;
    }
    img.width = info.width;
    img.height = info.height;
    img.channels = info.channels;
    img.bytes_per_sample = info.bits_per_sample / 8;
    const DicomPixelParams* d = src.dicom_params();
    if (d) {
        img.window_mode = R2P_WINDOW_DICOM16;
        std::memcpy(&img.dicom, d, sizeof(img.dicom));
    } else {
        img.window_mode = R2P_WINDOW_NONE;
    }
    img.level = clamp_level(cfg.deflate_level);
    img.strip_height = strip_rows(cfg);
    return true;
}

PngColorType color_type(int channels)
{
    return channels == 1 ? PngColorType::Gray : channels == 3 ? PngColorType::RGB : PngColorType::RGBA;
}

bool read_all(ImageSource& src, uint8_t* dst, int strip, size_t row_bytes)
{
    const int h = (int)src.info().height;
    for (int r = 0; r < h;) {
        const int n = src.read_strip(dst + (size_t)r * row_bytes, std::min(strip, h - r));
        if (n <= 0) {
            std::fprintf(stderr, "encode: source ended at row %d of %d\n", r, h);
            return false;
        }
        r += n;
    }
    return true;
}

bool encode_whole(ImageSource& src, const char* out, const PipelineConfig& cfg, const r2p_image& img)
{
    thread_local PinnedScratch raw_buf, png_buf;
    const ImageInfo& info = src.info();
    const size_t rb = (size_t)info.width * info.bpp;
    const size_t bound = r2p_png_bound(&img);
    uint8_t* raw = raw_buf.get(rb * info.height);
    uint8_t* png = png_buf.get(bound);
    r2p_engine* eng = thread_engine(cfg.device);
    if (!raw || !png || !eng || !read_all(src, raw, strip_rows(cfg), rb)) return false;
    size_t len = 0;
    if (!ok(r2p_encode_png(eng, &img, raw, png, bound, &len), "r2p_encode_png")) return false;
    if (cfg.idat_chunk > 0) return write_png_rechunked(out, png, len, (size_t)cfg.idat_chunk);
    FILE* f = std::fopen(out, "wb");
    if (!f) {
        std::fprintf(stderr, "cannot create '%s'\n", out);
        return false;
    }
    const bool good = std::fwrite(png, 1, len, f) == len;
    return (std::fclose(f) == 0) && good;
}

// Strip path as three overlapped stages, like the reference's modern
// pipeline (src/pipeline.cpp:445-853): a reader thread fills a ring of pinned
// strip buffers from the source, this thread runs each strip through the GPU
// filter (prior row carried on the device) and GpuDeflateBackend, and a
// writer thread appends the compressed strips to the PNG's IDAT chunks
// (modern_writer_stage, :826-848), so source reads and file writes overlap
// the GPU work.
bool encode_strips(ImageSource& src, const char* out, const PipelineConfig& cfg, const r2p_image& img)
{
    constexpr int kRing = 3;                      // strip buffers in flight
    const ImageInfo& info = src.info();
    const int H = (int)info.height;
    const int strip = strip_rows(cfg);
    const size_t rb = (size_t)info.width * info.bpp;
    const size_t slot_bytes = (size_t)strip * rb;
    const DicomPixelParams* dicom = src.dicom_params();
    GpuFilterContext* ctx = gpu_filter_create((int)info.width, info.bpp, strip, true);
    if (!ctx) return false;
    ParallelDeflateConfig dc;
    dc.num_threads = cfg.deflate_threads;
    dc.zlib_level = img.level;
    GpuDeflateBackend backend(dc, cfg.device);
    thread_local PinnedScratch ring_buf;
    uint8_t* ring = ring_buf.get(kRing * slot_bytes);
    PngWriter w;
    if (cfg.idat_chunk > 0) w.set_idat_chunk((size_t)cfg.idat_chunk);
    bool good = ring && backend.ok() &&
                w.open(out, info.width, info.height, (uint8_t)info.bits_per_sample, color_type(info.channels));
    if (good) {
        w.begin_idat();
        uint8_t hdr[2];
        zlib_header(img.level, hdr);
        w.write_idat_bytes(hdr, 2);
        struct StripIn {
            int slot = 0, rows = 0;
        };
        BoundedQueue<int> q_free(kRing);
        BoundedQueue<StripIn> q_in(kRing);
        BoundedQueue<std::vector<uint8_t>> q_out(kRing + 1);
        for (int k = 0; k < kRing; k++) q_free.push(k);
        std::atomic<bool> failed{false};
        std::thread reader([&] {
            for (int r = 0; r < H;) {
                int slot;
                if (!q_free.pop(slot)) break;
                const int n = src.read_strip(ring + slot * slot_bytes, std::min(strip, H - r));
                if (n <= 0) {
                    std::fprintf(stderr, "encode: source ended at row %d of %d\n", r, H);
                    failed = true;
                    break;
                }
                StripIn si;
                si.slot = slot;
                si.rows = n;
                if (!q_in.push(si)) break;
                r += n;
            }
            q_in.close();
        });
        std::thread writer([&] {
            std::vector<uint8_t> b;
            while (q_out.pop(b))
                if (!failed) w.write_idat_bytes(b.data(), b.size());
        });
        ParallelDeflateState st;
        gpu_filter_reset(ctx);
        int done = 0;
        StripIn si;
        while (!failed && q_in.pop(si)) {
            gpu_filter_process_from_host(ctx, ring + si.slot * slot_bytes, nullptr, si.rows, nullptr, dicom, true);
            const bool last = done + si.rows == H;
            // waits for the strip's stream: the upload from the slot is done after this
            DeflateResult dr = backend.compress_strip_device(gpu_filter_device_output(ctx),
                                                             gpu_filter_output_size(ctx, si.rows), last,
                                                             gpu_filter_stream(ctx));
            q_free.push(si.slot);
            if (dr.data.empty()) {
                failed = true;
                break;
            }
            accum_adler(st, dr);
            q_out.push(std::move(dr.data));
            done += si.rows;
        }
        if (done != H) failed = true;
        q_free.close();
        q_in.close();
        reader.join();
        if (!failed) {
            std::vector<uint8_t> trl(4);
            zlib_trailer(st, trl.data());
            q_out.push(std::move(trl));
        }
        q_out.close();
        writer.join();
        good = !failed;
        if (good) w.end_idat();
        w.close();
        good = good && !w.failed();
    }
    gpu_filter_destroy(ctx);
    if (!good) std::remove(out);
    return good;
}

// per-file times for the batch summary
std::mutex g_stats_mu;
std::vector<std::pair<long long, long long>> g_file_times;

}  // namespace

bool encode_source_to_png(ImageSource& src, const char* output_path, const PipelineConfig& cfg)
{
    if (cfg.format == ExportFormat::BMP) return encode_source_to_bmp(src, output_path);
    r2p_image img;
    if (!describe(src, cfg, img)) return false;
    const size_t bound = r2p_png_bound(&img);
    // one call holds the whole image: PNG below 2 GiB
    const bool whole = !cfg.strip_pipeline && bound > 0 && bound < ((size_t)1 << 31) - 4096;
    return whole ? encode_whole(src, output_path, cfg, img) : encode_strips(src, output_path, cfg, img);
}

namespace {

// The reference's BMP export of a source (run_bmp_from_source,
// src/pipeline.cpp:1944-2004) on the GPU: DICOM sources through the BMP
// path's own 16-bit gray window, others by the first byte of 16-bit samples
// or as they are.
bool bmp_from_source(ImageSource& src, const char* out, int device)
{
    thread_local PinnedScratch raw_buf;
    const ImageInfo& info = src.info();
    PipelineConfig cfg;
    r2p_image img;
    if (!describe(src, cfg, img)) return false;
    const size_t rb = (size_t)info.width * info.bpp;
    uint8_t* raw = raw_buf.get(rb * info.height);
    if (!raw || !read_all(src, raw, 64, rb)) return false;
    return write_bmp(img, raw, out, device);
}

}  // namespace

bool encode_source_to_bmp(ImageSource& src, const char* output_path)
{
    return bmp_from_source(src, output_path, 0);
}

bool encode_tiff_to_png(const char* input_path, const char* output_path, const PipelineConfig& cfg)
{
    const auto t0 = std::chrono::steady_clock::now();
    TiffSource src;
    if (!src.open(input_path)) {
        std::fprintf(stderr, "Cannot open TIFF: %s\n", input_path);
        return false;
    }
    const bool good = encode_source_to_png(src, output_path, cfg);
    pipeline_record_file_times(0, std::chrono::duration_cast<std::chrono::milliseconds>(
                                      std::chrono::steady_clock::now() - t0).count());
    return good;
}

bool encode_raw_to_png(const char* input_path, const char*, const PipelineConfig&)
{
    std::fprintf(stderr, "camera RAW input is not part of this build: %s\n", input_path);
    return false;
}

bool encode_dicom_to_bmp(const char* input_path, const char* output_path, const PipelineConfig& cfg)
{
    DicomSource src;
    if (!src.open(input_path)) {
        std::fprintf(stderr, "Cannot open DICOM: %s\n", input_path);
        return false;
    }
    const int frame = cfg.frame >= 0 ? cfg.frame : 0;
    if (frame >= src.num_frames()) {
        std::fprintf(stderr, "DICOM: requested frame %d but file has %d frame(s)\n", frame, src.num_frames());
        return false;
    }
    if (!src.load_frame(frame)) return false;
    return bmp_from_source(src, output_path, cfg.device);
}

bool encode_tiff_to_bmp(const char* input_path, const char* output_path, const PipelineConfig& cfg)
{
    TiffSource src;
    if (!src.open(input_path)) {
        std::fprintf(stderr, "Cannot open TIFF: %s\n", input_path);
        return false;
    }
    return bmp_from_source(src, output_path, cfg.device);
}

bool encode_raw_to_bmp(const char* input_path, const char*, const PipelineConfig&)
{
    std::fprintf(stderr, "camera RAW input is not part of this build: %s\n", input_path);
    return false;
}

bool encode_dicom_to_png(const char* input_path, const char* output_path, const PipelineConfig& cfg)
{
    using Clock = std::chrono::steady_clock;
    const auto t0 = Clock::now();
    DicomSource src;
    if (!src.open(input_path)) return false;
    const int frame = cfg.frame >= 0 ? cfg.frame : 0;
    if (frame >= src.num_frames()) {
        std::fprintf(stderr, "DICOM: requested frame %d but file has %d frame(s)\n", frame, src.num_frames());
        return false;
    }
    if (cfg.verbose && src.num_frames() > 1)
        std::printf("DICOM: %d frames; exporting frame %d\n", src.num_frames(), frame);
    if (!src.load_frame(frame)) return false;
    const auto t1 = Clock::now();
    const bool good = encode_source_to_png(src, output_path, cfg);
    const auto t2 = Clock::now();
    pipeline_record_file_times(std::chrono::duration_cast<std::chrono::milliseconds>(t1 - t0).count(),
                               std::chrono::duration_cast<std::chrono::milliseconds>(t2 - t0).count());
    if (cfg.verbose && good)
        std::printf("%s  %ux%u  ch=%d  bits=%d  level=%d  -> %s  (%.1f ms)\n", input_path, src.info().width,
                    src.info().height, src.info().channels, src.info().bits_per_sample, clamp_level(cfg.deflate_level),
                    output_path, std::chrono::duration<double, std::milli>(t2 - t0).count());
    return good;
}

bool encode_dicom_all_frames_to_png(const char* input_path, const char* output_dir, const PipelineConfig& cfg)
{
    DicomSource probe;
    if (!probe.open(input_path)) return false;
    const int n = probe.num_frames();
    std::error_code ec;
    std::filesystem::create_directories(output_dir, ec);
    if (ec) {
        std::fprintf(stderr, "Cannot create output folder '%s': %s\n", output_dir, ec.message().c_str());
        return false;
    }
    std::printf("Detected %d frame%s\n", n, n == 1 ? "" : "s");
    int workers = cfg.gpu_streams > 0 ? cfg.gpu_streams : 4;
    workers = std::max(1, std::min(workers, n));
    std::atomic<int> next{0};
    std::atomic<bool> all_ok{true};
    const std::string dir(output_dir);
    auto worker = [&]() {
        DicomSource src;
        if (!src.open(input_path)) {
            all_ok = false;
            return;
        }
        for (;;) {
            const int i = next.fetch_add(1);
            if (i >= n || !all_ok.load()) break;
            char name[32];
            std::snprintf(name, sizeof(name), "slice_%04d.png", i);
            const std::string out = (std::filesystem::path(dir) / name).string();
            if (!src.load_frame(i) || !encode_source_to_png(src, out.c_str(), cfg)) all_ok = false;
        }
    };
    std::vector<std::thread> th;
    for (int k = 0; k < workers; k++) th.emplace_back(worker);
    for (auto& t : th) t.join();
    return all_ok.load();
}

void pipeline_reset_gpu_batch_stats()
{
    std::lock_guard<std::mutex> lk(g_stats_mu);
    g_file_times.clear();
}

void pipeline_record_file_times(long long dicom_ms, long long total_ms)
{
    std::lock_guard<std::mutex> lk(g_stats_mu);
    g_file_times.emplace_back(dicom_ms, total_ms);
}

void pipeline_print_gpu_batch_summary(int total_files, int succeeded, double total_wall_s, long long sum_file_batch_ms,
                                      int num_workers)
{
    std::lock_guard<std::mutex> lk(g_stats_mu);
    long long sd = 0, st = 0;
    for (auto& t : g_file_times) {
        sd += t.first;
        st += t.second;
    }
    const size_t k = g_file_times.size();
    std::printf("GPU batch summary: %d/%d files OK in %.2f s (%.1f files/s), %d worker(s)\n", succeeded, total_files,
                total_wall_s, total_wall_s > 0 ? succeeded / total_wall_s : 0.0, num_workers);
    if (k)
        std::printf("  per file: decode %.1f ms, total %.1f ms (mean over %zu); batch-side sum %lld ms\n",
                    (double)sd / k, (double)st / k, k, sum_file_batch_ms);
}
