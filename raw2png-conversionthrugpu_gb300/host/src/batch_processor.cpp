// batch_processor.cpp -- folder batch mode (the reference's
// src/batch_processor.cpp:330-437, 482-737) on the continuous-batching server.
//
// Reader threads open files and submit their frames to one r2p_server as they
// go; the calling thread waits on the tickets in file order and writes the
// PNGs.  Output naming, the multi-frame subfolder and the 16-bit grayscale ->
// 8-bit rule follow the reference:
//   single-frame 16-bit 1-channel  -> <stem>.png, 8-bit (R2P_WINDOW_BATCH8:
//                                     Q15 map when eligible, else FP32 table)
//   other single-frame             -> <stem>.png at its own depth (R2P_WINDOW_DICOM16)
//   multi-frame                    -> <stem>/slice_NNNN.png, own depth
// With --format bmp single frames and TIFFs become <stem>.bmp, written by the
// reader thread through r2p_encode_bmp (the same 16->8 rule for 16-bit
// grayscale DICOM, src/batch_processor.cpp:389-434); multi-frame files stay
// PNG slices, as in the reference (:378-384).
#include "batch_processor.h"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "dicom_loader.h"
#include "file_type.h"
#include "image_source.h"
#include "host_common.h"

namespace fs = std::filesystem;

namespace {

struct FrameJob {
    uint64_t ticket = 0;
    std::string out;
};

struct FileJob {
    bool ready = false, ok = true;
    std::vector<FrameJob> frames;
};

bool write_file(const std::string& path, const uint8_t* p, size_t n)
{
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool good = std::fwrite(p, 1, n, f) == n;
    return (std::fclose(f) == 0) && good;
}

}  // namespace

bool encode_folder(const char* input_dir, const char* output_dir, const PipelineConfig& cfg,
                   const BatchConfig& batch_cfg)
{
    std::error_code ec;
    fs::create_directories(output_dir, ec);
    if (ec) {
        std::fprintf(stderr, "Cannot create output folder '%s': %s\n", output_dir, ec.message().c_str());
        return false;
    }
    std::vector<fs::path> files;
    for (auto& entry : fs::directory_iterator(input_dir, ec)) {
        if (ec) break;
        if (!entry.is_regular_file()) continue;
        const std::string p = entry.path().string();
        if (is_dicom_file(p.c_str()) || is_tiff_file(p.c_str()) || is_raw_file(p.c_str())) files.push_back(entry.path());
    }
    if (ec) {
        std::fprintf(stderr, "Cannot read input folder '%s': %s\n", input_dir, ec.message().c_str());
        return false;
    }
    if (files.empty()) {
        std::printf("No supported files found in '%s'\n", input_dir);
        return true;
    }
    std::sort(files.begin(), files.end());
    const bool bmp = cfg.format == ExportFormat::BMP;
    const std::string ext = bmp ? ".bmp" : ".png";
    int workers = batch_cfg.num_workers;
    if (workers <= 0) {
        const int hw = (int)std::thread::hardware_concurrency();
        workers = std::max(1, std::min({hw > 0 ? hw : 4, (int)files.size(), 4}));
    }
    r2p_server_config sc;
    std::memset(&sc, 0, sizeof(sc));
    sc.hbm_budget = (size_t)8 << 30;
    sc.host_pool_bytes = (size_t)2 << 30;
    sc.max_inflight_batches = 8;
    sc.max_batch_images = 256;
    r2p_server* srv = nullptr;
    if (!r2p_host::ok(r2p_server_create(cfg.device, &sc, &srv), "r2p_server_create")) return false;
    const int level = cfg.deflate_level < 0 ? 0 : cfg.deflate_level > 9 ? 9 : cfg.deflate_level;
    std::printf("Batch: %zu file(s), %d reader(s), format=%s\n", files.size(), workers, bmp ? "BMP" : "PNG");

    const int kMaxOutstanding = 256;            // frames submitted but not yet written
    std::vector<FileJob> jobs(files.size());
    std::mutex mu;
    std::condition_variable cv;
    int outstanding = 0;
    size_t next_file = 0;
    const fs::path outdir(output_dir);

    auto submit_frame = [&](DicomSource& src, int frame, int mode, const std::string& out, FileJob& job) -> bool {
        if (!src.load_frame(frame)) return false;
        const ImageInfo& info = src.info();
        r2p_image img;
        std::memset(&img, 0, sizeof(img));
        img.width = info.width;
        img.height = info.height;
        img.channels = info.channels;
        img.bytes_per_sample = info.bits_per_sample / 8;
        img.window_mode = mode;
        std::memcpy(&img.dicom, src.dicom_params(), sizeof(img.dicom));
        img.level = level;
        img.strip_height = cfg.strip_height > 0 ? cfg.strip_height : 1024;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return outstanding < kMaxOutstanding; });
            outstanding++;
        }
        uint64_t t = 0;
        if (!r2p_host::ok(r2p_server_submit(srv, &img, src.pixel_data_.data(), &t), "r2p_server_submit")) {
            std::lock_guard<std::mutex> lk(mu);
            outstanding--;
            cv.notify_all();
            return false;
        }
        FrameJob fj;
        fj.ticket = t;
        fj.out = out;
        job.frames.push_back(fj);
        return true;
    };

    // a BMP of one loaded DICOM frame, written by this (reader) thread
    auto write_frame_bmp = [&](DicomSource& src, int frame, int mode, const std::string& out) -> bool {
        if (!src.load_frame(frame)) return false;
        const ImageInfo& info = src.info();
        r2p_image img;
        std::memset(&img, 0, sizeof(img));
        img.width = info.width;
        img.height = info.height;
        img.channels = info.channels;
        img.bytes_per_sample = info.bits_per_sample / 8;
        img.window_mode = mode;
        std::memcpy(&img.dicom, src.dicom_params(), sizeof(img.dicom));
        return r2p_host::write_bmp(img, src.pixel_data_.data(), out.c_str(), cfg.device);
    };

    // a TIFF file: samples already in PNG order, no window
    auto submit_tiff = [&](const std::string& path, const std::string& out, FileJob& job) -> bool {
        TiffSource t;
        if (!t.open(path.c_str())) return false;
        const ImageInfo& info = t.info();
        std::vector<uint8_t> px((size_t)info.width * info.height * info.bpp);
        const size_t rb = (size_t)info.width * info.bpp;
        for (int r = 0; r < (int)info.height;) {
            const int n = t.read_strip(px.data() + (size_t)r * rb, (int)info.height - r);
            if (n <= 0) return false;
            r += n;
        }
        r2p_image img;
        std::memset(&img, 0, sizeof(img));
        img.width = info.width;
        img.height = info.height;
        img.channels = info.channels;
        img.bytes_per_sample = info.bits_per_sample / 8;
        img.window_mode = R2P_WINDOW_NONE;
        img.level = level;
        img.strip_height = cfg.strip_height > 0 ? cfg.strip_height : 1024;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return outstanding < kMaxOutstanding; });
            outstanding++;
        }
        uint64_t tk = 0;
        if (!r2p_host::ok(r2p_server_submit(srv, &img, px.data(), &tk), "r2p_server_submit")) {
            std::lock_guard<std::mutex> lk(mu);
            outstanding--;
            cv.notify_all();
            return false;
        }
        FrameJob fj;
        fj.ticket = tk;
        fj.out = out;
        job.frames.push_back(fj);
        return true;
    };

    auto reader = [&]() {
        for (;;) {
            size_t i;
            {
                std::lock_guard<std::mutex> lk(mu);
                if (next_file >= files.size()) return;
                i = next_file++;
            }
            FileJob job;
            const std::string path = files[i].string();
            const std::string stem = files[i].stem().string();
            DicomSource src;
            if (is_tiff_file(path.c_str())) {
                job.ok = bmp ? encode_tiff_to_bmp(path.c_str(), (outdir / (stem + ext)).string().c_str(), cfg)
                             : submit_tiff(path, (outdir / (stem + ext)).string(), job);
            } else if (!is_dicom_file(path.c_str())) {
                std::fprintf(stderr, "%s: camera RAW input is not part of this build\n", path.c_str());
                job.ok = false;
            } else if (!src.open(path.c_str())) {
                job.ok = false;
            } else if (src.num_frames() > 1) {
                const fs::path sub = outdir / stem;
                std::error_code e2;
                fs::create_directories(sub, e2);
                for (int f = 0; f < src.num_frames() && job.ok; f++) {
                    char name[32];
                    std::snprintf(name, sizeof(name), "slice_%04d.png", f);
                    job.ok = submit_frame(src, f, R2P_WINDOW_DICOM16, (sub / name).string(), job);
                }
            } else {
                const int frame = cfg.frame >= 0 ? cfg.frame : 0;
                const ImageInfo& info = src.info();
                const int mode = (info.channels == 1 && info.bits_per_sample == 16) ? R2P_WINDOW_BATCH8
                                                                                    : R2P_WINDOW_DICOM16;
                const std::string out = (outdir / (stem + ext)).string();
                job.ok = frame < src.num_frames() &&
                         (bmp ? write_frame_bmp(src, frame, mode, out) : submit_frame(src, frame, mode, out, job));
            }
            std::lock_guard<std::mutex> lk(mu);
            jobs[i] = std::move(job);
            jobs[i].ready = true;
            cv.notify_all();
        }
    };

    const auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> th;
    for (int k = 0; k < workers; k++) th.emplace_back(reader);
    int succeeded = 0;
    for (size_t i = 0; i < files.size(); i++) {
        const auto f0 = std::chrono::steady_clock::now();
        {
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return jobs[i].ready; });
        }
        bool good = jobs[i].ok;
        for (const FrameJob& fj : jobs[i].frames) {
            r2p_result res;
            std::memset(&res, 0, sizeof(res));
            const int rc = r2p_server_wait(srv, fj.ticket, -1, &res);
            if (rc == R2P_OK && res.png) {
                if (!write_file(fj.out, res.png, res.png_len)) {
                    std::fprintf(stderr, "cannot write '%s'\n", fj.out.c_str());
                    good = false;
                }
            } else {
                std::fprintf(stderr, "%s: %s\n", fj.out.c_str(), r2p_status_string(rc));
                good = false;
            }
            r2p_server_release(srv, fj.ticket);
            std::lock_guard<std::mutex> lk(mu);
            outstanding--;
            cv.notify_all();
        }
        succeeded += good ? 1 : 0;
        const long long ms =
            std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - f0).count();
        if (batch_cfg.batch_verbose)
            std::printf("[%zu/%zu] %-40s  %-6s  (%lld ms)\n", i + 1, files.size(), files[i].filename().string().c_str(),
                        good ? "OK" : "FAILED", ms);
        else
            std::printf("[%zu/%zu] %s  %s\n", i + 1, files.size(), files[i].filename().string().c_str(),
                        good ? "OK" : "FAILED");
    }
    for (auto& t : th) t.join();
    const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    r2p_server_stats st;
    r2p_server_get_stats(srv, &st);
    std::printf("Batch done: %d/%zu OK in %.3f s (%.1f files/s); %llu GPU batches, mean %.1f images, p50 %.2f ms, "
                "p99 %.2f ms\n",
                succeeded, files.size(), wall, wall > 0 ? succeeded / wall : 0.0, (unsigned long long)st.batches,
                st.mean_batch_images, st.p50_ms, st.p99_ms);
    r2p_server_destroy(srv);
    return succeeded == (int)files.size();
}
