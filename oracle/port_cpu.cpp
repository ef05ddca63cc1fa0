// port_cpu.cpp -- TEST INFRASTRUCTURE: the CPU restatement of the reference's
// legacy encode path (window -> filter -> strip-parallel zlib DEFLATE -> PNG
// container).  It is the checker's CPU pipeline and the timed CPU baseline
// ("port"); the product library never links or calls it.
//
// Restates:
//   deflate_strip        src/parallel_deflate.cpp:117-192 (chunking, flush modes,
//                        per-chunk Adler + adler32_combine)
//   compress_chunk       src/parallel_deflate.cpp:75-112 (deflateInit2(level,
//                        Z_DEFLATED, -15, 8, Z_DEFAULT_STRATEGY), deflateReset reuse)
//   accum_adler          src/parallel_deflate.cpp:197-209
//   zlib_header/trailer  src/parallel_deflate.cpp:214-237
//   PngWriter            src/png_writer.cpp:33-125 (signature, IHDR, 32 KB IDAT
//                        chunks, CRC over type+data, IEND)
//   run_one strip loop   src/pipeline.cpp:137-284 (strips of strip_height rows,
//                        is_last on the final strip, writer order)
// The zlib calls are the reference's own third-party dependency (zlib 1.3 on
// both build machines), so for equal inputs this port emits the same bytes as
// the reference build; tests/test_oracle.py::test_port_png_matches_reference_bytes
// checks that byte equality against the reference's own sources compiled into
// oracle/_ref.
#include <zlib.h>

#include <algorithm>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

extern "C" {
struct orc_params;
void orc_window_a2(const uint8_t* in, size_t nsamples, const orc_params* p, uint8_t* out);
int  orc_window8(const uint8_t* src_le, size_t n, const orc_params* p, uint8_t* dst8);
void orc_filter_rows(const uint8_t* img, const uint8_t* prior, int rows, int rb, int bpp,
                     uint8_t* out);
}

namespace {

// Fixed-size worker pool: run(n, fn) executes fn(0..n-1) across the workers
// and returns when all calls finished.  Mirrors the persistent ThreadPool
// of include/thread_pool.h (workers created once, reused for every strip).
class Pool {
public:
    explicit Pool(int n) {
        for (int i = 0; i < n; i++) ws_.emplace_back([this] { loop(); });
    }
    ~Pool() {
        { std::lock_guard<std::mutex> lk(m_); stop_ = true; }
        cv_.notify_all();
        for (auto& t : ws_) t.join();
    }
    void run(int n, const std::function<void(int)>& fn) {
        std::unique_lock<std::mutex> lk(m_);
        fn_ = &fn; next_ = 0; total_ = n; done_ = 0; gen_++;
        cv_.notify_all();
        done_cv_.wait(lk, [&] { return done_ == total_; });
        fn_ = nullptr;
    }
private:
    void loop() {
        uint64_t seen = 0;
        std::unique_lock<std::mutex> lk(m_);
        for (;;) {
            cv_.wait(lk, [&] { return stop_ || (gen_ != seen && next_ < total_); });
            if (stop_) return;
            while (fn_ && next_ < total_) {
                int i = next_++;
                const std::function<void(int)>* f = fn_;
                lk.unlock();
                (*f)(i);
                lk.lock();
                if (++done_ == total_) { seen = gen_; done_cv_.notify_all(); }
            }
            seen = gen_;
        }
    }
    std::vector<std::thread> ws_;
    std::mutex m_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(int)>* fn_ = nullptr;
    int next_ = 0, total_ = 0, done_ = 0;
    uint64_t gen_ = 0;
    bool stop_ = false;
};

struct Zs {
    z_stream zs{};
    int level = -1;
    bool inited = false;
    ~Zs() { if (inited) deflateEnd(&zs); }
    z_stream& acquire(int lvl) {                 // src/parallel_deflate.cpp:49-60
        if (inited && level == lvl) {
            deflateReset(&zs);
        } else {
            if (inited) deflateEnd(&zs);
            zs = z_stream{};
            deflateInit2(&zs, lvl, Z_DEFLATED, -15, 8, Z_DEFAULT_STRATEGY);
            level = lvl;
            inited = true;
        }
        return zs;
    }
};
thread_local Zs tl_zs;

struct Chunk {
    std::vector<uint8_t> data;
    unsigned long adler = 1;
    size_t in_size = 0;
};

const size_t MIN_CHUNK = 4096;                   // src/parallel_deflate.cpp:27

void compress_chunk(const uint8_t* in, size_t n, int level, int flush, Chunk& out)
{
    out.in_size = n;
    if (n == 0) { out.data.clear(); out.adler = 1; return; }
    z_stream& zs = tl_zs.acquire(level);
    const uLong bound = deflateBound(&zs, (uLong)n) + 64;
    out.data.resize((size_t)bound);
    zs.next_in = const_cast<Bytef*>(in);
    zs.avail_in = (uInt)n;
    zs.next_out = out.data.data();
    zs.avail_out = (uInt)bound;
    deflate(&zs, flush);
    out.data.resize((size_t)zs.total_out);
    out.adler = adler32(1L, in, (uInt)n);
}

struct StripOut {
    std::vector<uint8_t> data;
    unsigned long adler = 1;
    size_t in_size = 0;
};

void deflate_strip(const uint8_t* in, size_t n, int level, Pool& pool, int nthreads,
                   bool is_last, StripOut& res, std::vector<Chunk>& chunks)
{
    res.data.clear();
    res.in_size = n;
    res.adler = 1;
    if (n == 0) return;
    int nt = nthreads;                            // :133-136
    if ((size_t)nt > n / MIN_CHUNK) nt = (int)std::max<size_t>(1, n / MIN_CHUNK);
    nt = std::max(1, nt);
    const size_t cs = (n + (size_t)nt - 1) / (size_t)nt;
    int last_active = 0;                          // :141-144
    for (int i = nt - 1; i >= 0; i--)
        if ((size_t)i * cs < n) { last_active = i; break; }
    chunks.resize((size_t)nt);
    pool.run(nt, [&](int i) {
        const size_t s = (size_t)i * cs;
        if (s >= n) { chunks[i].in_size = 0; chunks[i].data.clear(); return; }
        const size_t e = std::min(s + cs, n);
        const bool last = is_last && (i == last_active);
        compress_chunk(in + s, e - s, level, last ? Z_FINISH : Z_FULL_FLUSH, chunks[i]);
    });
    bool started = false;                         // :167-190
    unsigned long running = 1;
    for (int i = 0; i < nt; i++) {
        Chunk& c = chunks[i];
        if (c.in_size == 0) continue;
        running = started ? adler32_combine(running, c.adler, (z_off_t)c.in_size) : c.adler;
        started = true;
        res.data.insert(res.data.end(), c.data.begin(), c.data.end());
    }
    res.adler = started ? running : 1UL;
}

// In-memory PngWriter (src/png_writer.cpp): 32 KB IDAT buffer, CRC per chunk.
struct MemPng {
    std::vector<uint8_t>& out;
    uint8_t idat[32768];
    size_t pos = 0;
    explicit MemPng(std::vector<uint8_t>& o) : out(o) {}
    void u32(uint32_t v) {
        uint8_t b[4] = {(uint8_t)(v >> 24), (uint8_t)(v >> 16), (uint8_t)(v >> 8), (uint8_t)v};
        out.insert(out.end(), b, b + 4);
    }
    void chunk(const char* type, const uint8_t* data, uint32_t len) {
        u32(len);
        out.insert(out.end(), type, type + 4);
        if (len && data) out.insert(out.end(), data, data + len);
        uLong crc = crc32(0L, nullptr, 0);
        crc = crc32(crc, (const Bytef*)type, 4);
        if (len && data) crc = crc32(crc, data, len);
        u32((uint32_t)crc);
    }
    void open(uint32_t w, uint32_t h, uint8_t depth, uint8_t ctype) {
        static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
        out.insert(out.end(), sig, sig + 8);
        uint8_t ihdr[13] = {(uint8_t)(w >> 24), (uint8_t)(w >> 16), (uint8_t)(w >> 8), (uint8_t)w,
                            (uint8_t)(h >> 24), (uint8_t)(h >> 16), (uint8_t)(h >> 8), (uint8_t)h,
                            depth, ctype, 0, 0, 0};
        chunk("IHDR", ihdr, 13);
        pos = 0;
    }
    void write(const uint8_t* d, size_t n) {
        while (n > 0) {
            const size_t take = std::min(n, sizeof(idat) - pos);
            memcpy(idat + pos, d, take);
            pos += take; d += take; n -= take;
            if (pos == sizeof(idat)) { chunk("IDAT", idat, (uint32_t)pos); pos = 0; }
        }
    }
    void close() {
        if (pos) { chunk("IDAT", idat, (uint32_t)pos); pos = 0; }
        chunk("IEND", nullptr, 0);
    }
};

void zlib_header(int level, uint8_t o[2])       // src/parallel_deflate.cpp:214-228
{
    uint8_t flg;
    if (level == 1) flg = 0x01;
    else if (level >= 2 && level <= 5) flg = 0x5E;
    else if (level >= 6 && level <= 7) flg = 0x9C;
    else flg = 0xDA;
    o[0] = 0x78; o[1] = flg;
}

uint8_t color_type(int channels)                 // src/pipeline.cpp:80-88
{
    switch (channels) { case 1: return 0; case 3: return 2; case 4: return 6; default: return 2; }
}

}  // namespace

extern "C" {

// Opaque CPU encoder holding the worker pool (threads created once).
struct port_encoder { Pool* pool; int threads; };

port_encoder* port_encoder_create(int threads)
{
    if (threads < 1) threads = 1;
    port_encoder* e = new port_encoder;
    e->pool = new Pool(threads);
    e->threads = threads;
    return e;
}

void port_encoder_destroy(port_encoder* e)
{
    if (!e) return;
    delete e->pool;
    delete e;
}

// Compress already-filtered scanlines (height rows of row_bytes+1 bytes) into
// a PNG in `out` (capacity cap).  Returns the PNG size, or 0 if cap is short.
size_t port_png_from_filtered(port_encoder* e, const uint8_t* filtered, uint32_t width,
                              uint32_t height, int row_bytes, int bit_depth, int channels,
                              int level, int strip_height, uint8_t* out, size_t cap)
{
    std::vector<uint8_t> png;
    png.reserve((size_t)height * (row_bytes + 1) / 2 + 1024);
    MemPng w(png);
    w.open(width, height, (uint8_t)bit_depth, color_type(channels));
    uint8_t zh[2];
    zlib_header(level, zh);
    w.write(zh, 2);
    unsigned long running = 1;
    bool started = false;
    StripOut so;
    std::vector<Chunk> chunks;
    const size_t frb = (size_t)row_bytes + 1;
    const int nstrips = ((int)height + strip_height - 1) / strip_height;
    for (int s = 0; s < nstrips; s++) {
        const int r0 = s * strip_height;
        const int rows = std::min(strip_height, (int)height - r0);
        deflate_strip(filtered + (size_t)r0 * frb, (size_t)rows * frb, level, *e->pool,
                      e->threads, s == nstrips - 1, so, chunks);
        if (so.in_size) {                         // accum_adler, :197-209
            running = started ? adler32_combine(running, so.adler, (z_off_t)so.in_size) : so.adler;
            started = true;
        }
        if (!so.data.empty()) w.write(so.data.data(), so.data.size());
    }
    uint8_t tr[4] = {(uint8_t)(running >> 24), (uint8_t)(running >> 16),
                     (uint8_t)(running >> 8), (uint8_t)running};
    w.write(tr, 4);
    w.close();
    if (png.size() > cap) return 0;
    memcpy(out, png.data(), png.size());
    return png.size();
}

// Whole CPU pipeline from raw samples.
//   window_mode 0: no windowing; input bytes are PNG-ordered already
//   window_mode 1: 16-bit-output DICOM window (gpu_filter.cu:71-162 restated)
//   window_mode 2: 8-bit-output batch window (batch_processor.cpp:397-409)
// filtered_out (optional, height*(rb+1) bytes) receives the filtered scanlines.
size_t port_encode_png(port_encoder* e, const uint8_t* raw, uint32_t width, uint32_t height,
                       int channels, int in_bytes_per_sample, int window_mode,
                       const orc_params* params, int level, int strip_height,
                       uint8_t* out, size_t cap, uint8_t* filtered_out)
{
    const size_t nsamp = (size_t)width * height * channels;
    int out_bps = in_bytes_per_sample;
    std::vector<uint8_t> win;
    const uint8_t* img = raw;
    if (window_mode == 1) {
        win.resize(nsamp * (size_t)in_bytes_per_sample);
        orc_window_a2(raw, nsamp, params, win.data());
        img = win.data();
    } else if (window_mode == 2) {
        win.resize(nsamp);
        orc_window8(raw, nsamp, params, win.data());
        img = win.data();
        out_bps = 1;
    }
    const int rb = (int)(width * channels * out_bps);
    const int bpp = channels * out_bps;
    std::vector<uint8_t> filt_local;
    uint8_t* filt = filtered_out;
    if (!filt) { filt_local.resize((size_t)height * (rb + 1)); filt = filt_local.data(); }
    // Row groups in parallel; each group's row above comes from the windowed image.
    const int groups = std::max(1, std::min<int>(e->threads * 4, (int)height));
    const int per = ((int)height + groups - 1) / groups;
    e->pool->run(groups, [&](int g) {
        const int r0 = g * per;
        const int rows = std::min(per, (int)height - r0);
        if (rows <= 0) return;
        orc_filter_rows(img + (size_t)r0 * rb, r0 ? img + (size_t)(r0 - 1) * rb : nullptr,
                        rows, rb, bpp, filt + (size_t)r0 * (rb + 1));
    });
    return port_png_from_filtered(e, filt, width, height, rb, out_bps * 8, channels, level,
                                  strip_height, out, cap);
}

}  // extern "C"
