// gpu_filter.cpp -- the reference's strip filter interface
// (include/gpu_filter.h, src/gpu_filter.cu:313-520) over the r2p C ABI.
#include "gpu_filter.h"

#include <cstring>
#include <utility>

#include "host_common.h"

struct GpuFilterContext {
    int width = 0, bpp = 0, strip_height = 0;
    size_t width_bytes = 0;
    r2p_engine* eng = nullptr;
    void* stream = nullptr;
    uint8_t* d_input = nullptr;
    uint8_t* d_prior = nullptr;        // row above the next strip
    uint8_t* d_prior_next = nullptr;   // receives this strip's last windowed row
    uint8_t* d_selected = nullptr;
    uint8_t* h_output = nullptr;
    void* ev[4] = {nullptr, nullptr, nullptr, nullptr};   // start, h2d done, kernels done, d2h done
};

static void release(GpuFilterContext* c)
{
    if (c->d_input) r2p_device_free(c->d_input);
    if (c->d_prior) r2p_device_free(c->d_prior);
    if (c->d_prior_next) r2p_device_free(c->d_prior_next);
    if (c->d_selected) r2p_device_free(c->d_selected);
    if (c->h_output) r2p_host_free_pinned(c->h_output);
    for (void* e : c->ev)
        if (e) r2p_event_destroy(e);
    if (c->stream) r2p_stream_destroy(c->stream);
    if (c->eng) r2p_engine_destroy(c->eng);
    delete c;
}

GpuFilterContext* gpu_filter_create(int width, int bpp, int strip_height, bool device_output_only)
{
    int ch, bps;
    if (width < 1 || strip_height < 1 || !r2p_host::split_bpp(bpp, 0, ch, bps)) {
        std::fprintf(stderr, "gpu_filter_create: bad geometry (width %d, bpp %d, strip %d)\n", width, bpp,
                     strip_height);
        return nullptr;
    }
    GpuFilterContext* c = new GpuFilterContext();
    c->width = width;
    c->bpp = bpp;
    c->strip_height = strip_height;
    c->width_bytes = (size_t)width * bpp;
    const size_t strip_bytes = (size_t)strip_height * c->width_bytes;
    const size_t out_bytes = (size_t)strip_height * (c->width_bytes + 1);
    void* p = nullptr;
    bool good = r2p_host::ok(r2p_engine_create(0, 0, &c->eng), "r2p_engine_create") &&
                r2p_host::ok(r2p_stream_create(&c->stream), "r2p_stream_create");
    good = good && r2p_host::ok(r2p_device_alloc(strip_bytes + 16, &p), "device alloc");
    c->d_input = static_cast<uint8_t*>(p);
    good = good && r2p_host::ok(r2p_device_alloc(c->width_bytes + 16, &p), "device alloc");
    c->d_prior = static_cast<uint8_t*>(p);
    good = good && r2p_host::ok(r2p_device_alloc(c->width_bytes + 16, &p), "device alloc");
    c->d_prior_next = static_cast<uint8_t*>(p);
    good = good && r2p_host::ok(r2p_device_alloc(out_bytes + 16, &p), "device alloc");
    c->d_selected = static_cast<uint8_t*>(p);
    if (good && !device_output_only) {
        good = r2p_host::ok(r2p_host_alloc_pinned(out_bytes, &p), "pinned alloc");
        c->h_output = static_cast<uint8_t*>(p);
    }
    for (int i = 0; i < 4 && good; i++) good = r2p_host::ok(r2p_event_create(&c->ev[i]), "r2p_event_create");
    good = good && r2p_host::ok(r2p_memset_device(c->d_prior, 0, c->width_bytes, c->stream), "memset") &&
           r2p_host::ok(r2p_stream_synchronize(c->stream), "sync");
    if (!good) {
        release(c);
        return nullptr;
    }
    return c;
}

void gpu_filter_destroy(GpuFilterContext* ctx)
{
    if (!ctx) return;
    r2p_stream_synchronize(ctx->stream);
    release(ctx);
}

uint8_t* gpu_filter_alloc_pinned(size_t bytes)
{
    void* p = nullptr;
    return r2p_host::ok(r2p_host_alloc_pinned(bytes, &p), "gpu_filter_alloc_pinned") ? static_cast<uint8_t*>(p)
                                                                                       : nullptr;
}

void gpu_filter_free_pinned(uint8_t* ptr)
{
    if (ptr) r2p_host_free_pinned(ptr);
}

void gpu_filter_reset(GpuFilterContext* ctx)
{
    if (!ctx) return;
    r2p_host::ok(r2p_memset_device(ctx->d_prior, 0, ctx->width_bytes, ctx->stream), "gpu_filter_reset");
}

size_t gpu_filter_output_size(const GpuFilterContext* ctx, int actual_rows)
{
    return (size_t)actual_rows * (ctx->width_bytes + 1);
}

const uint8_t* gpu_filter_device_output(const GpuFilterContext* ctx)
{
    return ctx->d_selected;
}

void* gpu_filter_stream(const GpuFilterContext* ctx)
{
    return ctx->stream;
}

void gpu_filter_copy_prior_row_to_host(const GpuFilterContext* ctx, uint8_t* h_dst)
{
    r2p_host::ok(r2p_memcpy(h_dst, ctx->d_prior, ctx->width_bytes, ctx->stream), "prior row copy");
    r2p_host::ok(r2p_stream_synchronize(ctx->stream), "sync");
}

// Window + filter the strip in d_input; the carry moves to this strip's last row.
static const uint8_t* run_strip(GpuFilterContext* c, int rows, GpuTimings* t, const DicomPixelParams* dicom,
                                bool skip_d2h)
{
    r2p_image img;
    std::memset(&img, 0, sizeof(img));
    img.width = (uint32_t)c->width;
    img.height = (uint32_t)rows;
    int ch = 0, bps = 0;
    if (dicom) {
        if (dicom->bits_allocated != 8 && dicom->bits_allocated != 16) {
            std::fprintf(stderr, "gpu_filter: bits_allocated %d not supported\n", dicom->bits_allocated);
            return nullptr;
        }
        if (!r2p_host::split_bpp(c->bpp, dicom->bits_allocated / 8, ch, bps)) {
            std::fprintf(stderr, "gpu_filter: bpp %d does not fit bits_allocated %d\n", c->bpp, dicom->bits_allocated);
            return nullptr;
        }
        img.window_mode = R2P_WINDOW_DICOM16;
        static_assert(sizeof(DicomPixelParams) == sizeof(r2p_dicom_params), "DicomPixelParams layout");
        std::memcpy(&img.dicom, dicom, sizeof(img.dicom));
    } else {
        r2p_host::split_bpp(c->bpp, 0, ch, bps);
        img.window_mode = R2P_WINDOW_NONE;
    }
    img.channels = ch;
    img.bytes_per_sample = bps;
    img.strip_height = c->strip_height;
    if (!r2p_host::ok(r2p_window_filter_device_ex(c->eng, &img, c->d_input, c->d_prior, c->d_selected,
                                                  c->d_prior_next, c->stream),
                      "r2p_window_filter_device_ex"))
        return nullptr;
    std::swap(c->d_prior, c->d_prior_next);
    r2p_event_record(c->ev[2], c->stream);
    const uint8_t* ret = nullptr;
    if (!skip_d2h && c->h_output) {
        if (!r2p_host::ok(r2p_memcpy(c->h_output, c->d_selected, gpu_filter_output_size(c, rows), c->stream),
                          "filtered strip download"))
            return nullptr;
        ret = c->h_output;
    }
    r2p_event_record(c->ev[3], c->stream);
    if (!skip_d2h && !r2p_host::ok(r2p_stream_synchronize(c->stream), "sync")) return nullptr;
    if (t) {
        if (skip_d2h) r2p_stream_synchronize(c->stream);
        r2p_event_elapsed_ms(c->ev[0], c->ev[1], &t->h2d_ms);
        r2p_event_elapsed_ms(c->ev[1], c->ev[2], &t->kernel_ms);
        r2p_event_elapsed_ms(c->ev[2], c->ev[3], &t->d2h_ms);
    }
    return ret;
}

static bool check_rows(const GpuFilterContext* c, int rows)
{
    if (rows >= 1 && rows <= c->strip_height) return true;
    std::fprintf(stderr, "gpu_filter: %d rows outside [1, %d]\n", rows, c->strip_height);
    return false;
}

const uint8_t* gpu_filter_process_from_device(GpuFilterContext* ctx, const uint8_t* d_input,
                                              const uint8_t* d_prior_row, int actual_rows, GpuTimings* timings,
                                              const DicomPixelParams* dicom)
{
    if (!ctx || !d_input || !check_rows(ctx, actual_rows)) return nullptr;
    r2p_event_record(ctx->ev[0], ctx->stream);
    if (!r2p_host::ok(r2p_memcpy(ctx->d_input, d_input, (size_t)actual_rows * ctx->width_bytes, ctx->stream),
                      "strip copy"))
        return nullptr;
    if (d_prior_row && !r2p_host::ok(r2p_memcpy(ctx->d_prior, d_prior_row, ctx->width_bytes, ctx->stream),
                                     "prior row copy"))
        return nullptr;
    r2p_event_record(ctx->ev[1], ctx->stream);
    return run_strip(ctx, actual_rows, timings, dicom, ctx->h_output == nullptr);
}

const uint8_t* gpu_filter_process_from_host(GpuFilterContext* ctx, const uint8_t* h_input,
                                            const uint8_t* h_prior_row, int actual_rows, GpuTimings* timings,
                                            const DicomPixelParams* dicom, bool device_output_only)
{
    if (!ctx || !h_input || !check_rows(ctx, actual_rows)) return nullptr;
    r2p_event_record(ctx->ev[0], ctx->stream);
    if (!r2p_host::ok(r2p_memcpy(ctx->d_input, h_input, (size_t)actual_rows * ctx->width_bytes, ctx->stream),
                      "strip upload"))
        return nullptr;
    if (h_prior_row && !r2p_host::ok(r2p_memcpy(ctx->d_prior, h_prior_row, ctx->width_bytes, ctx->stream),
                                     "prior row upload"))
        return nullptr;
    r2p_event_record(ctx->ev[1], ctx->stream);
    return run_strip(ctx, actual_rows, timings, dicom, device_output_only || ctx->h_output == nullptr);
}
