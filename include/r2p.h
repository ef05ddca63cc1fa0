/*
 * r2p.h -- C ABI of the GB300 raw-pixel -> PNG encoder (libr2p.so).
 *
 * Plain C types only: pointers, sizes, ints.  Device pointers are CUDA
 * device addresses on the current device; `stream` arguments are cudaStream_t
 * handles passed as void* (NULL = the legacy default stream).  Every entry
 * point returns an R2P_* status and never exits the process; the reference
 * printed and called exit(1) on every CUDA error (src/gpu_filter.cu:25-33).
 *
 * Each declaration names the reference interface it replaces (paths are
 * relative to the HeC-KriS/RAW2PNG-ConversionThruGPU project root).
 */
#ifndef R2P_H
#define R2P_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define R2P_OK        0
#define R2P_EINVAL    1   /* bad argument or unsupported geometry */
#define R2P_ENOMEM    2   /* device or pinned allocation failed */
#define R2P_EBUDGET   3   /* request exceeds the engine's HBM budget */
#define R2P_ECUDA     4   /* CUDA runtime error (message via r2p_last_error) */
#define R2P_ETIMEOUT  5   /* a bounded wait gave up */
#define R2P_ENOSPC    6   /* caller's output buffer is too small */
#define R2P_ECANCELED 7   /* request cancelled before it ran */
#define R2P_ENOTFOUND 8   /* unknown ticket */

/* ---- window modes ------------------------------------------------------ */
/* R2P_WINDOW_NONE: samples are already in PNG byte order (16-bit big-endian,
 *   as the TIFF/RAW loaders deliver them, src/image_loader.cpp:200-202).
 * R2P_WINDOW_SWAP16: 16-bit little-endian samples, byte-swapped only.
 * R2P_WINDOW_DICOM16: DICOM shift/mask/sign/rescale/window with output depth
 *   equal to BitsAllocated (dicom_preprocess_kernel, src/gpu_filter.cu:71-162).
 * R2P_WINDOW_BATCH8: 16-bit grayscale DICOM converted to 8 bits the way the
 *   folder batch does it (src/batch_processor.cpp:397-409: Q15 linear map
 *   when eligible, else the FP32 table). */
#define R2P_WINDOW_NONE    0
#define R2P_WINDOW_SWAP16  1
#define R2P_WINDOW_DICOM16 2
#define R2P_WINDOW_BATCH8  3

/* Same layout as DicomPixelParams (include/dicom_params.h:6-21). */
typedef struct r2p_dicom_params {
    int   bits_allocated;
    int   bits_stored;
    int   high_bit;
    int   pixel_rep;
    int   apply_rescale;
    float rescale_slope;
    float rescale_intercept;
    int   apply_window;
    float window_center;
    float window_width;
} r2p_dicom_params;

/* One image to encode.  level 0 = stored DEFLATE blocks; 1 = LZ77 with the
 * fixed Huffman code (the reference GPU encoder's format,
 * src/gpu_deflate_backend.cu:557-697); 2..9 = a per-block dynamic Huffman
 * code over a run-length parse (distance-1 matches, the strategy PNG
 * encoders use for filtered scanlines), smaller output at a lower rate.
 * Blocks are independent at every level (the zlib header's FLEVEL bits
 * follow the level exactly as src/parallel_deflate.cpp:214-228 sets them).
 * strip_height keeps the CLI's meaning for the strip-wise entry points; the
 * whole-image entry points hold the image resident and ignore it. */
typedef struct r2p_image {
    uint32_t width;
    uint32_t height;
    int      channels;          /* 1 gray, 3 RGB, 4 RGBA */
    int      bytes_per_sample;  /* input: 1 or 2 */
    int      window_mode;       /* R2P_WINDOW_* */
    r2p_dicom_params dicom;     /* used by DICOM16 / BATCH8 */
    int      level;             /* 0..9 */
    int      strip_height;
    int      block_size;        /* 0 = automatic (size-class table), else filtered bytes per DEFLATE block */
} r2p_image;

/* ---- library ----------------------------------------------------------- */
int         r2p_version(void);
const char* r2p_status_string(int status);
/* Message of the last R2P_ECUDA/R2P_EINVAL raised on the calling thread. */
const char* r2p_last_error(void);

/* ---- engine: device-owning encoder ------------------------------------- */
typedef struct r2p_engine r2p_engine;

/* Replaces the per-image GpuFilterContext/GpuDeflateContext/GpuAdler32Context/
 * GpuPngAssembleContext set built in run_pipeline (src/pipeline.cpp:1579-1648)
 * and its thread-local cache (:1527-1561).  hbm_budget = 0 means no limit. */
int  r2p_engine_create(int device, size_t hbm_budget, r2p_engine** out);
void r2p_engine_destroy(r2p_engine* eng);

/* Upper bound of the PNG size for an image under any tuning table (it assumes
 * 1024-byte DEFLATE blocks unless img->block_size is set); 0 on invalid
 * geometry. */
size_t r2p_png_bound(const r2p_image* img);

/* Encode one image from host memory to a PNG in host memory (blocking).
 * Replaces encode_source_to_png(ImageSource&, out, cfg)
 * (include/pipeline.h:110-112) minus the file write. */
int r2p_encode_png(r2p_engine* eng, const r2p_image* img, const void* h_pixels,
                   void* h_png, size_t png_cap, size_t* png_len);

/* Device-resident form: pixels and PNG stay in HBM; the PNG size is written
 * to *d_png_len (a device uint64) when the work on `stream` completes.  A
 * device-side failure writes (1 << 63) | status there instead (R2P_ENOSPC,
 * or R2P_ETIMEOUT when a bounded wait in a kernel gave up).
 * Replaces the modern path's filter -> gpu_deflate -> gpu_adler32 ->
 * gpu_png_assemble sequence (src/pipeline.cpp:581-830). */
int r2p_encode_png_device(r2p_engine* eng, const r2p_image* img, const void* d_pixels,
                          void* d_png, size_t png_cap, uint64_t* d_png_len, void* stream);

/* Batched form: n images in one launch sequence (one kernel per stage over a
 * device work list of row bands and DEFLATE blocks).  Replaces the folder
 * batch's per-file encode pool (src/batch_processor.cpp:482-737). */
int r2p_encode_batch_device(r2p_engine* eng, int n, const r2p_image* imgs,
                            const void* const* d_pixels, void* const* d_pngs,
                            const size_t* png_caps, uint64_t* d_png_lens, void* stream);

/* Reusable batch: the work list (row bands, DEFLATE blocks) and descriptors of
 * n images are planned and uploaded once, with the batch's own device
 * scratch (r2p_batch_device_bytes); r2p_batch_launch then issues only the
 * stage kernels, and r2p_batch_launch_graph captures that kernel sequence
 * once as a CUDA graph and replays it.  Pixels and PNG buffers are fixed at
 * creation.  Replaces the folder batch's per-file encode pool and thread-local
 * context cache (src/batch_processor.cpp:482-737, src/pipeline.cpp:1527-1561). */
typedef struct r2p_batch r2p_batch;
int    r2p_batch_create(r2p_engine* eng, int n, const r2p_image* imgs, const void* const* d_pixels,
                        void* const* d_pngs, const size_t* png_caps, uint64_t* d_png_lens, r2p_batch** out);
int    r2p_batch_launch(r2p_batch* b, void* stream);
int    r2p_batch_launch_graph(r2p_batch* b, void* stream);
size_t r2p_batch_device_bytes(const r2p_batch* b);
void   r2p_batch_destroy(r2p_batch* b);

/* Size-class tuning: per class of raw image bytes (sorted, the last class
 * takes everything larger), the DEFLATE block size used for a level-1 image
 * whose block_size is 0 (levels 0 and 2-9 keep 65520-byte blocks: fewer
 * stored headers, and per-block Huffman codes that pay for their header),
 * the filter's rows per work item of the shared-memory filter kernel (0 =
 * about 64 KB of filtered output per item; a work list with fewer items than
 * resident CTA slots is split evenly over them instead; the row-per-warp and
 * register-group kernels size their items from the row width) and
 * the LZ77 hash-table bits per image (9 or 10: 2^9 or 2^10 entries per
 * warp).  Set from the
 * autotuner's table; n = 0 restores the built-in one (the autotuner's GB300
 * result: 21760-byte level-1 blocks in every class, band rows 16 / auto / 32
 * / 32 / auto for classes up to 327680 / 1310720 / 6168576 / 14557184 raw
 * bytes / larger, 10 hash bits).  Replaces the fixed
 * strip-height/pool-size defaults (src/main.cpp:165-170, src/pipeline.cpp:1587). */
typedef struct r2p_tuning {
    uint64_t max_raw_bytes;
    int      block_size;
    int      band_rows;
    int      hash_bits;
} r2p_tuning;
int r2p_engine_set_tuning(r2p_engine* eng, int n, const r2p_tuning* classes);
int r2p_engine_get_tuning(r2p_engine* eng, int cap, r2p_tuning* out, int* n);

/* Encode n images from host memory (any mix of sizes and modes), each as by
 * r2p_encode_png, with the copies and kernels of up to R2P_MANY_SLOTS images
 * in flight at once (helper engines, each with its own arena and stream):
 * one host thread keeps the GPU busy across images.  Pinned host buffers let
 * copies overlap; pageable ones are correct but serialise.  statuses (may be
 * NULL) receives each image's status; returns R2P_OK or the first failure.
 * The reference encodes images one at a time per worker thread
 * (src/batch_processor.cpp:482-737, src/pipeline.cpp:1571). */
#define R2P_MANY_SLOTS 4
int r2p_encode_png_many(r2p_engine* eng, int n, const r2p_image* imgs, const void* const* h_pixels,
                        void* const* h_pngs, const size_t* png_caps, size_t* png_lens, int* statuses);

/* Stage entry point: window + adaptive filter of a whole image into
 * height*(row_bytes+1) filtered scanline bytes on the device.  d_prior (may
 * be NULL = zeros) is the windowed row above row 0.  Replaces
 * gpu_filter_process_from_device (include/gpu_filter.h:41-47). */
int r2p_window_filter_device(r2p_engine* eng, const r2p_image* img, const void* d_pixels,
                             const void* d_prior, void* d_filtered, void* stream);
/* As above; d_last_row (may be NULL) also receives the image's last row
 * after windowing (row_bytes bytes, PNG byte order): the row above the next
 * strip.  Replaces the carry that gpu_filter_process_* keeps between strips
 * and gpu_filter_copy_prior_row_to_host reads (src/gpu_filter.cu:428-434,
 * include/gpu_filter.h:76-90). */
int r2p_window_filter_device_ex(r2p_engine* eng, const r2p_image* img, const void* d_pixels,
                                const void* d_prior, void* d_filtered, void* d_last_row,
                                void* stream);

/* Stage entry point: zlib stream (header, DEFLATE blocks, Adler-32 trailer)
 * of already-filtered bytes, on the device.  Replaces gpu_deflate_compress_strip
 * + gpu_adler32 + zlib_header/trailer (include/gpu_deflate_backend.h:80-82,
 * include/gpu_adler32.h:25-31, src/parallel_deflate.cpp:214-237). */
int r2p_zlib_compress_device(r2p_engine* eng, const void* d_in, size_t len, int level,
                             int block_size, void* d_out, size_t out_cap,
                             uint64_t* d_out_len, void* stream);
size_t r2p_zlib_bound(size_t len, int level, int block_size);

/* Raw DEFLATE (no zlib header or trailer) of one part of a longer stream:
 * the strip contract of CompressionBackend::compress_strip
 * (include/compression_backend.h:33-43, src/parallel_deflate.cpp:141-170).
 * final_part = 0 leaves the stream open: no block has BFINAL set and the
 * part ends byte-aligned on an empty stored block, so parts concatenate into
 * one valid stream; final_part = 1 sets BFINAL on the last block.  The
 * input's Adler-32 follows the *d_out_len stream bytes as 4 big-endian bytes
 * (not counted).  out_cap >= r2p_zlib_bound(len, level, block_size). */
int r2p_deflate_raw_device(r2p_engine* eng, const void* d_in, size_t len, int level,
                           int block_size, int final_part, void* d_out, size_t out_cap,
                           uint64_t* d_out_len, void* stream);

/* Allocation-free form of r2p_zlib_compress_device, for callers that cannot
 * allocate device memory once running: code hosted in a framework that owns
 * all GPU memory and forbids allocation after start-up, and latency-bound
 * callers for which cudaMalloc/cudaFree would stall the device.  It has no
 * counterpart in the reference.  It needs no engine: its scratch (work
 * descriptors, per-block results, LZ77 block slots, CRC power table) lives in
 * a 2 MiB static device array that every GPU loading the library holds until
 * exit, so len is limited to 1 MiB (1048576 bytes); larger inputs are
 * rejected with R2P_EINVAL.  The first call on a device sets the array up
 * (looks up its address, builds the power table and waits for it): make that
 * call before any stream capture.  That set-up lasts for the process: after
 * cudaDeviceReset the entry point must not be called again.  All calls share
 * the array, so calls that overlap on the GPU race: issue them on one stream
 * or order them.  Output is
 * byte-identical to r2p_zlib_compress_device for the same input, level and
 * block_size. */
int r2p_zlib_compress_noalloc(const void* d_in, size_t len, int level, int block_size,
                              void* d_out, size_t out_cap, uint64_t* d_out_len, void* stream);

/* ---- BMP export -------------------------------------------------------- */
/* Uncompressed BMP file of an image, written on the device: replaces
 * run_bmp_from_source + BmpWriter (src/pipeline.cpp:1944-2004,
 * src/bmp_writer.cpp:36-131) behind encode_{dicom,tiff,raw,source}_to_bmp
 * (include/pipeline.h:97-122).  Layout: 14-byte file header, 40-byte info
 * header with negative height (rows top to bottom), a 256-entry gray palette
 * for one channel, rows padded with zeros to 4 bytes; one channel gives 8-bit
 * gray, three or four give 24-bit BGR (alpha dropped).  Pixel sources:
 *   DICOM16, 16-bit gray   the reference BMP path's own FP32 window formula
 *                          (src/pipeline.cpp:1894-1932; it divides by the
 *                          window range where the BATCH8 table multiplies)
 *   BATCH8                 the folder batch's 16->8-bit rule (Q15 or table),
 *                          as its BMP output does (src/batch_processor.cpp:389-422)
 *   NONE, 16-bit           the first byte of each sample (the high byte of the
 *                          big-endian samples the TIFF/RAW loaders produce)
 *   SWAP16                 the high byte of little-endian samples
 *   DICOM16, 16-bit colour the first byte of each sample, as the reference
 *   8-bit samples          as they are
 * 8-bit RGBA is refused (R2P_EINVAL).  level, strip_height and block_size are
 * ignored.  r2p_bmp_bound gives the exact file size (0 = not exportable). */
size_t r2p_bmp_bound(const r2p_image* img);
int r2p_encode_bmp(r2p_engine* eng, const r2p_image* img, const void* h_pixels, void* h_bmp,
                   size_t bmp_cap, size_t* bmp_len);
/* Device buffers; d_bmp must be 4-byte aligned and hold r2p_bmp_bound bytes. */
int r2p_encode_bmp_device(r2p_engine* eng, const r2p_image* img, const void* d_pixels, void* d_bmp,
                          size_t bmp_cap, void* stream);

/* ---- serving: continuous batching ------------------------------------- */
/* A server owns a device (an engine), a pooled device arena of hbm_budget
 * bytes and a pinned host pool.  Requests are admitted against the budget;
 * a dispatcher thread launches a batch of pending requests whenever one of
 * max_inflight_batches stream slots is free, so requests that arrive while
 * others run join the next batch and batches overlap on the device.  Results
 * come back to host memory owned by the server until r2p_server_release.
 * Replaces the reference's per-file worker pools and queues
 * (src/batch_processor.cpp:482-737, src/pipeline.cpp:445-1291). */
typedef struct r2p_server r2p_server;
typedef struct r2p_server_config {
    size_t hbm_budget;            /* device bytes for requests + scratch (0 = 40 GiB) */
    size_t host_pool_bytes;       /* pinned host bytes for pixels + PNGs (0 = 4 GiB) */
    int    max_inflight_batches;  /* concurrent batches / streams (0 = 8) */
    int    max_batch_images;      /* requests per batch at most (0 = 512) */
    size_t max_batch_bytes;       /* raw pixel bytes per batch at most, a single larger
                                     request excepted (0 = 96 MiB): small batches keep
                                     the streams' uploads, kernels and downloads
                                     overlapped */
} r2p_server_config;
typedef struct r2p_result {
    int            status;        /* R2P_OK, R2P_ECANCELED, or the failure */
    const uint8_t* png;           /* server-owned until r2p_server_release */
    size_t         png_len;
    double         latency_ms;    /* submit -> PNG in host memory */
    double         queue_ms;      /* submit -> dispatched in a batch */
} r2p_result;
typedef struct r2p_server_stats {
    uint64_t completed, failed, canceled, batches, pending;
    double   mean_batch_images;
    double   p50_ms, p99_ms, max_ms;
    size_t   device_bytes_in_use, device_bytes_peak;
} r2p_server_stats;
int  r2p_server_create(int device, const r2p_server_config* cfg, r2p_server** out);
int  r2p_server_set_tuning(r2p_server* srv, int n, const r2p_tuning* classes);
/* Copies the pixels; R2P_EBUDGET if the request can never fit the budget. */
int  r2p_server_submit(r2p_server* srv, const r2p_image* img, const void* h_pixels, uint64_t* ticket);
/* flags R2P_SUBMIT_BORROW: no copy -- the server reads h_pixels directly (best
 * from pinned memory), which must stay valid and unchanged until the request's
 * wait returns or it is cancelled. */
#define R2P_SUBMIT_BORROW 1u
int  r2p_server_submit_ex(r2p_server* srv, const r2p_image* img, const void* h_pixels, uint32_t flags,
                          uint64_t* ticket);
/* timeout_ms < 0 waits without limit; R2P_ETIMEOUT if still running. */
int  r2p_server_wait(r2p_server* srv, uint64_t ticket, int timeout_ms, r2p_result* res);
/* Only requests not yet dispatched can be cancelled. */
int  r2p_server_cancel(r2p_server* srv, uint64_t ticket);
int  r2p_server_release(r2p_server* srv, uint64_t ticket);
int  r2p_server_get_stats(r2p_server* srv, r2p_server_stats* st);
int  r2p_server_reset_stats(r2p_server* srv);
/* Drains in-flight work, then frees everything. */
void r2p_server_destroy(r2p_server* srv);

/* ---- diagnostics ------------------------------------------------------- */
/* Runs, on `device`, the time-bounded barrier wait that the TMA-staged
 * kernels use for their bulk copies, on a barrier that nothing completes
 * (arrive = 0) or that one arrival completes (arrive = 1).  *status receives
 * what the kernel reported: R2P_ETIMEOUT once limit_us (1..1000000) has
 * passed without completion, R2P_OK otherwise; the context stays usable.
 * No counterpart in the reference, whose waits have no limit. */
int r2p_selftest_bounded_wait(int device, int arrive, uint32_t limit_us, int* status);

/* ---- checksums (device data) ------------------------------------------- */
/* Replace gpu_adler32_compute (include/gpu_adler32.h:25) and
 * gpu_crc32_compute (include/gpu_crc32.h:29); results land in *d_result (a
 * device uint32) on `stream`. */
int r2p_adler32_device(r2p_engine* eng, const void* d_data, size_t len, uint32_t* d_result, void* stream);
int r2p_crc32_device(r2p_engine* eng, const void* d_data, size_t len, uint32_t* d_result, void* stream);
/* Host combine identities.  Replace gpu_crc32_combine (include/gpu_crc32.h:36)
 * and zlib's adler32_combine as used by accum_adler (src/parallel_deflate.cpp:197-209). */
uint32_t r2p_crc32_combine(uint32_t crc1, uint32_t crc2, uint64_t len2);
uint32_t r2p_adler32_combine(uint32_t adler1, uint32_t adler2, uint64_t len2);

/* ---- memory helpers (for callers without their own CUDA bindings) ------- */
int  r2p_device_alloc(size_t bytes, void** d_ptr);
int  r2p_device_free(void* d_ptr);
int  r2p_host_alloc_pinned(size_t bytes, void** h_ptr);   /* gpu_filter_alloc_pinned, include/gpu_filter.h:29 */
int  r2p_host_free_pinned(void* h_ptr);                   /* gpu_filter_free_pinned, include/gpu_filter.h:30 */
int  r2p_memcpy(void* dst, const void* src, size_t bytes, void* stream); /* any direction, async on stream */
int  r2p_memset_device(void* d_ptr, int value, size_t bytes, void* stream);
int  r2p_stream_create(void** stream);
int  r2p_stream_destroy(void* stream);
int  r2p_stream_synchronize(void* stream);
/* Events for device-side timing on a caller's stream. */
int  r2p_event_create(void** ev);
int  r2p_event_destroy(void* ev);
int  r2p_event_record(void* ev, void* stream);
int  r2p_event_elapsed_ms(void* ev_start, void* ev_end, float* ms);
int  r2p_stream_wait_event(void* stream, void* ev);   /* later work on stream waits for ev */
/* Stage timing: when enabled, each encode call (and each part of an
 * r2p_batch_launch of a batch created on the engine) records CUDA events on
 * its stream between its kernel launches; r2p_engine_stage_times() waits for
 * them, returns per-stage device milliseconds summed over the calls since the
 * last query (and how many launches each sum covers), and resets. */
#define R2P_STAGE_PREPARE  0   /* k_prepare_window: window tables (shared-memory filter, BMP) */
#define R2P_STAGE_FILTER   1   /* k_window_lut + k_filter_rows / k_window_filter_reg / k_window_filter: window + adaptive filter */
#define R2P_STAGE_STORED   2   /* k_stored_blocks: level-0 DEFLATE */
#define R2P_STAGE_LZ77     3   /* k_lz77_blocks (level 1) and k_rle_dyn_blocks (2..9) */
#define R2P_STAGE_FINALIZE 4   /* k_finish: block gather, checksum combine, PNG chunks */
#define R2P_STAGE_COPY     5   /* always 0: the block gather runs inside k_finish */
#define R2P_STAGE_COUNT    6
int r2p_engine_set_timing(r2p_engine* eng, int enable);
int r2p_engine_stage_times(r2p_engine* eng, double* ms, uint64_t* launches);
/* Kernels this library launched since the process started (all streams). */
uint64_t r2p_kernel_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* R2P_H */
