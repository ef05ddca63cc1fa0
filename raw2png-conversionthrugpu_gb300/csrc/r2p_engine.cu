// r2p_engine.cu -- host side of the encoder: the C ABI of include/r2p.h for
// engines, planning and the per-call encodes (batches: r2p_batch.cu; the
// request server: r2p_server.cu; shared internals: r2p_engine_impl.h).
//
// An engine owns one device's scratch memory (a reusable arena), a pinned
// staging area for work descriptors, and the CRC power table.  Every encode
// call builds a plan on the host (per image: geometry, window request, row
// bands for the filter kernel, DEFLATE blocks), uploads it in one copy, and
// launches one kernel per stage over the whole work list:
//   [k_window_lut -> k_filter_rows] | k_window_filter_reg | [k_prepare_window ->] k_window_filter
//   -> k_stored_blocks | k_lz77_blocks | k_rle_dyn_blocks -> k_finish
// (every image goes to one filter kernel: rows of kRowsMinRowBytes and more
// whose pixels a 16-byte load may read to k_filter_rows, after k_window_lut
// has built their window tables; other 16-byte-aligned rows of up to 8 KB to
// the register-group kernel, which builds its own table; the rest to the
// shared-memory kernel, whose tables k_prepare_window builds in HBM, as it
// does for the BMP export.  k_finish gathers the compressed blocks into the
// output, joins the per-block checksums and writes the PNG chunks.)
// Calls are ordered through the engine: each call waits (on the device, not
// the host) for the previous call's last kernel before reusing the arena.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "r2p_engine_impl.h"

namespace r2p {

static std::atomic<uint64_t> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

static thread_local std::string t_last_error;

int set_err(int code, const char* what)
{
    t_last_error = what ? what : "";
    return code;
}

int cuda_err(cudaError_t e, const char* where)
{
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s", where, cudaGetErrorString(e));
    t_last_error = buf;
    return e == cudaErrorMemoryAllocation ? R2P_ENOMEM : R2P_ECUDA;
}



// x^(8 * j * 2^(10 l)) mod P, l = 0..3, j = 0..1023 (see xpow8n)
static void build_xpow(std::vector<uint32_t>& tab)
{
    tab.assign(kXpowLevels * 1024, 0);
    uint32_t base = 1u << 23;   // x^8
    for (int l = 0; l < kXpowLevels; l++) {
        uint32_t v = 0x80000000u;   // x^0
        for (int j = 0; j < 1024; j++) {
            tab[l * 1024 + j] = v;
            v = gf2_mulmod(v, base);
        }
        for (int k = 0; k < 10; k++) base = gf2_mulmod(base, base);   // base^1024
    }
}

// ---------------------------------------------------------------------------
// planning
// ---------------------------------------------------------------------------

// Built-in size-class table: the autotuner's result on GB300 (tuning_gb300.json,
// written by autotune.py): 21760-byte level-1 blocks in every class (three LZ77
// CTAs per SM), filter rows per work item by class, 2^10-entry hash tables.
// Engines may load another table.
const std::vector<r2p_tuning> kDefaultTuning = {{327680, 21760, 16, 10},
                                                       {1310720, 21760, 0, 10},
                                                       {6168576, 21760, 32, 10},
                                                       {14557184, 21760, 32, 10},
                                                       {~0ull, 21760, 0, 10}};

static const r2p_tuning& tune_for(const std::vector<r2p_tuning>& t, uint64_t raw_bytes)
{
    for (const auto& c : t)
        if (raw_bytes <= c.max_raw_bytes) return c;
    return t.back();
}

int plan_image(const r2p_image& im, int out_kind, ImgPlan& ip, const std::vector<r2p_tuning>& tune)
{
    if (im.width < 1 || im.height < 1) return set_err(R2P_EINVAL, "width and height must be >= 1");
    if (im.channels != 1 && im.channels != 3 && im.channels != 4)
        return set_err(R2P_EINVAL, "channels must be 1, 3 or 4");
    if (im.bytes_per_sample != 1 && im.bytes_per_sample != 2)
        return set_err(R2P_EINVAL, "bytes_per_sample must be 1 or 2");
    if (im.level < 0 || im.level > 9) return set_err(R2P_EINVAL, "level must be 0..9");
    const r2p_dicom_params& p = im.dicom;
    int ob = im.bytes_per_sample;
    switch (im.window_mode) {
        case R2P_WINDOW_NONE:
            break;
        case R2P_WINDOW_SWAP16:
            if (im.bytes_per_sample != 2) return set_err(R2P_EINVAL, "SWAP16 needs 16-bit samples");
            break;
        case R2P_WINDOW_DICOM16:
            if (p.bits_allocated != 8 * im.bytes_per_sample)
                return set_err(R2P_EINVAL, "DICOM16: bits_allocated must match bytes_per_sample");
            if (p.bits_stored < 1 || p.bits_stored > p.bits_allocated)
                return set_err(R2P_EINVAL, "DICOM16: bits_stored out of range");
            break;
        case R2P_WINDOW_BATCH8:
            if (im.bytes_per_sample != 2 || im.channels != 1)
                return set_err(R2P_EINVAL, "BATCH8 needs 16-bit grayscale samples");
            if (p.bits_stored < 1 || p.bits_stored > 16 || p.high_bit - p.bits_stored + 1 < 0 ||
                p.high_bit > 15)
                return set_err(R2P_EINVAL, "BATCH8: bits_stored/high_bit out of range");
            ob = 1;
            break;
        default:
            return set_err(R2P_EINVAL, "unknown window_mode");
    }
    DevImage& d = ip.di;
    memset(&d, 0, sizeof(d));
    d.width = im.width;
    d.height = im.height;
    d.channels = im.channels;
    d.ib = im.bytes_per_sample;
    d.ob = ob;
    const uint64_t rb = (uint64_t)im.width * im.channels * ob;
    const uint64_t pitch = (uint64_t)im.width * im.channels * im.bytes_per_sample;
    if (rb > (1u << 20)) return set_err(R2P_EINVAL, "row too wide");
    d.rb = (int32_t)rb;
    d.bpp = im.channels * ob;
    d.in_pitch = (int32_t)pitch;
    const uint64_t F = (uint64_t)im.height * (rb + 1);
    d.filt_bytes = F;
    d.req_mode = im.window_mode;
    d.dp = im.dicom;
    d.level = im.level;
    const uint64_t raw_total = pitch * im.height;
    const r2p_tuning& tc = tune_for(tune, raw_total);
    // the tuned block size is the LZ77 kernel's; stored and dynamic-Huffman
    // blocks stay as large as DEFLATE allows unless the image says otherwise
    int bs = im.block_size ? im.block_size : im.level == 1 ? tc.block_size : kBlock64;
    ip.band_rows = tc.band_rows;
    ip.hash_bits = tc.hash_bits;
    if (bs < 1024 || bs > kBlock64 || (bs & 15)) return set_err(R2P_EINVAL, "block_size must be a multiple of 16 in [1024, 65520]");
    d.block_size = bs;
    const uint64_t nb = (F + bs - 1) / bs;
    d.nblocks = (int32_t)nb;
    d.out_kind = out_kind;
    d.prefix = out_kind == 0 ? kPngPrefix : out_kind == 1 ? 2 : 0;
    ip.raw_bytes = pitch * im.height;
    // worst-case table for the window request (resolved on the device)
    int entries = 0, esize = 0, mode_guess = W_COPY;
    if (im.window_mode == R2P_WINDOW_DICOM16) {
        entries = (im.bytes_per_sample == 2) ? (p.bits_stored < 16 ? (1 << p.bits_stored) : 65536) : 256;
        esize = ob;
        mode_guess = W_A2_LUT;
    } else if (im.window_mode == R2P_WINDOW_BATCH8) {
        entries = 1 << p.bits_stored;
        esize = 1;
        mode_guess = W_LUT8;
    }
    ip.lut_cap = align_up((uint64_t)entries * esize + 16, 256);
    ip.lreg = filter_lut_region(mode_guess, entries, esize);
    ip.smem = filter_smem_bytes(d.rb, d.in_pitch, mode_guess, entries, esize);
    if (ip.smem < 0) return set_err(R2P_EINVAL, "row too wide for the filter kernel");
    ip.reg_lut = entries * esize;
    ip.reg = reg_filter_eligible(d.rb, d.in_pitch, ip.reg_lut);
    ip.reg_w = reg_filter_warps(d.rb);
    ip.rows = d.rb >= kRowsMinRowBytes && rows_filter_eligible(d.in_pitch, ip.reg_lut);
    ip.png_bound = (uint64_t)d.prefix + F + (uint64_t)kStoredHdr * nb + (out_kind == 0 ? kPngSuffix : 4);
    if (F >= (1ull << 32) || ip.png_bound >= (1ull << 31) - 64)
        return set_err(R2P_EINVAL, "image too large for a single IDAT chunk");
    return R2P_OK;
}

// BMP export plan.  The window request maps onto the pixel sources of the
// reference's BMP path (src/pipeline.cpp:1965-2001): a 16-bit grayscale DICOM
// frame through its own FP32 formula (as a table), BATCH8 through the folder
// batch's 16->8-bit rule (src/batch_processor.cpp:389-422), other 16-bit
// samples by one byte (the first: big-endian data as the loaders leave it,
// and the reference's choice for 16-bit colour DICOM too), 8-bit samples as
// they are.
int plan_bmp(const r2p_image& im, ImgPlan& ip)
{
    if (im.width < 1 || im.height < 1) return set_err(R2P_EINVAL, "width and height must be >= 1");
    if (im.channels != 1 && im.channels != 3 && im.channels != 4)
        return set_err(R2P_EINVAL, "channels must be 1, 3 or 4");
    if (im.bytes_per_sample != 1 && im.bytes_per_sample != 2)
        return set_err(R2P_EINVAL, "bytes_per_sample must be 1 or 2");
    if (im.bytes_per_sample == 1 && im.channels == 4)
        return set_err(R2P_EINVAL, "8-bit RGBA has no BMP form here (the reference reads such rows as RGB triplets)");
    const r2p_dicom_params& p = im.dicom;
    DevImage& d = ip.di;
    memset(&d, 0, sizeof(d));
    d.width = im.width;
    d.height = im.height;
    d.channels = im.channels;
    d.ib = im.bytes_per_sample;
    d.ob = 1;
    d.in_pitch = (int32_t)((uint64_t)im.width * im.channels * im.bytes_per_sample);
    d.req_mode = R2P_WINDOW_NONE;
    d.dp = p;
    d.block_size = kBlock64;
    int entries = 0;
    d.bmp_kind = im.bytes_per_sample == 2 ? BMP_TAKE : BMP_BYTE;
    switch (im.window_mode) {
        case R2P_WINDOW_NONE:
            break;
        case R2P_WINDOW_SWAP16:
            if (im.bytes_per_sample != 2) return set_err(R2P_EINVAL, "SWAP16 needs 16-bit samples");
            d.bmp_off = 1;                        // little-endian samples: the high byte is second
            break;
        case R2P_WINDOW_DICOM16:
            if (p.bits_allocated != 8 * im.bytes_per_sample)
                return set_err(R2P_EINVAL, "DICOM16: bits_allocated must match bytes_per_sample");
            if (p.bits_stored < 1 || p.bits_stored > p.bits_allocated)
                return set_err(R2P_EINVAL, "DICOM16: bits_stored out of range");
            if (im.bytes_per_sample == 2 && im.channels == 1) {
                if (p.high_bit - p.bits_stored + 1 < 0 || p.high_bit > 15)
                    return set_err(R2P_EINVAL, "DICOM16: high_bit out of range");
                d.req_mode = kReqBmp8;
                d.bmp_kind = BMP_WINDOW;
                entries = 1 << p.bits_stored;
            }
            break;
        case R2P_WINDOW_BATCH8:
            if (im.bytes_per_sample != 2 || im.channels != 1)
                return set_err(R2P_EINVAL, "BATCH8 needs 16-bit grayscale samples");
            if (p.bits_stored < 1 || p.bits_stored > 16 || p.high_bit - p.bits_stored + 1 < 0 || p.high_bit > 15)
                return set_err(R2P_EINVAL, "BATCH8: bits_stored/high_bit out of range");
            d.req_mode = R2P_WINDOW_BATCH8;
            d.bmp_kind = BMP_WINDOW;
            entries = 1 << p.bits_stored;
            break;
        default:
            return set_err(R2P_EINVAL, "unknown window_mode");
    }
    d.bmp_oc = im.channels == 1 ? 1 : 3;
    const uint64_t stride = ((uint64_t)im.width * d.bmp_oc + 3) & ~3ull;
    const uint64_t pix_off = 54 + (d.bmp_oc == 1 ? 1024 : 0);
    const uint64_t size = pix_off + stride * im.height;
    if (size >= (1ull << 31)) return set_err(R2P_EINVAL, "BMP file would exceed 2 GiB");
    d.bmp_stride = (int32_t)stride;
    d.bmp_pix_off = (uint32_t)pix_off;
    d.bmp_size = (uint32_t)size;
    ip.raw_bytes = (uint64_t)d.in_pitch * im.height;
    ip.lut_cap = align_up((uint64_t)entries + 16, 256);
    ip.png_bound = size;
    ip.smem = 0;
    ip.lreg = 0;
    return R2P_OK;
}

}  // namespace r2p

using namespace r2p;



namespace r2p {


// Work list and memory layout of one call (or one batch) over n images.
void plan_work(r2p_engine* e, std::vector<ImgPlan>& plans, const CallBuffers& cb, size_t extra_bytes,
                      Prepared& P)
{
    const int n = (int)plans.size();
    // each image to one filter kernel: wide rows to the warp-per-row kernel,
    // rows that fit the register-group kernel (and whose pixels a bulk copy
    // may read: 16-byte aligned) there, the rest to the shared-memory kernel
    std::vector<char> use_reg((size_t)n, 0);
    int max_w = 0, nreg = 0;
    for (int i = 0; i < n; i++) {
        const bool aligned = i < (int)cb.raw.size() && (reinterpret_cast<uintptr_t>(cb.raw[i]) & 15) == 0;
        if (plans[i].rows && aligned) {
            // wide rows: one warp per row, items of whole CTAs' worth of rows
            plans[i].di.fpath = kFiltRows;
            P.wlut = std::max(P.wlut, plans[i].reg_lut);
            const DevImage& d = plans[i].di;
            const uint64_t rows = (uint64_t)rows_filter_rows_per_item();
            for (uint64_t r = 0; r < d.height; r += rows)
                P.witems.push_back(BandItem{(uint32_t)i, (uint32_t)r, (uint32_t)std::min<uint64_t>(d.height, r + rows)});
            continue;
        }
        use_reg[(size_t)i] = plans[i].reg && plans[i].smem > 0 && aligned;
        plans[i].di.fpath = use_reg[(size_t)i] ? kFiltReg : kFiltSmem;
        if (use_reg[(size_t)i]) {
            max_w = std::max(max_w, plans[i].reg_w);
            nreg++;
        } else {
            P.smem = std::max(P.smem, plans[i].smem);
        }
    }
    if (!P.witems.empty()) {
        // one stash size per launch: the largest any of its images can use
        // (an image whose rows need more is windowed again in pass 2)
        for (int i = 0; i < n; i++)
            if (plans[i].di.fpath == kFiltRows)
                P.wstash = std::max(P.wstash, rows_filter_stash(plans[i].di.rb, P.wlut));
        P.wsmem = rows_filter_smem(P.wlut, P.wstash);
        P.wslots = e->nsm * rows_filter_ctas_per_sm(P.wsmem);
    }
    const int cps = P.smem > 0 ? filter_ctas_per_sm(P.smem) : 1;
    P.slots_total = e->nsm * cps;
    if (nreg) {
        P.rnw = reg_filter_cta_warps(max_w);
        for (int i = 0; i < n; i++)
            if (use_reg[(size_t)i])
                P.rsmem = std::max(P.rsmem, reg_filter_smem(plans[i].di.rb, plans[i].di.in_pitch, plans[i].reg_lut,
                                                             P.rnw));
        P.rslots = e->nsm * reg_filter_ctas_per_sm(P.rnw, P.rsmem);
        // Bands of about 64 KB of filtered output (a property of the image
        // alone), or, when that leaves CTA slots idle, each image split evenly
        // over the slots; a CTA's band is cut into one run of rows per group
        // of warps, at least two rows each.
        auto reg_bands = [&](bool spread) {
            P.ritems.clear();
            for (int i = 0; i < n; i++) {
                if (!use_reg[(size_t)i]) continue;
                const DevImage& d = plans[i].di;
                const uint64_t G = (uint64_t)(P.rnw / plans[i].reg_w);
                uint64_t rows = std::max<uint64_t>(2 * G, (64 * 1024 + d.rb) / ((uint64_t)d.rb + 1));
                if (spread) {
                    const uint64_t share = std::max<uint64_t>(1, (uint64_t)P.rslots / (uint64_t)nreg + (nreg > 1));
                    rows = std::max<uint64_t>(2 * G, (d.height + share - 1) / share);
                }
                for (uint64_t r = 0; r < d.height; r += rows)
                    P.ritems.push_back(BandItem{(uint32_t)i, (uint32_t)r,
                                                (uint32_t)std::min<uint64_t>(d.height, r + rows)});
            }
        };
        reg_bands(false);
        if (P.ritems.size() < (size_t)P.rslots) reg_bands(true);
    }
    uint64_t lut_total = 0, filt_total = 0;
    bool any10 = false;
    // Row bands of the filter stage.  Batches use the tuned band height of
    // each image's size class (0 = about kAutoBandBytes of filtered output
    // per band: a property of the image, the same alone or in any batch).
    // When that would leave resident CTA slots idle (a lone image, a small
    // batch) every image is split evenly over the slots instead.
    constexpr uint64_t kAutoBandBytes = 64 * 1024;
    auto plan_bands = [&](bool tuned) {
        P.items.clear();
        if (P.smem <= 0) return;
        for (int i = 0; i < n; i++) {
            if (plans[i].di.fpath != kFiltSmem) continue;    // another kernel filters this image
            const DevImage& d = plans[i].di;
            const int T = filter_tile_rows(d.rb, d.in_pitch, P.smem, plans[i].lreg);
            const uint64_t ntiles = (d.height + T - 1) / T;
            uint64_t band_rows;
            if (tuned && plans[i].band_rows > 0) {
                band_rows = ((uint64_t)plans[i].band_rows + T - 1) / T * T;    // tuned, whole tiles
            } else if (tuned) {
                band_rows = std::max<uint64_t>(1, (kAutoBandBytes + d.rb) / ((uint64_t)d.rb + 1));
            } else {
                // about one band per resident CTA (a lone image), split evenly;
                // a band's last tile may be partial
                uint64_t nb = std::min<uint64_t>(ntiles, (uint64_t)P.slots_total);
                if (n > 1) nb = std::min<uint64_t>(ntiles, std::max<uint64_t>(1, (uint64_t)P.slots_total / n + 1));
                band_rows = (d.height + nb - 1) / nb;
            }
            for (uint64_t r = 0; r < d.height; r += band_rows)
                P.items.push_back(BandItem{(uint32_t)i, (uint32_t)r,
                                           (uint32_t)std::min<uint64_t>(d.height, r + band_rows)});
        }
    };
    plan_bands(true);
    if (P.items.size() < (size_t)P.slots_total) plan_bands(false);
    for (int i = 0; i < n; i++) {
        DevImage& d = plans[i].di;
        d.blk0 = P.nblk;
        for (int k = 0; k < d.nblocks; k++) {
            BlockOut bo;
            memset(&bo, 0, sizeof(bo));
            bo.img = (uint32_t)i;
            bo.in_off = (uint32_t)((uint64_t)k * d.block_size);
            bo.in_len = (uint32_t)std::min<uint64_t>(d.block_size, d.filt_bytes - (uint64_t)k * d.block_size);
            P.blocks.push_back(bo);
        }
        P.nblk += (uint32_t)d.nblocks;
        P.max_block = std::max(P.max_block, d.block_size);
        if (d.level == 0) P.any_stored = true;
        else if (d.level == 1) P.any_lz = true;
        else P.any_dyn = true;
        d.hash_bits = plans[i].hash_bits == 9 ? 9 : 10;
        if (d.level > 0 && d.hash_bits == 10) any10 = true;
        lut_total += plans[i].lut_cap;
        if (!cb.filt[i]) filt_total += align_up(d.filt_bytes + 64, 256);
        P.bmp_words = std::max(P.bmp_words, (d.bmp_size + 3u) / 4u);
    }
    // one hash-table size per launch: the one most blocks were tuned for
    P.hash_bits = any10 ? 10 : 9;      // LZ77 tables sized for the largest; each block uses its image's
    P.slot = (P.any_lz || P.any_dyn) ? lz77_slot_bytes(P.max_block) : 0;
    Layout L;
    P.o_img = L.take(sizeof(DevImage) * n);
    P.o_items = L.take(sizeof(BandItem) * std::max<size_t>(1, P.items.size()));
    P.o_ritems = L.take(sizeof(BandItem) * std::max<size_t>(1, P.ritems.size()));
    P.o_witems = L.take(sizeof(BandItem) * std::max<size_t>(1, P.witems.size()));
    P.o_blocks = L.take(sizeof(BlockOut) * std::max<size_t>(1, P.blocks.size()));
    P.desc_bytes = L.off;
    P.o_lut = L.take(lut_total);
    P.o_filt = L.take(filt_total);
    P.o_scratch = L.take(P.slot * P.nblk);
    P.o_extra = L.take(extra_bytes);
    P.total = L.off;
}

// Point the image descriptors at their buffers inside memory base A.
void fill_pointers(std::vector<ImgPlan>& plans, const CallBuffers& cb, const Prepared& P, uint8_t* A)
{
    uint64_t lut_off = P.o_lut, filt_off = P.o_filt;
    for (size_t i = 0; i < plans.size(); i++) {
        DevImage& d = plans[i].di;
        d.lut = A + lut_off;
        lut_off += plans[i].lut_cap;
        d.raw = cb.raw[i];
        d.prior = cb.prior[i];
        d.last_row = i < cb.last_row.size() ? cb.last_row[i] : nullptr;
        if (cb.filt[i]) {
            d.filt = cb.filt[i];
        } else {
            d.filt = A + filt_off;
            filt_off += align_up(d.filt_bytes + 64, 256);
        }
        d.png = cb.out[i];
        d.png_cap = cb.out_cap[i];
        d.png_len = cb.out_len[i];
    }
}

void write_descriptors(uint8_t* H, const std::vector<ImgPlan>& plans, const Prepared& P)
{
    for (size_t i = 0; i < plans.size(); i++) memcpy(H + P.o_img + i * sizeof(DevImage), &plans[i].di, sizeof(DevImage));
    if (!P.items.empty()) memcpy(H + P.o_items, P.items.data(), P.items.size() * sizeof(BandItem));
    if (!P.ritems.empty()) memcpy(H + P.o_ritems, P.ritems.data(), P.ritems.size() * sizeof(BandItem));
    if (!P.witems.empty()) memcpy(H + P.o_witems, P.witems.data(), P.witems.size() * sizeof(BandItem));
    if (!P.blocks.empty()) memcpy(H + P.o_blocks, P.blocks.data(), P.blocks.size() * sizeof(BlockOut));
}

// Launch the stage kernels over a planned, uploaded work list at base A.
// With tmask != null, tev[k] is recorded before stage k (and tev[6] after
// the last) and *tmask gets the stages that ran.
int launch_stages(r2p_engine* e, int n, const Prepared& P, uint8_t* A, int stages, cudaStream_t s,
                         cudaEvent_t* tev, uint32_t* tmask)
{
    DevImage* dimg = reinterpret_cast<DevImage*>(A + P.o_img);
    BandItem* ditems = reinterpret_cast<BandItem*>(A + P.o_items);
    BlockOut* dblocks = reinterpret_cast<BlockOut*>(A + P.o_blocks);
    auto mark = [&](int k, bool ran) -> cudaError_t {
        if (!tev) return cudaSuccess;
        if (ran) *tmask |= 1u << (k - 1);
        return cudaEventRecord(tev[k], s);
    };
    const bool filt = (stages & ST_FILTER) != 0, defl = (stages & ST_DEFLATE) != 0, bmp = (stages & ST_BMP) != 0;
    const bool old_filt = filt && !P.items.empty(), reg_filt = filt && !P.ritems.empty();
    const bool rows_filt = filt && !P.witems.empty();
    R2P_CU(mark(0, false), "event");
    // window tables in HBM: only the shared-memory filter kernel and the BMP
    // export read them (the register kernel builds its table per CTA)
    if (old_filt || bmp) R2P_CU(launch_prepare_window(dimg, n, s), "k_prepare_window");
    R2P_CU(mark(1, old_filt || bmp), "event");
    if (old_filt) {
        const int grid = (int)std::min<size_t>(P.items.size(), (size_t)P.slots_total);
        R2P_CU(launch_window_filter(dimg, ditems, (int)P.items.size(), grid, P.smem, s), "k_window_filter");
    }
    if (reg_filt) {
        BandItem* dritems = reinterpret_cast<BandItem*>(A + P.o_ritems);
        const int grid = (int)std::min<size_t>(P.ritems.size(), (size_t)P.rslots);
        R2P_CU(launch_window_filter_reg(dimg, dritems, (int)P.ritems.size(), grid, P.rnw, P.rsmem, s),
               "k_window_filter_reg");
    }
    if (rows_filt) {
        BandItem* dwitems = reinterpret_cast<BandItem*>(A + P.o_witems);
        const int grid = (int)std::min<size_t>(P.witems.size(), (size_t)P.wslots);
        R2P_CU(launch_filter_rows(dimg, n, P.wlut, P.wstash, dwitems, (int)P.witems.size(), grid, s),
               "k_filter_rows");
    }
    if (bmp) R2P_CU(launch_bmp(dimg, n, P.bmp_words, e->nsm, s), "k_bmp_file");   // timed in the filter's slot
    R2P_CU(mark(2, filt || bmp), "event");
    const int bgrid = (int)std::min<uint64_t>(P.nblk, (uint64_t)e->nsm * 8);
    if (defl && P.any_stored)
        R2P_CU(launch_stored(dimg, dblocks, (int)P.nblk, P.max_block, e->d_xpow, bgrid, s), "k_stored_blocks");
    R2P_CU(mark(3, defl && P.any_stored), "event");
    if (defl && P.any_lz)
        R2P_CU(launch_lz77(dimg, dblocks, (int)P.nblk, P.max_block, A + P.o_scratch, P.slot, e->d_xpow, bgrid,
                           P.hash_bits, s),
               "k_lz77_blocks");
    if (defl && P.any_dyn)
        R2P_CU(launch_dyn(dimg, dblocks, (int)P.nblk, P.max_block, A + P.o_scratch, P.slot, e->d_xpow, e->nsm, s),
               "k_rle_dyn_blocks");                      // timed in the LZ77 slot
    R2P_CU(mark(4, defl && (P.any_lz || P.any_dyn)), "event");
    if (defl) {
        const int parts = finish_parts((int)P.nblk, e->nsm);
        const int fgrid = (int)std::min<uint64_t>(P.nblk * (uint64_t)parts, (uint64_t)e->nsm * 8);
        R2P_CU(launch_finish(dimg, dblocks, (int)P.nblk, parts, A + P.o_scratch, P.slot, e->d_xpow, fgrid, s),
               "k_finish");
    }
    R2P_CU(mark(5, defl), "event");
    R2P_CU(mark(6, false), "event");   // the block gather runs inside k_finish
    return R2P_OK;
}

// A graph replay launches the captured kernels of a whole encode again.
void note_launch_graph(const Prepared& P)
{
    const bool lz = P.any_lz, dyn = P.any_dyn;
    const uint32_t n = (P.items.empty() ? 0u : 2u) + (P.ritems.empty() ? 0u : 1u) + (P.witems.empty() ? 0u : 2u) +
                       1u /* finish */ +
                       (P.any_stored ? 1u : 0u) + (lz ? 1u : 0u) + (dyn ? 1u : 0u);
    g_launches.fetch_add(n, std::memory_order_relaxed);
}

// Plan into the engine arena, make sure it and the staging area are large
// enough, and order this call after the previous one on `s`.  *extra
// receives extra_bytes of arena space for the caller.
int prepare(r2p_engine* e, std::vector<ImgPlan>& plans, const CallBuffers& cb, size_t extra_bytes,
                   cudaStream_t s, Prepared& P, uint8_t** extra)
{
    plan_work(e, plans, cb, extra_bytes, P);
    int rc = ensure_arena(e, P.total);
    if (rc) return rc;
    rc = ensure_stage(e, P.desc_bytes, &P.stage_slot);
    if (rc) return rc;
    if (e->have_done) R2P_CU(cudaStreamWaitEvent(s, e->done, 0), "order calls");
    if (extra) *extra = e->arena + P.o_extra;
    return R2P_OK;
}

// With stage timing on, the next record of R2P_STAGE_COUNT + 1 events (and
// its stage mask) for one launch of the stages; nothing when timing is off.
int timing_slot(r2p_engine* e, cudaEvent_t** tev, uint32_t** tmask)
{
    *tev = nullptr;
    *tmask = nullptr;
    if (!e->timing) return R2P_OK;
    if (e->tused == e->trec.size()) {
        std::vector<cudaEvent_t> v(R2P_STAGE_COUNT + 1);
        for (auto& ev : v) R2P_CU(cudaEventCreate(&ev), "cudaEventCreate");
        e->trec.push_back(v);
        e->tmask.push_back(0);
    }
    *tev = e->trec[e->tused].data();
    e->tmask[e->tused] = 0;
    *tmask = &e->tmask[e->tused];
    e->tused++;
    return R2P_OK;
}

// Fill the device pointers, upload the descriptors and launch the stages.
int launch(r2p_engine* e, std::vector<ImgPlan>& plans, const CallBuffers& cb, Prepared& P, int stages,
                  cudaStream_t s)
{
    const int n = (int)plans.size();
    uint8_t* A = e->arena;
    fill_pointers(plans, cb, P, A);
    const int k = P.stage_slot;
    write_descriptors(e->h_stage[k], plans, P);
    R2P_CU(cudaMemcpyAsync(A, e->h_stage[k], P.desc_bytes, cudaMemcpyHostToDevice, s), "descriptor upload");
    R2P_CU(cudaEventRecord(e->staged[k], s), "event");
    e->stage_used[k] = true;
    e->stage_idx = (k + 1) % r2p_engine::kStageRing;
    cudaEvent_t* tev = nullptr;
    uint32_t* tmask = nullptr;
    int rc = timing_slot(e, &tev, &tmask);
    if (rc) return rc;
    rc = launch_stages(e, n, P, A, stages, s, tev, tmask);
    if (rc) return rc;
    R2P_CU(cudaEventRecord(e->done, s), "event");
    e->have_done = true;
    return R2P_OK;
}

int run(r2p_engine* e, std::vector<ImgPlan>& plans, CallBuffers& cb, int stages, cudaStream_t s)
{
    Prepared P;
    int rc = prepare(e, plans, cb, 0, s, P, nullptr);
    if (rc) return rc;
    return launch(e, plans, cb, P, stages, s);
}

int bind(r2p_engine* e)
{
    R2P_CU(cudaSetDevice(e->device), "cudaSetDevice");
    return R2P_OK;
}

}  // namespace r2p


// status message hook for the other translation units of the library
int r2p_internal_set_error(int code, const char* msg) { return r2p::set_err(code, msg); }

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int r2p_version(void) { return 10000; }

const char* r2p_status_string(int st)
{
    switch (st) {
        case R2P_OK: return "ok";
        case R2P_EINVAL: return "invalid argument";
        case R2P_ENOMEM: return "out of memory";
        case R2P_EBUDGET: return "HBM budget exceeded";
        case R2P_ECUDA: return "CUDA error";
        case R2P_ETIMEOUT: return "timed out";
        case R2P_ENOSPC: return "output buffer too small";
        case R2P_ECANCELED: return "cancelled";
        case R2P_ENOTFOUND: return "unknown ticket";
        default: return "unknown status";
    }
}

const char* r2p_last_error(void) { return t_last_error.c_str(); }

uint64_t r2p_kernel_launch_count(void) { return g_launches.load(); }

int r2p_engine_create(int device, size_t hbm_budget, r2p_engine** out)
{
    if (!out) return set_err(R2P_EINVAL, "out is NULL");
    *out = nullptr;
    int ndev = 0;
    R2P_CU(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount");
    if (device < 0 || device >= ndev) return set_err(R2P_EINVAL, "no such device");
    r2p_engine* e = new r2p_engine();
    e->device = device;
    e->budget = hbm_budget;
    cudaError_t ce = cudaSetDevice(device);
    if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&e->nsm, cudaDevAttrMultiProcessorCount, device);
    std::vector<uint32_t> tab;
    build_xpow(tab);
    if (ce == cudaSuccess) ce = cudaMalloc(&e->d_xpow, tab.size() * 4);
    if (ce == cudaSuccess) ce = cudaMemcpy(e->d_xpow, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->done, cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&e->hstream, cudaStreamNonBlocking);
    for (int k = 0; k < r2p_engine::kStageRing && ce == cudaSuccess; k++)
        ce = cudaEventCreateWithFlags(&e->staged[k], cudaEventDisableTiming);
    if (ce != cudaSuccess) {
        r2p_engine_destroy(e);
        return cuda_err(ce, "r2p_engine_create");
    }
    *out = e;
    return R2P_OK;
}

void r2p_engine_destroy(r2p_engine* e)
{
    if (!e) return;
    cudaSetDevice(e->device);
    if (e->have_done) cudaEventSynchronize(e->done);
    if (e->arena) cudaFree(e->arena);
    if (e->d_xpow) cudaFree(e->d_xpow);
    for (int k = 0; k < r2p_engine::kStageRing; k++) {
        if (e->h_stage[k]) cudaFreeHost(e->h_stage[k]);
        if (e->staged[k]) cudaEventDestroy(e->staged[k]);
    }
    if (e->done) cudaEventDestroy(e->done);
    if (e->hstream) {
        cudaStreamSynchronize(e->hstream);
        cudaStreamDestroy(e->hstream);
    }
    for (r2p_engine* h : e->helpers) r2p_engine_destroy(h);
    for (int k = 0; k < R2P_MANY_SLOTS; k++) {
        if (e->many_dl[k]) {
            cudaStreamSynchronize(e->many_dl[k]);
            cudaStreamDestroy(e->many_dl[k]);
        }
        if (e->many_dl_ev[k]) cudaEventDestroy(e->many_dl_ev[k]);
    }
    for (auto ev : e->many_ev)
        if (ev) cudaEventDestroy(ev);
    if (e->many_lens) cudaFreeHost(e->many_lens);
    for (auto& v : e->trec)
        for (auto ev : v) cudaEventDestroy(ev);
    delete e;
}

size_t r2p_png_bound(const r2p_image* img)
{
    if (!img) return 0;
    // Any engine's tuning table may pick blocks down to 1024 bytes, each with
    // its 5-byte stored-block header, so bound with the smallest block unless
    // the image fixes its block size.
    r2p_image im = *img;
    if (im.block_size == 0) im.block_size = 1024;
    ImgPlan ip;
    if (plan_image(im, 0, ip)) return 0;
    return (size_t)ip.png_bound;
}

size_t r2p_zlib_bound(size_t len, int level, int block_size)
{
    (void)level;
    const int bs = block_size ? block_size : kBlock64;
    if (bs < 1024 || bs > kBlock64 || (bs & 15)) return 0;
    return 2 + len + (size_t)kStoredHdr * ((len + bs - 1) / bs + 1) + 4;
}

int r2p_encode_png_device(r2p_engine* e, const r2p_image* img, const void* d_pixels, void* d_png,
                          size_t png_cap, uint64_t* d_png_len, void* stream)
{
    if (!e || !img || !d_pixels || !d_png || !d_png_len) return set_err(R2P_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(e->mu);
    int rc = bind(e);
    if (rc) return rc;
    std::vector<ImgPlan> plans(1);
    rc = plan_image(*img, 0, plans[0], e->tuning);
    if (rc) return rc;
    if (png_cap < plans[0].png_bound) return set_err(R2P_ENOSPC, "png_cap below r2p_png_bound()");
    CallBuffers cb;
    cb.raw = {static_cast<const uint8_t*>(d_pixels)};
    cb.filt = {nullptr};
    cb.prior = {nullptr};
    cb.out = {static_cast<uint8_t*>(d_png)};
    cb.out_cap = {png_cap};
    cb.out_len = {d_png_len};
    return run(e, plans, cb, ST_ALL, static_cast<cudaStream_t>(stream));
}

int r2p_encode_batch_device(r2p_engine* e, int n, const r2p_image* imgs, const void* const* d_pixels,
                            void* const* d_pngs, const size_t* png_caps, uint64_t* d_png_lens, void* stream)
{
    if (!e || n < 1 || !imgs || !d_pixels || !d_pngs || !png_caps || !d_png_lens)
        return set_err(R2P_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(e->mu);
    int rc = bind(e);
    if (rc) return rc;
    std::vector<ImgPlan> plans((size_t)n);
    CallBuffers cb;
    for (int i = 0; i < n; i++) {
        rc = plan_image(imgs[i], 0, plans[i], e->tuning);
        if (rc) return rc;
        if (png_caps[i] < plans[i].png_bound) return set_err(R2P_ENOSPC, "png_cap below r2p_png_bound()");
        if (!d_pixels[i] || !d_pngs[i]) return set_err(R2P_EINVAL, "NULL buffer");
        cb.raw.push_back(static_cast<const uint8_t*>(d_pixels[i]));
        cb.filt.push_back(nullptr);
        cb.prior.push_back(nullptr);
        cb.out.push_back(static_cast<uint8_t*>(d_pngs[i]));
        cb.out_cap.push_back(png_caps[i]);
        cb.out_len.push_back(d_png_lens + i);
    }
    return run(e, plans, cb, ST_ALL, static_cast<cudaStream_t>(stream));
}

int r2p_encode_png(r2p_engine* e, const r2p_image* img, const void* h_pixels, void* h_png, size_t png_cap,
                   size_t* png_len)
{
    if (!e || !img || !h_pixels || !h_png || !png_len) return set_err(R2P_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(e->mu);
    int rc = bind(e);
    if (rc) return rc;
    std::vector<ImgPlan> plans(1);
    rc = plan_image(*img, 0, plans[0], e->tuning);
    if (rc) return rc;
    const size_t raw_bytes = (size_t)plans[0].raw_bytes;
    const size_t bound = (size_t)plans[0].png_bound;
    const size_t raw_region = align_up(raw_bytes + 16, 256), png_region = align_up(bound, 256);
    CallBuffers cb;
    cb.raw = {nullptr};
    cb.filt = {nullptr};
    cb.prior = {nullptr};
    cb.out = {nullptr};
    cb.out_cap = {bound};
    cb.out_len = {nullptr};
    cudaStream_t s = e->hstream;
    Prepared P;
    uint8_t* ext = nullptr;
    rc = prepare(e, plans, cb, raw_region + png_region + 256, s, P, &ext);
    if (rc) return rc;
    uint8_t* d_raw = ext;
    uint8_t* d_png = ext + raw_region;
    uint64_t* d_len = reinterpret_cast<uint64_t*>(d_png + png_region);
    cb.raw = {d_raw};
    cb.out = {d_png};
    cb.out_len = {d_len};
    R2P_CU(cudaMemcpyAsync(d_raw, h_pixels, raw_bytes, cudaMemcpyHostToDevice, s), "pixel upload");
    rc = launch(e, plans, cb, P, ST_ALL, s);
    if (rc) return rc;
    uint64_t len = 0;
    R2P_CU(cudaMemcpyAsync(&len, d_len, sizeof(len), cudaMemcpyDeviceToHost, s), "length download");
    R2P_CU(cudaStreamSynchronize(s), "sync");
    if (len >> 63) {
        const int st = (int)(len & 0xFF);
        return set_err(st, st == R2P_ETIMEOUT ? "a bounded device wait gave up (bulk copy did not land)"
                                              : "png buffer too small");
    }
    *png_len = (size_t)len;
    if (len > png_cap) return set_err(R2P_ENOSPC, "png_cap too small for the encoded PNG");
    R2P_CU(cudaMemcpyAsync(h_png, d_png, (size_t)len, cudaMemcpyDeviceToHost, s), "png download");
    R2P_CU(cudaStreamSynchronize(s), "sync");
    return R2P_OK;
}

// Extra arena bytes of one host-buffer image: raw pixels, the PNG, its length word.
static size_t host_call_extra(const ImgPlan& p)
{
    return align_up((size_t)p.raw_bytes + 16, 256) + align_up((size_t)p.png_bound, 256) + 256;
}

int r2p_encode_png_many(r2p_engine* e, int n, const r2p_image* imgs, const void* const* h_pixels,
                        void* const* h_pngs, const size_t* png_caps, size_t* png_lens, int* statuses)
{
    if (!e || n < 0 || (n > 0 && (!imgs || !h_pixels || !h_pngs || !png_caps || !png_lens)))
        return set_err(R2P_EINVAL, "NULL argument");
    if (n == 0) return R2P_OK;
    std::lock_guard<std::mutex> lk(e->mu);
    int rc = bind(e);
    if (rc) return rc;
    const int K = R2P_MANY_SLOTS;
    while ((int)e->helpers.size() < K) {
        r2p_engine* h = nullptr;
        rc = r2p_engine_create(e->device, e->budget, &h);
        if (rc) return rc;
        e->helpers.push_back(h);
    }
    if (!e->many_lens) R2P_CU(cudaMallocHost(&e->many_lens, sizeof(uint64_t) * K), "cudaMallocHost");
    for (int k = 0; k < K; k++) {
        if (!e->many_ev[k]) R2P_CU(cudaEventCreateWithFlags(&e->many_ev[k], cudaEventDisableTiming), "event");
        if (!e->many_dl[k]) R2P_CU(cudaStreamCreateWithFlags(&e->many_dl[k], cudaStreamNonBlocking), "stream");
        if (!e->many_dl_ev[k]) R2P_CU(cudaEventCreateWithFlags(&e->many_dl_ev[k], cudaEventDisableTiming), "event");
    }
    // plan every image first and size the helpers' arenas once: an arena must
    // not move while an earlier image's PNG download from it is queued
    std::vector<ImgPlan> plans(n);
    size_t need = 0;
    int first_err = R2P_OK;
    std::vector<int> st(n, R2P_OK);
    for (int i = 0; i < n; i++) {
        st[i] = plan_image(imgs[i], 0, plans[i], e->tuning);
        if (st[i]) {
            if (!first_err) first_err = st[i];
            continue;
        }
        std::vector<ImgPlan> one{plans[i]};
        CallBuffers cb;
        cb.raw = {nullptr}; cb.filt = {nullptr}; cb.prior = {nullptr}; cb.out = {nullptr};
        cb.out_cap = {plans[i].png_bound}; cb.out_len = {nullptr};
        Prepared P;
        plan_work(e, one, cb, host_call_extra(plans[i]), P);
        need = std::max(need, P.total);
    }
    for (r2p_engine* h : e->helpers) {
        std::lock_guard<std::mutex> hl(h->mu);
        h->tuning = e->tuning;
        rc = bind(h);
        if (!rc) rc = ensure_arena(h, need);
        if (rc) return rc;
    }
    struct Inflight {
        int img = -1;
        uint8_t* d_png = nullptr;
        bool dl = false;                  // a download from this slot's PNG region is queued
        size_t dl_len = 0;
    };
    std::vector<Inflight> fl(K);
    // the PNG of slot k's image: its length is on the host once the event fired
    auto finish = [&](int k) {
        const int j = fl[k].img;
        fl[k].img = -1;
        r2p_engine* h = e->helpers[k];
        const cudaError_t ce = cudaEventSynchronize(e->many_ev[k]);
        if (ce != cudaSuccess) {
            st[j] = cuda_err(ce, "length wait");
            return;
        }
        const uint64_t len = e->many_lens[k];
        if (len >> 63) {
            st[j] = set_err((int)(len & 0xFF), "device reported an error");
            return;
        }
        png_lens[j] = (size_t)len;
        if (len > png_caps[j]) {
            st[j] = set_err(R2P_ENOSPC, "png_cap too small for the encoded PNG");
            return;
        }
        // the length event fired, so the kernels that wrote the PNG are done
        cudaError_t c2 = cudaMemcpyAsync(h_pngs[j], fl[k].d_png, (size_t)len, cudaMemcpyDeviceToHost, e->many_dl[k]);
        if (c2 == cudaSuccess) c2 = cudaEventRecord(e->many_dl_ev[k], e->many_dl[k]);
        if (c2 != cudaSuccess) st[j] = cuda_err(c2, "png download");
        fl[k].dl = true;
        fl[k].dl_len = (size_t)len;
    };
    auto enqueue = [&](int k, int i) -> int {
        r2p_engine* h = e->helpers[k];
        std::lock_guard<std::mutex> hl(h->mu);
        std::vector<ImgPlan> one{plans[i]};
        const size_t raw_bytes = (size_t)plans[i].raw_bytes, bound = (size_t)plans[i].png_bound;
        const size_t raw_region = align_up(raw_bytes + 16, 256), png_region = align_up(bound, 256);
        CallBuffers cb;
        cb.raw = {nullptr}; cb.filt = {nullptr}; cb.prior = {nullptr}; cb.out = {nullptr};
        cb.out_cap = {bound}; cb.out_len = {nullptr};
        cudaStream_t s = h->hstream;
        Prepared P;
        uint8_t* ext = nullptr;
        int r = prepare(h, one, cb, host_call_extra(plans[i]), s, P, &ext);
        if (r) return r;
        uint8_t* d_raw = ext;
        uint8_t* d_png = ext + raw_region;
        uint64_t* d_len = reinterpret_cast<uint64_t*>(d_png + png_region);
        cb.raw = {d_raw}; cb.out = {d_png}; cb.out_len = {d_len};
        // the slot's previous PNG may still be downloading: the upload may run
        // beside it when it lands elsewhere in the arena (images of one size
        // share a layout), the kernels only after it
        const bool clash = fl[k].dl && d_raw < fl[k].d_png + fl[k].dl_len && fl[k].d_png < d_raw + raw_bytes;
        if (clash) R2P_CU(cudaStreamWaitEvent(s, e->many_dl_ev[k], 0), "order download");
        R2P_CU(cudaMemcpyAsync(d_raw, h_pixels[i], raw_bytes, cudaMemcpyHostToDevice, s), "pixel upload");
        if (fl[k].dl && !clash) R2P_CU(cudaStreamWaitEvent(s, e->many_dl_ev[k], 0), "order download");
        r = launch(h, one, cb, P, ST_ALL, s);
        if (r) return r;
        R2P_CU(cudaMemcpyAsync(e->many_lens + k, d_len, sizeof(uint64_t), cudaMemcpyDeviceToHost, s), "length");
        R2P_CU(cudaEventRecord(e->many_ev[k], s), "event");
        fl[k].img = i;
        fl[k].d_png = d_png;
        return R2P_OK;
    };
    int slot = 0;
    for (int i = 0; i < n; i++) {
        if (st[i]) continue;
        const int k = slot;
        slot = (slot + 1) % K;
        if (fl[k].img >= 0) finish(k);
        const int r = enqueue(k, i);
        if (r) st[i] = r;
    }
    for (int k = 0; k < K; k++)
        if (fl[k].img >= 0) finish(k);
    for (int k = 0; k < K; k++) {
        r2p_engine* h = e->helpers[k];
        cudaError_t ce = cudaStreamSynchronize(h->hstream);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->many_dl[k]);
        if (ce != cudaSuccess && !first_err) first_err = cuda_err(ce, "sync");
    }
    for (int i = 0; i < n; i++) {
        if (statuses) statuses[i] = st[i];
        if (st[i] && !first_err) first_err = st[i];
    }
    return first_err ? set_err(first_err, "at least one image failed") : R2P_OK;
}

int r2p_window_filter_device(r2p_engine* e, const r2p_image* img, const void* d_pixels, const void* d_prior,
                             void* d_filtered, void* stream)
{
    return r2p_window_filter_device_ex(e, img, d_pixels, d_prior, d_filtered, nullptr, stream);
}

int r2p_window_filter_device_ex(r2p_engine* e, const r2p_image* img, const void* d_pixels, const void* d_prior,
                                void* d_filtered, void* d_last_row, void* stream)
{
    if (!e || !img || !d_pixels || !d_filtered) return set_err(R2P_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(e->mu);
    int rc = bind(e);
    if (rc) return rc;
    std::vector<ImgPlan> plans(1);
    rc = plan_image(*img, 0, plans[0], e->tuning);
    if (rc) return rc;
    CallBuffers cb;
    cb.raw = {static_cast<const uint8_t*>(d_pixels)};
    cb.filt = {static_cast<uint8_t*>(d_filtered)};
    cb.prior = {static_cast<const uint8_t*>(d_prior)};
    cb.last_row = {static_cast<uint8_t*>(d_last_row)};
    cb.out = {nullptr};
    cb.out_cap = {0};
    cb.out_len = {nullptr};
    return run(e, plans, cb, ST_FILTER, static_cast<cudaStream_t>(stream));
}

size_t r2p_bmp_bound(const r2p_image* img)
{
    if (!img) return 0;
    ImgPlan ip;
    if (plan_bmp(*img, ip)) return 0;
    return (size_t)ip.png_bound;
}

int r2p_encode_bmp_device(r2p_engine* e, const r2p_image* img, const void* d_pixels, void* d_bmp, size_t bmp_cap,
                          void* stream)
{
    if (!e || !img || !d_pixels || !d_bmp) return set_err(R2P_EINVAL, "NULL argument");
    if (reinterpret_cast<uintptr_t>(d_bmp) & 3) return set_err(R2P_EINVAL, "d_bmp must be 4-byte aligned");
    std::lock_guard<std::mutex> lk(e->mu);
    int rc = bind(e);
    if (rc) return rc;
    std::vector<ImgPlan> plans(1);
    rc = plan_bmp(*img, plans[0]);
    if (rc) return rc;
    if (bmp_cap < plans[0].png_bound) return set_err(R2P_ENOSPC, "bmp_cap below r2p_bmp_bound()");
    CallBuffers cb;
    cb.raw = {static_cast<const uint8_t*>(d_pixels)};
    cb.filt = {nullptr};
    cb.prior = {nullptr};
    cb.out = {static_cast<uint8_t*>(d_bmp)};
    cb.out_cap = {bmp_cap};
    cb.out_len = {nullptr};
    return run(e, plans, cb, ST_BMP, static_cast<cudaStream_t>(stream));
}

int r2p_encode_bmp(r2p_engine* e, const r2p_image* img, const void* h_pixels, void* h_bmp, size_t bmp_cap,
                   size_t* bmp_len)
{
    if (!e || !img || !h_pixels || !h_bmp || !bmp_len) return set_err(R2P_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(e->mu);
    int rc = bind(e);
    if (rc) return rc;
    std::vector<ImgPlan> plans(1);
    rc = plan_bmp(*img, plans[0]);
    if (rc) return rc;
    const size_t raw_bytes = (size_t)plans[0].raw_bytes;
    const size_t size = (size_t)plans[0].png_bound;
    *bmp_len = size;
    if (bmp_cap < size) return set_err(R2P_ENOSPC, "bmp_cap below r2p_bmp_bound()");
    const size_t raw_region = align_up(raw_bytes + 16, 256);
    CallBuffers cb;
    cb.raw = {nullptr};
    cb.filt = {nullptr};
    cb.prior = {nullptr};
    cb.out = {nullptr};
    cb.out_cap = {size};
    cb.out_len = {nullptr};
    cudaStream_t s = e->hstream;
    Prepared P;
    uint8_t* ext = nullptr;
    rc = prepare(e, plans, cb, raw_region + align_up(size, 256), s, P, &ext);
    if (rc) return rc;
    uint8_t* d_raw = ext;
    uint8_t* d_bmp = ext + raw_region;
    cb.raw = {d_raw};
    cb.out = {d_bmp};
    R2P_CU(cudaMemcpyAsync(d_raw, h_pixels, raw_bytes, cudaMemcpyHostToDevice, s), "pixel upload");
    rc = launch(e, plans, cb, P, ST_BMP, s);
    if (rc) return rc;
    R2P_CU(cudaMemcpyAsync(h_bmp, d_bmp, size, cudaMemcpyDeviceToHost, s), "bmp download");
    R2P_CU(cudaStreamSynchronize(s), "sync");
    return R2P_OK;
}

// One DEFLATE stream over device bytes: a zlib stream (out_kind 1) or raw
// DEFLATE (out_kind 2, optionally left open for a following stream part).
static int deflate_bytes(r2p_engine* e, const void* d_in, size_t len, int level, int block_size, int out_kind,
                         int open_end, void* d_out, size_t out_cap, uint64_t* d_out_len, void* stream);

int r2p_zlib_compress_device(r2p_engine* e, const void* d_in, size_t len, int level, int block_size,
                             void* d_out, size_t out_cap, uint64_t* d_out_len, void* stream)
{
    return deflate_bytes(e, d_in, len, level, block_size, 1, 0, d_out, out_cap, d_out_len, stream);
}

int r2p_deflate_raw_device(r2p_engine* e, const void* d_in, size_t len, int level, int block_size, int final_part,
                           void* d_out, size_t out_cap, uint64_t* d_out_len, void* stream)
{
    return deflate_bytes(e, d_in, len, level, block_size, 2, final_part ? 0 : 1, d_out, out_cap, d_out_len, stream);
}

static int deflate_bytes(r2p_engine* e, const void* d_in, size_t len, int level, int block_size, int out_kind,
                         int open_end, void* d_out, size_t out_cap, uint64_t* d_out_len, void* stream)
{
    if (!e || !d_in || !d_out || !d_out_len) return set_err(R2P_EINVAL, "NULL argument");
    if (len == 0 || len >= (1ull << 31)) return set_err(R2P_EINVAL, "len must be in [1, 2^31)");
    if (level < 0 || level > 9) return set_err(R2P_EINVAL, "level must be 0..9");
    const int bs = block_size ? block_size : kBlock64;
    if (bs < 1024 || bs > kBlock64 || (bs & 15)) return set_err(R2P_EINVAL, "bad block_size");
    if (out_cap < r2p_zlib_bound(len, level, block_size)) return set_err(R2P_ENOSPC, "out_cap below r2p_zlib_bound()");
    std::lock_guard<std::mutex> lk(e->mu);
    int rc = bind(e);
    if (rc) return rc;
    // The bytes are planned as one "image" whose filtered stream is d_in; only
    // the DEFLATE stages run.
    std::vector<ImgPlan> plans(1);
    DevImage& d = plans[0].di;
    memset(&d, 0, sizeof(d));
    d.width = 1; d.height = 1; d.channels = 1; d.ib = 1; d.ob = 1; d.rb = 0; d.bpp = 1;
    d.filt_bytes = len;
    d.level = level;
    d.block_size = bs;
    d.nblocks = (int32_t)((len + bs - 1) / bs);
    d.out_kind = out_kind;
    d.open_end = open_end;
    d.prefix = out_kind == 1 ? 2 : 0;
    d.req_mode = R2P_WINDOW_NONE;
    plans[0].smem = 0;
    plans[0].lreg = 0;
    plans[0].lut_cap = 256;
    CallBuffers cb;
    cb.raw = {nullptr};
    cb.filt = {static_cast<uint8_t*>(const_cast<void*>(d_in))};
    cb.prior = {nullptr};
    cb.out = {static_cast<uint8_t*>(d_out)};
    cb.out_cap = {out_cap};
    cb.out_len = {d_out_len};
    return run(e, plans, cb, ST_DEFLATE, static_cast<cudaStream_t>(stream));
}

int r2p_selftest_bounded_wait(int device, int arrive, uint32_t limit_us, int* status)
{
    if (!status) return set_err(R2P_EINVAL, "NULL argument");
    if (limit_us == 0 || limit_us > 1000000u) return set_err(R2P_EINVAL, "limit_us must be in [1, 1000000]");
    R2P_CU(cudaSetDevice(device), "cudaSetDevice");
    int* d = nullptr;
    R2P_CU(cudaMalloc(&d, sizeof(int)), "cudaMalloc");
    int h = -1;
    cudaError_t ce = cudaMemset(d, 0xFF, sizeof(int));
    if (ce == cudaSuccess) ce = launch_wait_probe(arrive ? 1 : 0, (uint64_t)limit_us * 1000ull, d, nullptr);
    if (ce == cudaSuccess) ce = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (ce != cudaSuccess) return cuda_err(ce, "bounded-wait probe");
    *status = h;
    return R2P_OK;
}

int r2p_adler32_device(r2p_engine* e, const void* d_data, size_t len, uint32_t* d_result, void* stream)
{
    if (!e || (!d_data && len) || !d_result) return set_err(R2P_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(e->mu);
    int rc = bind(e);
    if (rc) return rc;
    rc = ensure_arena(e, checksum_scratch_bytes(len));
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (e->have_done) R2P_CU(cudaStreamWaitEvent(s, e->done, 0), "order calls");
    R2P_CU(launch_checksum(static_cast<const uint8_t*>(d_data), len, true, d_result, e->arena, e->d_xpow,
                           e->nsm * 4, s), "k_checksum");
    R2P_CU(cudaEventRecord(e->done, s), "event");
    e->have_done = true;
    return R2P_OK;
}

int r2p_crc32_device(r2p_engine* e, const void* d_data, size_t len, uint32_t* d_result, void* stream)
{
    if (!e || (!d_data && len) || !d_result) return set_err(R2P_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(e->mu);
    int rc = bind(e);
    if (rc) return rc;
    rc = ensure_arena(e, checksum_scratch_bytes(len));
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (e->have_done) R2P_CU(cudaStreamWaitEvent(s, e->done, 0), "order calls");
    R2P_CU(launch_checksum(static_cast<const uint8_t*>(d_data), len, false, d_result, e->arena, e->d_xpow,
                           e->nsm * 4, s), "k_checksum");
    R2P_CU(cudaEventRecord(e->done, s), "event");
    e->have_done = true;
    return R2P_OK;
}

int r2p_engine_set_timing(r2p_engine* e, int enable)
{
    if (!e) return set_err(R2P_EINVAL, "NULL engine");
    std::lock_guard<std::mutex> lk(e->mu);
    e->timing = enable != 0;
    e->tused = 0;
    return R2P_OK;
}

int r2p_engine_stage_times(r2p_engine* e, double* ms, uint64_t* launches)
{
    if (!e || !ms) return set_err(R2P_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(e->mu);
    int rc = bind(e);
    if (rc) return rc;
    for (int k = 0; k < R2P_STAGE_COUNT; k++) {
        ms[k] = 0.0;
        if (launches) launches[k] = 0;
    }
    for (size_t c = 0; c < e->tused; c++) {
        auto& v = e->trec[c];
        R2P_CU(cudaEventSynchronize(v[R2P_STAGE_COUNT]), "cudaEventSynchronize");
        for (int k = 0; k < R2P_STAGE_COUNT; k++) {
            if (!(e->tmask[c] & (1u << k))) continue;
            float t = 0.f;
            R2P_CU(cudaEventElapsedTime(&t, v[k], v[k + 1]), "cudaEventElapsedTime");
            ms[k] += t;
            if (launches) launches[k]++;
        }
    }
    e->tused = 0;
    return R2P_OK;
}


int r2p_engine_set_tuning(r2p_engine* e, int n, const r2p_tuning* classes)
{
    if (!e || n < 0 || (n > 0 && !classes)) return set_err(R2P_EINVAL, "bad tuning table");
    std::vector<r2p_tuning> t;
    for (int i = 0; i < n; i++) {
        const r2p_tuning& c = classes[i];
        if (c.block_size < 1024 || c.block_size > kBlock64 || (c.block_size & 15) || c.band_rows < 0 ||
            (c.hash_bits != 9 && c.hash_bits != 10) || (i > 0 && c.max_raw_bytes <= classes[i - 1].max_raw_bytes))
            return set_err(R2P_EINVAL, "tuning class out of range or not sorted by max_raw_bytes");
        t.push_back(c);
    }
    if (t.empty()) t = kDefaultTuning;
    t.back().max_raw_bytes = ~0ull;   // the last class takes everything larger
    std::lock_guard<std::mutex> lk(e->mu);
    e->tuning = t;
    return R2P_OK;
}

int r2p_engine_get_tuning(r2p_engine* e, int cap, r2p_tuning* out, int* n)
{
    if (!e || !n || (cap > 0 && !out)) return set_err(R2P_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(e->mu);
    *n = (int)e->tuning.size();
    for (int i = 0; i < cap && i < *n; i++) out[i] = e->tuning[i];
    return R2P_OK;
}

uint32_t r2p_crc32_combine(uint32_t crc1, uint32_t crc2, uint64_t len2)
{
    static CrcPow pw = [] { CrcPow t; crc_init_pow(t); return t; }();
    return crc32_combine(crc1, crc2, len2, pw.p);
}

uint32_t r2p_adler32_combine(uint32_t a1, uint32_t a2, uint64_t len2) { return r2p::adler32_combine(a1, a2, len2); }

int r2p_device_alloc(size_t bytes, void** p)
{
    if (!p) return set_err(R2P_EINVAL, "NULL argument");
    R2P_CU(cudaMalloc(p, bytes ? bytes : 1), "cudaMalloc");
    return R2P_OK;
}
int r2p_device_free(void* p)
{
    R2P_CU(cudaFree(p), "cudaFree");
    return R2P_OK;
}
int r2p_host_alloc_pinned(size_t bytes, void** p)
{
    if (!p) return set_err(R2P_EINVAL, "NULL argument");
    R2P_CU(cudaMallocHost(p, bytes ? bytes : 1), "cudaMallocHost");
    return R2P_OK;
}
int r2p_host_free_pinned(void* p)
{
    R2P_CU(cudaFreeHost(p), "cudaFreeHost");
    return R2P_OK;
}
int r2p_memcpy(void* dst, const void* src, size_t bytes, void* stream)
{
    R2P_CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, static_cast<cudaStream_t>(stream)), "cudaMemcpyAsync");
    return R2P_OK;
}
int r2p_memset_device(void* p, int v, size_t bytes, void* stream)
{
    R2P_CU(cudaMemsetAsync(p, v, bytes, static_cast<cudaStream_t>(stream)), "cudaMemsetAsync");
    return R2P_OK;
}
int r2p_stream_create(void** s)
{
    if (!s) return set_err(R2P_EINVAL, "NULL argument");
    cudaStream_t st;
    R2P_CU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    *s = st;
    return R2P_OK;
}
int r2p_stream_destroy(void* s)
{
    R2P_CU(cudaStreamDestroy(static_cast<cudaStream_t>(s)), "cudaStreamDestroy");
    return R2P_OK;
}
int r2p_stream_synchronize(void* s)
{
    R2P_CU(cudaStreamSynchronize(static_cast<cudaStream_t>(s)), "cudaStreamSynchronize");
    return R2P_OK;
}
int r2p_event_create(void** ev)
{
    if (!ev) return set_err(R2P_EINVAL, "NULL argument");
    cudaEvent_t e;
    R2P_CU(cudaEventCreate(&e), "cudaEventCreate");
    *ev = e;
    return R2P_OK;
}
int r2p_event_destroy(void* ev)
{
    R2P_CU(cudaEventDestroy(static_cast<cudaEvent_t>(ev)), "cudaEventDestroy");
    return R2P_OK;
}
int r2p_event_record(void* ev, void* s)
{
    R2P_CU(cudaEventRecord(static_cast<cudaEvent_t>(ev), static_cast<cudaStream_t>(s)), "cudaEventRecord");
    return R2P_OK;
}
int r2p_stream_wait_event(void* s, void* ev)
{
    R2P_CU(cudaStreamWaitEvent(static_cast<cudaStream_t>(s), static_cast<cudaEvent_t>(ev), 0), "cudaStreamWaitEvent");
    return R2P_OK;
}
int r2p_event_elapsed_ms(void* a, void* b, float* ms)
{
    if (!ms) return set_err(R2P_EINVAL, "NULL argument");
    R2P_CU(cudaEventSynchronize(static_cast<cudaEvent_t>(b)), "cudaEventSynchronize");
    R2P_CU(cudaEventElapsedTime(ms, static_cast<cudaEvent_t>(a), static_cast<cudaEvent_t>(b)), "cudaEventElapsedTime");
    return R2P_OK;
}

}  // extern "C"

