// r2p_engine_impl.h -- internals shared by the host-side translation units
// of the C ABI: the engine (r2p_engine.cu: planning, per-call encodes,
// checksums, tuning), batches and their CUDA graphs (r2p_batch.cu) and the
// request server (r2p_server.cu).  Not part of the public interface.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "r2p_common.h"
#include "r2p_device.h"
#include "r2p_kernels.h"

namespace r2p {

// status message for r2p_last_error(); returns code
int set_err(int code, const char* what);
// a CUDA failure as a status (R2P_ENOMEM for allocation failures, else R2P_ECUDA)
int cuda_err(cudaError_t e, const char* where);

#define R2P_CU(call, where)                                     \
    do {                                                        \
        cudaError_t _e = (call);                                \
        if (_e != cudaSuccess) return cuda_err(_e, where);      \
    } while (0)

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

struct ImgPlan {
    DevImage di;
    uint64_t raw_bytes = 0;
    uint64_t lut_cap = 0;
    uint64_t png_bound = 0;
    int smem = 0;      // filter smem wanted
    int lreg = 0;      // worst-case LUT region
    int band_rows = 0; // rows per filter work item (0 = about 64 KB of filtered output)
    int hash_bits = 10;
    bool reg = false;  // rows fit the register-resident filter kernel (k_filter_reg.cu)
    int reg_w = 0;     // its warps per row
    int reg_lut = 0;   // its worst-case window table bytes
    bool rows = false; // rows wide enough for the warp-per-row filter kernel (k_filter_rows.cu)
};

// Rows at least this wide (filtered bytes) go to the warp-per-row filter
// kernel; narrower ones to the register-group kernel.  On the 1000-slice CT
// batch, 2048 moved the 2048- and 3072-pixel slices over and cut the batch's
// filter stage from 6.1 to 4.9 ms; 1024 gave the same batch and a slightly
// slower per-image path.
constexpr int kRowsMinRowBytes = 2048;

// Built-in size-class table (the autotuner's GB300 result).
extern const std::vector<r2p_tuning> kDefaultTuning;

int plan_image(const r2p_image& im, int out_kind, ImgPlan& ip, const std::vector<r2p_tuning>& tune = kDefaultTuning);
int plan_bmp(const r2p_image& im, ImgPlan& ip);

}  // namespace r2p

struct r2p_engine {
    int device = 0;
    size_t budget = 0;
    int nsm = 1;
    uint32_t* d_xpow = nullptr;
    uint8_t* arena = nullptr;
    size_t arena_cap = 0;
    // pinned staging ring for descriptor uploads: the host may run up to
    // kStageRing calls ahead of the device before reusing a slot
    static constexpr int kStageRing = 8;
    uint8_t* h_stage[kStageRing] = {};
    size_t stage_cap[kStageRing] = {};
    cudaEvent_t staged[kStageRing] = {};   // upload of the call that last used the slot
    bool stage_used[kStageRing] = {};
    int stage_idx = 0;
    cudaEvent_t done = nullptr;     // last kernel of the previous call
    bool have_done = false;
    // stream of the host-buffer entry points: engines driven from different
    // threads overlap their copies and kernels instead of sharing the
    // legacy default stream
    cudaStream_t hstream = nullptr;
    // r2p_encode_png_many: helper engines (own arena and stream each), the
    // pinned length words they read back, and their events
    std::vector<r2p_engine*> helpers;
    uint64_t* many_lens = nullptr;
    cudaEvent_t many_ev[R2P_MANY_SLOTS] = {};
    // per slot: the PNG download runs on its own stream, so the next image's
    // upload overlaps it; the next image's kernels wait for its event
    cudaStream_t many_dl[R2P_MANY_SLOTS] = {};
    cudaEvent_t many_dl_ev[R2P_MANY_SLOTS] = {};
    std::mutex mu;
    // stage timing (events between stage launches on the call's stream)
    bool timing = false;
    std::vector<std::vector<cudaEvent_t>> trec;   // per timed call: R2P_STAGE_COUNT + 1 events
    std::vector<uint32_t> tmask;                  // stages each timed call launched
    size_t tused = 0;
    std::vector<r2p_tuning> tuning = r2p::kDefaultTuning;
};

namespace r2p {

// Bump allocator over one plan's arena layout.
struct Layout {
    size_t off = 0;
    size_t take(size_t bytes)
    {
        const size_t o = off;
        off = align_up(off + bytes, 256);
        return o;
    }
};

struct CallBuffers {
    // per image, caller-provided or arena
    std::vector<const uint8_t*> raw;
    std::vector<uint8_t*> filt;
    std::vector<const uint8_t*> prior;
    std::vector<uint8_t*> last_row;     // optional; empty = none
    std::vector<uint8_t*> out;
    std::vector<uint64_t> out_cap;
    std::vector<uint64_t*> out_len;
};

enum Stages { ST_FILTER = 1, ST_DEFLATE = 2, ST_ALL = 3, ST_BMP = 4 };

static int ensure_arena(r2p_engine* e, size_t need)
{
    if (need <= e->arena_cap) return R2P_OK;
    if (e->budget && need > e->budget) return set_err(R2P_EBUDGET, "request exceeds the engine's HBM budget");
    if (e->have_done) R2P_CU(cudaEventSynchronize(e->done), "arena wait");
    if (e->arena) cudaFree(e->arena);
    e->arena = nullptr;
    e->arena_cap = 0;
    size_t cap = align_up(need + need / 4, 1 << 20);
    if (e->budget && cap > e->budget) cap = need;
    R2P_CU(cudaMalloc(&e->arena, cap), "arena cudaMalloc");
    e->arena_cap = cap;
    return R2P_OK;
}

// Take the next staging slot, waiting for the upload that last used it and
// growing it to `need` bytes.
static int ensure_stage(r2p_engine* e, size_t need, int* slot)
{
    const int k = e->stage_idx;
    if (e->stage_used[k]) R2P_CU(cudaEventSynchronize(e->staged[k]), "staging wait");
    if (need > e->stage_cap[k]) {
        if (e->h_stage[k]) cudaFreeHost(e->h_stage[k]);
        e->h_stage[k] = nullptr;
        e->stage_cap[k] = 0;
        const size_t cap = align_up(need * 2, 1 << 16);
        R2P_CU(cudaMallocHost(&e->h_stage[k], cap), "staging cudaMallocHost");
        e->stage_cap[k] = cap;
    }
    *slot = k;
    return R2P_OK;
}

// One call's work list and memory layout.
struct Prepared {
    std::vector<BandItem> items;       // bands of the shared-memory filter kernel
    std::vector<BandItem> ritems;      // bands of the register-resident filter kernel
    std::vector<BandItem> witems;      // bands of the warp-per-row filter kernel
    std::vector<BlockOut> blocks;
    int smem = 0, slots_total = 0, max_block = 0;
    int rnw = 0, rsmem = 0, rslots = 0;   // register kernel: warps per CTA, shared memory, CTA slots
    int wsmem = 0, wslots = 0, wlut = 0;  // warp-per-row kernel: shared memory, CTA slots, largest table
    int wstash = 0;                       // its per-warp stash of windowed rows (bytes; 0 = none)
    uint32_t nblk = 0;
    bool any_lz = false, any_stored = false, any_dyn = false;
    uint64_t slot = 0;
    size_t o_img = 0, o_items = 0, o_ritems = 0, o_witems = 0, o_blocks = 0, desc_bytes = 0, o_lut = 0, o_filt = 0, o_scratch = 0,
           o_extra = 0;
    size_t total = 0;
    int hash_bits = 10;
    int stage_slot = 0;
    uint32_t bmp_words = 0;    // 4-byte words of the largest BMP file
};

void plan_work(r2p_engine* e, std::vector<ImgPlan>& plans, const CallBuffers& cb, size_t extra_bytes, Prepared& P);
void fill_pointers(std::vector<ImgPlan>& plans, const CallBuffers& cb, const Prepared& P, uint8_t* A);
void write_descriptors(uint8_t* H, const std::vector<ImgPlan>& plans, const Prepared& P);
int launch_stages(r2p_engine* e, int n, const Prepared& P, uint8_t* A, int stages, cudaStream_t s, cudaEvent_t* tev,
                  uint32_t* tmask);
void note_launch_graph(const Prepared& P);
int timing_slot(r2p_engine* e, cudaEvent_t** tev, uint32_t** tmask);
int prepare(r2p_engine* e, std::vector<ImgPlan>& plans, const CallBuffers& cb, size_t extra_bytes, cudaStream_t s,
            Prepared& P, uint8_t** extra);
int launch(r2p_engine* e, std::vector<ImgPlan>& plans, const CallBuffers& cb, Prepared& P, int stages,
           cudaStream_t s);
int run(r2p_engine* e, std::vector<ImgPlan>& plans, CallBuffers& cb, int stages, cudaStream_t s);
int bind(r2p_engine* e);

}  // namespace r2p

// One part of a batch: its own work list and memory, launched as its own
// branch of the batch's graph.
struct BatchPart {
    std::vector<r2p::ImgPlan> plans;
    r2p::CallBuffers cb;
    r2p::Prepared P;
    size_t off = 0;                   // of the part's descriptors + scratch in mem
};

struct r2p_batch {
    r2p_engine* eng = nullptr;
    int n = 0;
    std::vector<BatchPart> parts;
    uint8_t* mem = nullptr;           // descriptors + tables + scratch of every part, owned
    size_t total = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};
