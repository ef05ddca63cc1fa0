// r2p_batch.cu -- reusable batches: one plan over many images, launched
// directly or replayed as a CUDA graph (part of the C ABI of include/r2p.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "r2p_engine_impl.h"

using namespace r2p;

extern "C" {

// Batches of at least this many images are split into kBatchParts parts
// (size-balanced: images dealt out by decreasing size) whose stage kernels
// run as parallel branches of one graph, so one part's stage tails overlap
// another's work; each image's bytes do not depend on its part.
constexpr int kBatchParts = 4;
constexpr int kBatchSplitMin = 64;

int r2p_batch_create(r2p_engine* e, int n, const r2p_image* imgs, const void* const* d_pixels, void* const* d_pngs,
                     const size_t* png_caps, uint64_t* d_png_lens, r2p_batch** out)
{
    if (!e || n < 1 || !imgs || !d_pixels || !d_pngs || !png_caps || !d_png_lens || !out)
        return set_err(R2P_EINVAL, "NULL argument");
    *out = nullptr;
    std::lock_guard<std::mutex> lk(e->mu);
    int rc = bind(e);
    if (rc) return rc;
    std::vector<ImgPlan> all((size_t)n);
    for (int i = 0; i < n; i++) {
        rc = plan_image(imgs[i], 0, all[i], e->tuning);
        if (!rc && png_caps[i] < all[i].png_bound) rc = set_err(R2P_ENOSPC, "png_cap below r2p_png_bound()");
        if (!rc && (!d_pixels[i] || !d_pngs[i])) rc = set_err(R2P_EINVAL, "NULL buffer");
        if (rc) return rc;
    }
    const int K = n >= kBatchSplitMin ? kBatchParts : 1;
    std::vector<int> order((size_t)n);
    for (int i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int x, int y) { return all[x].raw_bytes > all[y].raw_bytes; });
    r2p_batch* b = new r2p_batch();
    b->eng = e;
    b->n = n;
    b->parts.resize((size_t)K);
    for (int j = 0; j < n; j++) {
        const int i = order[j];
        BatchPart& pt = b->parts[(size_t)(j % K)];
        pt.plans.push_back(all[i]);
        pt.cb.raw.push_back(static_cast<const uint8_t*>(d_pixels[i]));
        pt.cb.filt.push_back(nullptr);
        pt.cb.prior.push_back(nullptr);
        pt.cb.out.push_back(static_cast<uint8_t*>(d_pngs[i]));
        pt.cb.out_cap.push_back(png_caps[i]);
        pt.cb.out_len.push_back(d_png_lens + i);
    }
    for (BatchPart& pt : b->parts) {
        plan_work(e, pt.plans, pt.cb, 0, pt.P);
        pt.off = b->total;
        b->total += align_up(pt.P.total, 256);
    }
    if (e->budget && b->total > e->budget) {
        delete b;
        return set_err(R2P_EBUDGET, "batch exceeds the engine's HBM budget");
    }
    cudaError_t ce = cudaMalloc(&b->mem, b->total);
    if (ce != cudaSuccess) {
        delete b;
        return cuda_err(ce, "batch cudaMalloc");
    }
    for (BatchPart& pt : b->parts) {
        fill_pointers(pt.plans, pt.cb, pt.P, b->mem + pt.off);
        std::vector<uint8_t> host(pt.P.desc_bytes);
        write_descriptors(host.data(), pt.plans, pt.P);
        ce = cudaMemcpy(b->mem + pt.off, host.data(), pt.P.desc_bytes, cudaMemcpyHostToDevice);
        if (ce != cudaSuccess) {
            cudaFree(b->mem);
            delete b;
            return cuda_err(ce, "batch descriptor upload");
        }
    }
    *out = b;
    return R2P_OK;
}

int r2p_batch_launch(r2p_batch* b, void* stream)
{
    if (!b) return set_err(R2P_EINVAL, "NULL batch");
    int rc = bind(b->eng);
    if (rc) return rc;
    // parts one after another on the stream; with the engine's stage timing
    // on, each part's stages are timed like an encode call's
    for (BatchPart& pt : b->parts) {
        cudaEvent_t* tev = nullptr;
        uint32_t* tmask = nullptr;
        rc = timing_slot(b->eng, &tev, &tmask);
        if (rc) return rc;
        rc = launch_stages(b->eng, (int)pt.plans.size(), pt.P, b->mem + pt.off, ST_ALL,
                           static_cast<cudaStream_t>(stream), tev, tmask);
        if (rc) return rc;
    }
    return R2P_OK;
}

// Capture every part's stage kernels into one graph: part 0 on the capture
// stream, the others on forked streams joined back before the capture ends.
static int capture_batch(r2p_batch* b, cudaStream_t cs)
{
    const int K = (int)b->parts.size();
    std::vector<cudaStream_t> fs((size_t)K, nullptr);
    std::vector<cudaEvent_t> ev((size_t)K, nullptr);
    int rc = R2P_OK;
    cudaError_t ce = cudaSuccess;
    for (int k = 0; k < K && ce == cudaSuccess; k++) {
        ce = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
        if (ce == cudaSuccess && k > 0) ce = cudaStreamCreateWithFlags(&fs[k], cudaStreamNonBlocking);
    }
    if (ce == cudaSuccess) ce = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
        fs[0] = cs;
        if (K > 1) ce = cudaEventRecord(ev[0], cs);
        for (int k = 1; k < K && ce == cudaSuccess; k++) ce = cudaStreamWaitEvent(fs[k], ev[0], 0);
        for (int k = 0; k < K && ce == cudaSuccess && !rc; k++)
            rc = launch_stages(b->eng, (int)b->parts[k].plans.size(), b->parts[k].P, b->mem + b->parts[k].off,
                               ST_ALL, fs[k], nullptr, nullptr);
        for (int k = 1; k < K && ce == cudaSuccess && !rc; k++) {
            ce = cudaEventRecord(ev[k], fs[k]);
            if (ce == cudaSuccess) ce = cudaStreamWaitEvent(cs, ev[k], 0);
        }
        cudaGraph_t g = nullptr;
        const cudaError_t ce2 = cudaStreamEndCapture(cs, &g);
        if (ce == cudaSuccess) ce = ce2;
        if (!rc && ce == cudaSuccess) {
            b->graph = g;
            ce = cudaGraphInstantiate(&b->exec, g, 0);
        } else if (g) {
            cudaGraphDestroy(g);
        }
    }
    for (int k = 1; k < K; k++)
        if (fs[k]) cudaStreamDestroy(fs[k]);
    for (auto x : ev)
        if (x) cudaEventDestroy(x);
    if (rc) return rc;
    if (ce != cudaSuccess) return cuda_err(ce, "graph capture");
    return R2P_OK;
}

int r2p_batch_launch_graph(r2p_batch* b, void* stream)
{
    if (!b) return set_err(R2P_EINVAL, "NULL batch");
    int rc = bind(b->eng);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!b->exec) {
        // capture on a private stream so the caller's stream state is untouched
        cudaStream_t cs;
        R2P_CU(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "cudaStreamCreate");
        rc = capture_batch(b, cs);
        cudaStreamDestroy(cs);
        if (rc) return rc;
    }
    R2P_CU(cudaGraphLaunch(b->exec, s), "cudaGraphLaunch");
    for (const BatchPart& pt : b->parts) note_launch_graph(pt.P);
    return R2P_OK;
}

size_t r2p_batch_device_bytes(const r2p_batch* b) { return b ? b->total : 0; }

void r2p_batch_destroy(r2p_batch* b)
{
    if (!b) return;
    cudaSetDevice(b->eng->device);
    cudaDeviceSynchronize();
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->mem) cudaFree(b->mem);
    delete b;
}

}  // extern "C"
