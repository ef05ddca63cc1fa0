// ref_gpu_runner.cpp -- test infrastructure: launches the reference's own
// window and filter kernels (dicom_preprocess_kernel, filter_select_kernel of
// src/gpu_filter.cu, compiled from the reference sources into cubins by
// oracle/build_oracle.py) through the CUDA driver API, with the launch shape
// of the reference's host code (src/gpu_filter.cu:414-434: 256 threads, one
// thread per sample for the window, one CTA per row for the filter).  Used on
// a GPU to record golden vectors (tests/golden/gen_gpu_golden.py) and, as a
// reported baseline, to time those kernels beside this encoder's (bench.py);
// nothing in the product loads it.
#include <cuda.h>

#include <cstdio>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct Mod {
    CUmodule mod = nullptr;
    CUfunction pre = nullptr, filt = nullptr;
};

std::vector<Mod> g_mods;
CUcontext g_ctx = nullptr;
std::string g_err;

bool ck(CUresult r, const char* what)
{
    if (r == CUDA_SUCCESS) return true;
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    g_err = std::string(what) + ": " + (s ? s : "unknown error");
    return false;
}

}  // namespace

extern "C" {

const char* rgr_error(void) { return g_err.c_str(); }

// Load a cubin; returns a handle >= 0 or -1.
int rgr_open(const char* cubin)
{
    if (!g_ctx) {
        CUdevice dev;
        if (!ck(cuInit(0), "cuInit") || !ck(cuDeviceGet(&dev, 0), "cuDeviceGet") ||
            !ck(cuDevicePrimaryCtxRetain(&g_ctx, dev), "cuDevicePrimaryCtxRetain"))
            return -1;
    }
    if (!ck(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent")) return -1;
    Mod m;
    if (!ck(cuModuleLoad(&m.mod, cubin), "cuModuleLoad")) return -1;
    unsigned int n = 0;
    if (!ck(cuModuleGetFunctionCount(&n, m.mod), "cuModuleGetFunctionCount")) return -1;
    std::vector<CUfunction> fs(n);
    if (n && !ck(cuModuleEnumerateFunctions(fs.data(), n, m.mod), "cuModuleEnumerateFunctions")) return -1;
    for (CUfunction f : fs) {
        const char* name = nullptr;
        if (cuFuncGetName(&name, f) != CUDA_SUCCESS || !name) continue;
        if (std::strstr(name, "dicom_preprocess_kernel")) m.pre = f;
        if (std::strstr(name, "filter_select_kernel")) m.filt = f;
    }
    if (!m.pre || !m.filt) {
        g_err = "kernels not found in the cubin";
        return -1;
    }
    g_mods.push_back(m);
    return (int)g_mods.size() - 1;
}

// One strip through the reference kernels: input rows (rows * width_bytes,
// DICOM little-endian samples when params is non-null), the prior row
// (width_bytes, or null = zeros), params = the 40-byte DicomPixelParams or
// null.  Writes the filtered strip (rows * (width_bytes + 1)) and, if
// out_pre is non-null, the preprocessed rows.  0 on success.
int rgr_run(int h, const unsigned char* input, const unsigned char* prior, int width_bytes, int bpp, int rows,
            const void* params, unsigned char* out_filtered, unsigned char* out_pre)
{
    if (h < 0 || h >= (int)g_mods.size() || width_bytes < 1 || rows < 1) {
        g_err = "bad arguments";
        return 1;
    }
    if (!ck(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent")) return 2;
    const Mod& m = g_mods[h];
    const size_t in_bytes = (size_t)rows * width_bytes, out_bytes = (size_t)rows * (width_bytes + 1);
    CUdeviceptr d_in = 0, d_prior = 0, d_sel = 0;
    int rc = 0;
    if (!ck(cuMemAlloc(&d_in, in_bytes + 256), "cuMemAlloc") || !ck(cuMemAlloc(&d_prior, width_bytes + 256), "cuMemAlloc") ||
        !ck(cuMemAlloc(&d_sel, out_bytes + 256), "cuMemAlloc")) {
        rc = 3;
    } else {
        std::vector<unsigned char> zeros(width_bytes, 0);
        bool good = ck(cuMemcpyHtoD(d_in, input, in_bytes), "HtoD") &&
                    ck(cuMemcpyHtoD(d_prior, prior ? prior : zeros.data(), width_bytes), "HtoD");
        if (good && params) {
            unsigned char p[40];
            std::memcpy(p, params, 40);
            int bits_alloc;
            std::memcpy(&bits_alloc, p, 4);
            int total = (int)(in_bytes / (size_t)(bits_alloc / 8));
            void* args[] = {&d_in, &total, p};
            good = ck(cuLaunchKernel(m.pre, (unsigned)((total + 255) / 256), 1, 1, 256, 1, 1, 0, nullptr, args, nullptr),
                      "launch dicom_preprocess_kernel");
        }
        if (good) {
            int wb = width_bytes, bp = bpp, nr = rows;
            void* args[] = {&d_in, &d_prior, &d_sel, &wb, &bp, &nr};
            good = ck(cuLaunchKernel(m.filt, (unsigned)rows, 1, 1, 256, 1, 1, 0, nullptr, args, nullptr),
                      "launch filter_select_kernel") &&
                   ck(cuCtxSynchronize(), "synchronize") && ck(cuMemcpyDtoH(out_filtered, d_sel, out_bytes), "DtoH") &&
                   (!out_pre || ck(cuMemcpyDtoH(out_pre, d_in, in_bytes), "DtoH"));
        }
        if (!good) rc = 4;
    }
    if (d_in) cuMemFree(d_in);
    if (d_prior) cuMemFree(d_prior);
    if (d_sel) cuMemFree(d_sel);
    return rc;
}

// Time the reference kernels over a whole image in strips of strip_rows rows,
// each strip as the reference's modern path runs it (src/pipeline.cpp:575-640
// with src/gpu_filter.cu:411-434): the window kernel in place (one thread per
// sample, 256 per CTA; skipped when params is null), then the filter kernel
// (one 256-thread CTA per row) with the previous strip's last windowed row as
// its prior row.  reps passes after one warm-up; the raw image is uploaded
// again before each pass, outside the timed launches.  *ms_pre / *ms_filt:
// mean device milliseconds per pass, CUDA events around every launch.
int rgr_time(int h, const unsigned char* input, int width_bytes, int bpp, int rows, int strip_rows,
             const void* params, int reps, double* ms_pre, double* ms_filt)
{
    if (h < 0 || h >= (int)g_mods.size() || width_bytes < 1 || rows < 1 || strip_rows < 1 || reps < 1) {
        g_err = "bad arguments";
        return 1;
    }
    if (!ck(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent")) return 2;
    const Mod& m = g_mods[h];
    int bits_alloc = 8;
    unsigned char p[40] = {0};
    if (params) {
        std::memcpy(p, params, 40);
        std::memcpy(&bits_alloc, p, 4);
    }
    // input bytes per row: the raw samples (16-bit in when the window
    // narrows nothing: width_bytes is the output row, the same size here)
    const size_t in_row = (size_t)width_bytes;
    const size_t in_bytes = (size_t)rows * in_row, out_bytes = (size_t)rows * (width_bytes + 1);
    CUdeviceptr d_in = 0, d_zero = 0, d_sel = 0;
    const int nstrips = (rows + strip_rows - 1) / strip_rows;
    std::vector<CUevent> ev((size_t)nstrips * 3, nullptr);
    int rc = 0;
    double tp = 0.0, tf = 0.0;
    bool good = ck(cuMemAlloc(&d_in, in_bytes + 256), "cuMemAlloc") &&
                ck(cuMemAlloc(&d_zero, in_row + 256), "cuMemAlloc") &&
                ck(cuMemAlloc(&d_sel, out_bytes + 256), "cuMemAlloc") &&
                ck(cuMemsetD8(d_zero, 0, in_row + 256), "cuMemsetD8");
    for (size_t i = 0; good && i < ev.size(); i++) good = ck(cuEventCreate(&ev[i], CU_EVENT_DEFAULT), "cuEventCreate");
    for (int pass = 0; good && pass <= reps; pass++) {
        good = ck(cuMemcpyHtoD(d_in, input, in_bytes), "HtoD") && ck(cuCtxSynchronize(), "synchronize");
        for (int s = 0; good && s < nstrips; s++) {
            const int r0 = s * strip_rows, n = std::min(strip_rows, rows - r0);
            CUdeviceptr strip = d_in + (CUdeviceptr)((size_t)r0 * in_row);
            CUdeviceptr prior = r0 == 0 ? d_zero : strip - (CUdeviceptr)in_row;
            CUdeviceptr sel = d_sel + (CUdeviceptr)((size_t)r0 * (width_bytes + 1));
            good = ck(cuEventRecord(ev[3 * s], nullptr), "cuEventRecord");
            if (good && params) {
                int total = (int)((size_t)n * in_row / (size_t)(bits_alloc / 8));
                void* args[] = {&strip, &total, p};
                good = ck(cuLaunchKernel(m.pre, (unsigned)((total + 255) / 256), 1, 1, 256, 1, 1, 0, nullptr, args,
                                         nullptr), "launch dicom_preprocess_kernel");
            }
            good = good && ck(cuEventRecord(ev[3 * s + 1], nullptr), "cuEventRecord");
            if (good) {
                int wb = width_bytes, bp = bpp, nr = n;
                void* args[] = {&strip, &prior, &sel, &wb, &bp, &nr};
                good = ck(cuLaunchKernel(m.filt, (unsigned)n, 1, 1, 256, 1, 1, 0, nullptr, args, nullptr),
                          "launch filter_select_kernel");
            }
            good = good && ck(cuEventRecord(ev[3 * s + 2], nullptr), "cuEventRecord");
        }
        good = good && ck(cuCtxSynchronize(), "synchronize");
        for (int s = 0; good && pass > 0 && s < nstrips; s++) {
            float a = 0.f, b = 0.f;
            good = ck(cuEventElapsedTime(&a, ev[3 * s], ev[3 * s + 1]), "cuEventElapsedTime") &&
                   ck(cuEventElapsedTime(&b, ev[3 * s + 1], ev[3 * s + 2]), "cuEventElapsedTime");
            tp += a;
            tf += b;
        }
    }
    if (!good) rc = 4;
    for (CUevent e : ev)
        if (e) cuEventDestroy(e);
    if (d_in) cuMemFree(d_in);
    if (d_zero) cuMemFree(d_zero);
    if (d_sel) cuMemFree(d_sel);
    if (!rc) {
        *ms_pre = tp / reps;
        *ms_filt = tf / reps;
    }
    return rc;
}

}  // extern "C"
