// k_window.cuh -- the window/level transforms shared by the filter kernels.
//
// Reference semantics:
//   windowing, 16-bit out: dicom_preprocess_kernel   src/gpu_filter.cu:71-162
//   windowing, 8-bit out : try_apply_linear_window   src/batch_processor.cpp:202-266
//                          build/apply_dicom16_lut   src/batch_processor.cpp:100-185
//                          dispatch                  src/batch_processor.cpp:397-409
//
// Float arithmetic uses explicit IEEE intrinsics (no contraction), matching
// the oracle's -ffp-contract=off restatement bit for bit.
#pragma once
#include <cuda_runtime.h>

#include "r2p_common.h"
#include "r2p_device.h"

namespace r2p {
// ---------------------------------------------------------------------------
// Window formulas
// ---------------------------------------------------------------------------

// DICOM PS3.3 window with output depth = BitsAllocated (src/gpu_filter.cu:82-154),
// applied to an already shifted-and-masked stored value (16-bit) or raw byte (8-bit).
__device__ inline uint32_t a2_eval(uint32_t m, const r2p_dicom_params& p)
{
    const int out_max = (p.bits_allocated == 16) ? 65535 : 255;
    float val;
    if (p.bits_allocated == 16) {
        if (p.pixel_rep == 1) {
            int32_t sv;
            if (p.bits_stored == 16) {
                sv = (int32_t)(int16_t)(uint16_t)m;
            } else {
                const int half = 1 << (p.bits_stored - 1);
                sv = (int32_t)m;
                if (sv >= half) sv -= (1 << p.bits_stored);
            }
            val = (float)sv;
        } else {
            val = (float)m;
        }
    } else {
        val = (p.pixel_rep == 1) ? (float)(int8_t)(uint8_t)m : (float)m;
    }
    if (p.apply_rescale) val = __fadd_rn(__fmul_rn(val, p.rescale_slope), p.rescale_intercept);
    if (p.apply_window) {
        const float wm1 = __fsub_rn(p.window_width, 1.0f);
        const float cen = p.window_center;
        if (wm1 <= 0.0f) {
            val = (val >= cen) ? (float)out_max : 0.0f;
        } else {
            const float half = __fmul_rn(wm1, 0.5f);
            const float lo = __fsub_rn(__fsub_rn(cen, half), 0.5f);
            const float hi = __fsub_rn(__fadd_rn(cen, half), 0.5f);
            if (val <= lo) {
                val = 0.0f;
            } else if (val > hi) {
                val = (float)out_max;
            } else {
                const float t = __fadd_rn(__fsub_rn(val, cen), 0.5f);
                const float q = __fdiv_rn(t, wm1);
                val = __fmul_rn(__fadd_rn(q, 0.5f), (float)out_max);
            }
        }
    }
    const float hi = (float)out_max;
    float v = (val < hi) ? val : hi;   // NaN -> hi, as fminf(hi, NaN)
    v = (v > 0.0f) ? v : 0.0f;
    return __float2uint_rz(v);
}

// Index into a window table: the stored value after shift and mask.
__device__ __forceinline__ uint32_t win_index(uint32_t raw, int shift, uint32_t mask)
{
    return (raw >> shift) & mask;
}

// FP32 table entry of build_dicom16_lut (src/batch_processor.cpp:100-147);
// with divide, the per-pixel formula of the BMP export, dicom16_row_to_gray8
// (src/pipeline.cpp:1894-1932, normalisation constants :1953-1963): the same
// steps except that the window divides by (hi - lo) where the table
// multiplies by its reciprocal.
__device__ inline uint8_t lut8_eval(int i, int lut_size, const r2p_dicom_params& p, bool divide = false)
{
    const int mask = lut_size - 1;
    float norm_scale = 1.f, norm_offset = 0.f;
    if (!p.apply_window) {
        if (p.pixel_rep == 1) {
            const float half = (float)(lut_size >> 1);
            const float range = (float)lut_size;
            norm_scale = __fdiv_rn(1.f, range);
            norm_offset = __fdiv_rn(half, range);
        } else {
            norm_scale = __fdiv_rn(1.f, (float)(lut_size - 1));
        }
    }
    float lo = 0.f, inv_range = 1.f;
    if (p.apply_window) {
        lo = __fsub_rn(p.window_center, __fmul_rn(p.window_width, 0.5f));
        const float hi = __fadd_rn(p.window_center, __fmul_rn(p.window_width, 0.5f));
        inv_range = (hi > lo) ? __fdiv_rn(1.f, __fsub_rn(hi, lo)) : 0.f;
    }
    float val;
    if (p.pixel_rep == 1 && p.bits_stored < 16) {
        const int sign_bit = lut_size >> 1;
        int32_t s = i;
        if (s & sign_bit) s |= ~mask;
        val = (float)s;
    } else if (p.pixel_rep == 1) {
        val = (float)(int16_t)(uint16_t)(unsigned)i;
    } else {
        val = (float)(unsigned)i;
    }
    if (p.apply_rescale) val = __fadd_rn(__fmul_rn(val, p.rescale_slope), p.rescale_intercept);
    float norm;
    if (p.apply_window && divide) {
        const float hi = __fadd_rn(p.window_center, __fmul_rn(p.window_width, 0.5f));
        norm = (hi > lo) ? __fdiv_rn(__fsub_rn(val, lo), __fsub_rn(hi, lo)) : 0.f;
    } else {
        norm = p.apply_window ? __fmul_rn(__fsub_rn(val, lo), inv_range)
                              : __fadd_rn(__fmul_rn(val, norm_scale), norm_offset);
    }
    const int v = __float2int_rz(__fadd_rn(__fmul_rn(norm, 255.f), 0.5f));
    return (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v);
}

// Q15 coefficients of try_apply_linear_window (src/batch_processor.cpp:202-251).
// Returns false when the reference would decline and fall back to the table.
__device__ inline bool q15_coeffs(const r2p_dicom_params& p, int32_t& A, int32_t& B)
{
    if (p.high_bit - p.bits_stored + 1 != 0) return false;
    float A_f, B_f;
    const float slope = p.apply_rescale ? p.rescale_slope : 1.f;
    const float intercept = p.apply_rescale ? p.rescale_intercept : 0.f;
    if (p.apply_window && p.window_width > 0.f) {
        const float lo = __fsub_rn(p.window_center, __fmul_rn(p.window_width, 0.5f));
        A_f = __fdiv_rn(__fmul_rn(slope, 255.f), p.window_width);
        B_f = __fdiv_rn(__fmul_rn(__fsub_rn(intercept, lo), 255.f), p.window_width);
    } else if (!p.apply_window) {
        const float range = (float)(1u << p.bits_stored);
        if (p.pixel_rep == 1) {
            const float half = __fmul_rn(range, 0.5f);
            A_f = __fdiv_rn(__fmul_rn(slope, 255.f), range);
            B_f = __fdiv_rn(__fmul_rn(__fadd_rn(intercept, half), 255.f), range);
        } else {
            const float r1 = __fsub_rn(range, 1.f);
            A_f = __fdiv_rn(__fmul_rn(slope, 255.f), r1);
            B_f = __fdiv_rn(__fmul_rn(intercept, 255.f), r1);
        }
    } else {
        return false;
    }
    const float A_q15 = __fmul_rn(A_f, 32768.f);
    if (A_q15 < -32767.f || A_q15 > 32767.f) return false;
    A = (int32_t)(int16_t)__float2int_rz(A_q15);
    const float bs = __fmul_rn(B_f, 32768.f);
    float bq;
    if (A_f >= 0.f) bq = (A_q15 == (float)__float2int_rz(A_q15)) ? bs : __fadd_rn(bs, 0.5f);
    else            bq = __fsub_rn(bs, 0.5f);
    B = __float2int_rz(bq);
    return true;
}

// Resolved window of one image: the transform and its table parameters,
// decided from the request as the reference's dispatch does
// (src/batch_processor.cpp:397-409 for 8-bit output, src/gpu_filter.cu:411
// for the DICOM formula).
struct WinRes {
    int mode;
    int32_t qa, qb, shift;
    uint32_t mask;
    int entries, esize;
};

__device__ inline WinRes resolve_window(const DevImage& d)
{
    WinRes r = {W_COPY, 0, 0, 0, 0u, 0, 0};
    const r2p_dicom_params& p = d.dp;
    if (d.req_mode == R2P_WINDOW_SWAP16) {
        r.mode = (d.ib == 2) ? W_SWAP16 : W_COPY;
    } else if (d.req_mode == R2P_WINDOW_DICOM16) {
        int entries, shift = 0;
        uint32_t mask;
        if (d.ib == 2) {
            const int bs = p.bits_stored;
            const int sh = p.high_bit - bs + 1;
            shift = sh > 0 ? sh : 0;
            mask = (bs < 16) ? ((1u << bs) - 1u) : 0xFFFFu;
            entries = (int)mask + 1;
        } else {
            mask = 0xFFu;
            entries = 256;
        }
        r.shift = shift;
        r.mask = mask;
        r.entries = entries;
        r.esize = d.ob;
        r.mode = (entries * d.ob <= kMaxSmemLut) ? W_A2_LUT : W_A2_DIRECT;
    } else if (d.req_mode == kReqBmp8) {
        r.entries = 1 << p.bits_stored;
        r.esize = 1;
        r.shift = p.high_bit - p.bits_stored + 1;
        r.mask = (uint32_t)(r.entries - 1);
        r.mode = W_LUT8;
    } else if (d.req_mode == R2P_WINDOW_BATCH8) {
        int32_t A, B;
        if (q15_coeffs(p, A, B)) {
            r.qa = A;
            r.qb = B;
            r.mode = W_Q15;
        } else {
            r.entries = 1 << p.bits_stored;
            r.esize = 1;
            r.shift = p.high_bit - p.bits_stored + 1;
            r.mask = (uint32_t)(r.entries - 1);
            r.mode = W_LUT8;
        }
    }
    return r;
}

// Entries [i0, n) step `step` of an image's window table (mode W_A2_LUT or
// W_LUT8) into lut: 16-bit entries byte-swapped, so that a little-endian
// 16-bit store gives PNG byte order.
__device__ inline void fill_window_table(const DevImage& d, const WinRes& r, uint8_t* lut, int i0, int step)
{
    if (r.mode == W_A2_LUT) {
        for (int i = i0; i < r.entries; i += step) {
            const uint32_t v = a2_eval((uint32_t)i, d.dp);
            if (d.ob == 2) reinterpret_cast<uint16_t*>(lut)[i] = (uint16_t)(((v & 0xFF) << 8) | (v >> 8));
            else           lut[i] = (uint8_t)v;
        }
    } else if (r.mode == W_LUT8) {
        const bool divide = d.req_mode == kReqBmp8;
        for (int i = i0; i < r.entries; i += step) lut[i] = lut8_eval(i, r.entries, d.dp, divide);
    }
}

struct WinCtx {
    int mode, ib, ob, shift;
    uint32_t mask;
    int32_t qa, qb;
    const uint8_t* lut;         // shared or global table
    r2p_dicom_params dp;
};

// Windowing kinds: the resolved WinMode split by sample and table sizes, so
// each row loop is compiled for exactly one transform.
enum WinKind : int {
    K_COPY = 0,      // bytes unchanged
    K_SWAP16 = 1,    // 16-bit LE -> BE
    K_LUT16 = 2,     // 16-bit in/out through a u16 table (entries in PNG byte order)
    K_LUT8IN = 3,    // 8-bit in/out through a u8 table
    K_DIRECT = 4,    // DICOM formula per sample (table too large)
    K_Q15 = 5,       // 16-bit in, 8-bit out, Q15 linear map
    K_LUT8 = 6,      // 16-bit in, 8-bit out, FP32-built table
};

__device__ __forceinline__ int win_kind(const WinCtx& w)
{
    switch (w.mode) {
        case W_COPY: return K_COPY;
        case W_SWAP16: return K_SWAP16;
        case W_A2_LUT: return w.ib == 2 ? K_LUT16 : K_LUT8IN;
        case W_Q15: return K_Q15;
        case W_LUT8: return K_LUT8;
        default: return K_DIRECT;
    }
}

// DICOM formula on one sample, in PNG byte order (kept out of line: rare).
static __device__ __noinline__ uint32_t win_direct(const WinCtx& w, uint32_t raw)
{
    const uint32_t m = (w.ib == 2) ? win_index(raw, w.shift, w.mask) : raw;
    const uint32_t v = a2_eval(m, w.dp);
    return (w.ob == 2) ? (((v & 0xFF) << 8) | (v >> 8)) : v;
}

// One sample (16-bit LE value or byte) of kind K; output in the low ob bytes,
// PNG byte order.
template <int K>
__device__ __forceinline__ uint32_t win_sample(const WinCtx& w, uint32_t raw)
{
    if (K == K_COPY) return raw;
    if (K == K_SWAP16) return ((raw & 0xFF) << 8) | (raw >> 8);
    if (K == K_LUT16) return reinterpret_cast<const uint16_t*>(w.lut)[win_index(raw, w.shift, w.mask)];
    if (K == K_LUT8IN) return w.lut[raw & w.mask];
    if (K == K_Q15) {
        const int32_t x = (w.dp.pixel_rep == 1) ? (int32_t)(int16_t)(uint16_t)raw : (int32_t)raw;
        const int32_t v = (int32_t)((uint32_t)x * (uint32_t)w.qa + (uint32_t)w.qb) >> 15;
        return (uint32_t)(v < 0 ? 0 : v > 255 ? 255 : v);
    }
    if (K == K_LUT8) return w.lut[(raw >> w.shift) & w.mask];
    return win_direct(w, raw);
}

// 16 raw bytes (one aligned unit) -> windowed output: 16 bytes (same depth)
// or 8 bytes (16 -> 8 bit, in o[0..1]).
template <int K>
__device__ __forceinline__ void win_unit(const WinCtx& w, const uint4 v, uint32_t o[4])
{
    const uint32_t wv[4] = {v.x, v.y, v.z, v.w};
    if (K == K_COPY) {
#pragma unroll
        for (int k = 0; k < 4; k++) o[k] = wv[k];
    } else if (K == K_SWAP16) {
#pragma unroll
        for (int k = 0; k < 4; k++) o[k] = __byte_perm(wv[k], 0, 0x2301);
    } else if (K == K_Q15 || K == K_LUT8) {
#pragma unroll
        for (int k = 0; k < 2; k++)
            o[k] = win_sample<K>(w, wv[2 * k] & 0xFFFF) | (win_sample<K>(w, wv[2 * k] >> 16) << 8) |
                   (win_sample<K>(w, wv[2 * k + 1] & 0xFFFF) << 16) | (win_sample<K>(w, wv[2 * k + 1] >> 16) << 24);
        o[2] = o[3] = 0;
    } else if (K == K_LUT16 || K == K_DIRECT) {
        if (K == K_LUT16 || w.ib == 2) {                         // 16-bit samples
#pragma unroll
            for (int k = 0; k < 4; k++)
                o[k] = win_sample<K>(w, wv[k] & 0xFFFF) | (win_sample<K>(w, wv[k] >> 16) << 16);
            return;
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {                              // K_DIRECT on 8-bit samples
            uint32_t acc = 0;
#pragma unroll
            for (int q = 0; q < 4; q++) acc |= win_sample<K>(w, (wv[k] >> (8 * q)) & 0xFF) << (8 * q);
            o[k] = acc;
        }
    } else {                                                       // K_LUT8IN: 8-bit samples
#pragma unroll
        for (int k = 0; k < 4; k++) {
            uint32_t acc = 0;
#pragma unroll
            for (int q = 0; q < 4; q++) acc |= win_sample<K>(w, (wv[k] >> (8 * q)) & 0xFF) << (8 * q);
            o[k] = acc;
        }
    }
}

}  // namespace r2p
