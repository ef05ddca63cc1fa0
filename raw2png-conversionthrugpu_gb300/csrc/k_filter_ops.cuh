// k_filter_ops.cuh -- per-byte operations shared by the window+filter
// kernels that hold rows in registers (k_filter_reg.cu, k_filter_rows.cu):
// filter scores, the Paeth predictor, left neighbours, one windowed 16-byte
// unit of a row, and the DICOM window table.
//
// Reference semantics:
//   adaptive filter : filter_select_kernel   src/gpu_filter.cu:183-309
//   windowing       : dicom_preprocess_kernel src/gpu_filter.cu:71-162 and
//                     the 8-bit forms of src/batch_processor.cpp:100-266
//                     (formulas in k_window.cuh)
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include "k_window.cuh"
#include "r2p_common.h"
#include "r2p_device.h"

namespace r2p {

// Words of a row each lane holds per unit: one 16-byte unit.
constexpr int kWPL = 4;
constexpr uint32_t kFull = 0xFFFFFFFFu;

// Sum over the four bytes of |a - b| (unsigned), plus acc.
__device__ __forceinline__ uint32_t sad4(uint32_t a, uint32_t b, uint32_t acc)
{
    uint32_t r;
    asm("vabsdiff4.u32.u32.u32.add %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(acc));
    return r;
}

// Per-byte floor((a + b) / 2).
__device__ __forceinline__ uint32_t avg4_dev(uint32_t a, uint32_t b)
{
    return (a & b) + ((a ^ b) & 0xFEFEFEFEu) / 2u;
}

// Paeth predictor of four bytes (PNG specification 9.4: pa = |b - c|,
// pb = |a - c|, pc = |a + b - 2c|, a if pa <= pb and pa <= pc, else b if
// pb <= pc, else c).  The bytes become fp16 values 1024 + v (exact), so the
// differences (up to +-510) and the comparisons are exact in packed halves.
// al, bl, cl: two bytes of a, b, c widened; returns the a-mask, mb the b-mask.
__device__ __forceinline__ uint32_t paeth_masks(uint32_t al, uint32_t bl, uint32_t cl, uint32_t& mb)
{
    const __half2 a = *reinterpret_cast<const __half2*>(&al);
    const __half2 b = *reinterpret_cast<const __half2*>(&bl);
    const __half2 c = *reinterpret_cast<const __half2*>(&cl);
    const __half2 A = __hsub2(a, c), B = __hsub2(b, c);
    const __half2 pa = __habs2(B), pb = __habs2(A), pc = __habs2(__hadd2(A, B));
    mb = __hle2_mask(pb, pc);
    return __hle2_mask(pa, __hmin2(pb, pc));
}

__device__ __forceinline__ uint32_t widen_lo(uint32_t v) { return __byte_perm(v, 0x64646464u, 0x4140); }
__device__ __forceinline__ uint32_t widen_hi(uint32_t v) { return __byte_perm(v, 0x64646464u, 0x4342); }

__device__ __forceinline__ uint32_t paeth_word(uint32_t a, uint32_t b, uint32_t c, uint32_t al, uint32_t ah,
                                               uint32_t bl, uint32_t bh, uint32_t cl, uint32_t ch)
{
    uint32_t mbl, mbh;
    const uint32_t mal = paeth_masks(al, bl, cl, mbl);
    const uint32_t mah = paeth_masks(ah, bh, ch, mbh);
    // 16-bit lane masks -> byte masks (bytes 0, 1 from the low pair, 2, 3 from the high pair)
    const uint32_t ma = __byte_perm(mal, mah, 0x6420);
    const uint32_t mb = __byte_perm(mbl, mbh, 0x6420);
    const uint32_t t = (b & mb) | (c & ~mb);
    return (a & ma) | (t & ~ma);
}

// Word q of the bytes bpp to the left of the lane's words x[0..kWPL), given
// the two words before x (m2, m1); dw = words reached back (1 or 2).
__device__ __forceinline__ uint32_t left_word(const uint32_t x[kWPL], uint32_t m1, uint32_t m2, int dw, uint32_t sh,
                                              int q)
{
    const uint32_t p1 = q >= 1 ? x[q - 1] : m1;
    if (dw == 1) return __funnelshift_r(p1, x[q], sh);
    const uint32_t p2 = q >= 2 ? x[q - 2] : q == 1 ? m1 : m2;
    return __funnelshift_r(p2, p1, sh);
}

// Window kinds of this kernel: those of k_window.cuh, plus K_LUT16Z, the
// 16-bit table whose index is the sample masked (no shift), read by byte
// offset so that an index costs two instructions.
constexpr int K_LUT16Z = 16;

// Window the lane's unit u (16 output bytes) of a staged raw row.
template <int K>
__device__ __forceinline__ void win_unit_row(const WinCtx& w, const uint8_t* slot, int u, uint32_t x[4])
{
    constexpr bool to8 = (K == K_Q15 || K == K_LUT8);
    if (K == K_LUT16Z) {
        const uint4 v = *reinterpret_cast<const uint4*>(slot + 16 * u);
        const uint32_t m2 = w.mask << 1;
        const uint32_t wv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint32_t lo = *reinterpret_cast<const uint16_t*>(w.lut + ((wv[k] << 1) & m2));
            const uint32_t hi = *reinterpret_cast<const uint16_t*>(w.lut + ((wv[k] >> 15) & m2));
            x[k] = __byte_perm(lo, hi, 0x5410);
        }
    } else if (to8) {
        uint32_t o[4];
        win_unit<K>(w, *reinterpret_cast<const uint4*>(slot + 32 * u), o);
        x[0] = o[0];
        x[1] = o[1];
        win_unit<K>(w, *reinterpret_cast<const uint4*>(slot + 32 * u + 16), o);
        x[2] = o[0];
        x[3] = o[1];
    } else {
        win_unit<K>(w, *reinterpret_cast<const uint4*>(slot + 16 * u), x);
    }
}

__device__ __forceinline__ void window_unit(int kind, const WinCtx& w, const uint8_t* slot, int u, uint32_t x[4])
{
    switch (kind) {
        case K_LUT16Z: win_unit_row<K_LUT16Z>(w, slot, u, x); break;
        case K_COPY: win_unit_row<K_COPY>(w, slot, u, x); break;
        case K_SWAP16: win_unit_row<K_SWAP16>(w, slot, u, x); break;
        case K_LUT16: win_unit_row<K_LUT16>(w, slot, u, x); break;
        case K_LUT8IN: win_unit_row<K_LUT8IN>(w, slot, u, x); break;
        case K_Q15: win_unit_row<K_Q15>(w, slot, u, x); break;
        default: win_unit_row<K_LUT8>(w, slot, u, x); break;
    }
}

// The DICOM window table (W_A2_LUT) with the formula of a2_eval, its one
// division per entry, t / (w - 1), done by Markstein's method: with
// y = RN(1 / b) (an IEEE reciprocal, once per image), q = RN(a y) and the
// exact remainder r = a - b q (one fma), RN(q + r y) is the correctly rounded
// a / b (P. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Dev. 34(1), 1990).  The window branch
// keeps |a / b| <= 1/2 and |a| >= 2^-25 or 0, so nothing over- or
// underflows while b lies in [2^-20, 2^60]; other b take __fdiv_rn.
__device__ inline void fill_a2_table_fast(const DevImage& d, const WinRes& r, uint8_t* lut, int i0, int step)
{
    const r2p_dicom_params p = d.dp;           // by value: the stores below cannot alias it
    const int ob = d.ob, entries = r.entries;
    const int out_max = (p.bits_allocated == 16) ? 65535 : 255;
    const float wm1 = __fsub_rn(p.window_width, 1.0f);
    const float cen = p.window_center;
    const float half = __fmul_rn(wm1, 0.5f);
    const float lo = __fsub_rn(__fsub_rn(cen, half), 0.5f);
    const float hi = __fsub_rn(__fadd_rn(cen, half), 0.5f);
    const bool fast = p.apply_window && wm1 >= 0x1p-20f && wm1 <= 0x1p60f;
    const float y = __frcp_rn(wm1);
    const float fmax_ = (float)out_max;
    if (fast && p.bits_allocated == 16 && p.pixel_rep == 0 && !p.apply_rescale && ob == 2) {
        // unsigned 16-bit samples, no rescale (the common DICOM case)
        for (int i = i0; i < entries; i += step) {
            float val = (float)i;
            if (val <= lo) {
                val = 0.0f;
            } else if (val > hi) {
                val = fmax_;
            } else {
                const float t = __fadd_rn(__fsub_rn(val, cen), 0.5f);
                const float q0 = __fmul_rn(t, y);
                const float q = __fmaf_rn(__fmaf_rn(-q0, wm1, t), y, q0);
                val = __fmul_rn(__fadd_rn(q, 0.5f), fmax_);
            }
            float c = (val < fmax_) ? val : fmax_;
            c = (c > 0.0f) ? c : 0.0f;
            const uint32_t v = __float2uint_rz(c);
            reinterpret_cast<uint16_t*>(lut)[i] = (uint16_t)(((v & 0xFF) << 8) | (v >> 8));
        }
        return;
    }
    for (int i = i0; i < entries; i += step) {
        uint32_t v;
        if (!fast) {
            v = a2_eval((uint32_t)i, p);
        } else {
            float val;
            if (p.bits_allocated == 16) {
                if (p.pixel_rep == 1) {
                    int32_t sv;
                    if (p.bits_stored == 16) {
                        sv = (int32_t)(int16_t)(uint16_t)i;
                    } else {
                        sv = i;
                        if (sv >= (1 << (p.bits_stored - 1))) sv -= (1 << p.bits_stored);
                    }
                    val = (float)sv;
                } else {
                    val = (float)i;
                }
            } else {
                val = (p.pixel_rep == 1) ? (float)(int8_t)(uint8_t)i : (float)i;
            }
            if (p.apply_rescale) val = __fadd_rn(__fmul_rn(val, p.rescale_slope), p.rescale_intercept);
            if (val <= lo) {
                val = 0.0f;
            } else if (val > hi) {
                val = fmax_;
            } else {
                const float t = __fadd_rn(__fsub_rn(val, cen), 0.5f);
                const float q0 = __fmul_rn(t, y);
                const float rem = __fmaf_rn(-q0, wm1, t);
                const float q = __fmaf_rn(rem, y, q0);
                val = __fmul_rn(__fadd_rn(q, 0.5f), fmax_);
            }
            float c = (val < fmax_) ? val : fmax_;
            c = (c > 0.0f) ? c : 0.0f;
            v = __float2uint_rz(c);
        }
        if (ob == 2) reinterpret_cast<uint16_t*>(lut)[i] = (uint16_t)(((v & 0xFF) << 8) | (v >> 8));
        else         lut[i] = (uint8_t)v;
    }
}

// Byte mask of word q of a unit holding nvalid (< 16) valid bytes.
__device__ __forceinline__ uint32_t valid_mask(int nvalid, int q)
{
    const int k = nvalid - 4 * q;
    return k >= 4 ? kFull : k <= 0 ? 0u : ((1u << (8 * k)) - 1u);
}

}  // namespace r2p
