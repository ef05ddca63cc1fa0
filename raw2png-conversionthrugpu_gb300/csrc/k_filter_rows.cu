// k_filter_rows.cu -- window/level + adaptive PNG filter for wide rows, one
// warp per row.
//
// Reference semantics:
//   adaptive filter : filter_select_kernel   src/gpu_filter.cu:183-309
//                     (filters 0-4 on bytes, a = the byte bpp to the left,
//                     score = sum of min(v, 256 - v) over the filtered row,
//                     lowest score wins, ties to the lowest type)
//   windowing       : k_window.cuh (dicom_preprocess_kernel,
//                     try_apply_linear_window, build/apply_dicom16_lut)
//   prior-row carry : src/gpu_filter.cu:391-434 (row 0 sees the caller's
//                     windowed prior row, or zeros)
//
// Design.  Rows are independent once the row above is known, so a warp
// filters a whole row by itself: lane l holds the 16 output bytes of unit
// 32 c + l of each 512-byte chunk c, and a CTA of 8 warps takes an item of
// 8 consecutive rows.
//   pass 0  each row of the item is windowed once, straight from the raw
//           pixels (16-byte read-only loads, several chunks in flight), into
//           the CTA's stash in shared memory: slot 1 + w holds warp w's row,
//           slot 0 the row above the item (windowed by all 8 warps, or the
//           caller's prior row, or zeros); one CTA barrier follows;
//   pass 1  each warp sums the five filters' costs of its row from its own
//           slot and the slot before it (the row above): two instructions
//           per filter and word (vabsdiff4, then vabsdiff4 with .add against
//           0x80808080: min(v, 256 - v) = 128 - |d - 128| with d = |x - p|
//           per byte); five warp reductions (redux) and the argmin, the same
//           in every lane, pick the filter;
//   pass 2  the winner's residuals x - p, from the same two slots, stored as
//           aligned 4-byte words re-cut from the lane's unit and the previous
//           lane's last word (only a row's first and last few bytes are
//           stored bytewise).
// With an 8 KB table a CTA of 6 KB rows holds 64 KB, so three fit an SM.
// Rows too wide for that (C2's 36000-byte rows) skip the stash: pass 1
// windows the row and the row above from the raw pixels (one chunk ahead,
// the bytes to the left by a shuffle) and pass 2 windows them again.  The
// window table is built once per image by k_window_lut (a grid over the
// table's entries) and copied into each CTA's shared memory.
#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include <algorithm>

#include "k_filter_ops.cuh"
#include "k_window.cuh"
#include "r2p_common.h"
#include "r2p_device.h"
#include "r2p_kernels.h"

namespace r2p {

constexpr int kRowsWarps = 8;                  // warps per CTA: rows filtered side by side
constexpr int kRowsThreads = 32 * kRowsWarps;
constexpr int kRowsLutMax = 32768;             // table bytes a CTA keeps in shared memory
constexpr int kRowsSmemMax = 74 * 1024;        // dynamic shared memory of a CTA: three fit an SM
constexpr int kLutEntriesPerCta = 1024;        // k_window_lut: table bytes per CTA of 256 threads

// Everything a warp needs about its image, in registers.
struct RowsJob {
    const uint8_t* raw;
    uint8_t* filt;
    const uint8_t* prior;
    uint8_t* last_row;
    int rb, sp, height, nch;
    uint32_t sh;                               // funnel shift of the left neighbour
};

// Raw bytes of one unit: 16 (a = all; same depth in and out) or 32 (a, b;
// 16-bit samples to an 8-bit row).  The row walks issue these loads ahead of
// the arithmetic that uses them (one chunk ahead in the wide-row passes,
// four chunks at a time in pass 0 of the stash path).
struct RawU {
    uint4 a, b;
};

// Unit u of raw row `rowp`; nv = valid output bytes of the unit (rb - 16 u:
// a multiple of 8 here); zeros past them (a half unit reads only its own 16
// raw bytes).
template <int K>
__device__ __forceinline__ RawU fetch_unit(const uint8_t* __restrict__ rowp, int u, int nv)
{
    RawU r;
    r.a = r.b = make_uint4(0u, 0u, 0u, 0u);
    if (nv <= 0) return r;
    if (K == K_Q15 || K == K_LUT8) {
        r.a = __ldg(reinterpret_cast<const uint4*>(rowp + 32 * u));
        if (nv > 8) r.b = __ldg(reinterpret_cast<const uint4*>(rowp + 32 * u + 16));
    } else {
        r.a = __ldg(reinterpret_cast<const uint4*>(rowp + 16 * u));
    }
    return r;
}

// Unit u of the caller's prior row (windowed bytes in PNG order, any
// alignment), in a.
__device__ __noinline__ RawU fetch_prior(const uint8_t* prior, int u, int nv)
{
    uint32_t v[4] = {0u, 0u, 0u, 0u};
    for (int k = 0; k < 16 && k < nv; k++) v[k >> 2] |= (uint32_t)prior[16 * u + k] << (8 * (k & 3));
    RawU r;
    r.a = make_uint4(v[0], v[1], v[2], v[3]);
    r.b = make_uint4(0u, 0u, 0u, 0u);
    return r;
}

// The windowed output words of a fetched unit.
template <int K>
__device__ __forceinline__ void win_raw(const WinCtx& w, const RawU& r, int nv, uint32_t x[4])
{
    if (nv <= 0) {
        x[0] = x[1] = x[2] = x[3] = 0u;
        return;
    }
    if (K == K_Q15 || K == K_LUT8) {
        uint32_t o[4];
        win_unit<K>(w, r.a, o);
        x[0] = o[0];
        x[1] = o[1];
        if (nv > 8) {
            win_unit<K>(w, r.b, o);
            x[2] = o[0];
            x[3] = o[1];
        } else {
            x[2] = x[3] = 0u;
        }
    } else if (K == K_LUT16Z) {
        const uint32_t m2 = w.mask << 1;
        const uint32_t wv[4] = {r.a.x, r.a.y, r.a.z, r.a.w};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint32_t lo = *reinterpret_cast<const uint16_t*>(w.lut + ((wv[k] << 1) & m2));
            const uint32_t hi = *reinterpret_cast<const uint16_t*>(w.lut + ((wv[k] >> 15) & m2));
            x[k] = __byte_perm(lo, hi, 0x5410);
        }
    } else {
        win_unit<K>(w, r.a, x);
    }
}

// Where row j's "above" bytes come from: the raw row j - 1 (windowed here),
// the caller's prior row (already windowed), or zeros (image row 0).
enum AboveKind : int { kAboveRaw = 0, kAbovePrior = 1, kAboveZero = 2 };

// The row above row j, fetching side.
template <int K>
__device__ __forceinline__ RawU fetch_above(const RowsJob& J, const uint8_t* br, int am, int u, int nv)
{
    if (am == kAboveRaw) return fetch_unit<K>(br, u, nv);
    if (am == kAbovePrior && nv > 0) return fetch_prior(J.prior, u, nv);
    RawU r;
    r.a = r.b = make_uint4(0u, 0u, 0u, 0u);
    return r;
}

// The row above row j, windowing side.
template <int K>
__device__ __forceinline__ void win_above(const WinCtx& w, const RawU& r, int am, int nv, uint32_t b[4])
{
    if (am == kAboveRaw) {
        win_raw<K>(w, r, nv, b);
    } else {
        b[0] = r.a.x;
        b[1] = r.a.y;
        b[2] = r.a.z;
        b[3] = r.a.w;
    }
}

// The two words before the lane's unit (m1 = word -1, m2 = word -2) from the
// previous lane, or at lane 0 from the previous chunk's lane 31 (carried in
// c1, c2; zeros at the row start).  Updates the carries for the next chunk.
template <int DW>
__device__ __forceinline__ void left_of(const uint32_t v[4], int lane, uint32_t& c1, uint32_t& c2, uint32_t& m1,
                                        uint32_t& m2)
{
    m1 = __shfl_up_sync(kFull, v[3], 1);
    m2 = DW == 2 ? __shfl_up_sync(kFull, v[2], 1) : 0u;
    if (lane == 0) {
        m1 = c1;
        m2 = c2;
    }
    c1 = __shfl_sync(kFull, v[3], 31);
    if (DW == 2) c2 = __shfl_sync(kFull, v[2], 31);
}

// Residual words of unit u -> the output row (type byte at R, data byte i
// at R + 1 + i).  Aligned word k of the data (address A - s3 + 4k, A = R + 1,
// s3 = A mod 4) holds data bytes [4k - s3, 4k - s3 + 4); the lane of unit u
// writes words 4u .. 4u + 3 (the first built with the previous unit's last
// word rp), the lane of the last unit also word 4u + 4.  Words that reach
// outside the row's data are stored bytewise.
__device__ __forceinline__ void store_unit(uint8_t* R, int rb, int u, const uint32_t r[4], uint32_t rp)
{
    uint8_t* A = R + 1;
    const int s3 = (int)(reinterpret_cast<uintptr_t>(A) & 3u);
    const uint32_t fs = 8u * (uint32_t)s3;
    uint32_t* Aw = reinterpret_cast<uint32_t*>(A - s3) + 4 * u;
    const int lo = 16 * u - s3;                // data byte of word 4u's first byte
    if (lo >= 0 && (16 * u + 16 < rb || (16 * u + 16 == rb && s3 == 0))) {
        Aw[0] = __funnelshift_l(rp, r[0], fs);
        Aw[1] = __funnelshift_l(r[0], r[1], fs);
        Aw[2] = __funnelshift_l(r[1], r[2], fs);
        Aw[3] = __funnelshift_l(r[2], r[3], fs);
        return;
    }
    const bool last = 16 * u + 16 >= rb;
#pragma unroll
    for (int q = 0; q < 5; q++) {
        if (q == 4 && !last) break;
        const uint32_t pw = q == 0 ? rp : r[q - 1];
        const uint32_t cw = q < 4 ? r[q] : 0u;
        const uint32_t v = __funnelshift_l(pw, cw, fs);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int bi = lo + 4 * q + i;
            if (bi >= 0 && bi < rb) A[bi] = (uint8_t)(v >> (8 * i));
        }
    }
}

// Pass 2 for filter F: residuals of row j written to the output.
template <int K, int DW, int F>
__device__ __forceinline__ void emit_row(const WinCtx& w, const RowsJob& J, int j, int lane)
{
    const uint8_t* xr = J.raw + (size_t)j * J.sp;
    uint8_t* R = J.filt + (size_t)j * (size_t)(J.rb + 1);
    if (lane == 0) R[0] = (uint8_t)F;
    const bool keep_last = J.last_row != nullptr && j == J.height - 1;
    const uint8_t* br = xr - J.sp;
    const int am = j > 0 ? kAboveRaw : J.prior ? kAbovePrior : kAboveZero;
    uint32_t cx1 = 0, cx2 = 0, cb1 = 0, cb2 = 0, cr = 0;
    RawU nx = fetch_unit<K>(xr, lane, J.rb - 16 * lane), nb;
    if (F >= 2) nb = fetch_above<K>(J, br, am, lane, J.rb - 16 * lane);
#pragma unroll 1
    for (int c = 0; c < J.nch; c++) {
        const int u = 32 * c + lane;
        const int nv = J.rb - 16 * u;
        const RawU cx = nx;
        RawU cb;
        if (F >= 2) cb = nb;
        if (c + 1 < J.nch) {
            nx = fetch_unit<K>(xr, u + 32, nv - 512);
            if (F >= 2) nb = fetch_above<K>(J, br, am, u + 32, nv - 512);
        }
        uint32_t x[4], b[4] = {0u, 0u, 0u, 0u};
        win_raw<K>(w, cx, nv, x);
        if (F >= 2) win_above<K>(w, cb, am, nv, b);
        uint32_t xm1 = 0, xm2 = 0, bm1 = 0, bm2 = 0;
        if (F == 1 || F >= 3) left_of<DW>(x, lane, cx1, cx2, xm1, xm2);
        if (F == 4) left_of<DW>(b, lane, cb1, cb2, bm1, bm2);
        uint32_t r[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if (F == 0) {
                r[q] = x[q];
            } else if (F == 1) {
                r[q] = __vsub4(x[q], left_word(x, xm1, xm2, DW, J.sh, q));
            } else if (F == 2) {
                r[q] = __vsub4(x[q], b[q]);
            } else if (F == 3) {
                r[q] = __vsub4(x[q], avg4_dev(left_word(x, xm1, xm2, DW, J.sh, q), b[q]));
            } else {
                const uint32_t a = left_word(x, xm1, xm2, DW, J.sh, q);
                const uint32_t cq = left_word(b, bm1, bm2, DW, J.sh, q);
                r[q] = __vsub4(x[q], paeth_word(a, b[q], cq, widen_lo(a), widen_hi(a), widen_lo(b[q]),
                                                widen_hi(b[q]), widen_lo(cq), widen_hi(cq)));
            }
        }
        uint32_t rp = __shfl_up_sync(kFull, r[3], 1);
        if (lane == 0) rp = cr;
        cr = __shfl_sync(kFull, r[3], 31);
        if (nv > 0) {
            store_unit(R, J.rb, u, r, rp);
            if (keep_last) {
                for (int k = 0; k < 16 && k < nv; k++) J.last_row[16 * u + k] = (uint8_t)(x[k >> 2] >> (8 * (k & 3)));
            }
        }
    }
}

// One stashed row of nch chunks: its windowed bytes behind 16 zero bytes
// (what lies left of the row start).  A CTA's stash holds kRowsWarps + 1 of
// them: slot 0 the row above the item's first row, slot 1 + w warp w's row,
// so the row above warp w's row is slot w, written by the warp before it.
__host__ __device__ inline int rows_slot_bytes(int nch) { return 16 + 512 * nch; }
__host__ __device__ inline int rows_stash_bytes(int nch) { return (kRowsWarps + 1) * rows_slot_bytes(nch); }

// 16 and 8 bytes from shared memory at 32-bit shared address a.
__device__ __forceinline__ uint4 lds128(uint32_t a)
{
    uint4 v;
    asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(a));
    return v;
}
__device__ __forceinline__ uint2 lds64(uint32_t a)
{
    uint2 v;
    asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(a));
    return v;
}

// Pass 2 for filter F from the stash: row j's windowed bytes at shared
// address xa, the row above at ba (each with 16 zero bytes before it).  One
// copy per (DW, F), called once per row: it does not depend on the window.
template <int DW, int F>
__device__ __noinline__ void emit_stash(uint8_t* filt, uint8_t* last_row, int rb, int height, int nch, uint32_t sh,
                                        int j, int lane, uint32_t xa, uint32_t ba)
{
    uint8_t* R = filt + (size_t)j * (size_t)(rb + 1);
    if (lane == 0) R[0] = (uint8_t)F;
    const bool keep_last = last_row != nullptr && j == height - 1;
    uint32_t cr = 0;
#pragma unroll 1
    for (int c = 0; c < nch; c++) {
        const int u = 32 * c + lane;
        const int nv = rb - 16 * u;
        const uint4 xv = lds128(xa + 16 * u);
        const uint32_t x[4] = {xv.x, xv.y, xv.z, xv.w};
        uint32_t b[4] = {0u, 0u, 0u, 0u};
        uint32_t xm1 = 0, xm2 = 0, bm1 = 0, bm2 = 0;
        if (F == 1 || F >= 3) {
            const uint2 m = lds64(xa + 16 * u - 8);
            xm2 = m.x;
            xm1 = m.y;
        }
        if (F >= 2) {
            const uint4 bv = lds128(ba + 16 * u);
            b[0] = bv.x;
            b[1] = bv.y;
            b[2] = bv.z;
            b[3] = bv.w;
        }
        if (F == 4) {
            const uint2 m = lds64(ba + 16 * u - 8);
            bm2 = m.x;
            bm1 = m.y;
        }
        uint32_t r[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if (F == 0) {
                r[q] = x[q];
            } else if (F == 1) {
                r[q] = __vsub4(x[q], left_word(x, xm1, xm2, DW, sh, q));
            } else if (F == 2) {
                r[q] = __vsub4(x[q], b[q]);
            } else if (F == 3) {
                r[q] = __vsub4(x[q], avg4_dev(left_word(x, xm1, xm2, DW, sh, q), b[q]));
            } else {
                const uint32_t a = left_word(x, xm1, xm2, DW, sh, q);
                const uint32_t cq = left_word(b, bm1, bm2, DW, sh, q);
                r[q] = __vsub4(x[q], paeth_word(a, b[q], cq, widen_lo(a), widen_hi(a), widen_lo(b[q]),
                                                widen_hi(b[q]), widen_lo(cq), widen_hi(cq)));
            }
        }
        uint32_t rp = __shfl_up_sync(kFull, r[3], 1);
        if (lane == 0) rp = cr;
        cr = __shfl_sync(kFull, r[3], 31);
        if (nv > 0) {
            store_unit(R, rb, u, r, rp);
            if (keep_last) {
                for (int k = 0; k < 16 && k < nv; k++) last_row[16 * u + k] = (uint8_t)(x[k >> 2] >> (8 * (k & 3)));
            }
        }
    }
}

// Row j of the job: the five costs (pass 1), the winner, its residuals.
template <int K, int DW>
__device__ void filter_row(const WinCtx& w, const RowsJob& J, int j, int lane)
{
    const uint8_t* xr = J.raw + (size_t)j * J.sp;
    const uint32_t K80 = 0x80808080u;
    uint32_t S0 = 0, S1 = 0, S2 = 0, S3 = 0, S4 = 0;
    uint32_t cx1 = 0, cx2 = 0, cb1 = 0, cb2 = 0;
    const uint8_t* br = xr - J.sp;
    const int am = j > 0 ? kAboveRaw : J.prior ? kAbovePrior : kAboveZero;
    RawU nx = fetch_unit<K>(xr, lane, J.rb - 16 * lane);
    RawU nb = fetch_above<K>(J, br, am, lane, J.rb - 16 * lane);
#pragma unroll 1
    for (int c = 0; c < J.nch; c++) {
        const int u = 32 * c + lane;
        const int nv = J.rb - 16 * u;
        const RawU cx = nx, cb = nb;
        if (c + 1 < J.nch) {
            nx = fetch_unit<K>(xr, u + 32, nv - 512);
            nb = fetch_above<K>(J, br, am, u + 32, nv - 512);
        }
        uint32_t x[4], b[4];
        win_raw<K>(w, cx, nv, x);
        win_above<K>(w, cb, am, nv, b);
        uint32_t xm1, xm2, bm1, bm2;
        left_of<DW>(x, lane, cx1, cx2, xm1, xm2);
        left_of<DW>(b, lane, cb1, cb2, bm1, bm2);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const uint32_t a = left_word(x, xm1, xm2, DW, J.sh, q);
            const uint32_t cq = left_word(b, bm1, bm2, DW, J.sh, q);
            const uint32_t av = avg4_dev(a, b[q]);
            const uint32_t pp = paeth_word(a, b[q], cq, widen_lo(a), widen_hi(a), widen_lo(b[q]), widen_hi(b[q]),
                                           widen_lo(cq), widen_hi(cq));
            uint32_t d1 = __vabsdiffu4(x[q], a), d2 = __vabsdiffu4(x[q], b[q]);
            uint32_t d3 = __vabsdiffu4(x[q], av), d4 = __vabsdiffu4(x[q], pp);
            if (nv < 16) {
                // bytes past the row end: x = 0 and d = 0 add 128 - |0 - 128| = 0
                const uint32_t m = valid_mask(nv, q);
                d1 &= m;
                d2 &= m;
                d3 &= m;
                d4 &= m;
            }
            S0 = sad4(x[q], K80, S0);
            S1 = sad4(d1, K80, S1);
            S2 = sad4(d2, K80, S2);
            S3 = sad4(d3, K80, S3);
            S4 = sad4(d4, K80, S4);
        }
    }
    // every word a lane held, valid or not, added 512 - (its cost) to S
    const uint32_t base = 2048u * (uint32_t)J.nch;
    const uint32_t t0 = __reduce_add_sync(kFull, base - S0);
    const uint32_t t1 = __reduce_add_sync(kFull, base - S1);
    const uint32_t t2 = __reduce_add_sync(kFull, base - S2);
    const uint32_t t3 = __reduce_add_sync(kFull, base - S3);
    const uint32_t t4 = __reduce_add_sync(kFull, base - S4);
    int f = 0;
    uint32_t best = t0;
    if (t1 < best) { best = t1; f = 1; }
    if (t2 < best) { best = t2; f = 2; }
    if (t3 < best) { best = t3; f = 3; }
    if (t4 < best) { f = 4; }
    switch (f) {
        case 0: emit_row<K, DW, 0>(w, J, j, lane); break;
        case 1: emit_row<K, DW, 1>(w, J, j, lane); break;
        case 2: emit_row<K, DW, 2>(w, J, j, lane); break;
        case 3: emit_row<K, DW, 3>(w, J, j, lane); break;
        default: emit_row<K, DW, 4>(w, J, j, lane); break;
    }
}

// Chunks c0, c0 + step, ... of raw row `rowp` windowed into a stash slot's
// data at dst (32 units a chunk, zeros past the row end).  Windowing costs
// few instructions per load, so four chunks' loads (two for 16-bit samples to
// 8-bit rows) are issued before any of them is windowed.
template <int K>
__device__ __forceinline__ void window_into(const WinCtx& w, const RowsJob& J, const uint8_t* rowp, int lane,
                                            uint8_t* dst, int c0, int step)
{
    constexpr int G = (K == K_Q15 || K == K_LUT8) ? 2 : 4;    // 32 raw bytes a unit there
#pragma unroll 1
    for (int c = c0; c < J.nch; c += G * step) {
        RawU r[G];
#pragma unroll
        for (int k = 0; k < G; k++) {
            const int u = 32 * (c + k * step) + lane;
            r[k] = fetch_unit<K>(rowp, u, c + k * step < J.nch ? J.rb - 16 * u : 0);
        }
#pragma unroll
        for (int k = 0; k < G; k++) {
            if (c + k * step < J.nch) {
                const int u = 32 * (c + k * step) + lane;
                uint32_t x[4];
                win_raw<K>(w, r[k], J.rb - 16 * u, x);
                *reinterpret_cast<uint4*>(dst + 16 * u) = make_uint4(x[0], x[1], x[2], x[3]);
            }
        }
    }
}

// Rows [r0, r1) (at most kRowsWarps) through the CTA's stash: pass 0 windows
// warp w's row r0 + w into slot 1 + w, and every warp a share of the chunks
// of the row above r0 into slot 0 (the windowed raw row, the caller's prior
// row, or zeros); after one CTA barrier pass 1 scores each row from its slot
// and the slot before it, and pass 2 forms the winner's residuals from the
// same two slots.  Every row is windowed once.  All warps of the CTA call
// this.
template <int K, int DW>
__device__ void filter_item_stash(const WinCtx& w, const RowsJob& J, int r0, int r1, int warp, int lane,
                                  uint8_t* stash)
{
    const int slot = rows_slot_bytes(J.nch);
    const int j = r0 + warp;
    const bool has = j < r1;
    uint8_t* xs = stash + (1 + warp) * slot;
    if (lane == 0) *reinterpret_cast<uint4*>(xs) = make_uint4(0u, 0u, 0u, 0u);
    if (warp == 0 && lane == 1) *reinterpret_cast<uint4*>(stash) = make_uint4(0u, 0u, 0u, 0u);
    if (has) window_into<K>(w, J, J.raw + (size_t)j * J.sp, lane, xs + 16, 0, 1);
    uint8_t* bs = stash + 16;
    if (r0 > 0) {
        if (warp < J.nch) window_into<K>(w, J, J.raw + (size_t)(r0 - 1) * J.sp, lane, bs, warp, kRowsWarps);
    } else {
#pragma unroll 1
        for (int u = 32 * warp + lane; u < 32 * J.nch; u += 32 * kRowsWarps) {
            const int nv = J.rb - 16 * u;
            const RawU r = (J.prior && nv > 0) ? fetch_prior(J.prior, u, nv)
                                               : RawU{make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u)};
            *reinterpret_cast<uint4*>(bs + 16 * u) = r.a;
        }
    }
    __syncthreads();
    if (!has) return;
    const uint8_t* xrow = xs + 16;
    const uint8_t* brow = xs - slot + 16;
    const uint32_t K80 = 0x80808080u;
    uint32_t S0 = 0, S1 = 0, S2 = 0, S3 = 0, S4 = 0;
#pragma unroll 1
    for (int c = 0; c < J.nch; c++) {
        const int u = 32 * c + lane;
        const int nv = J.rb - 16 * u;
        const uint4 xv = *reinterpret_cast<const uint4*>(xrow + 16 * u);
        const uint4 bv = *reinterpret_cast<const uint4*>(brow + 16 * u);
        const uint2 xm = *reinterpret_cast<const uint2*>(xrow + 16 * u - 8);
        const uint2 bm = *reinterpret_cast<const uint2*>(brow + 16 * u - 8);
        const uint32_t x[4] = {xv.x, xv.y, xv.z, xv.w}, b[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const uint32_t a = left_word(x, xm.y, xm.x, DW, J.sh, q);
            const uint32_t cq = left_word(b, bm.y, bm.x, DW, J.sh, q);
            const uint32_t av = avg4_dev(a, b[q]);
            const uint32_t pp = paeth_word(a, b[q], cq, widen_lo(a), widen_hi(a), widen_lo(b[q]), widen_hi(b[q]),
                                           widen_lo(cq), widen_hi(cq));
            uint32_t d1 = __vabsdiffu4(x[q], a), d2 = __vabsdiffu4(x[q], b[q]);
            uint32_t d3 = __vabsdiffu4(x[q], av), d4 = __vabsdiffu4(x[q], pp);
            if (nv < 16) {
                // bytes past the row end: x = 0 and d = 0 add 128 - |0 - 128| = 0
                const uint32_t m = valid_mask(nv, q);
                d1 &= m;
                d2 &= m;
                d3 &= m;
                d4 &= m;
            }
            S0 = sad4(x[q], K80, S0);
            S1 = sad4(d1, K80, S1);
            S2 = sad4(d2, K80, S2);
            S3 = sad4(d3, K80, S3);
            S4 = sad4(d4, K80, S4);
        }
    }
    const uint32_t base = 2048u * (uint32_t)J.nch;
    const uint32_t t0 = __reduce_add_sync(kFull, base - S0);
    const uint32_t t1 = __reduce_add_sync(kFull, base - S1);
    const uint32_t t2 = __reduce_add_sync(kFull, base - S2);
    const uint32_t t3 = __reduce_add_sync(kFull, base - S3);
    const uint32_t t4 = __reduce_add_sync(kFull, base - S4);
    int f = 0;
    uint32_t best = t0;
    if (t1 < best) { best = t1; f = 1; }
    if (t2 < best) { best = t2; f = 2; }
    if (t3 < best) { best = t3; f = 3; }
    if (t4 < best) { f = 4; }
    const uint32_t xa = (uint32_t)__cvta_generic_to_shared(xrow), ba = (uint32_t)__cvta_generic_to_shared(brow);
    switch (f) {
        case 0: emit_stash<DW, 0>(J.filt, J.last_row, J.rb, J.height, J.nch, J.sh, j, lane, xa, ba); break;
        case 1: emit_stash<DW, 1>(J.filt, J.last_row, J.rb, J.height, J.nch, J.sh, j, lane, xa, ba); break;
        case 2: emit_stash<DW, 2>(J.filt, J.last_row, J.rb, J.height, J.nch, J.sh, j, lane, xa, ba); break;
        case 3: emit_stash<DW, 3>(J.filt, J.last_row, J.rb, J.height, J.nch, J.sh, j, lane, xa, ba); break;
        default: emit_stash<DW, 4>(J.filt, J.last_row, J.rb, J.height, J.nch, J.sh, j, lane, xa, ba); break;
    }
}

template <int K>
__device__ __forceinline__ void filter_rows_k(const WinCtx& w, const RowsJob& J, int r0, int r1, int warp, int nw,
                                              int lane, int dw, uint8_t* stash)
{
    if (stash) {
        if (dw == 1) filter_item_stash<K, 1>(w, J, r0, r1, warp, lane, stash);
        else         filter_item_stash<K, 2>(w, J, r0, r1, warp, lane, stash);
        return;
    }
    for (int j = r0 + warp; j < r1; j += nw) {
        if (dw == 1) filter_row<K, 1>(w, J, j, lane);
        else         filter_row<K, 2>(w, J, j, lane);
    }
}

// Dynamic shared memory: the window table (lut_region bytes), then the CTA's
// stash of `stash` bytes (0: no stash; rows are then windowed again in
// pass 2).
__global__ void __launch_bounds__(kRowsThreads, 3)
k_filter_rows(DevImage* __restrict__ imgs, const BandItem* __restrict__ items, int nitems, int lut_region, int stash)
{
    extern __shared__ __align__(16) uint8_t lut[];
    __shared__ int s_img;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_img = -1;
    __syncthreads();
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const BandItem bi = items[it];
        DevImage& d = imgs[bi.img];
        // the image's table into shared memory when the image changes; every
        // thread reads s_img before the barrier, thread 0 rewrites it after
        const bool new_img = (int)bi.img != s_img;
        __syncthreads();
        const int tbytes = (d.mode == W_A2_LUT || d.mode == W_LUT8) ? d.lut_entries * d.lut_esize : 0;
        if (new_img) {
            if (tbytes <= kRowsLutMax) {
                const uint4* src = reinterpret_cast<const uint4*>(d.lut);
                for (int i = tid; i < (tbytes + 15) / 16; i += kRowsThreads) reinterpret_cast<uint4*>(lut)[i] = src[i];
            }
            if (tid == 0) s_img = (int)bi.img;
            __syncthreads();
        }
        WinCtx wc;
        wc.mode = d.mode;
        wc.ib = d.ib;
        wc.ob = d.ob;
        wc.shift = d.lut_shift;
        wc.mask = d.lut_mask;
        wc.qa = d.qa;
        wc.qb = d.qb;
        wc.dp = d.dp;
        wc.lut = lut;
        int kind = win_kind(wc);
        if (kind == K_LUT16 && wc.shift == 0) kind = K_LUT16Z;
        // the host routes here only rows whose pixels a 16-byte load may read
        // and whose table fits; anything else is reported, not guessed
        if (kind == K_DIRECT || tbytes > kRowsLutMax || (reinterpret_cast<uintptr_t>(d.raw) & 15) ||
            (d.in_pitch & 15)) {
            if (tid == 0) atomicExch(&d.status, R2P_EINVAL);
            continue;
        }
        RowsJob J;
        J.raw = d.raw;
        J.filt = d.filt;
        J.prior = d.prior;
        J.last_row = d.last_row;
        J.rb = d.rb;
        J.sp = d.in_pitch;
        J.height = (int)d.height;
        J.nch = (d.rb + 511) / 512;
        const int dw = (d.bpp + 3) >> 2;
        J.sh = 8u * (uint32_t)(4 * dw - d.bpp);
        const int r0 = (int)bi.r0, r1 = (int)bi.r1;
        // the stash path takes an item of at most one row per warp (the
        // host's items); the condition is the same in every thread
        uint8_t* xs = (stash >= rows_stash_bytes(J.nch) && r1 - r0 <= kRowsWarps) ? lut + lut_region : nullptr;
        switch (kind) {
            case K_LUT16Z: filter_rows_k<K_LUT16Z>(wc, J, r0, r1, warp, kRowsWarps, lane, dw, xs); break;
            case K_COPY: filter_rows_k<K_COPY>(wc, J, r0, r1, warp, kRowsWarps, lane, dw, xs); break;
            case K_SWAP16: filter_rows_k<K_SWAP16>(wc, J, r0, r1, warp, kRowsWarps, lane, dw, xs); break;
            case K_LUT16: filter_rows_k<K_LUT16>(wc, J, r0, r1, warp, kRowsWarps, lane, dw, xs); break;
            case K_LUT8IN: filter_rows_k<K_LUT8IN>(wc, J, r0, r1, warp, kRowsWarps, lane, dw, xs); break;
            case K_Q15: filter_rows_k<K_Q15>(wc, J, r0, r1, warp, kRowsWarps, lane, dw, xs); break;
            default: filter_rows_k<K_LUT8>(wc, J, r0, r1, warp, kRowsWarps, lane, dw, xs); break;
        }
    }
}

// Window tables of the images filtered by k_filter_rows: blockIdx.x = image,
// the image's blockIdx.y CTAs share its entries (thread t of CTA y takes
// entries y * 256 + t, stepping by all of them); the first CTA of an image
// also records the resolved window in its descriptor.
__global__ void __launch_bounds__(256) k_window_lut(DevImage* __restrict__ imgs)
{
    DevImage& d = imgs[blockIdx.x];
    if (d.fpath != kFiltRows) return;
    const WinRes r = resolve_window(d);
    if (blockIdx.y == 0 && threadIdx.x == 0) {
        d.mode = r.mode;
        d.qa = r.qa;
        d.qb = r.qb;
        d.lut_shift = r.shift;
        d.lut_mask = r.mask;
        d.lut_entries = r.entries;
        d.lut_esize = r.esize;
    }
    const int i0 = (int)(blockIdx.y * blockDim.x + threadIdx.x), step = (int)(gridDim.y * blockDim.x);
    if (r.mode == W_A2_LUT) fill_a2_table_fast(d, r, d.lut, i0, step);
    else                    fill_window_table(d, r, d.lut, i0, step);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
bool rows_filter_eligible(int in_pitch, int lut_bytes) { return (in_pitch & 15) == 0 && lut_bytes <= kRowsLutMax; }

int rows_filter_rows_per_item() { return kRowsWarps; }

int rows_filter_lut_region(int lut_bytes) { return (std::min(lut_bytes, kRowsLutMax) + 15) & ~15; }

// A CTA's stash for rows of rb filtered bytes, or 0 when the launch could
// then not keep three CTAs on an SM (rows of more than about 7 KB with an
// 8 KB table): those rows are windowed again in pass 2 instead.
int rows_filter_stash(int rb, int lut_bytes)
{
    const int st = rows_stash_bytes((rb + 511) / 512);
    return rows_filter_lut_region(lut_bytes) + st <= kRowsSmemMax ? st : 0;
}

int rows_filter_smem(int lut_bytes, int stash) { return rows_filter_lut_region(lut_bytes) + stash; }

int rows_filter_ctas_per_sm(int smem)
{
    int n = 0;
    cudaFuncSetAttribute(k_filter_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, kRowsSmemMax);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_filter_rows, kRowsThreads, smem) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

cudaError_t launch_filter_rows(DevImage* imgs, int n, int lut_bytes, int stash, const BandItem* items, int nitems,
                               int grid, cudaStream_t s)
{
    const int slices = std::max(1, (lut_bytes + kLutEntriesPerCta - 1) / kLutEntriesPerCta);
    k_window_lut<<<dim3((unsigned)n, (unsigned)slices), 256, 0, s>>>(imgs);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_filter_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, kRowsSmemMax);
    if (e != cudaSuccess) return e;
    const int lr = rows_filter_lut_region(lut_bytes);
    k_filter_rows<<<grid, kRowsThreads, rows_filter_smem(lut_bytes, stash), s>>>(imgs, items, nitems, lr, stash);
    note_launch();
    return cudaGetLastError();
}

}  // namespace r2p
