// k_filter_reg.cu -- window/level + adaptive PNG filter for rows of up to
// 8 KB, each row held in registers across a group of warps.
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
// Design.  A group of W warps owns a run of consecutive rows of one image;
// lane l of warp w owns the kLB = 16 output bytes at kLB * (32 w + l) of
// every row (one "unit"), so a row of up to 512 W bytes lies in the group's
// registers and walks down the image with it: the windowed row
// becomes the next row's "above" bytes (b), and the bytes bpp to the left
// (a, and c for the row above) are funnel shifts of words already held, with
// the two words before the lane's first from its neighbour.
//
// Per row and unit, in registers:
//   - raw bytes staged by bulk copies (TMA, one row per copy, kRegRing rows
//     ahead, an mbarrier per ring slot, bounded waits) and windowed by the
//     image's transform (table in shared memory);
//   - the bytes to the left (a) from the neighbouring lane (shuffle) or, at a
//     warp's first lane, from the previous warp through shared memory;
//   - scores: with d = |x - p| per byte (vabsdiff4), min(v, 256 - v) of the
//     filtered byte v = (x - p) mod 256 equals 128 - |d - 128|, so a word's
//     four costs are 512 minus one sum-of-absolute-differences instruction
//     (vabsdiff4 with .add) against 0x80808080: two instructions per filter
//     and word, one for filter 0;
//   - the Paeth predictor: a, b, c widened to fp16 pairs (exact), the
//     comparisons |b-c| <= |a-c|, |a+b-2c| done as packed half compares, the
//     masks narrowed back to bytes and the predictor selected bytewise;
//   - lane costs summed by warp reductions (redux), warps' sums through
//     shared memory and one named barrier per row, the argmin taken by every
//     lane;
//   - the residual x - p of the winner (its predictor kept from scoring, no
//     second filtering pass) stored to a shared-memory row buffer, and one row
//     later (after the next row's barrier) written to HBM as 16-byte aligned
//     chunks re-cut from two adjacent units; the few bytes at a row's ends
//     that do not fill an aligned chunk are stored bytewise by their owners.
// The next row is windowed before the barrier, so the barrier waits overlap
// useful work.  A CTA of NW warps holds NW / W groups, each on its own part
// of the CTA's band.
#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include <algorithm>

#include "k_filter_ops.cuh"
#include "k_window.cuh"
#include "r2p_common.h"
#include "r2p_device.h"
#include "r2p_kernels.h"
#include "r2p_tma.cuh"

namespace r2p {

constexpr int kRegMaxWarps = 16;   // warps per CTA at most
constexpr int kRegRing = 4;        // raw rows staged per group
constexpr int kRegLutMax = 16384;  // window table bytes kept in shared memory
constexpr uint64_t kRegWaitNs = 200ull * 1000 * 1000;        // one row copy
constexpr uint64_t kRegDrainNs = 2000ull * 1000 * 1000;      // outstanding copies after a timeout

// Words of a row each lane holds: kWPL, one 16-byte unit.  (Two units per
// lane halve the per-row bookkeeping per byte but need 112 registers a thread;
// measured on the 3072x3072 16-bit image that ran 49 us against 40 us for one
// unit, as only 18 warps fit an SM instead of 24.)
constexpr int kLB = 4 * kWPL;      // bytes per lane per row
constexpr int kNU = kWPL / 4;      // 16-byte units per lane

__host__ __device__ inline int reg_warps(int rb) { return (rb + 32 * kLB - 1) / (32 * kLB); }
__host__ __device__ inline int reg_resid_bytes(int rb) { return 16 + kLB * 32 * reg_warps(rb); }
// One group's shared memory: kRegRing staged raw rows and two residual rows.
__host__ __device__ inline int reg_group_bytes(int rb, int in_pitch)
{
    return kRegRing * in_pitch + 2 * reg_resid_bytes(rb);
}
__host__ __device__ inline int reg_lut_bytes(int entries, int esize)
{
    return (entries * esize + 15) & ~15;
}

struct __align__(16) RegShared {
    uint64_t bar[kRegMaxWarps][kRegRing];   // per group, per ring slot
    uint32_t seq[kRegMaxWarps];             // copies issued so far per group (mbarrier phases)
    uint32_t part[2][kRegMaxWarps][8];      // per warp: five lane-summed costs of a row
    uint32_t xch[3][kRegMaxWarps][2];       // per warp: last two windowed words (row parity; 2 = row above)
    WinRes res;
    int img;                                // image whose window table is in shared memory
};

// Group barrier: a named barrier over the group's W warps (ids 1..8), or the
// warp alone; returns whether `bad` was set in any of its threads, so every
// thread of the group takes the same branch after it.
__device__ __forceinline__ bool group_bar(int g, int W, bool bad)
{
    if (W == 1) {
        __syncwarp();
        return __any_sync(kFull, bad);
    }
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\t"
        "barrier.red.or.pred q, %2, %3, p;\n\tselp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"(bad ? 1u : 0u), "r"(1 + g), "r"(32 * W)
        : "memory");
    return r != 0;
}

// One chunk's words: bytes [o, o + 16) of the 32 bytes in w0 (low 16) and w1.
__device__ __forceinline__ uint4 cut16(const uint4 w0, const uint4 w1, int o)
{
    const uint32_t W[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
    const uint32_t sh = 8u * (uint32_t)(o & 3);
    uint4 r;
    switch (o >> 2) {
        case 0:
            r = make_uint4(__funnelshift_r(W[0], W[1], sh), __funnelshift_r(W[1], W[2], sh),
                           __funnelshift_r(W[2], W[3], sh), __funnelshift_r(W[3], W[4], sh));
            break;
        case 1:
            r = make_uint4(__funnelshift_r(W[1], W[2], sh), __funnelshift_r(W[2], W[3], sh),
                           __funnelshift_r(W[3], W[4], sh), __funnelshift_r(W[4], W[5], sh));
            break;
        case 2:
            r = make_uint4(__funnelshift_r(W[2], W[3], sh), __funnelshift_r(W[3], W[4], sh),
                           __funnelshift_r(W[4], W[5], sh), __funnelshift_r(W[5], W[6], sh));
            break;
        case 3:
            r = make_uint4(__funnelshift_r(W[3], W[4], sh), __funnelshift_r(W[4], W[5], sh),
                           __funnelshift_r(W[5], W[6], sh), __funnelshift_r(W[6], W[7], sh));
            break;
        default:
            r = w1;
            break;
    }
    return r;
}

// Bytes [k0, k1) of the 16 held in v0..v3 (little-endian) to dst + k0.
__device__ __noinline__ void store_bytes(uint8_t* dst, uint32_t v0, uint32_t v1, uint32_t v2, uint32_t v3, int k0,
                                         int k1)
{
    for (int k = k0; k < k1; k++) {
        const uint32_t w = k < 8 ? (k < 4 ? v0 : v1) : (k < 12 ? v2 : v3);
        dst[k] = (uint8_t)(w >> (8 * (k & 3)));
    }
}

// Output geometry of one row: its type byte at R, data byte i at R + 1 + i;
// h = data bytes before the first 16-byte aligned address, nch = aligned
// 16-byte chunks wholly inside the data, t0 = first data byte after them.
struct RowOut {
    uint8_t* R;
    int h, nch, t0;
};

__device__ __forceinline__ RowOut row_out(uint8_t* R, int rb)
{
    RowOut o;
    o.R = R;
    o.h = (int)((15u - (uint32_t)reinterpret_cast<uintptr_t>(R)) & 15u);   // (16 - (R + 1) % 16) % 16
    o.nch = rb >= o.h ? (rb - o.h) >> 4 : 0;
    o.t0 = o.h + 16 * o.nch;
    return o;
}

// Aligned chunks of a finished row from its residual buffer: the lane of
// unit u writes chunk u - (h > 0), re-cut from units u - 1 and u.
__device__ __forceinline__ void store_chunks(const RowOut& o, const uint8_t* resid, int u)
{
    const int c = u - (o.h > 0 ? 1 : 0);
    if (c < 0 || c >= o.nch) return;
    const uint4 w0 = *reinterpret_cast<const uint4*>(resid + 16 * u);
    const uint4 w1 = *reinterpret_cast<const uint4*>(resid + 16 * u + 16);
    *reinterpret_cast<uint4*>(o.R + 1 + o.h + 16 * c) = cut16(w0, w1, o.h ? o.h : 16);
}

// Spin until the copy of ring sequence number q has landed (bounded).
__device__ __forceinline__ bool wait_row(RegShared& S, int g, uint32_t q)
{
    return mbar_wait_bounded(&S.bar[g][q % kRegRing], (q / kRegRing) & 1u, kRegWaitNs);
}

// Table bytes reserved for an image's window (the largest its request can
// resolve to); the host plans shared memory with the same figure.
__host__ __device__ inline int reg_lut_reserve(int req_mode, int ib, int ob, int bits_stored)
{
    if (req_mode == R2P_WINDOW_DICOM16)
        return (ib == 2 ? (bits_stored < 16 ? (1 << bits_stored) : 65536) : 256) * ob;
    if (req_mode == R2P_WINDOW_BATCH8) return 1 << bits_stored;
    return 0;
}

// Everything one group needs about its image and its rows, in registers.
struct GroupJob {
    const uint8_t* raw;
    uint8_t* filt;
    const uint8_t* prior;
    uint8_t* last_row;
    int rb, sp, height, bpp, kind;
    int s0, s1, q0;
    uint8_t* ring;
    uint8_t* resid0;
    uint8_t* resid1;
    uint32_t seq0;
};

// The group's rows [s0, s1).  FULL: every lane of the group holds kLB valid
// bytes (rb = kLB * 32 * W), so no lane tests its bounds.
template <bool FULL>
__device__ __forceinline__ void group_rows(RegShared& S, const GroupJob& J, const WinCtx& wc, int g, int W, int wg,
                                           int lane, int warp, int& nissued, bool& abort)
{
    const int lp = 32 * wg + lane;             // the lane's place in the row
    const int off0 = kLB * lp;                 // its first byte
    const int rb = J.rb;
    const int nvalid = rb - off0;              // its valid bytes (>= kLB: all)
    const bool active = FULL || nvalid > 0;
    const bool leader = (wg == 0 && lane == 0);
    const int dw = (J.bpp + 3) >> 2;
    const uint32_t sh = 8u * (uint32_t)(4 * dw - J.bpp);
    const int L = J.s1 - J.q0;                 // rows staged through the ring
    const uint32_t K80 = 0x80808080u;
    const int wprev = warp > 0 ? warp - 1 : 0;
    // ring: row q0 + k is copy seq0 + k in slot (seq0 + k) % kRegRing; a slot
    // is reused once its row has been windowed and a group barrier has passed
    auto refill = [&](int consumed) {
        const int target = min(L, consumed + kRegRing);
        if (leader) {
            for (int k = nissued; k < target; k++) {
                const uint32_t q = J.seq0 + (uint32_t)k;
                uint64_t* bar = &S.bar[g][q % kRegRing];
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(bar, (uint32_t)J.sp);
                bulk_g2s(J.ring + (size_t)(q % kRegRing) * J.sp, J.raw + (size_t)(J.q0 + k) * J.sp, (uint32_t)J.sp,
                         bar);
            }
        }
        nissued = max(nissued, target);
    };
    auto slot_of = [&](int row) { return J.ring + (size_t)((J.seq0 + (uint32_t)(row - J.q0)) % kRegRing) * J.sp; };
    // the lane's kWPL windowed words of a staged row; bytes past the row end are zero
    auto window_lane = [&](const uint8_t* slot, uint32_t v[kWPL]) {
#pragma unroll
        for (int k = 0; k < kNU; k++) {
            if (FULL || 16 * k < nvalid) {
                window_unit(J.kind, wc, slot, kNU * lp + k, v + 4 * k);
            } else {
#pragma unroll
                for (int q = 0; q < 4; q++) v[4 * k + q] = 0u;
            }
        }
        if (!FULL && nvalid < kLB) {
#pragma unroll
            for (int q = 0; q < kWPL; q++) v[q] &= valid_mask(nvalid, q);
        }
    };

    bool bad = false;
    uint32_t x[kWPL], b[kWPL];
#pragma unroll
    for (int q = 0; q < kWPL; q++) x[q] = b[q] = 0u;
    // row above the group's first row: windowed raw, the caller's prior row, or zeros
    if (J.s0 > 0) {
        bad = !wait_row(S, g, J.seq0);
        if (active) window_lane(slot_of(J.s0 - 1), b);
    } else if (J.prior && active) {
#pragma unroll
        for (int q = 0; q < kWPL; q++) {
            uint32_t v = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int i = off0 + 4 * q + k;
                if (i < rb) v |= (uint32_t)J.prior[i] << (8 * k);
            }
            b[q] = v;
        }
    }
    if (lane == 31) *reinterpret_cast<uint2*>(S.xch[2][warp]) = make_uint2(b[kWPL - 2], b[kWPL - 1]);
    bad = !wait_row(S, g, J.seq0 + (uint32_t)(J.s0 - J.q0)) || bad;
    if (active) window_lane(slot_of(J.s0), x);
    if (lane == 31) *reinterpret_cast<uint2*>(S.xch[J.s0 & 1][warp]) = make_uint2(x[kWPL - 2], x[kWPL - 1]);
    abort = group_bar(g, W, bad);
    // the two words left of b and of x: the previous lane's last two, or the
    // previous warp's (through shared memory), zeros at the row start
    uint32_t bm1, bm2, xm1, xm2;
    {
        const uint2 pb = *reinterpret_cast<const uint2*>(S.xch[2][wprev]);
        const uint2 px = *reinterpret_cast<const uint2*>(S.xch[J.s0 & 1][wprev]);
        bm1 = __shfl_up_sync(kFull, b[kWPL - 1], 1);
        bm2 = __shfl_up_sync(kFull, b[kWPL - 2], 1);
        xm1 = __shfl_up_sync(kFull, x[kWPL - 1], 1);
        xm2 = __shfl_up_sync(kFull, x[kWPL - 2], 1);
        if (lane == 0) {
            bm1 = wg > 0 ? pb.y : 0u;
            bm2 = wg > 0 ? pb.x : 0u;
            xm1 = wg > 0 ? px.y : 0u;
            xm2 = wg > 0 ? px.x : 0u;
        }
    }
    if (abort) return;
    refill(J.s0 - J.q0 + 1);

    // output geometry of the previous row, carried from step to step
    RowOut prev = row_out(J.filt + (size_t)J.s0 * (size_t)(rb + 1), rb);
    uint8_t* Rj = prev.R;
#pragma unroll 1
    for (int j = J.s0; j < J.s1; j++) {
        // ---- scores of row j: a and c are x and b shifted left by bpp bytes
        uint32_t S0 = 0, S1 = 0, S2 = 0, S3 = 0, S4 = 0;
        uint32_t av[kWPL], pp[kWPL];
#pragma unroll
        for (int q = 0; q < kWPL; q++) {
            const uint32_t aq = left_word(x, xm1, xm2, dw, sh, q);
            const uint32_t cq = left_word(b, bm1, bm2, dw, sh, q);
            av[q] = avg4_dev(aq, b[q]);
            pp[q] = paeth_word(aq, b[q], cq, widen_lo(aq), widen_hi(aq), widen_lo(b[q]), widen_hi(b[q]),
                               widen_lo(cq), widen_hi(cq));
            uint32_t d1 = __vabsdiffu4(x[q], aq), d2 = __vabsdiffu4(x[q], b[q]);
            uint32_t d3 = __vabsdiffu4(x[q], av[q]), d4 = __vabsdiffu4(x[q], pp[q]);
            if (!FULL && nvalid < kLB) {
                // bytes past the row end: x = 0 and d = 0, which add 128 - |0 - 128| = 0
                const uint32_t m = valid_mask(nvalid, q);
                d1 &= m; d2 &= m; d3 &= m; d4 &= m;
            }
            S0 = sad4(x[q], K80, S0);
            S1 = sad4(d1, K80, S1);
            S2 = sad4(d2, K80, S2);
            S3 = sad4(d3, K80, S3);
            S4 = sad4(d4, K80, S4);
        }
        // every byte a lane holds, valid or not, added 128 - |d - 128| (0 for
        // the masked ones) to its cost: kLB * 128 - S per filter
        const uint32_t base = (uint32_t)kLB * 128u;
        uint32_t t0s = __reduce_add_sync(kFull, base - S0);
        uint32_t t1s = __reduce_add_sync(kFull, base - S1);
        uint32_t t2s = __reduce_add_sync(kFull, base - S2);
        uint32_t t3s = __reduce_add_sync(kFull, base - S3);
        uint32_t t4s = __reduce_add_sync(kFull, base - S4);
        {
            // every lane holds the same sums: all store the same words
            uint32_t* p = S.part[j & 1][warp];
            *reinterpret_cast<uint4*>(p) = make_uint4(t0s, t1s, t2s, t3s);
            p[4] = t4s;
        }
        // ---- window row j + 1 while the other warps finish row j
        uint32_t xn[kWPL];
#pragma unroll
        for (int q = 0; q < kWPL; q++) xn[q] = 0u;
        const bool more = j + 1 < J.s1;
        bad = false;
        if (more) {
            bad = !wait_row(S, g, J.seq0 + (uint32_t)(j + 1 - J.q0));
            if (active) window_lane(slot_of(j + 1), xn);
            if (lane == 31) *reinterpret_cast<uint2*>(S.xch[(j + 1) & 1][warp]) = make_uint2(xn[kWPL - 2], xn[kWPL - 1]);
        }
        abort = group_bar(g, W, bad);
        if (abort) return;
        // ---- the row's winner
        if (W > 1) {
            const uint32_t* p = S.part[j & 1][warp - wg + (lane < W ? lane : 0)];
            const uint4 t = *reinterpret_cast<const uint4*>(p);
            const uint32_t t4 = p[4];
            const bool in = lane < W;
            t0s = __reduce_add_sync(kFull, in ? t.x : 0u);
            t1s = __reduce_add_sync(kFull, in ? t.y : 0u);
            t2s = __reduce_add_sync(kFull, in ? t.z : 0u);
            t3s = __reduce_add_sync(kFull, in ? t.w : 0u);
            t4s = __reduce_add_sync(kFull, in ? t4 : 0u);
        }
        int f = 0;
        {
            uint32_t best = t0s;
            if (t1s < best) { best = t1s; f = 1; }
            if (t2s < best) { best = t2s; f = 2; }
            if (t3s < best) { best = t3s; f = 3; }
            if (t4s < best) { f = 4; }
        }
        // ---- left words of row j + 1; its ring slot is free again
        uint32_t nm1, nm2;
        {
            const uint2 pn = *reinterpret_cast<const uint2*>(S.xch[(j + 1) & 1][wprev]);
            nm1 = __shfl_up_sync(kFull, xn[kWPL - 1], 1);
            nm2 = __shfl_up_sync(kFull, xn[kWPL - 2], 1);
            if (lane == 0) { nm1 = wg > 0 ? pn.y : 0u; nm2 = wg > 0 ? pn.x : 0u; }
        }
        if (more) refill(j + 1 - J.q0 + 1);
        // ---- row j - 1's aligned chunks (its residuals are visible since this barrier)
        if (j > J.s0 && active) {
            const uint8_t* rp = ((j - 1) & 1) ? J.resid1 : J.resid0;
#pragma unroll
            for (int k = 0; k < kNU; k++) store_chunks(prev, rp, kNU * lp + k);
        }
        // ---- row j's residuals: x minus the winner's predictor (f is the
        // same in every lane of the group)
        uint32_t r[kWPL];
        switch (f) {
            case 0:
#pragma unroll
                for (int q = 0; q < kWPL; q++) r[q] = x[q];
                break;
            case 1:
#pragma unroll
                for (int q = 0; q < kWPL; q++) r[q] = sub4(x[q], left_word(x, xm1, xm2, dw, sh, q));
                break;
            case 2:
#pragma unroll
                for (int q = 0; q < kWPL; q++) r[q] = sub4(x[q], b[q]);
                break;
            case 3:
#pragma unroll
                for (int q = 0; q < kWPL; q++) r[q] = sub4(x[q], av[q]);
                break;
            default:
#pragma unroll
                for (int q = 0; q < kWPL; q++) r[q] = sub4(x[q], pp[q]);
                break;
        }
        const RowOut o = row_out(Rj, rb);
        if (active) {
            uint8_t* rp = ((j & 1) ? J.resid1 : J.resid0) + 16 + off0;
#pragma unroll
            for (int k = 0; k < kNU; k++)
                reinterpret_cast<uint4*>(rp)[k] = make_uint4(r[4 * k], r[4 * k + 1], r[4 * k + 2], r[4 * k + 3]);
        }
        // bytes outside the aligned chunks: the type byte and the row's first
        // h data bytes (lane 0 of the first warp), and its tail from t0 on
        // (the last lanes)
        if (wg == 0 || kLB * 32 * (wg + 1) > o.t0) {
            int k0 = kLB, k1 = 0;
            if (lp == 0) {
                o.R[0] = (uint8_t)f;
                k0 = 0;
                k1 = min(o.h, rb);
            }
            if (active && off0 + kLB > o.t0) {
                k0 = min(k0, max(0, o.t0 - off0));
                k1 = min(kLB, rb - off0);
            }
            for (int k = k0; k < k1; k++) {
                if (off0 + k >= o.h && off0 + k < o.t0) continue;      // inside an aligned chunk
                uint32_t w = r[0];
#pragma unroll
                for (int q = 1; q < kWPL; q++)
                    if ((k >> 2) == q) w = r[q];
                o.R[1 + off0 + k] = (uint8_t)(w >> (8 * (k & 3)));
            }
        }
        if (J.last_row && j == J.height - 1 && active) {
#pragma unroll
            for (int k = 0; k < kNU; k++)
                store_bytes(J.last_row + off0 + 16 * k, x[4 * k], x[4 * k + 1], x[4 * k + 2], x[4 * k + 3], 0,
                            max(0, min(16, rb - off0 - 16 * k)));
        }
        prev = o;
        Rj += rb + 1;
        // ---- slide down: row j becomes the row above
#pragma unroll
        for (int q = 0; q < kWPL; q++) {
            b[q] = x[q];
            x[q] = xn[q];
        }
        bm1 = xm1;
        bm2 = xm2;
        xm1 = nm1;
        xm2 = nm2;
    }
    abort = group_bar(g, W, false);
    if (active) {
        const uint8_t* rp = ((J.s1 - 1) & 1) ? J.resid1 : J.resid0;
#pragma unroll
        for (int k = 0; k < kNU; k++) store_chunks(prev, rp, kNU * lp + k);
    }
}

__global__ void __maxnreg__(80)
k_window_filter_reg(DevImage* __restrict__ imgs, const BandItem* __restrict__ items, int nitems)
{
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ RegShared S;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int NW = blockDim.x >> 5;
    if (tid < kRegMaxWarps * kRegRing) mbar_init(&S.bar[tid / kRegRing][tid % kRegRing], 1);
    if (tid < kRegMaxWarps) S.seq[tid] = 0;
    if (tid == 0) S.img = -1;
    fence_mbar_init();
    __syncthreads();

    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const BandItem bi = items[it];
        DevImage& d = imgs[bi.img];
        GroupJob J;
        J.raw = d.raw;
        J.filt = d.filt;
        J.prior = d.prior;
        J.last_row = d.last_row;
        J.rb = d.rb;
        J.sp = d.in_pitch;
        J.height = (int)d.height;
        J.bpp = d.bpp;
        const int W = reg_warps(J.rb);
        const int G = NW / W;
        const int lreg = reg_lut_bytes(reg_lut_reserve(d.req_mode, d.ib, d.ob, d.dp.bits_stored), 1);
        // the host routes only tables that fit, and bulk-copyable rows, here
        if (G == 0 || (reinterpret_cast<uintptr_t>(J.raw) & 15) || (J.sp & 15) || lreg > kRegLutMax) {
            if (tid == 0) atomicExch(&d.status, R2P_EINVAL);
            continue;                                // uniform: every thread skips the item
        }
        const int g = warp / W, wg = warp - g * W;
        const int nrows = (int)(bi.r1 - bi.r0);
        const int per = (nrows + G - 1) / G;
        J.s0 = (int)bi.r0 + min(nrows, g * per);
        J.s1 = (int)bi.r0 + min(nrows, g * per + per);
        J.q0 = J.s0 > 0 ? J.s0 - 1 : J.s0;         // first staged row: the row above when there is one
        J.ring = smem + lreg + (size_t)(g < G ? g : 0) * reg_group_bytes(J.rb, J.sp);
        J.resid0 = J.ring + kRegRing * J.sp;
        J.resid1 = J.resid0 + reg_resid_bytes(J.rb);
        J.seq0 = S.seq[g < G ? g : 0];
        int nissued = 0;
        // first raw rows in flight before the window table is built
        if (g < G && J.s0 < J.s1 && wg == 0 && lane == 0) {
            const int pre = min(kRegRing, J.s1 - J.q0);
            fence_proxy_async_smem();
            for (int k = 0; k < pre; k++) {
                const uint32_t q = J.seq0 + (uint32_t)k;
                uint64_t* bar = &S.bar[g][q % kRegRing];
                mbar_arrive_expect_tx(bar, (uint32_t)J.sp);
                bulk_g2s(J.ring + (size_t)(q % kRegRing) * J.sp, J.raw + (size_t)(J.q0 + k) * J.sp, (uint32_t)J.sp,
                         bar);
            }
        }
        if (g < G && J.s0 < J.s1) nissued = min(kRegRing, J.s1 - J.q0);
        // resolve the window and build its table once per image; every
        // thread reads S.img before the barrier, thread 0 rewrites it after
        const bool new_img = (int)bi.img != S.img;
        __syncthreads();
        if (new_img) {
            if (tid == 0) {
                S.res = resolve_window(d);
                S.img = (int)bi.img;
            }
            __syncthreads();
            if (S.res.mode == W_A2_LUT) fill_a2_table_fast(d, S.res, smem, tid, blockDim.x);
            else                        fill_window_table(d, S.res, smem, tid, blockDim.x);
            __syncthreads();
        }
        const WinRes res = S.res;
        WinCtx wc;
        wc.mode = res.mode; wc.ib = d.ib; wc.ob = d.ob; wc.shift = res.shift; wc.mask = res.mask;
        wc.qa = res.qa; wc.qb = res.qb; wc.dp = d.dp;
        wc.lut = smem;
        J.kind = win_kind(wc);
        if (J.kind == K_LUT16 && res.shift == 0) J.kind = K_LUT16Z;
        if (g < G && J.s0 < J.s1) {
            bool abort = false;
            if (J.kind == K_DIRECT) {
                abort = true;                        // never routed here; report instead of guessing
            } else if (kLB * 32 * W == J.rb) {
                group_rows<true>(S, J, wc, g, W, wg, lane, warp, nissued, abort);
            } else {
                group_rows<false>(S, J, wc, g, W, wg, lane, warp, nissued, abort);
            }
            if (abort) {
                // a copy did not land in time: report, and stay until every
                // copy issued into this group's ring has landed (bounded)
                if (wg == 0 && lane == 0) {
                    atomicExch(&d.status, J.kind == K_DIRECT ? R2P_EINVAL : R2P_ETIMEOUT);
                    for (int k = 0; k < nissued; k++)
                        mbar_wait_bounded(&S.bar[g][(J.seq0 + k) % kRegRing], ((J.seq0 + k) / kRegRing) & 1u,
                                          kRegDrainNs);
                }
            }
            if (wg == 0 && lane == 0) S.seq[g] = J.seq0 + (uint32_t)nissued;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int reg_filter_warps(int rb) { return reg_warps(rb); }

bool reg_filter_eligible(int rb, int in_pitch, int lut_bytes)
{
    return rb >= 1 && reg_warps(rb) <= kRegMaxWarps && (in_pitch & 15) == 0 && lut_bytes <= kRegLutMax;
}

int reg_filter_max_row_bytes() { return kRegMaxWarps * 32 * kLB; }

// Warps per CTA for a launch whose widest row needs max_w warps: a multiple
// of every smaller row's warp count (12 = 1, 2, 3, 4, 6, 12), else the
// widest row's own.  At 80 registers a thread, two 12-warp CTAs fit an SM.
int reg_filter_cta_warps(int max_w) { return max_w <= 12 ? 12 : kRegMaxWarps; }

int reg_filter_smem(int rb, int in_pitch, int lut_bytes, int nw)
{
    const int W = reg_warps(rb);
    return reg_lut_bytes(lut_bytes, 1) + (nw / W) * reg_group_bytes(rb, in_pitch) + 64;
}

int reg_filter_ctas_per_sm(int nw, int smem)
{
    int n = 0;
    cudaFuncSetAttribute(k_window_filter_reg, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_window_filter_reg, nw * 32, smem) != cudaSuccess)
        return 1;
    return n > 0 ? n : 1;
}

cudaError_t launch_window_filter_reg(DevImage* imgs, const BandItem* items, int nitems, int grid, int nw, int smem,
                                     cudaStream_t s)
{
    cudaError_t e = cudaFuncSetAttribute(k_window_filter_reg, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         200 * 1024);
    if (e != cudaSuccess) return e;
    k_window_filter_reg<<<grid, nw * 32, smem, s>>>(imgs, items, nitems);
    note_launch();
    return cudaGetLastError();
}

}  // namespace r2p
