// k_filter.cu -- window/level + adaptive PNG filter, fused in one pass.
//
// Reference semantics:
//   windowing, 16-bit out: dicom_preprocess_kernel   src/gpu_filter.cu:71-162
//   windowing, 8-bit out : try_apply_linear_window   src/batch_processor.cpp:202-266
//                          build/apply_dicom16_lut   src/batch_processor.cpp:100-185
//                          dispatch                  src/batch_processor.cpp:397-409
//   adaptive filter      : filter_select_kernel      src/gpu_filter.cu:183-309
//
// Design.  One CTA owns a band of consecutive rows of one image.  It windows
// the raw rows into a ring of shared-memory row slots (16-byte coalesced loads
// where the rows allow it) and keeps the last windowed row of a tile as the
// "row above" of the next tile, so every raw byte is read once per band (plus
// one row per band).  Each row is then scored for the five PNG filters by a
// group of warps: four bytes per lane per step in SWAR arithmetic, costs summed
// with a signed dp4a, warp shuffles for the reduction.  The winning filter is
// recomputed and written straight to HBM with 4-byte stores realigned by a
// funnel shift, so the filtered row never round-trips through shared memory.
// Float arithmetic uses explicit IEEE intrinsics (no contraction), matching
// the oracle's -ffp-contract=off restatement bit for bit.
#include <cuda_runtime.h>

#include <algorithm>

#include "r2p_common.h"
#include "r2p_device.h"
#include "r2p_kernels.h"
#include "r2p_tma.cuh"
#include "k_window.cuh"

namespace r2p {

// Resolve each image's window request into a WinMode and build its table.
// One CTA per image.
__global__ void k_prepare_window(DevImage* imgs, int n)
{
    DevImage& d = imgs[blockIdx.x];
    __shared__ WinRes s_res;
    if (threadIdx.x == 0) {
        const WinRes r = resolve_window(d);
        d.mode = r.mode;
        d.qa = r.qa;
        d.qb = r.qb;
        d.lut_shift = r.shift;
        d.lut_mask = r.mask;
        d.lut_entries = r.entries;
        d.lut_esize = r.esize;
        s_res = r;
    }
    __syncthreads();
    fill_window_table(d, s_res, d.lut, threadIdx.x, blockDim.x);
}

// ---------------------------------------------------------------------------
// Fused window + filter
// ---------------------------------------------------------------------------
constexpr int kFiltThreads = 256;
constexpr int kFiltWarps = kFiltThreads / 32;

__host__ __device__ inline int warps_per_row(int rb)
{
    return rb <= 4096 ? 1 : rb <= 8192 ? 2 : rb <= 16384 ? 4 : 8;
}

__host__ __device__ inline int slot_stride(int rb)
{
    return 16 + ((rb + 15) & ~15) + 16;
}

// Raw bytes per row a bulk-copy tile stages (0 when rows are not 16-byte
// multiples: plain loads then).
__host__ __device__ inline int staged_pitch(int in_pitch) { return (in_pitch & 15) ? 0 : in_pitch; }

// Rows per tile for staging pitch sp in smem bytes of dynamic shared memory:
// the most rows, up to cap_rows, whose staging + (rows+1) slots fit.
__host__ __device__ inline int tile_rows_sp(int rb, int sp, int smem, int lreg, int cap_rows)
{
    const int stride = slot_stride(rb);
    for (int t = cap_rows; t >= 1; t--)
        if (lreg + t * sp + (t + 1) * stride <= smem) return t;
    return 0;
}

// Staging pitch actually used at a given shared-memory size: rows too wide to
// stage even one row next to two ring slots are windowed from global memory
// straight into the ring.  Host planning and the kernel both decide here.
__host__ __device__ inline int staged_pitch_for(int rb, int in_pitch, int smem, int lreg)
{
    const int sp = staged_pitch(in_pitch);
    return (sp && tile_rows_sp(rb, sp, smem, lreg, 1) >= 1) ? sp : 0;
}

__host__ __device__ inline int tile_rows_for(int rb, int in_pitch, int smem, int lreg, int cap_rows)
{
    return tile_rows_sp(rb, staged_pitch_for(rb, in_pitch, smem, lreg), smem, lreg, cap_rows);
}

__host__ __device__ inline int lut_region_bytes(int mode, int entries, int esize)
{
    const bool lut = (mode == W_A2_LUT) || (mode == W_LUT8);
    const int b = entries * esize;
    return (lut && b <= kMaxSmemLut) ? ((b + 15) & ~15) : 0;
}


// Window raw row `r` of image d into smem row `dst` (rb bytes) with plain
// global loads and zero its tail.  aligned: rows are 16-byte multiples at a
// 16-byte aligned base (whole units); otherwise one 4-byte output group per
// thread from byte loads.
template <int K>
__device__ void window_row_k(const DevImage& d, const WinCtx& w, int r, uint8_t* dst, int tid, int nthr, bool aligned)
{
    const uint8_t* src = d.raw + (size_t)r * (size_t)d.in_pitch;
    constexpr bool to8 = (K == K_Q15 || K == K_LUT8);
    if (aligned) {
        const int units = d.in_pitch >> 4;
        const uint4* s4 = reinterpret_cast<const uint4*>(src);
        for (int u = tid; u < units; u += nthr) {
            uint32_t o[4];
            win_unit<K>(w, __ldg(s4 + u), o);
            if (to8) *reinterpret_cast<uint2*>(dst + 8 * u) = make_uint2(o[0], o[1]);
            else     *reinterpret_cast<uint4*>(dst + 16 * u) = make_uint4(o[0], o[1], o[2], o[3]);
        }
    } else {
        const int groups = (d.rb + 3) >> 2;
        for (int g = tid; g < groups; g += nthr) {
            uint32_t o = 0;
            const int b0 = 4 * g;
            if (to8) {
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int so = 2 * (b0 + j);
                    if (b0 + j < d.rb)
                        o |= win_sample<K>(w, (uint32_t)__ldg(src + so) | ((uint32_t)__ldg(src + so + 1) << 8)) << (8 * j);
                }
            } else if (d.ib == 2) {
#pragma unroll
                for (int j = 0; j < 2; j++) {
                    const int bo = b0 + 2 * j;
                    if (bo < d.rb) {
                        const uint32_t raw = (uint32_t)__ldg(src + bo) | ((uint32_t)__ldg(src + bo + 1) << 8);
                        // K_COPY keeps memory order: the little-endian pair is the bytes as they lie
                        o |= win_sample<K>(w, raw) << (16 * j);
                    }
                }
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int bo = b0 + j;
                    if (bo < d.rb) o |= win_sample<K>(w, __ldg(src + bo)) << (8 * j);
                }
            }
            if (b0 + 4 <= d.rb) {
                *reinterpret_cast<uint32_t*>(dst + b0) = o;
            } else {
                for (int j = 0; b0 + j < d.rb; j++) dst[b0 + j] = (uint8_t)(o >> (8 * j));
            }
        }
    }
    // zero the tail so the last partial word and the word after it read zeros
    const int tail0 = d.rb, tail1 = ((d.rb + 15) & ~15) + 16;
    for (int i = tail0 + tid; i < tail1; i += nthr) dst[i] = 0;
}

__device__ void window_row_range(const DevImage& d, const WinCtx& w, int r, uint8_t* dst, int tid, int nthr,
                                 bool aligned)
{
    switch (win_kind(w)) {
        case K_COPY: window_row_k<K_COPY>(d, w, r, dst, tid, nthr, aligned); break;
        case K_SWAP16: window_row_k<K_SWAP16>(d, w, r, dst, tid, nthr, aligned); break;
        case K_LUT16: window_row_k<K_LUT16>(d, w, r, dst, tid, nthr, aligned); break;
        case K_LUT8IN: window_row_k<K_LUT8IN>(d, w, r, dst, tid, nthr, aligned); break;
        case K_Q15: window_row_k<K_Q15>(d, w, r, dst, tid, nthr, aligned); break;
        case K_LUT8: window_row_k<K_LUT8>(d, w, r, dst, tid, nthr, aligned); break;
        default: window_row_k<K_DIRECT>(d, w, r, dst, tid, nthr, aligned); break;
    }
}

__device__ __forceinline__ uint8_t filtered_byte(const uint8_t* xr, const uint8_t* ur, int i, int bpp, int f)
{
    const uint32_t x = xr[i], b = ur[i];
    const uint32_t a = (i >= bpp) ? xr[i - bpp] : 0u, c = (i >= bpp) ? ur[i - bpp] : 0u;
    return (uint8_t)filter_word(f, x, a, b, c);
}


// Window n staged raw rows (16-byte multiples, in shared memory) into their
// ring slots.  All threads; rows outer, 16-byte units inner.
template <int K>
__device__ void window_staged_k(const DevImage& d, const WinCtx& w, const uint8_t* stage, int n, uint8_t* ring,
                                int stride, int slots, int rel0, int tid, int nthr)
{
    constexpr bool to8 = (K == K_Q15 || K == K_LUT8);
    const int units = d.in_pitch >> 4;
    const int tail0 = d.rb, tail1 = ((d.rb + 15) & ~15) + 16;
    for (int j = 0; j < n; j++) {
        const uint4* s4 = reinterpret_cast<const uint4*>(stage + (size_t)j * d.in_pitch);
        uint8_t* dst = ring + ((rel0 + j) % slots) * stride + 16;
        for (int u = tid; u < units; u += nthr) {
            uint32_t o[4];
            win_unit<K>(w, s4[u], o);
            if (to8) reinterpret_cast<uint2*>(dst)[u] = make_uint2(o[0], o[1]);
            else     reinterpret_cast<uint4*>(dst)[u] = make_uint4(o[0], o[1], o[2], o[3]);
        }
        for (int i = tail0 + tid; i < tail1; i += nthr) dst[i] = 0;
    }
}

__device__ void window_staged_rows(const DevImage& d, const WinCtx& w, const uint8_t* stage, int n, uint8_t* ring,
                                   int stride, int slots, int rel0, int tid, int nthr)
{
    switch (win_kind(w)) {
        case K_COPY: window_staged_k<K_COPY>(d, w, stage, n, ring, stride, slots, rel0, tid, nthr); break;
        case K_SWAP16: window_staged_k<K_SWAP16>(d, w, stage, n, ring, stride, slots, rel0, tid, nthr); break;
        case K_LUT16: window_staged_k<K_LUT16>(d, w, stage, n, ring, stride, slots, rel0, tid, nthr); break;
        case K_LUT8IN: window_staged_k<K_LUT8IN>(d, w, stage, n, ring, stride, slots, rel0, tid, nthr); break;
        case K_Q15: window_staged_k<K_Q15>(d, w, stage, n, ring, stride, slots, rel0, tid, nthr); break;
        case K_LUT8: window_staged_k<K_LUT8>(d, w, stage, n, ring, stride, slots, rel0, tid, nthr); break;
        default: window_staged_k<K_DIRECT>(d, w, stage, n, ring, stride, slots, rel0, tid, nthr); break;
    }
}

// One 16-byte unit of a windowed row (u >= 0) and the two words before it
// (the slot's 16 guard bytes are zero, so unit 0 sees zeros on its left).
struct RowUnit {
    uint32_t m2, m1, w[4];
};

__device__ __forceinline__ RowUnit load_unit(const uint8_t* row, int u)
{
    const uint4 v = *reinterpret_cast<const uint4*>(row + 16 * u);
    const uint2 p = *reinterpret_cast<const uint2*>(row + 16 * u - 8);
    RowUnit r;
    r.m2 = p.x; r.m1 = p.y;
    r.w[0] = v.x; r.w[1] = v.y; r.w[2] = v.z; r.w[3] = v.w;
    return r;
}

// Words of the bytes bpp to the left of the unit's four words.  DW = words
// reached back (1 for bpp <= 4, 2 for bpp 6 or 8); sh = 8 * (4 * DW - bpp).
template <int DW>
__device__ __forceinline__ void left_words(const RowUnit& r, uint32_t sh, uint32_t out[4])
{
    if (DW == 1) {
        out[0] = fshr(r.m1, r.w[0], sh);
        out[1] = fshr(r.w[0], r.w[1], sh);
        out[2] = fshr(r.w[1], r.w[2], sh);
        out[3] = fshr(r.w[2], r.w[3], sh);
    } else {
        out[0] = fshr(r.m2, r.m1, sh);
        out[1] = fshr(r.m1, r.w[0], sh);
        out[2] = fshr(r.w[0], r.w[1], sh);
        out[3] = fshr(r.w[1], r.w[2], sh);
    }
}

// Byte mask of word q of a unit with nvalid valid bytes.
__device__ __forceinline__ uint32_t unit_word_mask(int nvalid, int q)
{
    const int k = nvalid - 4 * q;
    return k >= 4 ? 0xFFFFFFFFu : k <= 0 ? 0u : ((1u << (8 * k)) - 1u);
}

// Scores of units [us, ue) of one row, this warp's share.
template <int DW>
__device__ __forceinline__ Score5 score_units(const uint8_t* xr, const uint8_t* ur, int us, int ue, int rb, uint32_t sh,
                                              int lane)
{
    Score5 s = {0u, 0u, 0u, 0u, 0u};
    for (int u = us + lane; u < ue; u += 32) {
        const RowUnit X = load_unit(xr, u), B = load_unit(ur, u);
        uint32_t a[4], c[4];
        left_words<DW>(X, sh, a);
        left_words<DW>(B, sh, c);
        const int nvalid = rb - 16 * u;
        if (nvalid >= 16) {
#pragma unroll
            for (int q = 0; q < 4; q++) score_word(s, X.w[q], a[q], B.w[q], c[q], 0xFFFFFFFFu);
        } else {
#pragma unroll
            for (int q = 0; q < 4; q++) score_word(s, X.w[q], a[q], B.w[q], c[q], unit_word_mask(nvalid, q));
        }
    }
    return s;
}

// Filtered word of filter type F (compile-time).
template <int F>
__device__ __forceinline__ uint32_t filter_word_t(uint32_t x, uint32_t a, uint32_t b, uint32_t c)
{
    if (F == 0) return x;
    if (F == 1) return sub4(x, a);
    if (F == 2) return sub4(x, b);
    if (F == 3) return sub4(x, avg4(a, b));
    return sub4(x, R2P_PAETH4(a, b, c));
}

// Filtered words (type F) of units [us, ue), stored as 4-byte words aligned to
// the output: gw = the aligned word holding data byte 0 minus e bytes, words
// klo..khi lie wholly inside the row; the rest is written byte-wise by the caller.
template <int DW, int F>
__device__ __forceinline__ void store_units_t(const uint8_t* xr, const uint8_t* ur, int us, int ue, uint32_t sh,
                                              uint32_t* gw, int e, int klo, int khi, int lane)
{
    uint32_t carry = 0;                       // last filtered word of the unit before this lane's
    if (us > 0) {
        const RowUnit X = load_unit(xr, us - 1), B = load_unit(ur, us - 1);
        uint32_t a[4], c[4];
        left_words<DW>(X, sh, a);
        left_words<DW>(B, sh, c);
        carry = filter_word_t<F>(X.w[3], a[3], B.w[3], c[3]);
    }
    const uint32_t es = 8u * (uint32_t)e;
    for (int u0 = us; u0 < ue; u0 += 32) {
        const int u = u0 + lane;
        uint32_t Fw[4] = {0u, 0u, 0u, 0u};
        if (u < ue) {
            const RowUnit X = load_unit(xr, u), B = load_unit(ur, u);
            uint32_t a[4], c[4];
            left_words<DW>(X, sh, a);
            left_words<DW>(B, sh, c);
#pragma unroll
            for (int q = 0; q < 4; q++) Fw[q] = filter_word_t<F>(X.w[q], a[q], B.w[q], c[q]);
        }
        uint32_t Fp = __shfl_up_sync(0xFFFFFFFFu, Fw[3], 1);
        const uint32_t last = __shfl_sync(0xFFFFFFFFu, Fw[3], 31);
        if (lane == 0) Fp = carry;
        carry = last;
        if (u < ue) {
            const int k0 = 4 * u;
            if (k0 >= klo && k0 + 3 <= khi) {             // the whole unit is interior
                if (e) {
                    gw[k0] = __funnelshift_l(Fp, Fw[0], es);
                    gw[k0 + 1] = __funnelshift_l(Fw[0], Fw[1], es);
                    gw[k0 + 2] = __funnelshift_l(Fw[1], Fw[2], es);
                    gw[k0 + 3] = __funnelshift_l(Fw[2], Fw[3], es);
                } else {
                    gw[k0] = Fw[0]; gw[k0 + 1] = Fw[1]; gw[k0 + 2] = Fw[2]; gw[k0 + 3] = Fw[3];
                }
            } else {
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int k = k0 + q;
                    const uint32_t prevw = q == 0 ? Fp : Fw[q - 1];
                    if (k >= klo && k <= khi) gw[k] = e ? __funnelshift_l(prevw, Fw[q], es) : Fw[q];
                }
            }
        }
    }
}

template <int DW>
__device__ __forceinline__ void store_units(const uint8_t* xr, const uint8_t* ur, int us, int ue, uint32_t sh, int f,
                                            uint32_t* gw, int e, int klo, int khi, int lane)
{
    switch (f) {
        case 0: store_units_t<DW, 0>(xr, ur, us, ue, sh, gw, e, klo, khi, lane); break;
        case 1: store_units_t<DW, 1>(xr, ur, us, ue, sh, gw, e, klo, khi, lane); break;
        case 2: store_units_t<DW, 2>(xr, ur, us, ue, sh, gw, e, klo, khi, lane); break;
        case 3: store_units_t<DW, 3>(xr, ur, us, ue, sh, gw, e, klo, khi, lane); break;
        default: store_units_t<DW, 4>(xr, ur, us, ue, sh, gw, e, klo, khi, lane); break;
    }
}

// Barrier over the nthreads threads (a multiple of 32) of one row group; ids
// 1..15 (0 is __syncthreads).  Every warp of the group executes the same
// sequence of these.
__device__ __forceinline__ void group_sync(int id, int nthreads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Time limit for one bulk copy of a tile to land in shared memory, and the
// further wait for it after a timeout before the CTA gives its memory back.
constexpr uint64_t kBulkWaitNs = 200ull * 1000 * 1000;
constexpr uint64_t kBulkDrainNs = 2000ull * 1000 * 1000;

__global__ void __launch_bounds__(kFiltThreads)
k_window_filter(DevImage* __restrict__ imgs, const BandItem* __restrict__ items, int nitems, int smem_bytes)
{
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ uint32_t red[kFiltWarps][5];
    __shared__ __align__(8) uint64_t bar;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    uint32_t phase = 0;

    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const BandItem bi = items[it];
        DevImage& d = imgs[bi.img];
        const int rb = d.rb, bpp = d.bpp;
        const int lreg = lut_region_bytes(d.mode, d.lut_entries, d.lut_esize);
        const int stride = slot_stride(rb);
        const int G = warps_per_row(rb);
        const int rpp = kFiltWarps / G;                     // rows per pass
        const int T = tile_rows_for(rb, d.in_pitch, smem_bytes, lreg, 2 * rpp);
        const int slots = T + 1;
        const int sp = staged_pitch_for(rb, d.in_pitch, smem_bytes, lreg);
        uint8_t* stage = smem + lreg;
        uint8_t* ring = stage + (size_t)T * sp;
        // bulk copies need a 16-byte aligned source; otherwise plain loads
        const bool bulk = sp > 0 && ((reinterpret_cast<uintptr_t>(d.raw) & 15) == 0);

        WinCtx w;
        w.mode = d.mode; w.ib = d.ib; w.ob = d.ob; w.shift = d.lut_shift; w.mask = d.lut_mask;
        w.qa = d.qa; w.qb = d.qb; w.dp = d.dp;
        w.lut = (lreg > 0) ? smem : d.lut;

        __syncthreads();   // previous item finished with shared memory
        if (bulk && tid == 0) {                            // first tile's raw rows
            const int n0 = min(T, (int)bi.r1 - (int)bi.r0);
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&bar, (uint32_t)(n0 * sp));
            bulk_g2s(stage, d.raw + (size_t)bi.r0 * d.in_pitch, (uint32_t)(n0 * sp), &bar);
        }
        if (lreg > 0) {
            const uint4* s = reinterpret_cast<const uint4*>(d.lut);
            uint4* t = reinterpret_cast<uint4*>(smem);
            for (int i = tid; i < lreg / 16; i += kFiltThreads) t[i] = s[i];
        }
        for (int i = tid; i < slots * 4; i += kFiltThreads)
            reinterpret_cast<uint32_t*>(ring + (i >> 2) * stride)[i & 3] = 0u;
        __syncthreads();

        const bool aligned = ((d.in_pitch & 15) == 0) && ((reinterpret_cast<uintptr_t>(d.raw) & 15) == 0);
        // row above the band: windowed raw row, caller's prior row, or zeros
        {
            uint8_t* dst = ring + 16;                        // slot of rel 0
            const int r = (int)bi.r0 - 1;
            if (r >= 0) {
                window_row_range(d, w, r, dst, tid, kFiltThreads, aligned);
            } else {
                const int tail1 = ((rb + 15) & ~15) + 16;
                for (int i = tid; i < tail1; i += kFiltThreads)
                    dst[i] = (d.prior && i < rb) ? d.prior[i] : 0;
            }
        }

        for (int t0 = (int)bi.r0; t0 < (int)bi.r1; t0 += T) {
            const int n = min(T, (int)bi.r1 - t0);
            const int rel0 = t0 - (int)bi.r0 + 1;            // rel of the tile's first row
            if (bulk) {
                const bool ok = mbar_wait_bounded(&bar, phase, kBulkWaitNs);
                if (__syncthreads_or(!ok)) {
                    // the copy did not land in time: report it, and keep the
                    // CTA (and its shared memory) until the copy has landed,
                    // for up to kBulkDrainNs more; only a copy engine that
                    // stopped answering altogether outlasts that
                    if (tid == 0) {
                        atomicExch(&d.status, R2P_ETIMEOUT);
                        mbar_wait_bounded(&bar, phase, kBulkDrainNs);
                    }
                    __syncthreads();
                    return;
                }
                phase ^= 1u;
                window_staged_rows(d, w, stage, n, ring, stride, slots, rel0, tid, kFiltThreads);
                __syncthreads();
                const int t1 = t0 + n;
                if (t1 < (int)bi.r1 && tid == 0) {           // prefetch the next tile during filtering
                    const int n1 = min(T, (int)bi.r1 - t1);
                    fence_proxy_async_smem();
                    mbar_arrive_expect_tx(&bar, (uint32_t)(n1 * sp));
                    bulk_g2s(stage, d.raw + (size_t)t1 * d.in_pitch, (uint32_t)(n1 * sp), &bar);
                }
            } else {
                for (int j = warp; j < n; j += kFiltWarps) {
                    uint8_t* dst = ring + ((rel0 + j) % slots) * stride + 16;
                    window_row_range(d, w, t0 + j, dst, lane, 32, aligned);
                }
                __syncthreads();
            }

            const int nunits = (rb + 15) >> 4;
            const int g = warp / G, wg = warp % G;
            const int useg = (nunits + G - 1) / G;
            const int us = min(nunits, wg * useg), ue = min(nunits, us + useg);
            const int dw = (bpp + 3) >> 2;                   // words reached back: 1 or 2
            const uint32_t sh = 8u * (uint32_t)(4 * dw - bpp);
            for (int pass = 0; pass * rpp < n; pass++) {
                const int j = pass * rpp + g;                // tile row index of this group
                const bool active = j < n;
                const int rel = rel0 + j;
                const uint8_t* xr = ring + (rel % slots) * stride + 16;
                const uint8_t* ur = ring + ((rel - 1 + slots) % slots) * stride + 16;
                Score5 s = {0u, 0u, 0u, 0u, 0u};
                if (active)
                    s = dw == 1 ? score_units<1>(xr, ur, us, ue, rb, sh, lane) : score_units<2>(xr, ur, us, ue, rb, sh, lane);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    s.s0 += __shfl_xor_sync(0xFFFFFFFFu, s.s0, o);
                    s.s1 += __shfl_xor_sync(0xFFFFFFFFu, s.s1, o);
                    s.s2 += __shfl_xor_sync(0xFFFFFFFFu, s.s2, o);
                    s.s3 += __shfl_xor_sync(0xFFFFFFFFu, s.s3, o);
                    s.s4 += __shfl_xor_sync(0xFFFFFFFFu, s.s4, o);
                }
                if (G > 1) {                                 // combine the group's warps
                    if (lane == 0) {
                        red[warp][0] = s.s0; red[warp][1] = s.s1; red[warp][2] = s.s2;
                        red[warp][3] = s.s3; red[warp][4] = s.s4;
                    }
                    group_sync(1 + g, 32 * G);
                    Score5 t = {0u, 0u, 0u, 0u, 0u};
                    for (int q = g * G; q < g * G + G; q++) {
                        t.s0 += red[q][0]; t.s1 += red[q][1]; t.s2 += red[q][2];
                        t.s3 += red[q][3]; t.s4 += red[q][4];
                    }
                    s = t;
                    group_sync(1 + g, 32 * G);                   // red[] is reused by the next pass
                }
                if (!active) continue;
                const int f = best_filter(s);
                const int r = t0 + j;
                if (d.last_row && r == (int)d.height - 1) {   // the next strip's row above
                    for (int i = wg * 32 + lane; i < rb; i += 32 * G) d.last_row[i] = xr[i];
                }
                uint8_t* orow = d.filt + (size_t)r * (size_t)(rb + 1);
                const uintptr_t data_addr = reinterpret_cast<uintptr_t>(orow + 1);
                const int e = (int)(data_addr & 3);
                uint32_t* gw = reinterpret_cast<uint32_t*>(data_addr - (uintptr_t)e);   // global word of data byte 0
                // interior words: k in [klo, khi]
                const int klo = (e > 0) ? 1 : 0;
                const int khi = (e + rb - 4) >> 2;
                if (dw == 1) store_units<1>(xr, ur, us, ue, sh, f, gw, e, klo, khi, lane);
                else         store_units<2>(xr, ur, us, ue, sh, f, gw, e, klo, khi, lane);
                // type byte, head bytes before the first interior word, tail bytes after the last
                if (wg == 0 && lane == 0) {
                    orow[0] = (uint8_t)f;
                    const int head = (e > 0) ? min(4 - e, rb) : 0;
                    for (int i = 0; i < head; i++) orow[1 + i] = filtered_byte(xr, ur, i, bpp, f);
                }
                if (wg == G - 1 && lane == 31) {
                    const int head = (e > 0) ? min(4 - e, rb) : 0;
                    const int tail_start = max(head, (khi >= klo) ? 4 * (khi + 1) - e : head);
                    for (int i = tail_start; i < rb; i++) orow[1 + i] = filtered_byte(xr, ur, i, bpp, f);
                }
            }
            __syncthreads();
        }
    }
}

// ---------------------------------------------------------------------------
// BMP export
// ---------------------------------------------------------------------------
// File layout of the reference's BmpWriter (src/bmp_writer.cpp:36-96 header
// and palette, :98-131 rows): BITMAPFILEHEADER (14) + BITMAPINFOHEADER (40,
// negative height: rows top to bottom) + a 256-entry gray palette (8-bit
// output only) + rows of width * oc bytes (BGR for colour) zero-padded to a
// multiple of 4.  Pixel sources follow run_bmp_from_source
// (src/pipeline.cpp:1965-2001).

// Byte fb (< 54) of the two headers, little-endian fields.
__device__ uint32_t bmp_header_byte(const DevImage& d, uint32_t fb)
{
    if (fb < 2) return fb == 0 ? 0x42u : 0x4Du;            // "BM"
    uint32_t field;
    uint32_t at;
    if (fb < 6) { field = d.bmp_size; at = 2; }
    else if (fb < 10) return 0u;                         // reserved
    else if (fb < 14) { field = d.bmp_pix_off; at = 10; }
    else if (fb < 18) { field = 40u; at = 14; }          // biSize
    else if (fb < 22) { field = d.width; at = 18; }
    else if (fb < 26) { field = (uint32_t)(-(int32_t)d.height); at = 22; }
    else if (fb < 28) { field = 1u; at = 26; }           // biPlanes
    else if (fb < 30) { field = d.bmp_oc == 1 ? 8u : 24u; at = 28; }
    else if (fb >= 46 && fb < 50) { field = d.bmp_oc == 1 ? 256u : 0u; at = 46; }   // biClrUsed
    else return 0u;
    return (field >> (8 * (fb - at))) & 0xFFu;
}

// One output pixel byte: row r, byte col (< width * oc) of the unpadded row.
__device__ __forceinline__ uint32_t bmp_pixel_byte(const DevImage& d, const WinCtx& w, uint32_t r, uint32_t col)
{
    const uint32_t oc = (uint32_t)d.bmp_oc;
    const uint32_t x = oc == 1 ? col : col / 3u;
    const uint32_t c = col - x * oc;
    const uint32_t si = x * (uint32_t)d.channels + (oc == 3 ? 2u - c : 0u);   // RGB -> BGR
    const uint8_t* row = d.raw + (size_t)r * (size_t)d.in_pitch;
    if (d.bmp_kind == BMP_BYTE) return __ldg(row + si);
    if (d.bmp_kind == BMP_TAKE) return __ldg(row + 2 * si + d.bmp_off);
    const uint32_t raw = (uint32_t)__ldg(row + 2 * si) | ((uint32_t)__ldg(row + 2 * si + 1) << 8);
    return d.mode == W_Q15 ? win_sample<K_Q15>(w, raw) : win_sample<K_LUT8>(w, raw);
}

// Whole BMP files, one 4-byte file word per thread (image blockIdx.y); the
// output buffer is 4-byte aligned.
__global__ void __launch_bounds__(256) k_bmp_file(const DevImage* __restrict__ imgs)
{
    const DevImage& d = imgs[blockIdx.y];
    WinCtx w;
    w.mode = d.mode; w.ib = d.ib; w.ob = 1; w.shift = d.lut_shift; w.mask = d.lut_mask;
    w.qa = d.qa; w.qb = d.qb; w.dp = d.dp;
    w.lut = d.lut;
    const uint32_t nwords = (d.bmp_size + 3u) >> 2;
    const uint32_t rowbytes = d.width * (uint32_t)d.bmp_oc, stride = (uint32_t)d.bmp_stride;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nwords; k += gridDim.x * blockDim.x) {
        const uint32_t fb0 = 4u * k;
        uint32_t word = 0;
        // row and column of the word's first pixel byte, stepped per byte
        uint32_t r = 0, col = 0;
        if (fb0 + 3u >= d.bmp_pix_off) {
            const uint32_t pb = fb0 > d.bmp_pix_off ? fb0 - d.bmp_pix_off : 0u;
            r = pb / stride;
            col = pb - r * stride;
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const uint32_t fb = fb0 + (uint32_t)j;
            uint32_t v = 0;
            if (fb < 54u) {
                v = bmp_header_byte(d, fb);
            } else if (fb < d.bmp_pix_off) {
                const uint32_t q = fb - 54u;                    // gray palette: B = G = R = i, 0
                v = (q & 3u) == 3u ? 0u : (q >> 2);
            } else if (fb < d.bmp_size) {
                if (col < rowbytes) v = bmp_pixel_byte(d, w, r, col);
                if (++col == stride) { col = 0; r++; }
            }
            word |= v << (8 * j);
        }
        uint8_t* out = d.png + fb0;
        if (fb0 + 4u <= d.bmp_size) {
            *reinterpret_cast<uint32_t*>(out) = word;
        } else {
            for (uint32_t j = 0; fb0 + j < d.bmp_size; j++) out[j] = (uint8_t)(word >> (8 * j));
        }
    }
}

}  // namespace r2p

namespace r2p {

// ---------------------------------------------------------------------------
// launch wrappers
// ---------------------------------------------------------------------------
constexpr int kFilterSmemCap = 226 * 1024;   // below the 227 KB opt-in limit minus static smem

int filter_lut_region(int mode, int lut_entries, int lut_esize)
{
    return lut_region_bytes(mode, lut_entries, lut_esize);
}

// Per-CTA shared memory aimed at three CTAs per SM; wider rows take more.
constexpr int kFilterSmemTarget = 72 * 1024;

// Dynamic shared memory wanted for an image: LUT region, the staged raw rows
// of one tile and tile+1 row slots, with the most rows (up to two passes of
// the warp groups) that fit the three-CTA target, else the cap; -1 if even
// one row does not fit.
int filter_smem_bytes(int rb, int in_pitch, int mode, int lut_entries, int lut_esize)
{
    const int lreg = lut_region_bytes(mode, lut_entries, lut_esize);
    const int stride = slot_stride(rb);
    const int rpp = kFiltWarps / warps_per_row(rb);
    int smem = kFilterSmemTarget;
    int t = tile_rows_for(rb, in_pitch, smem, lreg, 2 * rpp);
    if (t == 0) {
        smem = kFilterSmemCap;
        t = tile_rows_for(rb, in_pitch, smem, lreg, 2 * rpp);
    }
    if (t == 0) return -1;
    return lreg + t * staged_pitch_for(rb, in_pitch, smem, lreg) + (t + 1) * stride;
}

int filter_tile_rows(int rb, int in_pitch, int smem, int lut_region)
{
    const int rpp = kFiltWarps / warps_per_row(rb);
    return tile_rows_for(rb, in_pitch, smem, lut_region, 2 * rpp);
}

int filter_ctas_per_sm(int smem)
{
    int n = 0;
    cudaFuncSetAttribute(k_window_filter, cudaFuncAttributeMaxDynamicSharedMemorySize, kFilterSmemCap);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_window_filter, kFiltThreads, smem) != cudaSuccess)
        return 1;
    return n > 0 ? n : 1;
}

cudaError_t launch_prepare_window(DevImage* imgs, int n, cudaStream_t s)
{
    k_prepare_window<<<n, 1024, 0, s>>>(imgs, n);      // 4096-entry tables: four entries per thread
    note_launch();
    return cudaGetLastError();
}

// The time-bounded barrier wait of the TMA-staged kernels, on a barrier whose
// phase completes only if `arrive` (one thread arrives) -- otherwise nothing
// ever completes it and the wait must give up after limit_ns and report.
__global__ void k_wait_probe(int arrive, uint64_t limit_ns, int* status)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (arrive && threadIdx.x == 0) mbar_arrive(&bar);
    const bool ok = mbar_wait_bounded(&bar, 0, limit_ns);
    if (threadIdx.x == 0) *status = ok ? R2P_OK : R2P_ETIMEOUT;
}

cudaError_t launch_wait_probe(int arrive, uint64_t limit_ns, int* d_status, cudaStream_t s)
{
    k_wait_probe<<<1, 32, 0, s>>>(arrive, limit_ns, d_status);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_bmp(DevImage* imgs, int n, uint32_t max_words, int nsm, cudaStream_t s)
{
    const uint32_t want = (max_words + 255u) / 256u;
    const dim3 grid((unsigned)std::max<uint32_t>(1u, std::min<uint32_t>(want, (uint32_t)nsm * 8u)), (unsigned)n);
    k_bmp_file<<<grid, 256, 0, s>>>(imgs);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_window_filter(DevImage* imgs, const BandItem* items, int nitems, int grid, int smem,
                                 cudaStream_t s)
{
    cudaError_t e = cudaFuncSetAttribute(k_window_filter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kFilterSmemCap);
    if (e != cudaSuccess) return e;
    k_window_filter<<<grid, kFiltThreads, smem, s>>>(imgs, items, nitems, smem);
    note_launch();
    return cudaGetLastError();
}

}  // namespace r2p
