// k_deflate.cuh -- device routines shared by the DEFLATE-side kernels
// (stored blocks, LZ77 blocks, the finish pass, copies, checksums).
#pragma once
#include <cuda_runtime.h>

#include "r2p_common.h"
#include "r2p_device.h"

namespace r2p {

// x^(8n) mod P from a 4-level table in global memory (built on the host by
// crc_build_xpow): tab[l*1024 + j] = x^(8 * j * 2^(10 l)), so any byte count
// below 2^40 costs at most three GF(2) products.
__device__ __forceinline__ uint32_t xpow8n(uint64_t n, const uint32_t* __restrict__ tab)
{
    uint32_t r = __ldg(tab + (n & 1023));
#pragma unroll
    for (int l = 1; l < kXpowLevels; l++) {
        const uint32_t j = (uint32_t)(n >> (10 * l)) & 1023u;
        if (j) r = gf2_mulmod(r, __ldg(tab + l * 1024 + j));
    }
    return r;
}

constexpr int kCrcChunk = 252;      // bytes per thread chunk: 63 words, an odd
                                    // word stride so smem reads hit distinct banks

// Slicing-by-4 tables in shared memory (4 KB), built by the CTA.
__device__ __forceinline__ void build_crc_tables(uint32_t (*t)[256])
{
    for (int n = threadIdx.x; n < 256; n += blockDim.x) {
        uint32_t c = (uint32_t)n;
        for (int k = 0; k < 8; k++) c = (c & 1u) ? kCrcPoly ^ (c >> 1) : c >> 1;
        t[0][n] = c;
    }
    __syncthreads();
    for (int n = threadIdx.x; n < 256; n += blockDim.x) {
        uint32_t c = t[0][n];
        for (int k = 1; k < 4; k++) {
            c = (c >> 8) ^ t[0][c & 0xFF];
            t[k][n] = c;
        }
    }
    __syncthreads();
}

__device__ __forceinline__ uint32_t crc_word(uint32_t crc, uint32_t w, const uint32_t (*t)[256])
{
    crc ^= w;
    return t[3][crc & 0xFF] ^ t[2][(crc >> 8) & 0xFF] ^ t[1][(crc >> 16) & 0xFF] ^ t[0][crc >> 24];
}

__device__ __forceinline__ uint32_t crc_byte(uint32_t crc, uint32_t b, const uint32_t (*t)[256])
{
    return t[0][(crc ^ b) & 0xFF] ^ (crc >> 8);
}

// a * b mod P with the slicing tables at hand: the 63-bit carry-less
// product (clmul32), moved up one bit, holds x^0..x^31 in its high word and
// x^32..x^63 in its low word; the low word times x^32 is four zero bytes
// through the CRC register (one crc_word step).  About 50 independent
// instructions and four table reads, where gf2_mulmod is 32 dependent steps.
__device__ __forceinline__ uint32_t gf2_mulmod_t(uint32_t a, uint32_t b, const uint32_t (*t)[256])
{
    const uint64_t r = clmul32(a, b) << 1;
    return (uint32_t)(r >> 32) ^ crc_word((uint32_t)r, 0u, t);
}

// xpow8n with the table-assisted product.
__device__ __forceinline__ uint32_t xpow8n_t(uint64_t n, const uint32_t* __restrict__ tab, const uint32_t (*t)[256])
{
    uint32_t r = __ldg(tab + (n & 1023));
#pragma unroll
    for (int l = 1; l < kXpowLevels; l++) {
        const uint32_t j = (uint32_t)(n >> (10 * l)) & 1023u;
        if (j) r = gf2_mulmod_t(r, __ldg(tab + l * 1024 + j), t);
    }
    return r;
}

// finalised crc32 of a few bytes (thread-local)
__device__ __forceinline__ uint32_t crc_small(const uint8_t* p, int n, const uint32_t (*t)[256])
{
    uint32_t c = 0xFFFFFFFFu;
    for (int i = 0; i < n; i++) c = crc_byte(c, p[i], t);
    return c ^ 0xFFFFFFFFu;
}

template <int NT>
__device__ __forceinline__ uint32_t cta_xor(uint32_t v, uint32_t* red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v ^= __shfl_xor_sync(0xFFFFFFFFu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    uint32_t r = 0;
    for (int i = 0; i < NT / 32; i++) r ^= red[i];
    __syncthreads();
    return r;
}

template <int NT>
__device__ __forceinline__ uint64_t cta_sum64(uint64_t v, uint64_t* red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    uint64_t r = 0;
    for (int i = 0; i < NT / 32; i++) r += red[i];
    __syncthreads();
    return r;
}

// CRC-32 (finalised) of n bytes in shared memory `buf` (4-byte aligned), and
// optionally the Adler sums S1 = sum d_i and S2 = sum (n - i) d_i.  Whole CTA.
// Each thread takes contiguous CH-byte chunks (CH / 4 odd, so the lanes read
// distinct banks); chunk CRCs are shifted to their place with a table lookup
// and at most three table-assisted GF(2) products and XOR-reduced.
template <int NT, int CH = kCrcChunk>
__device__ void cta_crc_adler(const uint8_t* buf, int n, bool want_adler, const uint32_t (*t)[256],
                              const uint32_t* __restrict__ xpow, uint32_t& crc_out, uint32_t& s1_out,
                              uint64_t& s2_out, uint64_t* red64, uint32_t* red32)
{
    const int nch = (n + CH - 1) / CH;
    const int last = nch - 1;
    const int len_last = n - last * CH;
    uint32_t crc_acc = 0;
    uint64_t s1 = 0, s2 = 0;
    for (int ch = threadIdx.x; ch < nch; ch += NT) {
        const int o = ch * CH;
        const int L = (ch == last) ? len_last : CH;
        const uint32_t* w = reinterpret_cast<const uint32_t*>(buf + o);
        uint32_t c = 0xFFFFFFFFu;
        uint32_t cs1 = 0;
        uint64_t cw = 0;
        const int nw = L >> 2;
        for (int k = 0; k < nw; k++) {
            const uint32_t v = w[k];
            c = crc_word(c, v, t);
            if (want_adler) {
                const uint32_t bs = bytesum4(v);
                cs1 += bs;
                cw += (uint64_t)(L - 4 * k) * bs - bytewsum4(v);
            }
        }
        for (int i = nw * 4; i < L; i++) {
            const uint32_t b = buf[o + i];
            c = crc_byte(c, b, t);
            if (want_adler) { cs1 += b; cw += (uint64_t)(L - i) * b; }
        }
        c ^= 0xFFFFFFFFu;
        // shift past the bytes that follow this chunk
        if (ch != last) c = gf2_mulmod_t(c, xpow8n_t((uint64_t)(n - o - L), xpow, t), t);
        crc_acc ^= c;
        if (want_adler) {
            const uint64_t after = (uint64_t)(n - o - L);
            s1 += cs1;
            s2 += cw + after * cs1;
        }
    }
    crc_out = cta_xor<NT>(crc_acc, red32);
    if (want_adler) {
        s1_out = (uint32_t)cta_sum64<NT>(s1, red64);
        s2_out = cta_sum64<NT>(s2, red64);
    }
}

// Copy n bytes from a 4-byte-aligned source (shared or global) to an
// arbitrary global destination that does not overlap it, 16-byte stores for
// the aligned interior.  Each thread loads two chunks before it stores them,
// so two load round trips are in flight per thread.
template <int NT>
__device__ void cta_copy_to_global(uint8_t* __restrict__ dst, const uint8_t* __restrict__ src, int n)
{
    if (n <= 0) return;
    const uintptr_t d0 = reinterpret_cast<uintptr_t>(dst);
    const uintptr_t a0 = (d0 + 15) & ~(uintptr_t)15;              // first aligned dst
    const uintptr_t a1 = (d0 + (uintptr_t)n) & ~(uintptr_t)15;    // end of aligned part
    const int head = (int)min((uintptr_t)n, a0 - d0);
    const uint32_t* __restrict__ sw = reinterpret_cast<const uint32_t*>(src);
    if (a1 > a0) {
        const int o0 = (int)(a0 - d0);                           // data index of first aligned byte
        const uint32_t sh = (uint32_t)(o0 & 3) << 3;
        const int nchunks = (int)((a1 - a0) >> 4);
        // chunk c: source words q..q+4 (word q+4 holds bytes needed when the
        // shift is non-zero; it is loaded whenever it contains a valid byte,
        // so the copy never reads past that word)
        auto load = [&](int c, uint32_t* v) {
            const int q = (o0 + 16 * c) >> 2;
            v[0] = sw[q]; v[1] = sw[q + 1]; v[2] = sw[q + 2]; v[3] = sw[q + 3];
            v[4] = (4 * (q + 4) < n) ? sw[q + 4] : 0u;
        };
        auto store = [&](int c, const uint32_t* v) {
            uint4 o4;
            o4.x = fshr(v[0], v[1], sh);
            o4.y = fshr(v[1], v[2], sh);
            o4.z = fshr(v[2], v[3], sh);
            o4.w = fshr(v[3], v[4], sh);
            *reinterpret_cast<uint4*>(a0 + 16 * (uintptr_t)c) = o4;
        };
        int c = threadIdx.x;
        for (; c + NT < nchunks; c += 2 * NT) {
            uint32_t v[5], u[5];
            load(c, v);
            load(c + NT, u);
            store(c, v);
            store(c + NT, u);
        }
        if (c < nchunks) {
            uint32_t v[5];
            load(c, v);
            store(c, v);
        }
        const int tail0 = (int)(a1 - d0);
        for (int i = threadIdx.x; i < head; i += NT) dst[i] = src[i];
        for (int i = tail0 + threadIdx.x; i < n; i += NT) dst[i] = src[i];
    } else {
        for (int i = threadIdx.x; i < n; i += NT) dst[i] = src[i];
    }
}

}  // namespace r2p
