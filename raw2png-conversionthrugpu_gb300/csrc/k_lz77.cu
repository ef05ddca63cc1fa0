// k_lz77.cu -- LZ77 + fixed-Huffman DEFLATE on independent blocks.
//
// Reference semantics (what a block must decode to, not how it is found):
//   fixed Huffman code + length/distance tables   src/gpu_deflate_backend.cu:76-175
//   one BTYPE=01 block per unit, LSB-first packing src/gpu_deflate_backend.cu:557-697
//   greedy LZ77, min match 3..max 258, dist 32768 src/gpu_deflate_backend.cu:208-210,727-841
//   Z_FULL_FLUSH between units (empty stored block) src/parallel_deflate.cpp:155-157
// Only inflate-equality is required of the compressed bytes.
//
// Design.  One CTA per DEFLATE block (<= 65520 filtered bytes, staged in
// shared memory).  Its 16 warps each parse a 1/16 segment greedily with a
// private shared-memory hash table (most recent position per 4-byte hash,
// seeded from the 4 KB before the segment) and may reference any earlier byte
// of the block within 32 KB.  A warp examines 32 positions per step: every
// lane tests three candidates (distance 1, the same column one scanline up,
// the hash head) with word compares, a ballot chains the earliest matches
// through the window, and a match that reaches the per-lane limit is extended
// cooperatively (32 bytes per ballot).  Code lengths are prefix-summed across
// the warp and each lane ORs its code into the warp's bitstream.  The 16
// bitstreams are stitched at their bit offsets behind the 3-bit block header;
// an end-of-block code and an empty stored block byte-align the output, so
// blocks are independent and join by plain concatenation.  A block whose
// Huffman form would not be smaller is emitted as a stored block.  The CTA
// also leaves the block's Adler-32 sums (input) and CRC-32 (output).
#include <cuda_runtime.h>

#include "k_deflate.cuh"
#include "r2p_kernels.h"

namespace r2p {

constexpr int kLzWarps = 16;
constexpr int kLzThreads = kLzWarps * 32;
constexpr int kHashBits = 10;
constexpr int kHashSize = 1 << kHashBits;
constexpr int kPrefill = 4096;        // history bytes hashed before a segment
constexpr int kLaneCap = 16;          // per-lane match length before cooperative extension
constexpr int kMaxDist = 32768;
constexpr int kMaxMatch = 258;
constexpr uint32_t FULL = 0xFFFFFFFFu;

__host__ __device__ inline int lz_seg_bytes(int block_size) { return (block_size + kLzWarps - 1) / kLzWarps; }
__host__ __device__ inline int lz_out_words(int block_size) { return (lz_seg_bytes(block_size) * 9 + 31) / 32 + 8; }
__host__ __device__ inline int lz_in_bytes(int block_size) { return ((block_size + 15) & ~15) + 64; }

static int lz_smem_bytes(int block_size)
{
    return 4096 + lz_in_bytes(block_size) + kLzWarps * (lz_out_words(block_size) + kHashSize) * 4 + 256;
}

uint64_t lz77_slot_bytes(int block_size) { return (uint64_t)((block_size + kStoredHdr + 64 + 255) & ~255); }

// Unaligned 4-byte little-endian load from shared memory.
__device__ __forceinline__ uint32_t ld32u(const uint8_t* base, int p)
{
    const uint32_t* w = reinterpret_cast<const uint32_t*>(base);
    const int q = p >> 2;
    return fshr(w[q], w[q + 1], (uint32_t)(p & 3) << 3);
}

__device__ __forceinline__ uint32_t hash4(uint32_t v) { return (v * 2654435761u) >> (32 - kHashBits); }

// Length of the match between positions c < p, up to maxl (<= kLaneCap
// checked here with word compares); 0 if the first four bytes differ.
__device__ __forceinline__ int match_len(const uint8_t* in, int c, int p, uint32_t wp, int maxl)
{
    uint32_t x = ld32u(in, c) ^ wp;
    if (x) return 0;
    int L = 4;
#pragma unroll
    for (int k = 4; k < kLaneCap; k += 4) {
        x = ld32u(in, c + k) ^ ld32u(in, p + k);
        if (x) { L = k + ((__ffs(x) - 1) >> 3); break; }
        L = k + 4;
    }
    return L < maxl ? L : maxl;
}

// Cooperative extension of a match beyond L (warp-uniform arguments).
__device__ __forceinline__ int extend_match(const uint8_t* in, int p, int c, int L, int maxl, int lane)
{
    while (L < maxl) {
        const int k = L + lane;
        const bool eq = (k < maxl) && in[c + k] == in[p + k];
        const uint32_t ne = __ballot_sync(FULL, !eq);
        if (ne) return L + __ffs(ne) - 1;
        L += 32;
    }
    return maxl;
}

__device__ __forceinline__ uint32_t lane_range(int a, int b)   // bits [a, b), 0 <= a <= b <= 32
{
    const uint32_t hi = (b >= 32) ? FULL : ((1u << b) - 1u);
    const uint32_t lo = (a >= 32) ? FULL : ((1u << a) - 1u);
    return hi & ~lo;
}

// Fixed-Huffman code of a literal byte: reversed code and its length.
__device__ __forceinline__ void lit_code(uint32_t b, uint32_t& v, int& n)
{
    if (b < 144) { v = __brev(0x30u + b) >> 24; n = 8; }
    else         { v = __brev(0x190u + b - 144u) >> 23; n = 9; }
}

// Length/distance pair -> packed bits (length code, extra, 5-bit distance code, extra).
__device__ __forceinline__ void match_code(int len, int dist, uint32_t& v, int& n)
{
    int idx, lne, lex;
    if (len == 258) { idx = 28; lne = 0; lex = 0; }
    else {
        const int l = len - 3;
        if (l < 8) { idx = l; lne = 0; lex = 0; }
        else {
            const int lg = 31 - __clz(l);
            lne = lg - 2;
            idx = 4 * lne + 4 + ((l >> lne) & 3);
            lex = l & ((1 << lne) - 1);
        }
    }
    const int sym = 257 + idx;
    uint32_t code;
    int cl;
    if (sym <= 279) { code = __brev((uint32_t)(sym - 256)) >> 25; cl = 7; }
    else            { code = __brev((uint32_t)(0xC0 + sym - 280)) >> 24; cl = 8; }
    const int d = dist - 1;
    int dc, dne, dex;
    if (d < 4) { dc = d; dne = 0; dex = 0; }
    else {
        const int lg = 31 - __clz(d);
        dne = lg - 1;
        dc = 2 * dne + 2 + ((d >> dne) & 1);
        dex = d & ((1 << dne) - 1);
    }
    v = code | ((uint32_t)lex << cl) | ((__brev((uint32_t)dc) >> 27) << (cl + lne)) |
        ((uint32_t)dex << (cl + lne + 5));
    n = cl + lne + 5 + dne;
}

// Greedy parse of in[s0, s1) by one warp into bitstream `out` (zeroed words).
// Returns the number of bits written.
__device__ uint32_t parse_segment(const uint8_t* in, int n, int s0, int s1, int rb1, uint32_t* tab, uint32_t* out,
                                  int lane)
{
    const int pf0 = s0 > kPrefill ? s0 - kPrefill : 0;
    for (int q0 = pf0; q0 < s0; q0 += 32) {
        const int q = q0 + lane;
        if (q < s0 && q + 4 <= n) atomicMax(&tab[hash4(ld32u(in, q))], (uint32_t)(q + 1));
    }
    __syncwarp();
    uint32_t bp = 0;
    int pos = s0;
    while (pos < s1) {
        const int p = pos + lane;
        const int wlen = min(32, s1 - pos);
        const bool can = (lane < wlen) && (p + 4 <= s1);
        int bestL = 0, bestD = 0;
        uint32_t h = 0;
        if (can) {
            const uint32_t w = ld32u(in, p);
            h = hash4(w);
            const int maxl = min(kMaxMatch, s1 - p);
            if (p >= 1) {
                const int L = match_len(in, p - 1, p, w, maxl);
                if (L > bestL) { bestL = L; bestD = 1; }
            }
            if (rb1 > 1 && rb1 <= kMaxDist && p >= rb1) {
                const int L = match_len(in, p - rb1, p, w, maxl);
                if (L > bestL) { bestL = L; bestD = rb1; }
            }
            const uint32_t t = tab[h];
            if (t) {
                const int c = (int)t - 1;
                const int dist = p - c;
                if (dist > 1 && dist <= kMaxDist && dist != rb1) {
                    const int L = match_len(in, c, p, w, maxl);
                    if (L > bestL) { bestL = L; bestD = dist; }
                }
            }
        }
        const uint32_t mm = __ballot_sync(FULL, bestL >= 4);
        // resolve the greedy chain of tokens through this window
        uint32_t lits = 0, starts = 0;
        int myL = bestL;
        int t = 0;
        while (t < wlen) {
            const uint32_t cand = mm & ~lane_range(0, t);
            if (!cand) { lits |= lane_range(t, wlen); t = wlen; break; }
            const int j = __ffs(cand) - 1;
            lits |= lane_range(t, j);
            int L = __shfl_sync(FULL, bestL, j);
            const int D = __shfl_sync(FULL, bestD, j);
            const int pj = pos + j;
            if (L >= kLaneCap) L = extend_match(in, pj, pj - D, L, min(kMaxMatch, s1 - pj), lane);
            if (lane == j) myL = L;
            starts |= 1u << j;
            t = j + L;
        }
        // insert this window's examined positions that precede the next token
        if (can && lane < t) atomicMax(&tab[h], (uint32_t)(p + 1));
        // emit
        uint32_t v = 0;
        int nb = 0;
        if (lits & (1u << lane)) lit_code(in[p], v, nb);
        else if (starts & (1u << lane)) match_code(myL, bestD, v, nb);
        int incl = nb;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        const int total = __shfl_sync(FULL, incl, 31);
        if (nb) {
            const uint32_t b = bp + (uint32_t)(incl - nb);
            const uint32_t q = b >> 5, sh = b & 31;
            atomicOr(&out[q], v << sh);
            if (sh + (uint32_t)nb > 32) atomicOr(&out[q + 1], v >> (32 - sh));
        }
        bp += (uint32_t)total;
        pos += t;
        __syncwarp();
    }
    return bp;
}

// Adler sums of n bytes in shared memory (whole CTA).
template <int NT>
__device__ void cta_adler_sums(const uint8_t* buf, int n, uint32_t& s1_out, uint64_t& s2_out, uint64_t* red64)
{
    // word k covers bytes 4k..4k+3 with weights n - 4k - j
    const uint32_t* w = reinterpret_cast<const uint32_t*>(buf);
    const int nw = n >> 2;
    uint64_t s1 = 0, s2 = 0;
    for (int k = threadIdx.x; k < nw; k += NT) {
        const uint32_t v = w[k];
        const uint32_t bs = bytesum4(v);
        s1 += bs;
        s2 += (uint64_t)(n - 4 * k) * bs - bytewsum4(v);
    }
    for (int i = nw * 4 + threadIdx.x; i < n; i += NT) {
        s1 += buf[i];
        s2 += (uint64_t)(n - i) * buf[i];
    }
    s1_out = (uint32_t)cta_sum64<NT>(s1, red64);
    s2_out = cta_sum64<NT>(s2, red64);
}

__global__ void __launch_bounds__(kLzThreads, 1)
k_lz77_blocks(const DevImage* __restrict__ imgs, BlockOut* __restrict__ blocks, int nblocks, int max_block,
              uint8_t* __restrict__ scratch, uint64_t slot_bytes, const uint32_t* __restrict__ xpow)
{
    extern __shared__ __align__(16) uint8_t sm[];
    uint32_t (*ctab)[256] = reinterpret_cast<uint32_t (*)[256]>(sm);
    uint8_t* in = sm + 4096;
    const int in_bytes = lz_in_bytes(max_block);
    const int ow = lz_out_words(max_block);
    uint32_t* outs = reinterpret_cast<uint32_t*>(in + in_bytes);
    uint32_t* tabs = outs + kLzWarps * ow;
    __shared__ uint64_t red64[kLzWarps];
    __shared__ uint32_t red32[kLzWarps];
    __shared__ uint32_t seg_bits[kLzWarps];
    __shared__ uint32_t s_info[4];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    build_crc_tables(ctab);
    uint32_t* myout = outs + warp * ow;
    uint32_t* mytab = tabs + warp * kHashSize;

    for (int b = blockIdx.x; b < nblocks; b += gridDim.x) {
        BlockOut& bo = blocks[b];
        const DevImage& d = imgs[bo.img];
        if (d.level == 0) continue;
        const int n = (int)bo.in_len;
        const uint8_t* src = d.filt + bo.in_off;
        const bool last = ((int)(b - d.blk0) == d.nblocks - 1);
        __syncthreads();
        // stage the block (+ zero padding) and clear the per-warp state
        if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
            for (int i = tid; i < (n >> 4); i += kLzThreads)
                reinterpret_cast<uint4*>(in)[i] = __ldg(reinterpret_cast<const uint4*>(src) + i);
            for (int i = (n & ~15) + tid; i < n; i += kLzThreads) in[i] = src[i];
        } else {
            for (int i = tid; i < n; i += kLzThreads) in[i] = src[i];
        }
        for (int i = n + tid; i < in_bytes; i += kLzThreads) in[i] = 0;
        for (int i = lane; i < ow; i += 32) myout[i] = 0;
        for (int i = lane; i < kHashSize; i += 32) mytab[i] = 0;
        __syncthreads();
        uint32_t s1;
        uint64_t s2;
        cta_adler_sums<kLzThreads>(in, n, s1, s2, red64);
        // parse
        const int seg = (n + kLzWarps - 1) / kLzWarps;
        const int s0 = min(n, warp * seg), se = min(n, s0 + seg);
        const int rb1 = d.rb + 1;
        const uint32_t nbits = (s0 < se) ? parse_segment(in, n, s0, se, rb1, mytab, myout, lane) : 0u;
        if (lane == 0) seg_bits[warp] = nbits;
        __syncthreads();
        if (tid == 0) {
            uint32_t tot = 3;
            for (int w = 0; w < kLzWarps; w++) tot += seg_bits[w];
            tot += 7;                                              // end-of-block code
            const uint32_t huff = last ? (tot + 7) / 8 : (tot + 3 + 7) / 8 + 4;
            const uint32_t stored = (uint32_t)n + kStoredHdr;
            s_info[0] = tot;
            s_info[1] = (huff < stored) ? huff : 0u;               // 0 = stored block
        }
        __syncthreads();
        const uint32_t tot = s_info[0], huff = s_info[1];
        uint8_t* slot = scratch + (size_t)b * slot_bytes;
        uint32_t crc;
        if (huff) {
            // stitch the warp bitstreams behind the 3-bit header into `in`
            uint32_t* region = reinterpret_cast<uint32_t*>(in);
            const int rwords = (int)((huff + 3) / 4) + 2;
            for (int i = tid; i < rwords; i += kLzThreads) region[i] = 0;
            __syncthreads();
            uint32_t off = 3;
            for (int w = 0; w < warp; w++) off += seg_bits[w];
            const int nw = (int)((nbits + 31) / 32);
            for (int j = lane; j < nw; j += 32) {
                const uint32_t v = myout[j];
                const uint32_t bpos = off + 32u * (uint32_t)j;
                const uint32_t q = bpos >> 5, sh = bpos & 31;
                if (v) {
                    atomicOr(&region[q], v << sh);
                    if (sh) atomicOr(&region[q + 1], v >> (32 - sh));
                }
            }
            if (tid == 0) atomicOr(&region[0], last ? 3u : 2u);     // BFINAL, BTYPE = 01
            __syncthreads();
            if (!last && tid == 0) {
                // empty stored block: 3 zero bits, pad to a byte, LEN 0000, NLEN FFFF
                const uint32_t k = (tot + 3 + 7) / 8;
                in[k + 2] = 0xFF;
                in[k + 3] = 0xFF;
            }
            __syncthreads();
            uint32_t s1d;
            uint64_t s2d;
            cta_crc_adler<kLzThreads>(in, (int)huff, false, ctab, xpow, crc, s1d, s2d, red64, red32);
            const uint4* s4 = reinterpret_cast<const uint4*>(in);
            for (int i = tid; i < (int)((huff + 15) / 16); i += kLzThreads) reinterpret_cast<uint4*>(slot)[i] = s4[i];
        } else {
            uint8_t hdr[kStoredHdr] = {(uint8_t)(last ? 1 : 0), (uint8_t)(n & 0xFF), (uint8_t)(n >> 8),
                                       (uint8_t)(~n & 0xFF), (uint8_t)((~n >> 8) & 0xFF)};
            if (tid < kStoredHdr) slot[tid] = hdr[tid];
            cta_copy_to_global<kLzThreads>(slot + kStoredHdr, in, n);
            uint32_t cd, s1d;
            uint64_t s2d;
            cta_crc_adler<kLzThreads>(in, n, false, ctab, xpow, cd, s1d, s2d, red64, red32);
            crc = gf2_mulmod(crc_small(hdr, kStoredHdr, ctab), xpow8n((uint64_t)n, xpow)) ^ cd;
        }
        if (tid == 0) {
            bo.out_len = huff ? huff : (uint32_t)(n + kStoredHdr);
            bo.crc = crc;
            bo.s1 = s1;
            bo.s2 = s2;
        }
    }
}

cudaError_t launch_lz77(const DevImage* imgs, BlockOut* blocks, int nblocks, int max_block, uint8_t* scratch,
                        uint64_t slot_bytes, const uint32_t* xpow, int grid, cudaStream_t s)
{
    const int smem = lz_smem_bytes(max_block);
    cudaError_t e = cudaFuncSetAttribute(k_lz77_blocks, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    k_lz77_blocks<<<grid, kLzThreads, smem, s>>>(imgs, blocks, nblocks, max_block, scratch, slot_bytes, xpow);
    note_launch();
    return cudaGetLastError();
}

}  // namespace r2p
