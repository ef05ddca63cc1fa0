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
// shared memory).  Every one of the CTA's 1024 threads parses its own
// 68-byte sub-range of the block sequentially (32 warps per SM: the parse is
// latency-bound, so the warps hide each other's dependency chains) -- a
// greedy LZ77 with three candidates per position: distance 1 (a run), the
// same column one scanline up, and the head of a 4-byte hash table shared by
// the 32 lanes of a warp (seeded from the ~2 KB before the warp's range).
// Matches may reach any earlier byte of the block within 32 KB but end inside
// the thread's sub-range, and are extended by word compares.  Each thread
// packs its fixed-Huffman codes LSB-first into a 64-bit register (codes from
// per-CTA tables) and spills whole words to a private shared-memory buffer
// (an odd word stride keeps the 32 lanes on distinct banks), so no atomics
// are needed while parsing.  A CTA-wide scan of the per-thread bit counts
// places the bitstreams behind the 3-bit block header; an end-of-block code
// and an empty stored block byte-align the output, so blocks are independent
// and join by plain concatenation.  A block whose Huffman form would not be
// smaller is emitted as a stored block.  The CTA also leaves the block's
// Adler-32 sums (input) and CRC-32 (output).
#include <cuda_runtime.h>

#include "k_deflate.cuh"
#include "r2p_huff.h"
#include "r2p_kernels.h"

namespace r2p {

constexpr int kLzWarps = 32;
constexpr int kLzThreads = kLzWarps * 32;
constexpr int kPrefill = 4096;        // history bytes hashed before a warp's range
constexpr int kMaxDist = 32768;
constexpr int kMaxMatch = 258;
constexpr uint32_t FULL = 0xFFFFFFFFu;

// Bytes each thread parses: a multiple of 4 whose word count is odd, so the 32
// lanes of a warp, reading at the same offset of their sub-ranges, hit 32
// distinct shared-memory banks.  Output words per thread use an odd stride too.
__host__ __device__ inline int lz_sub_bytes(int block_size)
{
    const int w = ((block_size + kLzThreads - 1) / kLzThreads + 3) >> 2;
    return 4 * (w | 1);
}
__host__ __device__ inline int lz_lane_words(int block_size) { return ((lz_sub_bytes(block_size) * 9 + 31) / 32) | 1; }
__host__ __device__ inline int lz_in_bytes(int block_size) { return ((block_size + 15) & ~15) + 64; }

static int lz_smem_bytes(int block_size, int hash_bits)
{
    return 4096 + lz_in_bytes(block_size) + kLzThreads * lz_lane_words(block_size) * 4 +
           kLzWarps * (1 << hash_bits) * 2 + 256;
}

uint64_t lz77_slot_bytes(int block_size) { return (uint64_t)((block_size + kStoredHdr + 64 + 255) & ~255); }

// Unaligned 4-byte little-endian load from shared memory.
__device__ __forceinline__ uint32_t ld32u(const uint8_t* base, int p)
{
    const uint32_t* w = reinterpret_cast<const uint32_t*>(base);
    const int q = p >> 2;
    return fshr(w[q], w[q + 1], (uint32_t)(p & 3) << 3);
}

// Multiplicative hash of 4 bytes to hb bits.
__device__ __forceinline__ uint32_t hash4(uint32_t v, int hb) { return (v * 2654435761u) >> (32 - hb); }

// An image's hash table bits: 9 or 10 (32 warps of 2^10 u16 entries fit beside
// a 64 KB block; 11 bits would not).
__device__ __forceinline__ int lz_hash_bits(const DevImage& d) { return d.hash_bits == 9 ? 9 : 10; }

// Fixed-Huffman code of a literal byte: reversed code and its length.
__device__ __forceinline__ void lit_code(uint32_t b, uint32_t& v, int& n)
{
    if (b < 144) { v = __brev(0x30u + b) >> 24; n = 8; }
    else         { v = __brev(0x190u + b - 144u) >> 23; n = 9; }
}

// Code tables for matches (RFC 1951 3.2.5-3.2.6), built per CTA in shared
// memory from the definitions below:
//   length entry  [len - 3]           reversed code | bits << 8 | extra bits << 12 | base (len - 3) << 16
//   distance entry [d < 256 ? d : 256 + (d >> 7)], d = distance - 1
//                                     reversed 5-bit code | extra bits << 8 | base d << 12
// (for d >= 256 a code has >= 7 extra bits, so d >> 7 fixes the code).
constexpr int kLenTab = 256, kDistTab = 512;

__device__ uint32_t len_entry(int len)
{
    int idx, lne, base;
    const int l = len - 3;
    if (len == 258) { idx = 28; lne = 0; base = l; }
    else if (l < 8) { idx = l; lne = 0; base = l; }
    else {
        const int lg = 31 - __clz(l);
        lne = lg - 2;
        idx = 4 * lne + 4 + ((l >> lne) & 3);
        base = l & ~((1 << lne) - 1);
    }
    const int sym = 257 + idx;
    uint32_t code;
    int cl;
    if (sym <= 279) { code = __brev((uint32_t)(sym - 256)) >> 25; cl = 7; }
    else            { code = __brev((uint32_t)(0xC0 + sym - 280)) >> 24; cl = 8; }
    return code | ((uint32_t)cl << 8) | ((uint32_t)lne << 12) | ((uint32_t)base << 16);
}

__device__ uint32_t dist_entry(int i)
{
    const int d = i < 256 ? i : (i - 256) << 7;
    int dc, dne, base;
    if (d < 4) { dc = d; dne = 0; base = d; }
    else {
        const int lg = 31 - __clz(d);
        dne = lg - 1;
        dc = 2 * dne + 2 + ((d >> dne) & 1);
        base = d & ~((1 << dne) - 1);
    }
    return (__brev((uint32_t)dc) >> 27) | ((uint32_t)dne << 8) | ((uint32_t)base << 12);
}

// Length/distance pair -> packed bits (length code, extra, 5-bit distance code, extra).
__device__ __forceinline__ void match_code(int len, int dist, const uint32_t* lt, const uint32_t* dt, uint32_t& v,
                                           int& n)
{
    const uint32_t le = lt[len - 3];
    const uint32_t cl = (le >> 8) & 15u, lne = (le >> 12) & 15u;
    const uint32_t lex = (uint32_t)(len - 3) - (le >> 16);
    const int d = dist - 1;
    const uint32_t de = dt[d < 256 ? d : 256 + (d >> 7)];
    const uint32_t dne = (de >> 8) & 15u;
    const uint32_t dex = (uint32_t)d - (de >> 12);
    v = (le & 0xFFu) | (lex << cl) | ((de & 31u) << (cl + lne)) | (dex << (cl + lne + 5));
    n = (int)(cl + lne + 5 + dne);
}

// 4 bytes at i >= -3 with bytes at negative indices read as zero.
__device__ __forceinline__ uint32_t ld32z(const uint8_t* base, int i)
{
    if (i >= 0) return ld32u(base, i);
    return i > -4 ? ld32u(base, 0) << (8 * -i) : 0u;
}

// Greedy parse of in[s, e) by one thread into the word buffer `ob`.
// `tab` is the warp's shared hash table (latest position + 1 per hash).
// Returns the number of bits written; the last partial word is stored too.
//
// The thread keeps three sliding registers -- w (bytes p..p+3), the byte
// before p, and wv (bytes p-rb1..p-rb1+3, the scanline above) -- so a literal
// step reads one new byte per stream instead of two words per candidate.
__device__ uint32_t parse_lane(const uint8_t* in, int s, int e, int rb1, int hb, uint16_t* tab, uint32_t* ob,
                               const uint32_t* lt, const uint32_t* dt)
{
    const bool vert = rb1 > 1 && rb1 <= kMaxDist;
    uint64_t acc = 0;
    int nacc = 0, nw = 0;
    uint32_t bits = 0;
    int p = s;
    // sliding state for position p (bytes past the block end read the zero padding)
    uint32_t w = ld32u(in, p);
    // at the block start no run can match: a "previous byte" unequal to w's first byte
    uint32_t prev = p > 0 ? (uint32_t)in[p - 1] : ((w & 0xFFu) ^ 1u);
    // exact once p >= rb1 (the only positions it is compared at)
    uint32_t wv = vert ? ld32z(in, max(p - rb1, -4)) : 0u;
    while (p < e) {
        int L = 0, D = 0;
        if (p + 4 <= e) {
            const uint32_t h = hash4(w, hb);
            const int t = tab[h];
            tab[h] = (uint16_t)(p + 1);
            if (w == prev * 0x01010101u) {
                D = 1;
            } else if (vert && p >= rb1 && wv == w) {
                D = rb1;
            } else if (t) {
                const int dist = p - (t - 1);
                if (dist > 0 && dist <= kMaxDist && ld32u(in, t - 1) == w) D = dist;
            }
            if (D) {
                // extend by words, then bytes, up to the sub-range end
                const int maxl = min(kMaxMatch, e - p);
                const int c = p - D;
                L = 4;
                bool more = true;
                while (more && L + 4 <= maxl) {
                    const uint32_t x = ld32u(in, c + L) ^ ld32u(in, p + L);
                    if (x) { L += (__ffs(x) - 1) >> 3; more = false; }
                    else L += 4;
                }
                while (more && L < maxl && in[c + L] == in[p + L]) L++;
            }
        }
        uint32_t v;
        int nb;
        if (L >= 4) {
            match_code(L, D, lt, dt, v, nb);
            p += L;
            w = ld32u(in, p);
            prev = in[p - 1];
            wv = vert ? ld32z(in, max(p - rb1, -4)) : 0u;
        } else {
            lit_code(w & 0xFFu, v, nb);
            prev = w & 0xFFu;
            w = (w >> 8) | ((uint32_t)in[p + 4] << 24);
            if (vert) {
                const int q = p + 4 - rb1;
                wv = (wv >> 8) | ((uint32_t)(q >= 0 ? in[q] : 0) << 24);
            }
            p += 1;
        }
        acc |= (uint64_t)v << nacc;
        nacc += nb;
        bits += (uint32_t)nb;
        if (nacc >= 32) {
            ob[nw++] = (uint32_t)acc;
            acc >>= 32;
            nacc -= 32;
        }
    }
    if (nacc > 0) ob[nw] = (uint32_t)acc;
    return bits;
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
    const int lw = lz_lane_words(max_block);
    uint32_t* outs = reinterpret_cast<uint32_t*>(in + in_bytes);
    uint16_t* tabs = reinterpret_cast<uint16_t*>(outs + kLzThreads * lw);
    __shared__ uint64_t red64[kLzWarps];
    __shared__ uint32_t red32[kLzWarps];
    __shared__ uint32_t wsum[kLzWarps];
    __shared__ uint32_t s_info[4];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __shared__ uint32_t s_len[kLenTab], s_dist[kDistTab];
    build_crc_tables(ctab);
    for (int i = threadIdx.x; i < kLenTab; i += kLzThreads) s_len[i] = len_entry(i + 3);
    for (int i = threadIdx.x; i < kDistTab; i += kLzThreads) s_dist[i] = dist_entry(i);
    uint32_t* myout = outs + tid * lw;

    for (int b = blockIdx.x; b < nblocks; b += gridDim.x) {
        BlockOut& bo = blocks[b];
        const DevImage& d = imgs[bo.img];
        if (d.level != 1) continue;                 // level 0: stored; >= 2: dynamic blocks
        const int n = (int)bo.in_len;
        const uint8_t* src = d.filt + bo.in_off;
        const bool last = ((int)(b - d.blk0) == d.nblocks - 1) && !d.open_end;
        const int hb = lz_hash_bits(d);
        uint16_t* mytab = tabs + (warp << hb);      // the launch sized the tables for the largest hb
        __syncthreads();
        // stage the block (+ zero padding), clear the hash tables
        if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
            for (int i = tid; i < (n >> 4); i += kLzThreads)
                reinterpret_cast<uint4*>(in)[i] = __ldg(reinterpret_cast<const uint4*>(src) + i);
            for (int i = (n & ~15) + tid; i < n; i += kLzThreads) in[i] = src[i];
        } else {
            for (int i = tid; i < n; i += kLzThreads) in[i] = src[i];
        }
        for (int i = n + tid; i < in_bytes; i += kLzThreads) in[i] = 0;
        for (int i = tid; i < (kLzWarps << hb) / 2; i += kLzThreads) reinterpret_cast<uint32_t*>(tabs)[i] = 0u;
        __syncthreads();
        uint32_t s1;
        uint64_t s2;
        cta_adler_sums<kLzThreads>(in, n, s1, s2, red64);
        // seed the warp's table from the bytes before its range, oldest first
        const int sub = lz_sub_bytes(n);
        const int ws0 = min(n, warp * 32 * sub);
        const int prefill = min(kPrefill, d.block_size / kLzWarps);    // ~one warp range of history
        for (int q0 = max(0, ws0 - prefill); q0 < ws0; q0 += 32) {
            const int q = q0 + lane;
            if (q < ws0 && q + 4 <= n) mytab[hash4(ld32u(in, q), hb)] = (uint16_t)(q + 1);
            __syncwarp();
        }
        // parse this thread's sub-range
        const int s = min(n, tid * sub), e = min(n, s + sub);
        const uint32_t nbits = (s < e) ? parse_lane(in, s, e, d.rb + 1, hb, mytab, myout, s_len, s_dist) : 0u;
        // CTA-wide exclusive scan of the bit counts
        uint32_t incl = nbits;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        uint32_t wbase = 0, tot = 3;
        for (int k = 0; k < kLzWarps; k++) {
            if (k < warp) wbase += wsum[k];
            tot += wsum[k];
        }
        tot += 7;                                                  // end-of-block code
        const uint32_t off = 3 + wbase + incl - nbits;             // bit offset of this thread's stream
        if (tid == 0) {
            const uint32_t huff = last ? (tot + 7) / 8 : (tot + 3 + 7) / 8 + 4;
            const uint32_t stored = (uint32_t)n + kStoredHdr;
            s_info[1] = (huff < stored) ? huff : 0u;               // 0 = stored block
        }
        __syncthreads();
        const uint32_t huff = s_info[1];
        uint8_t* slot = scratch + (size_t)b * slot_bytes;
        uint32_t crc;
        if (huff) {
            // place the 512 bitstreams behind the 3-bit header, into `in`
            uint32_t* region = reinterpret_cast<uint32_t*>(in);
            const int rwords = (int)((huff + 3) / 4) + 2;
            for (int i = tid; i < rwords; i += kLzThreads) region[i] = 0;
            __syncthreads();
            const int nw = (int)((nbits + 31) / 32);
            const uint32_t sh = off & 31, q0 = off >> 5;
            for (int j = 0; j < nw; j++) {
                const uint32_t v = myout[j];
                if (!v) continue;
                // first and last words are shared with the neighbouring streams
                atomicOr(&region[q0 + j], v << sh);
                if (sh) atomicOr(&region[q0 + j + 1], v >> (32 - sh));
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

// ---------------------------------------------------------------------------
// Levels 2-9: dynamic-Huffman blocks (BTYPE = 10) over a run-length parse.
//
// Filtered scanlines are mostly small residuals and runs; coding them with a
// per-block Huffman code (RFC 1951 3.2.7) matters far more than a match
// search (zlib's run-length strategy, distance-1 matches only, is what PNG
// encoders use for this data).  One 256-thread CTA per block, two per SM:
//   1. stage the block; each thread parses its sub-range (tokens: a literal,
//      or a run of 3..258 copies of the previous byte = length, distance 1)
//      into per-warp symbol histograms;
//   2. one thread builds the literal/length code (lengths <= 15, r2p_huff.h),
//      the canonical codes and the block header, and sizes the block; the
//      block is stored instead when that is smaller;
//   3. every thread re-parses to count its bits, a CTA scan gives each its
//      bit offset, and a third parse writes its codes straight into the
//      block's slot (shared atomics only for the words at stream ends);
//   4. end-of-block code, the empty stored block of non-final blocks, CRC.
// ---------------------------------------------------------------------------
constexpr int kDynThreads = 256;
constexpr int kDynWarps = kDynThreads / 32;

// Bytes per thread: a multiple of 4 with an odd word count (distinct banks).
__host__ __device__ inline int dyn_sub_bytes(int block_size)
{
    const int w = ((block_size + kDynThreads - 1) / kDynThreads + 3) >> 2;
    return 4 * (w | 1);
}

struct DynLayout {
    int in, hist, freq, wt, lt, sorted, lltab, lens, codes, hw, lsym, total;
};

__host__ __device__ inline DynLayout dyn_layout(int max_block)
{
    DynLayout L;
    int o = 4096;                                   // CRC tables
    L.in = o;     o += lz_in_bytes(max_block);
    L.hist = o;   o += kDynWarps * kLLSyms * 4;
    L.freq = o;   o += kLLSyms * 4;
    L.wt = o;     o += kLLSyms * 4;
    L.lt = o;     o += kLLSyms * 4;
    L.sorted = o; o += ((kLLSyms * 2 + 15) & ~15);
    L.lltab = o;  o += kLLSyms * 4;
    L.lens = o;   o += ((kLLSyms + kDSyms + 15) & ~15);
    L.codes = o;  o += (((kLLSyms + kDSyms) * 2 + 15) & ~15);
    L.hw = o;     o += kHdrWords * 4;
    L.lsym = o;   o += 256 * 4;
    L.total = o;
    return L;
}

// Run-length parse of in[s, e): calls f.lit(byte) or f.match(len 3..258).
template <class F>
__device__ __forceinline__ void rle_parse(const uint8_t* in, int s, int e, F& f)
{
    uint32_t prev = s > 0 ? (uint32_t)in[s - 1] : 0x100u;   // no run at the block start
    int p = s;
    while (p < e) {
        const uint32_t b = in[p];
        if (b == prev) {
            const int maxl = min(kMaxMatch, e - p);
            const uint32_t pat = prev * 0x01010101u;
            int L = 1;
            bool more = true;
            while (more && L + 4 <= maxl) {
                const uint32_t x = ld32u(in, p + L) ^ pat;
                if (x) {
                    L += (__ffs(x) - 1) >> 3;
                    more = false;
                } else {
                    L += 4;
                }
            }
            while (more && L < maxl && in[p + L] == prev) L++;
            if (L >= 3) {
                f.match(L);
                p += L;
                continue;
            }
        }
        f.lit(b);
        prev = b;
        p++;
    }
}

// lsym[len - 3] = length symbol | extra bit count << 9 | extra value << 12
struct RleHist {
    uint32_t* h;
    const uint32_t* lsym;
    uint32_t matches, extra;
    __device__ void lit(uint32_t b) { atomicAdd(&h[b], 1u); }
    __device__ void match(int L)
    {
        const uint32_t e = lsym[L - 3];
        atomicAdd(&h[e & 511u], 1u);
        matches++;
        extra += (e >> 9) & 7u;
    }
};

// tab[sym] = reversed code | length << 16
struct RleCount {
    const uint32_t* tab;
    const uint32_t* lsym;
    uint32_t dlen, bits;
    __device__ void lit(uint32_t b) { bits += tab[b] >> 16; }
    __device__ void match(int L)
    {
        const uint32_t e = lsym[L - 3];
        bits += (tab[e & 511u] >> 16) + ((e >> 9) & 7u) + dlen;
    }
};

// Writes a thread's codes from bit `off` of the zeroed output words: whole
// words by plain stores, the first (when it starts mid-word) and the last
// partial word by atomicOr, as the neighbouring streams share them.
struct RleEmit {
    const uint32_t* tab;
    const uint32_t* lsym;
    uint32_t dcode, dlen;
    uint32_t* out;
    uint64_t acc;
    uint32_t nacc, q, q_first;
    bool first_shared;
    __device__ void init(uint32_t* o, uint32_t off)
    {
        out = o;
        acc = 0;
        nacc = off & 31u;
        q = q_first = off >> 5;
        first_shared = nacc != 0;
    }
    __device__ void put(uint32_t v, uint32_t n)
    {
        acc |= (uint64_t)v << nacc;
        nacc += n;
        if (nacc >= 32u) {
            const uint32_t w = (uint32_t)acc;
            if (q == q_first && first_shared) atomicOr(out + q, w);
            else out[q] = w;
            q++;
            acc >>= 32;
            nacc -= 32u;
        }
    }
    __device__ void lit(uint32_t b)
    {
        const uint32_t t = tab[b];
        put(t & 0xFFFFu, t >> 16);
    }
    __device__ void match(int L)
    {
        const uint32_t e = lsym[L - 3];
        const uint32_t t = tab[e & 511u];
        put(t & 0xFFFFu, t >> 16);
        const uint32_t ne = (e >> 9) & 7u;
        if (ne) put(e >> 12, ne);
        put(dcode, dlen);
    }
    __device__ void finish()
    {
        if (nacc > 0) atomicOr(out + q, (uint32_t)acc);    // the next stream may start in this word
    }
};

// OR n <= 25 bits into global words at bit pos (words shared with other writers).
__device__ __forceinline__ void or_bits_global(uint32_t* w, uint32_t pos, uint32_t v, uint32_t n)
{
    const uint32_t q = pos >> 5, sh = pos & 31u;
    atomicOr(w + q, v << sh);
    if (sh + n > 32u) atomicOr(w + q + 1, v >> (32u - sh));
}

__global__ void __launch_bounds__(kDynThreads)
k_rle_dyn_blocks(const DevImage* __restrict__ imgs, BlockOut* __restrict__ blocks, int nblocks, int max_block,
                 uint8_t* __restrict__ scratch, uint64_t slot_bytes, const uint32_t* __restrict__ xpow)
{
    extern __shared__ __align__(16) uint8_t sm[];
    const DynLayout Ly = dyn_layout(max_block);
    uint32_t (*ctab)[256] = reinterpret_cast<uint32_t (*)[256]>(sm);
    uint8_t* in = sm + Ly.in;
    const int in_bytes = lz_in_bytes(max_block);
    uint32_t* hist = reinterpret_cast<uint32_t*>(sm + Ly.hist);
    uint32_t* freq = reinterpret_cast<uint32_t*>(sm + Ly.freq);
    uint32_t* wt = reinterpret_cast<uint32_t*>(sm + Ly.wt);
    uint32_t* lt = reinterpret_cast<uint32_t*>(sm + Ly.lt);
    uint16_t* sorted = reinterpret_cast<uint16_t*>(sm + Ly.sorted);
    uint32_t* lltab = reinterpret_cast<uint32_t*>(sm + Ly.lltab);
    uint8_t* ll_len = sm + Ly.lens;
    uint8_t* d_len = ll_len + kLLSyms;
    uint16_t* ll_code = reinterpret_cast<uint16_t*>(sm + Ly.codes);
    uint16_t* d_code = ll_code + kLLSyms;
    uint32_t* hw = reinterpret_cast<uint32_t*>(sm + Ly.hw);
    uint32_t* lsym = reinterpret_cast<uint32_t*>(sm + Ly.lsym);
    __shared__ uint64_t red64[kDynWarps];
    __shared__ uint32_t red32[kDynWarps];
    __shared__ uint32_t wsum[kDynWarps];
    __shared__ uint32_t s_info[4];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    build_crc_tables(ctab);
    for (int i = tid; i < 256; i += kDynThreads) {
        int sym, ne, ex;
        length_symbol(i + 3, sym, ne, ex);
        lsym[i] = (uint32_t)sym | ((uint32_t)ne << 9) | ((uint32_t)ex << 12);
    }

    for (int b = blockIdx.x; b < nblocks; b += gridDim.x) {
        BlockOut& bo = blocks[b];
        const DevImage& d = imgs[bo.img];
        if (d.level < 2) continue;
        const int n = (int)bo.in_len;
        const uint8_t* src = d.filt + bo.in_off;
        const bool last = ((int)(b - d.blk0) == d.nblocks - 1) && !d.open_end;
        __syncthreads();
        if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
            for (int i = tid; i < (n >> 4); i += kDynThreads)
                reinterpret_cast<uint4*>(in)[i] = __ldg(reinterpret_cast<const uint4*>(src) + i);
            for (int i = (n & ~15) + tid; i < n; i += kDynThreads) in[i] = src[i];
        } else {
            for (int i = tid; i < n; i += kDynThreads) in[i] = src[i];
        }
        for (int i = n + tid; i < in_bytes; i += kDynThreads) in[i] = 0;
        for (int i = tid; i < kDynWarps * kLLSyms; i += kDynThreads) hist[i] = 0u;
        for (int i = tid; i < kLLSyms + kDSyms; i += kDynThreads) ll_len[i] = 0;
        __syncthreads();
        uint32_t s1;
        uint64_t s2;
        cta_adler_sums<kDynThreads>(in, n, s1, s2, red64);
        const int sub = dyn_sub_bytes(n);
        const int s = min(n, tid * sub), e = min(n, s + sub);
        // 1. histogram
        RleHist H{hist + warp * kLLSyms, lsym, 0u, 0u};
        rle_parse(in, s, e, H);
        const uint32_t matches = (uint32_t)cta_sum64<kDynThreads>(H.matches, red64);
        const uint64_t extra = cta_sum64<kDynThreads>(H.extra, red64);
        for (int i = tid; i < kLLSyms; i += kDynThreads) {
            uint32_t f = (i == 256) ? 1u : 0u;        // one end-of-block code
            for (int w = 0; w < kDynWarps; w++) f += hist[w * kLLSyms + i];
            freq[i] = f;
        }
        __syncthreads();
        // 2. used symbols sorted by (frequency, symbol): each thread ranks its own
        for (int i = tid; i < kLLSyms; i += kDynThreads) {
            const uint32_t f = freq[i];
            if (!f) continue;
            int r = 0;
            for (int j = 0; j < kLLSyms; j++) {
                const uint32_t g = freq[j];
                r += (g && (g < f || (g == f && j < i))) ? 1 : 0;
            }
            sorted[r] = (uint16_t)i;
        }
        __syncthreads();
        if (tid == 0) {
            int nu = 0;
            for (int i = 0; i < kLLSyms; i++) nu += freq[i] ? 1 : 0;
            for (int i = 0; i < nu; i++) wt[i] = freq[sorted[i]];
            if (nu >= 2) limited_lengths(wt, nu, kMaxCodeLen, lt);
            else lt[0] = 1;                            // (a block always has a literal and the end code)
            s_info[3] = (uint32_t)nu;
        }
        __syncthreads();
        const int nu = (int)s_info[3];
        for (int i = tid; i < nu; i += kDynThreads) ll_len[sorted[i]] = (uint8_t)lt[i];
        __syncthreads();
        if (tid == 0) {
            d_len[0] = matches ? 1 : 0;
            canonical_codes(ll_len, kLLSyms, ll_code);
            canonical_codes(d_len, kDSyms, d_code);
            for (int k = 0; k < kHdrWords; k++) hw[k] = 0u;
            uint32_t pos = 0;
            put_bits(hw, pos, last ? 5u : 4u, 3);      // BFINAL, BTYPE = 10
            const uint32_t hend = build_dyn_header(ll_len, d_len, hw, pos);
            uint64_t body = 0;
            for (int i = 0; i < kLLSyms; i++) body += (uint64_t)freq[i] * ll_len[i];
            const uint64_t total = hend + body + extra + (uint64_t)matches * d_len[0];
            const uint64_t dyn = last ? (total + 7) / 8 : (total + 3 + 7) / 8 + 4;
            s_info[0] = (dyn < (uint64_t)(n + kStoredHdr)) ? (uint32_t)dyn : 0u;   // 0 = stored block
            s_info[1] = hend;
            s_info[2] = (uint32_t)total;
        }
        __syncthreads();
        for (int i = tid; i < kLLSyms; i += kDynThreads) lltab[i] = (uint32_t)ll_code[i] | ((uint32_t)ll_len[i] << 16);
        const uint32_t dyn = s_info[0];
        uint8_t* slot = scratch + (size_t)b * slot_bytes;
        uint32_t crc;
        if (dyn) {
            const uint32_t hend = s_info[1], total = s_info[2];
            uint32_t* out = reinterpret_cast<uint32_t*>(slot);
            const int owords = (int)((dyn + 3) / 4) + 1;
            for (int i = tid; i < owords; i += kDynThreads) out[i] = 0u;
            __syncthreads();
            // 3. bit counts, offsets, codes
            RleCount C{lltab, lsym, (uint32_t)d_len[0], 0u};
            rle_parse(in, s, e, C);
            uint32_t incl = C.bits;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += y;
            }
            if (lane == 31) wsum[warp] = incl;
            if (tid == 0)
                for (int k = 0; k < (int)((hend + 31) / 32); k++) out[k] = hw[k];
            __syncthreads();
            uint32_t wbase = 0;
            for (int k = 0; k < warp; k++) wbase += wsum[k];
            RleEmit E;
            E.tab = lltab;
            E.lsym = lsym;
            E.dcode = d_code[0];
            E.dlen = d_len[0];
            E.init(out, hend + wbase + incl - C.bits);
            rle_parse(in, s, e, E);
            E.finish();
            __syncthreads();
            if (tid == 0) {
                const uint32_t eob = lltab[256];
                or_bits_global(out, total - (eob >> 16), eob & 0xFFFFu, eob >> 16);
                if (!last) {                               // empty stored block: 3 zero bits, pad, 0000 FFFF
                    const uint32_t k = (total + 3 + 7) / 8;
                    slot[k + 2] = 0xFF;
                    slot[k + 3] = 0xFF;
                }
            }
            __syncthreads();
            uint32_t s1d;
            uint64_t s2d;
            cta_crc_adler<kDynThreads>(slot, (int)dyn, false, ctab, xpow, crc, s1d, s2d, red64, red32);
        } else {
            uint8_t hdr[kStoredHdr] = {(uint8_t)(last ? 1 : 0), (uint8_t)(n & 0xFF), (uint8_t)(n >> 8),
                                       (uint8_t)(~n & 0xFF), (uint8_t)((~n >> 8) & 0xFF)};
            if (tid < kStoredHdr) slot[tid] = hdr[tid];
            cta_copy_to_global<kDynThreads>(slot + kStoredHdr, in, n);
            uint32_t cd, s1d;
            uint64_t s2d;
            cta_crc_adler<kDynThreads>(in, n, false, ctab, xpow, cd, s1d, s2d, red64, red32);
            crc = gf2_mulmod(crc_small(hdr, kStoredHdr, ctab), xpow8n((uint64_t)n, xpow)) ^ cd;
        }
        if (tid == 0) {
            bo.out_len = dyn ? dyn : (uint32_t)(n + kStoredHdr);
            bo.crc = crc;
            bo.s1 = s1;
            bo.s2 = s2;
        }
    }
}

int dyn_ctas_per_sm(int max_block)
{
    int n = 0;
    const int smem = dyn_layout(max_block).total;
    cudaFuncSetAttribute(k_rle_dyn_blocks, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_rle_dyn_blocks, kDynThreads, smem) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

cudaError_t launch_dyn(const DevImage* imgs, BlockOut* blocks, int nblocks, int max_block, uint8_t* scratch,
                       uint64_t slot_bytes, const uint32_t* xpow, int grid, cudaStream_t s)
{
    const int smem = dyn_layout(max_block).total;
    cudaError_t e = cudaFuncSetAttribute(k_rle_dyn_blocks, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    k_rle_dyn_blocks<<<grid, kDynThreads, smem, s>>>(imgs, blocks, nblocks, max_block, scratch, slot_bytes, xpow);
    note_launch();
    return cudaGetLastError();
}

// hash_bits: the largest table size among the launch's images (9 or 10).
cudaError_t launch_lz77(const DevImage* imgs, BlockOut* blocks, int nblocks, int max_block, uint8_t* scratch,
                        uint64_t slot_bytes, const uint32_t* xpow, int grid, int hash_bits, cudaStream_t s)
{
    const int smem = lz_smem_bytes(max_block, hash_bits == 9 ? 9 : 10);
    cudaError_t e = cudaFuncSetAttribute(k_lz77_blocks, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    k_lz77_blocks<<<grid, kLzThreads, smem, s>>>(imgs, blocks, nblocks, max_block, scratch, slot_bytes, xpow);
    note_launch();
    return cudaGetLastError();
}

}  // namespace r2p
