// k_lz77.cu -- DEFLATE on independent blocks: LZ77 + fixed Huffman (level 1,
// k_lz77_blocks) and dynamic Huffman over a run-length parse (levels 2-9,
// k_rle_dyn_blocks, further down).
//
// Reference semantics (what a block must decode to, not how it is found):
//   fixed Huffman code + length/distance tables   src/gpu_deflate_backend.cu:76-175
//   one BTYPE=01 block per unit, LSB-first packing src/gpu_deflate_backend.cu:557-697
//   greedy LZ77, min match 3..max 258, dist 32768 src/gpu_deflate_backend.cu:208-210,727-841
//   Z_FULL_FLUSH between units (empty stored block) src/parallel_deflate.cpp:155-157
// Only inflate-equality is required of the compressed bytes.
//
// Design.  One CTA per DEFLATE block (<= 65520 filtered bytes, staged in
// shared memory): 1024 threads for blocks above 32 KB (one CTA per SM), 512
// for blocks up to 32 KB (two CTAs per SM) and 320 for blocks up to 21760
// bytes (three CTAs per SM), so that one CTA's barrier phases run beside the
// others' parses.  Every thread parses its own 68-byte sub-range
// of the block sequentially (32 warps per SM: the parse is latency-bound, so
// the warps hide each other's dependency chains) -- a
// greedy LZ77 with two candidates per position: distance 1 (a run) and the
// head of a 3-byte hash table shared by the 32 lanes of a warp (seeded from
// the ~2 KB before the warp's range); a match is taken when it is at least 4
// bytes long, or 3 within 4096 bytes back (where its code, at most 22 bits,
// is shorter than three literals).  A thread steps two positions at a time
// (a match, a literal and a match, or two literals), which halves the steps
// of the literal-heavy lanes a warp waits for.  The PNG filter has already taken the
// scanline above out of the bytes, so a third candidate one scanline up found
// almost nothing the hash did not (990 of 12.55 M bytes on a 3072x3072 16-bit
// image) and cost a tenth of the launch; it is not searched.
// Matches reach back into the warp's range and the history hashed before it
// but end inside the thread's sub-range; runs are extended by aligned word
// compares against the repeated byte, other matches by unaligned word
// compares.  Each thread packs its fixed-Huffman codes LSB-first into a 64-bit
// register (codes from per-CTA tables) and spills whole words to a private
// shared-memory buffer (an odd word stride keeps the 32 lanes on distinct
// banks), so no atomics are needed while parsing; each thread then adds up
// the Adler-32 sums of its sub-range, so warps that finish early do that work.
// A CTA-wide scan of the per-thread bit counts
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
constexpr int kFar3 = 4096;           // farthest 3-byte match taken: nearer ones are shorter than 3 literals
constexpr uint32_t FULL = 0xFFFFFFFFu;

// Bytes each thread parses in a block of n bytes: a multiple of 4 whose word
// count is odd, so the 32 lanes of a warp, reading at the same offset of their
// sub-ranges, hit 32 distinct shared-memory banks; 68 for blocks above 21760
// bytes (at most 320, 482 or 964 threads busy in the three CTA sizes), n / 320
// rounded up that way below.  It depends on the block alone, not on the CTA
// size a launch picks, so a block encodes to the same bytes in any batch.
__host__ __device__ constexpr int lz_sub_bytes(int n)
{
    const int m = n < 21760 ? n : 21760;
    const int w = ((m + 319) / 320 + 3) >> 2;
    return 4 * (w | 1);
}
// Output words per thread: an odd stride (distinct banks for the 32 lanes)
// for the 1024-thread CTA; the smaller CTAs drop that word so that two or
// three CTAs fit one SM's shared memory (their lanes' spills meet in pairs).
__host__ __device__ inline int lz_lane_words(int block_size, int nt = kLzThreads)
{
    return ((lz_sub_bytes(block_size) * 9 + 31) / 32) | (nt == kLzThreads ? 1 : 0);
}
// A warp's hash table holds positions of its own range and of the history
// hashed before it, so every candidate lies within the 32 KB window.
static_assert(32 * lz_sub_bytes(kBlock64) + kPrefill <= kMaxDist, "hash candidates stay within the window");
__host__ __device__ inline int lz_in_bytes(int block_size) { return ((block_size + 15) & ~15) + 64; }

static int lz_smem_bytes(int block_size, int hash_bits, int nt = kLzThreads)
{
    return 4096 + lz_in_bytes(block_size) + nt * lz_lane_words(block_size, nt) * 4 +
           (nt / 32) * (1 << hash_bits) * 2 + 256;
}

uint64_t lz77_slot_bytes(int block_size) { return (uint64_t)((block_size + kStoredHdr + 64 + 255) & ~255); }

// Unaligned 4-byte little-endian load from shared memory.
__device__ __forceinline__ uint32_t ld32u(const uint8_t* base, int p)
{
    const uint32_t* w = reinterpret_cast<const uint32_t*>(base);
    const int q = p >> 2;
    return fshr(w[q], w[q + 1], (uint32_t)(p & 3) << 3);
}

// Multiplicative hash of the low 3 bytes (the shortest match) to hb bits.
__device__ __forceinline__ uint32_t hash3(uint32_t v, int hb) { return ((v & 0xFFFFFFu) * 2654435761u) >> (32 - hb); }

// An image's hash table bits: 9 or 10 (32 warps of 2^10 u16 entries fit beside
// a 64 KB block; 11 bits would not).
__device__ __forceinline__ int lz_hash_bits(const DevImage& d) { return d.hash_bits == 9 ? 9 : 10; }

// Fixed-Huffman code of a literal byte (RFC 1951 3.2.6): 0-143 are the 8-bit
// codes 0x30.., 144-255 the 9-bit codes 0x190..; reversed for LSB-first
// packing.  2b + 0x60 is 0x30 + b one bit up, so both reverse with >> 23.
__device__ __forceinline__ void lit_code(uint32_t b, uint32_t& v, int& n)
{
    const bool nine = b >= 144u;
    v = __brev(nine ? b + 0x100u : 2u * b + 0x60u) >> 23;
    n = 8 + (int)nine;
}

// Length codes for matches (RFC 1951 3.2.5-3.2.6), built per CTA in shared
// memory: entry [len - 3] = the reversed length code with its extra bits
// above it (low 16 bits) | the total bit count << 16.
constexpr int kLenTab = 256;

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
    return (code | ((uint32_t)(l - base) << cl)) | ((uint32_t)(cl + lne) << 16);
}

// Code of a match: length entry `le` (from the table), distance D >= 1 coded
// in place -- d = D - 1 below 4 is its own 5-bit code, otherwise the code is
// 2 * e + 2 + the bit below the top one, with e = floor(log2 d) - 1 extra
// bits (RFC 1951 3.2.5).  Returns the bits; *n gets their count (<= 31).
__device__ __forceinline__ uint32_t match_code(uint32_t le, uint32_t D, int& n)
{
    const uint32_t d = D - 1u;
    const int lg = 31 - __clz((int)(d | 1u));
    const int dne = d < 4u ? 0 : lg - 1;
    const uint32_t dc = d < 4u ? d : (uint32_t)(2 * dne + 2) + ((d >> dne) & 1u);
    const uint32_t dx = d & ((1u << dne) - 1u);
    const int ln = (int)(le >> 16);
    n = ln + 5 + dne;
    return (le & 0xFFFFu) | (((__brev(dc) >> 27) | (dx << 5)) << ln);
}

// Append n <= 32 bits to the thread's LSB-first bit accumulator; whole words
// go to its buffer `ob`.
__device__ __forceinline__ void put_bits(uint64_t& acc, int& nacc, int& nw, uint32_t* ob, uint32_t v, int n)
{
    acc |= (uint64_t)v << nacc;
    nacc += n;
    if (nacc >= 32) {
        ob[nw++] = (uint32_t)acc;
        acc >>= 32;
        nacc -= 32;
    }
}

// Match candidates at position p (bytes w = p..p+3, the byte before = prev,
// hash-head entry t): a run (distance 1) of 4 or more, the hash head with 4
// or more equal bytes, or the hash head with 3 equal bytes within kFar3.
// L = 4 means "at least 4: extend", 3 exactly 3, 0 none.
__device__ __forceinline__ void match_at(const uint8_t* in, int p, int e, uint32_t w, uint32_t prev, int t, int& L,
                                         int& D)
{
    const uint32_t rx = w ^ (prev * 0x01010101u);
    const int dist = p - (t - 1);              // <= 0: a later position of another lane, or empty
    const uint32_t hx = dist > 0 ? (ld32u(in, t - 1) ^ w) : 1u;
    L = 0;
    D = 0;
    if (rx == 0u) { D = 1; L = 4; }
    else if (hx == 0u) { D = dist; L = 4; }
    else if ((hx & 0xFFFFFFu) == 0u && dist <= kFar3) { D = dist; L = 3; }
    if (p + 4 > e) L = 0;                      // a match must leave its 4 bytes inside the sub-range
}

// Length of a match of at least 4 bytes at ps, distance D, up to the
// sub-range end e (and 258): runs by aligned words against the repeated byte
// `rb`, other matches by unaligned word compares, then bytes.
__device__ __forceinline__ int extend_match(const uint8_t* in, int ps, int e, int D, uint32_t rb)
{
    const uint32_t* W = reinterpret_cast<const uint32_t*>(in);
    const int maxl = min(kMaxMatch, e - ps);
    if (D == 1) {
        const uint32_t rep = rb * 0x01010101u;
        const int i = ps + 4, lim = ps + maxl;
        int q = i >> 2;
        uint32_t x = (W[q] ^ rep) & (0xFFFFFFFFu << (8 * (i & 3)));
        while (!x && 4 * q + 4 < lim) x = W[++q] ^ rep;
        const int end = x ? 4 * q + ((__ffs(x) - 1) >> 3) : 4 * q + 4;
        return min(end, lim) - ps;
    }
    const int c = ps - D;
    int L = 4;
    bool more = true;
    while (more && L + 4 <= maxl) {
        const uint32_t x = ld32u(in, c + L) ^ ld32u(in, ps + L);
        if (x) { L += (__ffs(x) - 1) >> 3; more = false; }
        else L += 4;
    }
    while (more && L < maxl && in[c + L] == in[ps + L]) L++;
    return L;
}

// Greedy parse of in[s, e) by one thread into the word buffer `ob`, two
// positions per step: each step looks up (and enters into the warp's hash
// table `tab`: latest position + 1 per hash, 0xFFFF when empty) position p,
// and p+1 when p is a literal, then emits a match at p, or a literal at p
// and a match at p+1, or two literals.  A literal-heavy lane -- the one a
// warp waits for -- so takes half as many steps, and literals and matches
// share one coding path (the selects below), so the lanes of a warp only
// diverge in match extension.
// Every lane of the warp calls it (lanes with nothing to parse too): after
// kProbeSteps steps the warp votes, and if its lanes' codes so far take 8 or
// more bits per input byte -- no better than stored bytes, as on noise --
// the warp codes the rest of its range as plain literals, skipping the
// match search.  The vote depends on the block's bytes alone.
// Returns the number of bits written; the last partial word is stored too.
constexpr int kProbeSteps = 8;

__device__ uint32_t parse_lane(const uint8_t* in, int s, int e, int hb, uint16_t* tab, uint32_t* ob,
                               const uint32_t* lt)
{
    const uint32_t* W = reinterpret_cast<const uint32_t*>(in);
    uint64_t acc = 0;
    int nacc = 0, nw = 0;
    int p = s;
    // at the block start no run can match: a "previous byte" unequal to byte 0
    const uint32_t prev0 = p > 0 ? (uint32_t)in[p - 1] : ((uint32_t)in[0] ^ 1u);
    auto step = [&]() {
        // bytes p-1 .. p+6 from three aligned words (bytes past the block end
        // read the zero padding)
        uint32_t wlo, whi;
        {
            const int pm = max(p - 1, 0);
            const int q = pm >> 2;
            const uint32_t sh = (uint32_t)(pm & 3) << 3;
            const uint32_t a = W[q], b = W[q + 1], c = W[q + 2];
            wlo = __funnelshift_r(a, b, sh);
            whi = __funnelshift_r(b, c, sh);
            if (p == 0) {
                whi = __funnelshift_l(wlo, whi, 8);
                wlo = (wlo << 8) | prev0;
            }
        }
        const uint32_t prev = wlo & 0xFFu;
        const uint32_t w0 = __funnelshift_r(wlo, whi, 8);     // bytes p .. p+3
        const uint32_t w1 = __funnelshift_r(wlo, whi, 16);    // bytes p+1 .. p+4
        const uint32_t h0 = hash3(w0, hb);
        const int t0 = tab[h0];
        tab[h0] = (uint16_t)(p + 1);
        int L0, D0, L1 = 0, D1 = 0;
        match_at(in, p, e, w0, prev, t0, L0, D0);
        const bool m0 = L0 != 0;
        if (!m0) {                                // p+1 is looked up (and entered) only if p is a literal
            const uint32_t h1 = hash3(w1, hb);
            const int t1 = tab[h1];
            if (p + 5 <= e) tab[h1] = (uint16_t)(p + 2);
            match_at(in, p + 1, e, w1, w0 & 0xFFu, t1, L1, D1);
        }
        const bool m1 = !m0 && L1 != 0;
        const int ps = m0 ? p : p + 1;
        const int D = m0 ? D0 : D1;
        int L = m0 ? L0 : L1;
        if (L == 4) L = extend_match(in, ps, e, D, m0 ? prev : (w0 & 0xFFu));
        int mn, ln0, ln1;
        const uint32_t mv = match_code(lt[(m0 || m1) ? L - 3 : 0], (m0 || m1) ? (uint32_t)D : 1u, mn);
        uint32_t lv0, lv1;
        lit_code(w0 & 0xFFu, lv0, ln0);
        lit_code(w1 & 0xFFu, lv1, ln1);
        put_bits(acc, nacc, nw, ob, m0 ? mv : lv0, m0 ? mn : ln0);
        if (!m0) put_bits(acc, nacc, nw, ob, m1 ? mv : lv1, m1 ? mn : ln1);
        p += m0 ? L : (m1 ? 1 + L : 2);
    };
    for (int k = 0; k < kProbeSteps && p + 4 <= e; k++) step();
    const uint32_t wbits = __reduce_add_sync(FULL, (uint32_t)(nw * 32 + nacc));
    const uint32_t wbytes = __reduce_add_sync(FULL, (uint32_t)(p - s));
    if (wbits < 8u * wbytes || wbytes == 0u)
        while (p + 4 <= e) step();
    for (; p < e; p++) {                        // the last bytes: literals
        uint32_t v;
        int nb;
        lit_code(in[p], v, nb);
        put_bits(acc, nacc, nw, ob, v, nb);
    }
    if (nacc > 0) ob[nw] = (uint32_t)acc;
    return (uint32_t)(nw * 32 + nacc);
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

template <int NT>
__global__ void __launch_bounds__(NT, 1024 / NT)
k_lz77_blocks(const DevImage* __restrict__ imgs, BlockOut* __restrict__ blocks, int nblocks, int max_block,
              uint8_t* __restrict__ scratch, uint64_t slot_bytes, const uint32_t* __restrict__ xpow)
{
    extern __shared__ __align__(16) uint8_t sm[];
    uint32_t (*ctab)[256] = reinterpret_cast<uint32_t (*)[256]>(sm);
    uint8_t* in = sm + 4096;
    const int in_bytes = lz_in_bytes(max_block);
    const int lw = lz_lane_words(max_block, NT);
    uint32_t* outs = reinterpret_cast<uint32_t*>(in + in_bytes);
    uint16_t* tabs = reinterpret_cast<uint16_t*>(outs + NT * lw);
    __shared__ uint64_t red64[(NT / 32)];
    __shared__ uint32_t red32[(NT / 32)];
    __shared__ uint32_t wsum[(NT / 32)], wa1[(NT / 32)], wa2[(NT / 32)];
    __shared__ uint32_t s_info[4];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __shared__ uint32_t s_len[kLenTab];
    build_crc_tables(ctab);
    for (int i = threadIdx.x; i < kLenTab; i += NT) s_len[i] = len_entry(i + 3);
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
            for (int i = tid; i < (n >> 4); i += NT)
                reinterpret_cast<uint4*>(in)[i] = __ldg(reinterpret_cast<const uint4*>(src) + i);
            for (int i = (n & ~15) + tid; i < n; i += NT) in[i] = src[i];
        } else {
            for (int i = tid; i < n; i += NT) in[i] = src[i];
        }
        for (int i = n + tid; i < in_bytes; i += NT) in[i] = 0;
        // empty entries hold 0xFFFF: position 65534, never before p (p < 65520)
        for (int i = tid; i < ((NT / 32) << hb) / 2; i += NT) reinterpret_cast<uint32_t*>(tabs)[i] = 0xFFFFFFFFu;
        __syncthreads();
        // seed the warp's table from the bytes before its range, oldest first
        const int sub = lz_sub_bytes(n);
        const int ws0 = min(n, warp * 32 * sub);
        const int prefill = min(kPrefill, 32 * sub);          // one warp range of history
        // four positions per lane per step, from two aligned words
        for (int q0 = max(0, ws0 - prefill) & ~3; q0 < ws0; q0 += 128) {
            const int q = q0 + 4 * lane;
            if (q < ws0) {
                const uint32_t* w32 = reinterpret_cast<const uint32_t*>(in);
                const uint32_t lo = w32[q >> 2], hi = w32[(q >> 2) + 1];
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (q + j + 4 <= n) mytab[hash3(fshr(lo, hi, 8u * j), hb)] = (uint16_t)(q + j + 1);
            }
            __syncwarp();
        }
        // parse this thread's sub-range
        const int s = min(n, tid * sub), e = min(n, s + sub);
        const uint32_t nbits = parse_lane(in, s, e, hb, mytab, myout, s_len);
        // Adler sums of the sub-range, taken while slower warps still parse:
        // S1 = sum d_i, S2 = sum (n - i) d_i mod 65521 (< 2^31 before the
        // reduction: at most 17 words of weight <= 65520)
        uint32_t a1 = 0, a2 = 0;
        {
            const int e4 = s + ((e - s) & ~3);
            for (int i = s; i < e4; i += 4) {
                const uint32_t v = reinterpret_cast<const uint32_t*>(in)[i >> 2];
                const uint32_t bs = bytesum4(v);
                a1 += bs;
                a2 += (uint32_t)(n - i) * bs - bytewsum4(v);
            }
            for (int i = e4; i < e; i++) {
                a1 += in[i];
                a2 += (uint32_t)(n - i) * in[i];
            }
            a2 %= kAdlerMod;
        }
        a1 = __reduce_add_sync(FULL, a1);
        a2 = __reduce_add_sync(FULL, a2);
        // CTA-wide exclusive scan of the bit counts
        uint32_t incl = nbits;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) { wsum[warp] = incl; wa1[warp] = a1; wa2[warp] = a2; }
        __syncthreads();
        // the warps' bases: lane k of every warp scans warp k's bit count
        const uint32_t ws = lane < NT / 32 ? wsum[lane] : 0u;
        uint32_t wx = ws;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, wx, o);
            if (lane >= o) wx += y;
        }
        const uint32_t wbase = __shfl_sync(FULL, wx - ws, warp);
        const uint32_t tot = 3 + __shfl_sync(FULL, wx, 31) + 7;   // header, streams, end-of-block code
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
            // place the 1024 bitstreams behind the 3-bit header, into `in`
            uint32_t* region = reinterpret_cast<uint32_t*>(in);
            const int rwords = (int)((huff + 3) / 4) + 2;
            for (int i = tid; i < rwords; i += NT) region[i] = 0;
            __syncthreads();
            const int nw = (int)((nbits + 31) / 32);
            const uint32_t sh = off & 31, q0 = off >> 5;
            if (nw > 0) {
                // the first and last words are shared with the neighbouring
                // streams; the words between hold this stream's bits alone
                uint32_t v = myout[0];
                atomicOr(&region[q0], v << sh);
                uint32_t carry = sh ? v >> (32 - sh) : 0u;
                for (int j = 1; j < nw; j++) {
                    v = myout[j];
                    const uint32_t u = (v << sh) | carry;
                    carry = sh ? v >> (32 - sh) : 0u;
                    if (32u * (j + 1) <= sh + nbits) region[q0 + j] = u;     // whole word of this stream
                    else atomicOr(&region[q0 + j], u);
                }
                if (sh) atomicOr(&region[q0 + nw], carry);
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
            // 124-byte chunks: ~120 chains of 31 words for a 21760-byte block
            cta_crc_adler<NT, 124>(in, (int)huff, false, ctab, xpow, crc, s1d, s2d, red64, red32);
            const uint4* s4 = reinterpret_cast<const uint4*>(in);
            for (int i = tid; i < (int)((huff + 15) / 16); i += NT) reinterpret_cast<uint4*>(slot)[i] = s4[i];
        } else {
            uint8_t hdr[kStoredHdr] = {(uint8_t)(last ? 1 : 0), (uint8_t)(n & 0xFF), (uint8_t)(n >> 8),
                                       (uint8_t)(~n & 0xFF), (uint8_t)((~n >> 8) & 0xFF)};
            if (tid < kStoredHdr) slot[tid] = hdr[tid];
            cta_copy_to_global<NT>(slot + kStoredHdr, in, n);
            uint32_t cd, s1d;
            uint64_t s2d;
            cta_crc_adler<NT>(in, n, false, ctab, xpow, cd, s1d, s2d, red64, red32);
            crc = gf2_mulmod_t(crc_small(hdr, kStoredHdr, ctab), xpow8n_t((uint64_t)n, xpow, ctab), ctab) ^ cd;
        }
        if (tid == 0) {
            uint32_t s1 = 0, s2 = 0;
            for (int k = 0; k < (NT / 32); k++) { s1 += wa1[k]; s2 += wa2[k]; }
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
// encoders use for this data).  One 1024-thread CTA per block:
//   1. stage the block; each thread parses its 68-byte chunks (tokens: a
//      literal, or a run of 3..258 copies of the previous byte = a length at
//      distance 1) into its warp's symbol histogram;
//   2. the literal/length code: used symbols ranked by (count, symbol) in
//      parallel; the pairing phase of the in-place minimum-redundancy
//      computation on one thread, internal-node depths by pointer jumping and
//      leaves per depth level in parallel (r2p_huff.h states both forms);
//      counts halved and the code rebuilt while it is deeper than 15;
//      canonical codes per symbol in parallel;
//   3. the CTA writes the block header (cta_dyn_header) and counts each
//      thread's code bits; a CTA scan gives each thread its bit offset, the block is
//      stored instead when that is smaller, and a last parse writes the codes
//      straight into the block's slot (atomics only for the words that
//      neighbouring streams share);
//   4. end-of-block code, the empty stored block of non-final blocks, CRC.
// ---------------------------------------------------------------------------
constexpr int kDynRounds = 9;                  // pointer-jumping rounds: depths < 512

// Bytes per chunk for NT chunks: a multiple of 4 with an odd word count (the
// lanes of a warp start on distinct banks).
template <int NT>
__host__ __device__ inline int dyn_sub_bytes(int block_size)
{
    const int w = ((block_size + NT - 1) / NT + 3) >> 2;
    return 4 * (w | 1);
}

// Shared memory of the dynamic kernel with NT threads: fixed-size tables
// first (compile-time offsets), the staged block last.
template <int NT>
struct DynSmem {
    static constexpr int Warps = NT / 32;
    static constexpr int Hist = 4096;                            // after the CRC tables
    static constexpr int Freq = Hist + Warps * kLLSyms * 4;
    static constexpr int Wt = Freq + kLLSyms * 4;
    static constexpr int Par = Wt + kLLSyms * 4;
    static constexpr int Dep = Par + kLLSyms * 4;
    static constexpr int Sorted = Dep + kLLSyms * 4;
    static constexpr int Lltab = Sorted + ((kLLSyms * 2 + 15) & ~15);
    static constexpr int Lens = Lltab + kLLSyms * 4;
    static constexpr int Hw = Lens + ((kLLSyms + kDSyms + 15) & ~15);
    static constexpr int Lsym = Hw + kHdrWords * 4;
    static constexpr int Lvl = Lsym + 256 * 4;                   // per depth: internal count, leaves so far; per length
    static constexpr int All = Lvl + 3 * 64 * 4;                 // header: code lengths in order
    static constexpr int Rs = All + 320;                         //   run-length symbols
    static constexpr int Rx = Rs + 320;                          //   their extra values
    static constexpr int Cl = Rx + 320;                          //   CL counts (19 u32), lengths, codes
    static constexpr int In = (Cl + 19 * 4 + 32 + 48 + 15) & ~15;  // 16-byte staging stores
    static_assert(In % 16 == 0 && Hw % 4 == 0 && Lsym % 4 == 0 && Lltab % 4 == 0 && NT >= 512, "layout");
    static int bytes(int max_block) { return In + lz_in_bytes(max_block); }
};

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

// The block's tokens do not depend on the CTA size: it is cut into 1024
// chunks of dyn_sub_bytes<1024> bytes (runs end at chunk ends) and thread t
// of NT parses chunks t * (1024 / NT) onward, so its bits stay contiguous.
template <int NT, class F>
__device__ __forceinline__ void rle_parse_chunks(const uint8_t* in, int n, F& f)
{
    constexpr int kChunks = 1024 / NT;
    const int sub = dyn_sub_bytes<1024>(n);
#pragma unroll
    for (int c = 0; c < kChunks; c++) {
        const int s = min(n, ((int)threadIdx.x * kChunks + c) * sub);
        rle_parse(in, s, min(n, s + sub), f);
    }
}

// lsym[len - 3] = length symbol | extra bit count << 9 | extra value << 12
struct RleHist {
    uint32_t* h;
    const uint32_t* lsym;
    uint32_t matches;
    __device__ void lit(uint32_t b) { atomicAdd(&h[b], 1u); }
    __device__ void match(int L)
    {
        atomicAdd(&h[lsym[L - 3] & 511u], 1u);
        matches++;
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

// Exclusive CTA-wide prefix sum of v (and the total); all threads call it.
template <int NT>
__device__ __forceinline__ uint32_t cta_excl_scan(uint32_t v, uint32_t* wsum, uint32_t& total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    uint32_t base = 0, tot = 0;
    for (int k = 0; k < NT / 32; k++) {
        const uint32_t w = wsum[k];
        base += k < warp ? w : 0u;
        tot += w;
    }
    __syncthreads();
    total = tot;
    return base + incl - v;
}

// The block's header (BFINAL, BTYPE = 10 and what build_dyn_header writes,
// bit for bit) built by the whole CTA: the thread at the first entry of each
// run of equal code lengths writes that run's symbols at its scanned
// position, one thread builds the 19-symbol code-length code, and every
// symbol then ORs its code and extra bits in at its scanned bit offset.
// hw (kHdrWords words) is zeroed here; returns the header's end bit.
template <int NT>
__device__ uint32_t cta_dyn_header(const uint8_t* ll_len, const uint8_t* d_len, uint32_t* hw, bool last, uint8_t* sm,
                                   uint32_t* wsum, uint32_t* s_hdr)
{
    using S = DynSmem<NT>;
    const int tid = threadIdx.x;
    uint8_t* all = sm + S::All;
    uint8_t* rs = sm + S::Rs;
    uint8_t* rx = sm + S::Rx;
    uint32_t* cf = reinterpret_cast<uint32_t*>(sm + S::Cl);
    uint8_t* cl_len = sm + S::Cl + 19 * 4;
    uint16_t* cl_code = reinterpret_cast<uint16_t*>(sm + S::Cl + 19 * 4 + 32);
    for (int k = tid; k < kHdrWords; k += NT) hw[k] = 0u;
    if (tid < kCLSyms) cf[tid] = 0u;
    if (tid < 2) s_hdr[tid] = 0u;
    __syncthreads();
    if (tid < kLLSyms && ll_len[tid]) atomicMax(&s_hdr[0], (uint32_t)tid + 1u);
    if (tid < kDSyms && d_len[tid]) atomicMax(&s_hdr[1], (uint32_t)tid + 1u);
    __syncthreads();
    const int nll = max(257, (int)s_hdr[0]), nd = max(1, (int)s_hdr[1]), n = nll + nd;
    if (tid < n) all[tid] = tid < nll ? ll_len[tid] : d_len[tid - nll];
    __syncthreads();
    int l = 0, run = 0;
    uint32_t k = 0;
    if (tid < n && (tid == 0 || all[tid] != all[tid - 1])) {
        l = all[tid];
        run = 1;
        while (tid + run < n && all[tid + run] == l) run++;
        k = (uint32_t)rle_run_count(l, run);
    }
    uint32_t nr;
    const uint32_t at = cta_excl_scan<NT>(k, wsum, nr);
    if (k) rle_run_write(l, run, rs + at, rx + at);
    __syncthreads();
    if (tid < (int)nr) atomicAdd(&cf[rs[tid]], 1u);
    __syncthreads();
    if (tid == 0) {
        const int ncl = cl_code_build(cf, cl_len, cl_code);
        uint32_t pos = 0;
        put_bits(hw, pos, last ? 5u : 4u, 3);
        put_header_counts(hw, pos, nll, nd, ncl, cl_len);
        s_hdr[2] = pos;
    }
    __syncthreads();
    uint32_t nb = 0, v = 0;
    if (tid < (int)nr) {
        const int sym = rs[tid];
        nb = (uint32_t)(cl_len[sym] + cl_extra_bits(sym));
        v = (uint32_t)cl_code[sym] | ((uint32_t)rx[tid] << cl_len[sym]);
    }
    uint32_t tot;
    const uint32_t off = s_hdr[2] + cta_excl_scan<NT>(nb, wsum, tot);
    if (nb) {
        const uint32_t q = off >> 5, sh = off & 31u;
        atomicOr(&hw[q], v << sh);
        if (sh + nb > 32u) atomicOr(&hw[q + 1], v >> (32u - sh));
    }
    __syncthreads();
    return s_hdr[2] + tot;
}

// NT threads: 1024 (one CTA per SM, the shortest per-block latency) for
// launches with at most one block per SM, 512 (two CTAs per SM, one's
// single-thread phases hidden behind the other's parses) for more; both
// write the same bytes (rle_parse_chunks).
template <int NT>
__global__ void __launch_bounds__(NT, 1024 / NT)
k_rle_dyn_blocks(const DevImage* __restrict__ imgs, BlockOut* __restrict__ blocks, int nblocks, int max_block,
                 uint8_t* __restrict__ scratch, uint64_t slot_bytes, const uint32_t* __restrict__ xpow)
{
    using S = DynSmem<NT>;
    constexpr int kDynThreads = NT, kDynWarps = NT / 32;
    extern __shared__ __align__(16) uint8_t sm[];
    uint32_t (*ctab)[256] = reinterpret_cast<uint32_t (*)[256]>(sm);
    uint8_t* in = sm + S::In;
    const int in_bytes = lz_in_bytes(max_block);
    uint32_t* hist = reinterpret_cast<uint32_t*>(sm + S::Hist);
    uint32_t* freq = reinterpret_cast<uint32_t*>(sm + S::Freq);
    uint32_t* P = reinterpret_cast<uint32_t*>(sm + S::Wt);       // weights, then parents (phase 1)
    uint32_t* par = reinterpret_cast<uint32_t*>(sm + S::Par);
    uint32_t* dep = reinterpret_cast<uint32_t*>(sm + S::Dep);
    uint16_t* sorted = reinterpret_cast<uint16_t*>(sm + S::Sorted);
    uint32_t* lltab = reinterpret_cast<uint32_t*>(sm + S::Lltab);
    uint8_t* ll_len = sm + S::Lens;
    uint8_t* d_len = ll_len + kLLSyms;
    uint32_t* hw = reinterpret_cast<uint32_t*>(sm + S::Hw);
    uint32_t* lsym = reinterpret_cast<uint32_t*>(sm + S::Lsym);
    uint32_t* cnt = reinterpret_cast<uint32_t*>(sm + S::Lvl);   // internal nodes per depth
    uint32_t* cum = cnt + 64;                                    // leaves at depth <= d
    uint32_t* blc = cnt + 128;                                   // codes per length, then next code
    __shared__ uint64_t red64[kDynWarps];
    __shared__ uint32_t red32[kDynWarps];
    __shared__ uint32_t wsum[kDynWarps];
    __shared__ uint32_t s_info[4];
    __shared__ uint32_t s_hdr[4];
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
        uint8_t* slot = scratch + (size_t)b * slot_bytes;
        uint32_t* out = reinterpret_cast<uint32_t*>(slot);
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
        for (int i = tid; i < (n + kStoredHdr + 3) / 4 + 2; i += kDynThreads) out[i] = 0u;   // any dynamic size
        __syncthreads();
        uint32_t s1;
        uint64_t s2;
        cta_adler_sums<kDynThreads>(in, n, s1, s2, red64);
        // 1. histogram
        RleHist H{hist + warp * kLLSyms, lsym, 0u};
        rle_parse_chunks<NT>(in, n, H);
        const uint32_t matches = (uint32_t)cta_sum64<kDynThreads>(H.matches, red64);
        uint32_t f = 0;
        if (tid < kLLSyms) {
            f = (tid == 256) ? 1u : 0u;                  // one end-of-block code
            for (int w = 0; w < kDynWarps; w++) f += hist[w * kLLSyms + tid];
            freq[tid] = f;
        }
        const int nu = __syncthreads_count(f != 0u);
        // 2. used symbols sorted by (count, symbol): bitonic sort of 512 keys
        //    count << 9 | symbol (unused symbols sort last) in the free histograms
        uint32_t* keys = hist;
        if (tid < 512) keys[tid] = (tid < kLLSyms && f) ? ((f << 9) | (uint32_t)tid) : 0xFFFFFFFFu;
        __syncthreads();
        for (int k = 2; k <= 512; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                if (tid < 256) {
                    const int i = 2 * tid - (tid & (j - 1)), ix = i + j;
                    const uint32_t a = keys[i], c = keys[ix];
                    if ((a > c) == ((i & k) == 0)) {
                        keys[i] = c;
                        keys[ix] = a;
                    }
                }
                __syncthreads();
            }
        }
        if (tid < nu) sorted[tid] = (uint16_t)(keys[tid] & 511u);
        __syncthreads();
        const int root = nu - 2;                        // nu >= 2: a literal and the end code
        for (uint32_t sh = 0;; sh++) {
            if (tid < nu) P[tid] = (uint32_t)(((uint64_t)freq[sorted[tid]] + (1u << sh) - 1u) >> sh);
            if (tid < 64) cnt[tid] = 0u;
            __syncthreads();
            if (tid == 0) mk_phase1(P, nu);
            __syncthreads();
            // depths of the internal nodes 0..nu-2 by pointer jumping
            if (tid <= root) {
                par[tid] = tid == root ? (uint32_t)root : P[tid];
                dep[tid] = tid == root ? 0u : 1u;
            }
            __syncthreads();
            for (int r = 0; r < kDynRounds; r++) {
                uint32_t nd = 0, np = 0;
                if (tid <= root) {
                    const uint32_t pk = par[tid];
                    nd = dep[tid] + dep[pk];
                    np = par[pk];
                }
                __syncthreads();
                if (tid <= root) {
                    dep[tid] = nd;
                    par[tid] = np;
                }
                __syncthreads();
            }
            if (tid <= root) atomicAdd(&cnt[min(dep[tid], 63u)], 1u);   // depths stay below 24 for 64 KB blocks
            __syncthreads();
            if (tid == 0) {                              // leaves per depth level, from the top
                uint32_t places = 1, leaves = 0;
                int dmax = 0;
                for (int dd = 0; dd < 64; dd++) {
                    const uint32_t lv = places - cnt[dd];
                    leaves += lv;
                    cum[dd] = leaves;
                    if (lv) dmax = dd;
                    places = 2 * cnt[dd];
                }
                s_info[3] = (uint32_t)dmax;
            }
            __syncthreads();
            if ((int)s_info[3] <= kMaxCodeLen) break;
            __syncthreads();
        }
        // leaf tid (ascending count) takes the depth whose range holds it
        if (tid < nu) {
            const uint32_t from_top = (uint32_t)(nu - tid);
            int dd = 1;
            while (cum[dd] < from_top) dd++;
            ll_len[sorted[tid]] = (uint8_t)dd;
        }
        if (tid < 16) blc[tid] = 0u;
        __syncthreads();
        // 3. canonical codes; the header (one thread) while the rest count bits
        const int myl = tid < kLLSyms ? ll_len[tid] : 0;
        if (myl) atomicAdd(&blc[myl], 1u);
        __syncthreads();
        if (tid == 0) {
            uint32_t c = 0;
            for (int l = 1; l <= kMaxCodeLen; l++) {
                c = (c + (l > 1 ? blc[l - 1] : 0u)) << 1;
                blc[16 + l] = c;                         // first code of length l
            }
            d_len[0] = matches ? 1 : 0;
        }
        __syncthreads();
        // a symbol's rank among the earlier symbols of its length: ballots per
        // length within the warp, per-warp counts for the warps before
        constexpr int kSymWarps = (kLLSyms + 31) / 32;
        uint32_t rank_in_warp = 0;
        if (warp < kSymWarps) {
            const uint32_t lt_mask = (1u << lane) - 1u;
            for (int l = 1; l <= kMaxCodeLen; l++) {
                const uint32_t bl = __ballot_sync(FULL, myl == l);
                if (myl == l) rank_in_warp = __popc(bl & lt_mask);
                if (lane == 0) dep[warp * 16 + l] = __popc(bl);     // (9 x 16 <= kLLSyms entries, free now)
            }
        }
        __syncthreads();
        if (tid < kLLSyms) {
            uint32_t code = 0;
            if (myl) {
                uint32_t r = rank_in_warp;
                for (int w = 0; w < warp; w++) r += dep[w * 16 + myl];
                code = bitrev(blc[16 + myl] + r, myl);
            }
            lltab[tid] = code | ((uint32_t)myl << 16);
        }
        __syncthreads();
        const uint32_t hend = cta_dyn_header<NT>(ll_len, d_len, hw, last, sm, wsum, s_hdr);
        RleCount C{lltab, lsym, (uint32_t)d_len[0], 0u};
        rle_parse_chunks<NT>(in, n, C);
        uint32_t incl = C.bits;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        if (tid == 0) {
            uint32_t body = 0;
            for (int k = 0; k < kDynWarps; k++) body += wsum[k];
            const uint32_t total = hend + body + (lltab[256] >> 16);
            const uint32_t dyn = last ? (total + 7) / 8 : (total + 3 + 7) / 8 + 4;
            s_info[0] = (dyn < (uint32_t)(n + kStoredHdr)) ? dyn : 0u;    // 0 = stored block
            s_info[2] = total;
            if (s_info[0])
                for (int k = 0; k < (int)((hend + 31) / 32); k++) out[k] = hw[k];
        }
        __syncthreads();
        const uint32_t dyn = s_info[0];
        uint32_t crc;
        if (dyn) {
            const uint32_t total = s_info[2];
            uint32_t wbase = 0;
            for (int k = 0; k < warp; k++) wbase += wsum[k];
            RleEmit E;
            E.tab = lltab;
            E.lsym = lsym;
            E.dcode = 0;                                 // the one distance code, length 1
            E.dlen = d_len[0];
            E.init(out, hend + wbase + incl - C.bits);
            rle_parse_chunks<NT>(in, n, E);
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
            // the staged block is no longer needed: CRC the slot from a shared copy
            for (int i = tid; i < (int)((dyn + 15) / 16); i += kDynThreads)
                reinterpret_cast<uint4*>(in)[i] = reinterpret_cast<const uint4*>(slot)[i];
            __syncthreads();
            uint32_t s1d;
            uint64_t s2d;
            cta_crc_adler<kDynThreads>(in, (int)dyn, false, ctab, xpow, crc, s1d, s2d, red64, red32);
        } else {
            uint8_t hdr[kStoredHdr] = {(uint8_t)(last ? 1 : 0), (uint8_t)(n & 0xFF), (uint8_t)(n >> 8),
                                       (uint8_t)(~n & 0xFF), (uint8_t)((~n >> 8) & 0xFF)};
            if (tid < kStoredHdr) slot[tid] = hdr[tid];
            cta_copy_to_global<kDynThreads>(slot + kStoredHdr, in, n);
            uint32_t cd, s1d;
            uint64_t s2d;
            cta_crc_adler<kDynThreads>(in, n, false, ctab, xpow, cd, s1d, s2d, red64, red32);
            crc = gf2_mulmod_t(crc_small(hdr, kStoredHdr, ctab), xpow8n_t((uint64_t)n, xpow, ctab), ctab) ^ cd;
        }
        if (tid == 0) {
            bo.out_len = dyn ? dyn : (uint32_t)(n + kStoredHdr);
            bo.crc = crc;
            bo.s1 = s1;
            bo.s2 = s2;
        }
    }
}

// Threads per CTA for a launch of nblocks blocks on nsm SMs (1024 while the
// blocks fit one CTA per SM, else 512 with two CTAs per SM) and its grid.
int dyn_grid(int nblocks, int nsm, int* threads)
{
    *threads = nblocks <= nsm ? 1024 : 512;
    return std::max(1, std::min(nblocks, *threads == 1024 ? nsm : 2 * nsm));
}

template <int NT>
static cudaError_t launch_dyn_t(const DevImage* imgs, BlockOut* blocks, int nblocks, int max_block, uint8_t* scratch,
                                uint64_t slot_bytes, const uint32_t* xpow, int grid, cudaStream_t s)
{
    const int smem = DynSmem<NT>::bytes(max_block);
    cudaError_t e = cudaFuncSetAttribute(k_rle_dyn_blocks<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    k_rle_dyn_blocks<NT><<<grid, NT, smem, s>>>(imgs, blocks, nblocks, max_block, scratch, slot_bytes, xpow);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_dyn(const DevImage* imgs, BlockOut* blocks, int nblocks, int max_block, uint8_t* scratch,
                       uint64_t slot_bytes, const uint32_t* xpow, int nsm, cudaStream_t s)
{
    int nt;
    const int grid = dyn_grid(nblocks, nsm, &nt);
    return nt == 1024 ? launch_dyn_t<1024>(imgs, blocks, nblocks, max_block, scratch, slot_bytes, xpow, grid, s)
                      : launch_dyn_t<512>(imgs, blocks, nblocks, max_block, scratch, slot_bytes, xpow, grid, s);
}

// hash_bits: the largest table size among the launch's images (9 or 10).
cudaError_t launch_lz77(const DevImage* imgs, BlockOut* blocks, int nblocks, int max_block, uint8_t* scratch,
                        uint64_t slot_bytes, const uint32_t* xpow, int grid, int hash_bits, cudaStream_t s)
{
    const int hb = hash_bits == 9 ? 9 : 10;
    cudaError_t e;
    if (max_block <= 21760) {           // three 320-thread CTAs per SM
        const int smem = lz_smem_bytes(max_block, hb, 320);
        e = cudaFuncSetAttribute(k_lz77_blocks<320>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        k_lz77_blocks<320><<<grid, 320, smem, s>>>(imgs, blocks, nblocks, max_block, scratch, slot_bytes, xpow);
    } else if (max_block <= 32768) {           // two 512-thread CTAs per SM
        const int smem = lz_smem_bytes(max_block, hb, 512);
        e = cudaFuncSetAttribute(k_lz77_blocks<512>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        k_lz77_blocks<512><<<grid, 512, smem, s>>>(imgs, blocks, nblocks, max_block, scratch, slot_bytes, xpow);
    } else {
        const int smem = lz_smem_bytes(max_block, hb);
        e = cudaFuncSetAttribute(k_lz77_blocks<kLzThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        k_lz77_blocks<kLzThreads><<<grid, kLzThreads, smem, s>>>(imgs, blocks, nblocks, max_block, scratch, slot_bytes, xpow);
    }
    note_launch();
    return cudaGetLastError();
}

}  // namespace r2p
