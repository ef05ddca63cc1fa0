// r2p_common.h -- arithmetic shared by the CUDA kernels and the host code.
//
// Everything here is plain integer code that compiles both under nvcc (device
// and host) and under g++ (host-only unit tests), so the CPU test suite can
// check it exhaustively against the oracle and zlib without a GPU.
#pragma once
#include <stddef.h>
#include <stdint.h>

#if defined(__CUDACC__)
#include <cuda_fp16.h>
#define R2P_HD __host__ __device__ __forceinline__
#else
#define R2P_HD static inline
#endif

namespace r2p {

// ---------------------------------------------------------------------------
// SWAR helpers: four independent bytes in one 32-bit word.
// ---------------------------------------------------------------------------
constexpr uint32_t kHi = 0x80808080u;
constexpr uint32_t kLo7 = 0x7F7F7F7Fu;
constexpr uint32_t kOnes = 0x01010101u;

// Per-byte wraparound subtraction (x - y) mod 256 in every byte.
R2P_HD uint32_t sub4(uint32_t x, uint32_t y)
{
    return ((x | kHi) - (y & kLo7)) ^ ((x ^ ~y) & kHi);
}

// Per-byte floor average (a + b) >> 1 without carries between bytes.
R2P_HD uint32_t avg4(uint32_t a, uint32_t b)
{
    return (a & b) + (((a ^ b) >> 1) & kLo7);
}

// Bit 7 of each byte set where a >= b (unsigned bytes).
R2P_HD uint32_t ge4_hi(uint32_t a, uint32_t b)
{
    const uint32_t d = sub4(a, b);
    // borrow out of bit 7 of (a - b): (~a & b) | (~(a ^ b) & d)
    const uint32_t borrow = (~a & b) | (~(a ^ b) & d);
    return ~borrow & kHi;
}

// Expand bit 7 of each byte to a full 0x00/0xFF byte mask.
R2P_HD uint32_t hi_to_mask(uint32_t h)
{
    return (h >> 7) * 0xFFu;
}

// Per-byte |a - b| for unsigned bytes.
R2P_HD uint32_t absdiff4(uint32_t a, uint32_t b)
{
    const uint32_t m = hi_to_mask(ge4_hi(a, b));
    return (sub4(a, b) & m) | (sub4(b, a) & ~m);
}

// Per-byte Paeth predictor (PNG specification 9.4), selection order a, b, c.
// With A = a - c and B = b - c: pa = |B|, pb = |A|, pc = |A + B|.  When A and
// B have the same sign pc = pa + pb, so the choice is pa <= pb ? a : b; when
// they differ pc = |pa - pb|, giving a if 2*pa <= pb, else b if 2*pb <= pa,
// else c.  A zero difference satisfies both branches identically.
R2P_HD uint32_t paeth4(uint32_t a, uint32_t b, uint32_t c)
{
    const uint32_t ga = ge4_hi(a, c);               // A >= 0
    const uint32_t gb = ge4_hi(b, c);               // B >= 0
    const uint32_t pa = absdiff4(b, c);
    const uint32_t pb = absdiff4(a, c);
    const uint32_t same = hi_to_mask(~(ga ^ gb) & kHi);
    const uint32_t ha = (pb >> 1) & kLo7;           // floor(pb / 2)
    const uint32_t hb = (pa >> 1) & kLo7;           // floor(pa / 2)
    const uint32_t a_le_b = hi_to_mask(ge4_hi(pb, pa));
    const uint32_t a_opp = hi_to_mask(ge4_hi(ha, pa));
    const uint32_t b_opp = hi_to_mask(ge4_hi(hb, pb));
    const uint32_t sel_a = (same & a_le_b) | (~same & a_opp);
    const uint32_t sel_b = ~sel_a & ((same & ~a_le_b) | (~same & b_opp));
    const uint32_t sel_c = ~(sel_a | sel_b);
    return (a & sel_a) | (b & sel_b) | (c & sel_c);
}

#if defined(__CUDA_ARCH__)
// Device Paeth on packed halves: bytes become fp16 values 1024 + b (a byte
// permute with 0x64 high bytes), whose differences up to +-510 are exact.
// pa = |b - c|, pb = |a - c|, pc = |a + b - 2c| and the a, b, c selection
// order of the PNG definition; the winner's low byte is the predictor.
// Checked against the scalar definition on all 2^24 (a, b, c).
__device__ __forceinline__ uint32_t paeth_h2(uint32_t a, uint32_t b, uint32_t c)
{
    const __half2 ha = *reinterpret_cast<const __half2*>(&a);
    const __half2 hb = *reinterpret_cast<const __half2*>(&b);
    const __half2 hc = *reinterpret_cast<const __half2*>(&c);
    const __half2 A = __hsub2(ha, hc), B = __hsub2(hb, hc);
    const __half2 pa = __habs2(B), pb = __habs2(A), pc = __habs2(__hadd2(A, B));
    const uint32_t ma = __hle2_mask(pa, pb) & __hle2_mask(pa, pc);
    const uint32_t mb = __hle2_mask(pb, pc);
    return (a & ma) | (~ma & ((b & mb) | (c & ~mb)));
}

__device__ __forceinline__ uint32_t paeth4_dev(uint32_t a, uint32_t b, uint32_t c)
{
    const uint32_t K = 0x64646464u;
    const uint32_t lo = paeth_h2(__byte_perm(a, K, 0x4140), __byte_perm(b, K, 0x4140), __byte_perm(c, K, 0x4140));
    const uint32_t hi = paeth_h2(__byte_perm(a, K, 0x4342), __byte_perm(b, K, 0x4342), __byte_perm(c, K, 0x4342));
    return __byte_perm(lo, hi, 0x6420);
}
#define R2P_PAETH4 paeth4_dev
#else
#define R2P_PAETH4 paeth4
#endif

// Sum over the four bytes of |int8(v)| = min(v, 256 - v), added to acc.
R2P_HD uint32_t cost4_acc(uint32_t v, uint32_t acc)
{
    // sign = +1 or -1 per byte, then a signed byte dot product.
#if defined(__CUDA_ARCH__)
    // PTX prmt (default mode): a selector nibble with its top bit set
    // replicates the selected byte's sign bit, so 0xBA98 gives 0x00 or 0xFF
    // per byte of v; OR 1 makes that +1 / -1 as signed bytes.
    uint32_t neg;
    asm("prmt.b32 %0, %1, 0, 0xBA98;" : "=r"(neg) : "r"(v));
    const uint32_t sgn = neg | kOnes;
    return (uint32_t)__dp4a((int)v, (int)sgn, (int)acc);
#else
    const uint32_t neg = (v >> 7) & kOnes;
    const uint32_t sgn = neg * 0xFEu + kOnes;
    int s = (int)acc;
    for (int k = 0; k < 4; k++)
        s += (int)(int8_t)(v >> (8 * k)) * (int)(int8_t)(sgn >> (8 * k));
    return (uint32_t)s;
#endif
}

// Sum of the four bytes of v (unsigned).
R2P_HD uint32_t bytesum4(uint32_t v)
{
#if defined(__CUDA_ARCH__)
    return (uint32_t)__dp4a(v, kOnes, 0u);
#else
    return (v & 0xFF) + ((v >> 8) & 0xFF) + ((v >> 16) & 0xFF) + (v >> 24);
#endif
}

// Sum of byte_k * k for k = 0..3 (byte 0 is the lowest address).
R2P_HD uint32_t bytewsum4(uint32_t v)
{
#if defined(__CUDA_ARCH__)
    return (uint32_t)__dp4a(v, 0x03020100u, 0u);
#else
    return ((v >> 8) & 0xFF) + 2 * ((v >> 16) & 0xFF) + 3 * (v >> 24);
#endif
}

// (hi:lo) >> sh for sh in 0..31, the low 32 bits.
R2P_HD uint32_t fshr(uint32_t lo, uint32_t hi, uint32_t sh)
{
#if defined(__CUDA_ARCH__)
    return __funnelshift_r(lo, hi, sh);
#else
    return sh ? ((lo >> sh) | (hi << (32 - sh))) : lo;
#endif
}

// Scores of the five PNG filters for one word: x (current), a (left by bpp),
// b (above), c (above-left).  mask keeps only valid bytes.
struct Score5 {
    uint32_t s0, s1, s2, s3, s4;
};

R2P_HD void score_word(Score5& s, uint32_t x, uint32_t a, uint32_t b, uint32_t c, uint32_t mask)
{
    s.s0 = cost4_acc(x & mask, s.s0);
    s.s1 = cost4_acc(sub4(x, a) & mask, s.s1);
    s.s2 = cost4_acc(sub4(x, b) & mask, s.s2);
    s.s3 = cost4_acc(sub4(x, avg4(a, b)) & mask, s.s3);
    s.s4 = cost4_acc(sub4(x, R2P_PAETH4(a, b, c)) & mask, s.s4);
}

// Filtered word for filter type f (0..4).
R2P_HD uint32_t filter_word(int f, uint32_t x, uint32_t a, uint32_t b, uint32_t c)
{
    switch (f) {
        case 0: return x;
        case 1: return sub4(x, a);
        case 2: return sub4(x, b);
        case 3: return sub4(x, avg4(a, b));
        default: return sub4(x, R2P_PAETH4(a, b, c));
    }
}

// Argmin over the five sums; strict '<' so the lowest type wins ties.
R2P_HD int best_filter(const Score5& s)
{
    int best = 0;
    uint32_t b = s.s0;
    if (s.s1 < b) { b = s.s1; best = 1; }
    if (s.s2 < b) { b = s.s2; best = 2; }
    if (s.s3 < b) { b = s.s3; best = 3; }
    if (s.s4 < b) { best = 4; }
    return best;
}

// ---------------------------------------------------------------------------
// CRC-32 (polynomial 0xEDB88320, reflected) arithmetic in GF(2)[x]/P.
// A CRC value is a polynomial in reflected bit order: bit 31 is x^0.
// ---------------------------------------------------------------------------
constexpr uint32_t kCrcPoly = 0xEDB88320u;

// Carry-less product of two 32-bit words (63 bits) from integer multiplies:
// each operand is split into four words holding every fourth bit, so in any
// partial product a column gathers at most 8 ones; the column sum then fits
// the 4 bits up to the next column of the same class, and its low bit is the
// XOR of the column (the "integer multiplies with holes" method, as BearSSL
// uses for GHASH).
R2P_HD uint64_t clmul32(uint32_t a, uint32_t b)
{
    const uint64_t a0 = a & 0x11111111u, a1 = a & 0x22222222u, a2 = a & 0x44444444u, a3 = a & 0x88888888u;
    const uint64_t b0 = b & 0x11111111u, b1 = b & 0x22222222u, b2 = b & 0x44444444u, b3 = b & 0x88888888u;
    const uint64_t z0 = (a0 * b0) ^ (a1 * b3) ^ (a2 * b2) ^ (a3 * b1);
    const uint64_t z1 = (a0 * b1) ^ (a1 * b0) ^ (a2 * b3) ^ (a3 * b2);
    const uint64_t z2 = (a0 * b2) ^ (a1 * b1) ^ (a2 * b0) ^ (a3 * b3);
    const uint64_t z3 = (a0 * b3) ^ (a1 * b2) ^ (a2 * b1) ^ (a3 * b0);
    return (z0 & 0x1111111111111111ull) | (z1 & 0x2222222222222222ull) | (z2 & 0x4444444444444444ull) |
           (z3 & 0x8888888888888888ull);
}

// a * b mod P (reflected representation), bit by bit.
R2P_HD uint32_t gf2_mulmod(uint32_t a, uint32_t b)
{
    uint32_t m = 1u << 31;   // x^0
    uint32_t p = 0;
    for (int i = 0; i < 32; i++) {
        if (a & m) p ^= b;
        m >>= 1;
        b = (b & 1u) ? (b >> 1) ^ kCrcPoly : b >> 1;   // b *= x
    }
    return p;
}

// x^(2^k * 8) mod P for k = 0..63 (byte-count powers), filled by crc_init_pow.
struct CrcPow {
    uint32_t p[64];
};

static inline void crc_init_pow(CrcPow& t)
{
    uint32_t x8 = 1u << 23;            // x^8 in reflected form (bit 31 - 8)
    t.p[0] = x8;
    for (int k = 1; k < 64; k++) t.p[k] = gf2_mulmod(t.p[k - 1], t.p[k - 1]);
}

// crc * x^(8 * nbytes) mod P: the CRC of a message shifted past nbytes more
// bytes of zeros, the building block of CRC concatenation.
R2P_HD uint32_t crc_shift(uint32_t crc, uint64_t nbytes, const uint32_t* pow)
{
    int k = 0;
    while (nbytes) {
        if (nbytes & 1u) crc = gf2_mulmod(pow[k], crc);
        nbytes >>= 1;
        k++;
    }
    return crc;
}

// crc32(A || B) from crc32(A), crc32(B) and len(B) (finalised CRC values, as
// zlib's crc32() returns them).
R2P_HD uint32_t crc32_combine(uint32_t crc_a, uint32_t crc_b, uint64_t len_b, const uint32_t* pow)
{
    return crc_shift(crc_a, len_b, pow) ^ crc_b;
}

// Byte-at-a-time table for the reflected polynomial.
static inline void crc_init_table(uint32_t* t256)
{
    for (uint32_t n = 0; n < 256; n++) {
        uint32_t c = n;
        for (int k = 0; k < 8; k++) c = (c & 1u) ? kCrcPoly ^ (c >> 1) : c >> 1;
        t256[n] = c;
    }
}

// ---------------------------------------------------------------------------
// Adler-32 (RFC 1950).  For bytes d_0..d_{n-1}:
//   A = 1 + S1,  B = n + S2  (mod 65521)
//   S1 = sum d_i,  S2 = sum (n - i) d_i
// Concatenation (A1,B1,n1) . (A2,B2,n2) = (A1 + A2 - 1, B1 + B2 + n2*(A1 - 1)).
// ---------------------------------------------------------------------------
constexpr uint32_t kAdlerMod = 65521u;

R2P_HD uint32_t adler_from_sums(uint64_t s1, uint64_t s2, uint64_t n)
{
    const uint32_t a = (uint32_t)((1u + s1 % kAdlerMod) % kAdlerMod);
    const uint32_t b = (uint32_t)((n % kAdlerMod + s2 % kAdlerMod) % kAdlerMod);
    return (b << 16) | a;
}

R2P_HD uint32_t adler32_combine(uint32_t ad1, uint32_t ad2, uint64_t len2)
{
    const uint64_t a1 = ad1 & 0xFFFF, b1 = ad1 >> 16;
    const uint64_t a2 = ad2 & 0xFFFF, b2 = ad2 >> 16;
    const uint64_t rem = len2 % kAdlerMod;
    const uint64_t a = (a1 + a2 + kAdlerMod - 1) % kAdlerMod;
    const uint64_t b = (b1 + b2 + rem * ((a1 + kAdlerMod - 1) % kAdlerMod)) % kAdlerMod;
    return (uint32_t)((b << 16) | a);
}

// ---------------------------------------------------------------------------
// DEFLATE fixed Huffman code (RFC 1951 3.2.6), codes bit-reversed for an
// LSB-first bit writer, and the length/distance symbol tables (3.2.5).
// ---------------------------------------------------------------------------
R2P_HD uint32_t bitrev(uint32_t v, int n)
{
    uint32_t r = 0;
    for (int i = 0; i < n; i++) { r = (r << 1) | (v & 1u); v >>= 1; }
    return r;
}

// Literal/length symbol 0..287 -> (reversed code, length).
R2P_HD void fixed_code(int sym, uint32_t& code, int& len)
{
    if (sym < 144)      { len = 8; code = bitrev(0x30u + (uint32_t)sym, 8); }
    else if (sym < 256) { len = 9; code = bitrev(0x190u + (uint32_t)(sym - 144), 9); }
    else if (sym < 280) { len = 7; code = bitrev((uint32_t)(sym - 256), 7); }
    else                { len = 8; code = bitrev(0xC0u + (uint32_t)(sym - 280), 8); }
}

// Match length 3..258 -> length symbol index 0..28 (symbol 257 + idx),
// extra-bit count and extra value.
R2P_HD void length_code(int len, int& idx, int& nextra, int& extra)
{
    if (len == 258) { idx = 28; nextra = 0; extra = 0; return; }
    const int l = len - 3;                     // 0..254
    if (l < 8) { idx = l; nextra = 0; extra = 0; return; }
    // For l >= 8: nextra = floor(log2(l)) - 2, four codes per extra-bit count.
    int lg = 31;
    while (!((uint32_t)l >> lg)) lg--;
    nextra = lg - 2;
    idx = 4 * nextra + 4 + ((l >> nextra) & 3);
    extra = l & ((1 << nextra) - 1);
}

// Distance 1..32768 -> distance code 0..29, extra-bit count and value.
R2P_HD void dist_code(int dist, int& code, int& nextra, int& extra)
{
    const int d = dist - 1;                    // 0..32767
    if (d < 4) { code = d; nextra = 0; extra = 0; return; }
    int lg = 31;
    while (!((uint32_t)d >> lg)) lg--;
    nextra = lg - 1;
    code = 2 * nextra + 2 + ((d >> nextra) & 1);
    extra = d & ((1 << nextra) - 1);
}

}  // namespace r2p
