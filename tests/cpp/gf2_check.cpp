// The table-assisted GF(2) product of the CRC kernels (gf2_mulmod_t in
// csrc/k_deflate.cuh): the carry-less product clmul32(a, b), moved up one
// bit, then its low word through one slicing-by-4 CRC step, must equal the
// bit-by-bit gf2_mulmod(a, b) for every a, b.  This restates that step with
// host tables and checks random and edge-case operands.
#include <cstdint>
#include <cstdio>
#include <random>
#include "r2p_common.h"
using namespace r2p;
static uint32_t T[4][256];
static uint32_t crc_word0(uint32_t c) { return T[3][c & 0xFF] ^ T[2][(c >> 8) & 0xFF] ^ T[1][(c >> 16) & 0xFF] ^ T[0][c >> 24]; }
int main()
{
    for (int n = 0; n < 256; n++) { uint32_t c = n; for (int k = 0; k < 8; k++) c = (c & 1u) ? kCrcPoly ^ (c >> 1) : c >> 1; T[0][n] = c; }
    for (int n = 0; n < 256; n++) { uint32_t c = T[0][n]; for (int k = 1; k < 4; k++) { c = (c >> 8) ^ T[0][c & 0xFF]; T[k][n] = c; } }
    std::mt19937_64 rng(3);
    for (long i = 0; i < 2000000; i++) {
        uint32_t a = (uint32_t)rng(), b = (uint32_t)rng();
        if (i % 7 == 0) a = 0xFFFFFFFFu; if (i % 11 == 0) b = 0xFFFFFFFFu; if (i % 13 == 0) a = 1u << (rng() % 32);
        const uint64_t R = clmul32(a, b) << 1;
        const uint32_t fast = (uint32_t)(R >> 32) ^ crc_word0((uint32_t)R);
        if (fast != gf2_mulmod(a, b)) { printf("MISMATCH %08x %08x\n", a, b); return 1; }
    }
    printf("ok\n");
    return 0;
}
