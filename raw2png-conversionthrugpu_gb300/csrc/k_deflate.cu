// k_deflate.cu -- stored DEFLATE blocks, the finish pass (block gather, checksum combine, PNG chunks),
// and standalone Adler-32 / CRC-32 over device data.
//
// Reference semantics:
//   stored level-0 stream   zlib level 0 via deflate_strip (src/parallel_deflate.cpp:55,155-157)
//   Adler-32 of filtered    adler32_partial_kernel + host combine (src/gpu_adler32.cu:39-56,106-125)
//   CRC-32 of IDAT          crc32_partial_kernel / host crc32 (src/gpu_crc32.cu:61-76,
//                           src/gpu_png_assemble.cu:126-154, src/png_writer.cpp:113-125)
//   zlib header FLEVEL      zlib_header (src/parallel_deflate.cpp:214-228)
//   PNG container           PngWriter::open/close (src/png_writer.cpp:33-101),
//                           colour type from channels (src/pipeline.cpp:80-88)
//
// Every block kernel leaves per-block partials (output length, CRC of its
// output bytes, Adler sums of its input bytes); k_finish joins them with the
// combine identities and gathers the blocks, so no kernel waits on another
// block.
#include <cuda_runtime.h>

#include <algorithm>

#include "k_deflate.cuh"
#include "r2p_kernels.h"

namespace r2p {

constexpr int kStoredThreads = 256;

// Level 0: one stored block per BlockOut, written straight to its final place
// in the PNG (block offsets are fixed: every block but the last is full).
__global__ void __launch_bounds__(kStoredThreads)
k_stored_blocks(const DevImage* __restrict__ imgs, BlockOut* __restrict__ blocks, int nblocks,
                const uint32_t* __restrict__ xpow)
{
    extern __shared__ __align__(16) uint8_t sm[];
    uint32_t (*tab)[256] = reinterpret_cast<uint32_t (*)[256]>(sm);
    uint8_t* buf = sm + 4096;
    __shared__ uint64_t red64[kStoredThreads / 32];
    __shared__ uint32_t red32[kStoredThreads / 32];
    build_crc_tables(tab);
    const int tid = threadIdx.x;
    for (int b = blockIdx.x; b < nblocks; b += gridDim.x) {
        BlockOut& bo = blocks[b];
        const DevImage& d = imgs[bo.img];
        if (d.level != 0) continue;
        const int n = (int)bo.in_len;
        const uint8_t* src = d.filt + bo.in_off;
        __syncthreads();
        if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
            for (int i = tid; i < (n >> 4); i += kStoredThreads)
                reinterpret_cast<uint4*>(buf)[i] = __ldg(reinterpret_cast<const uint4*>(src) + i);
            for (int i = (n & ~15) + tid; i < n; i += kStoredThreads) buf[i] = src[i];
        } else {
            for (int i = tid; i < n; i += kStoredThreads) buf[i] = src[i];
        }
        __syncthreads();
        const int local = (int)(b - d.blk0);
        const bool last = (local == d.nblocks - 1) && !d.open_end;
        uint8_t* dst = d.png + d.prefix + (size_t)local * (size_t)(kStoredHdr + d.block_size);
        uint8_t hdr[kStoredHdr] = {(uint8_t)(last ? 1 : 0), (uint8_t)(n & 0xFF), (uint8_t)(n >> 8),
                                   (uint8_t)(~n & 0xFF), (uint8_t)((~n >> 8) & 0xFF)};
        if (tid < kStoredHdr) dst[tid] = hdr[tid];
        cta_copy_to_global<kStoredThreads>(dst + kStoredHdr, buf, n);
        uint32_t crc, s1;
        uint64_t s2;
        cta_crc_adler<kStoredThreads>(buf, n, true, tab, xpow, crc, s1, s2, red64, red32);
        if (tid == 0) {
            const uint32_t ch = crc_small(hdr, kStoredHdr, tab);
            bo.crc = gf2_mulmod_t(ch, xpow8n_t((uint64_t)n, xpow, tab), tab) ^ crc;
            bo.out_len = (uint32_t)(n + kStoredHdr);
            bo.s1 = s1;
            bo.s2 = s2;
        }
    }
}

// zlib FLG byte for a level (src/parallel_deflate.cpp:219-223)
__device__ __forceinline__ uint8_t zlib_flg(int level)
{
    if (level == 1) return 0x01;
    if (level >= 2 && level <= 5) return 0x5E;
    if (level >= 6 && level <= 7) return 0x9C;
    return 0xDA;
}

__device__ __forceinline__ void put_be32(uint8_t* p, uint32_t v)
{
    p[0] = (uint8_t)(v >> 24); p[1] = (uint8_t)(v >> 16); p[2] = (uint8_t)(v >> 8); p[3] = (uint8_t)v;
}

constexpr int kFinThreads = 1024;   // standalone checksum combine: one partial per thread
constexpr int kFinishThreads = 256;

// Exclusive scan of a per-thread u64 value across an NT-thread CTA; returns
// the exclusive prefix and writes the CTA total to *total.
template <int NT>
__device__ uint64_t cta_exscan64(uint64_t v, uint64_t* sw, uint64_t* total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sw[warp] = x;
    __syncthreads();
    uint64_t base = 0, tot = 0;
#pragma unroll
    for (int i = 0; i < NT / 32; i++) {
        if (i < warp) base += sw[i];
        tot += sw[i];
    }
    __syncthreads();
    *total = tot;
    return base + x - v;
}

// Bytes an image's output needs for a DEFLATE stream of Ls bytes: the PNG
// chunks around it, the zlib header and Adler trailer, or for raw DEFLATE the
// stream and the input's Adler-32 after it.
__device__ __forceinline__ uint64_t output_need(const DevImage& d, uint64_t Ls)
{
    return d.out_kind == 0 ? (uint64_t)kPngPrefix + Ls + kPngSuffix : d.out_kind == 2 ? Ls + 4 : 2 + Ls + 4;
}

// One image's stream offsets, Adler-32 of the filtered bytes, CRC-32 of the
// IDAT chunk, and the PNG chunks around the DEFLATE stream of Ls bytes.
// Output layout: sig | IHDR | IDAT len,type | zlib hdr | stream | adler | crc | IEND.
// Whole CTA; tab holds the slicing tables.
template <int NT>
__device__ void finish_image(DevImage& d, BlockOut* B, uint64_t Ls, const uint32_t* __restrict__ xpow,
                             const uint32_t (*tab)[256], uint64_t* sw, uint64_t* red64, uint32_t* red32)
{
    const int nb = d.nblocks;
    const uint64_t F = d.filt_bytes;
    uint64_t s1 = 0, s2 = 0, carry = 0;
    uint32_t cx = 0;
    for (int base = 0; base < nb; base += NT) {
        const int i = base + threadIdx.x;
        const uint64_t len = (i < nb) ? B[i].out_len : 0;
        uint64_t tot;
        const uint64_t off = carry + cta_exscan64<NT>(len, sw, &tot);
        carry += tot;
        if (i < nb) {
            BlockOut& bo = B[i];
            bo.out_off = off;
            const uint64_t after_in = F - (uint64_t)bo.in_off - bo.in_len;
            s1 += bo.s1;
            s2 = (s2 + bo.s2 % kAdlerMod + (after_in % kAdlerMod) * (bo.s1 % kAdlerMod)) % kAdlerMod;
            const uint64_t after_out = Ls - off - len + 4;   // + Adler trailer
            cx ^= gf2_mulmod_t(bo.crc, xpow8n_t(after_out, xpow, tab), tab);
        }
    }
    s1 = cta_sum64<NT>(s1, red64);
    s2 = cta_sum64<NT>(s2, red64);
    cx = cta_xor<NT>(cx, red32);
    if (threadIdx.x != 0) return;
    const bool png = (d.out_kind == 0), raw = (d.out_kind == 2);
    const uint64_t total = raw ? Ls : output_need(d, Ls);   // raw: the Adler word is not counted
    if (d.status == 0 && output_need(d, Ls) > d.png_cap) d.status = R2P_ENOSPC;
    if (d.status) {                    // error word: top bit set, status in the low bits
        *d.png_len = (1ull << 63) | (uint64_t)d.status;
        return;
    }
    const uint32_t adler = adler_from_sums(s1, s2 % kAdlerMod, F);
    uint8_t* p = d.png;
    uint8_t head[6] = {'I', 'D', 'A', 'T', 0x78, zlib_flg(d.level)};
    uint8_t trl[4];
    put_be32(trl, adler);
    uint8_t* q = p + d.prefix + Ls;
    for (int i = 0; i < 4; i++) q[i] = trl[i];
    if (raw) {
        *d.png_len = total;
        return;
    }
    if (!png) {
        p[0] = head[4];
        p[1] = head[5];
        *d.png_len = total;
        return;
    }
    const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    for (int i = 0; i < 8; i++) p[i] = sig[i];
    uint8_t ihdr[17] = {'I', 'H', 'D', 'R'};
    put_be32(ihdr + 4, d.width);
    put_be32(ihdr + 8, d.height);
    ihdr[12] = (uint8_t)(8 * d.ob);
    ihdr[13] = (uint8_t)(d.channels == 1 ? 0 : d.channels == 3 ? 2 : d.channels == 4 ? 6 : 2);
    ihdr[14] = 0; ihdr[15] = 0; ihdr[16] = 0;
    put_be32(p + 8, 13);
    for (int i = 0; i < 17; i++) p[12 + i] = ihdr[i];
    put_be32(p + 29, crc_small(ihdr, 17, tab));
    put_be32(p + 33, (uint32_t)(Ls + 6));
    for (int i = 0; i < 6; i++) p[37 + i] = head[i];
    const uint32_t ch = crc_small(head, 6, tab);
    const uint32_t ct = crc_small(trl, 4, tab);
    const uint32_t crc = gf2_mulmod_t(ch, xpow8n_t(Ls + 4, xpow, tab), tab) ^ cx ^ ct;
    put_be32(q + 4, crc);
    const uint8_t iend[12] = {0, 0, 0, 0, 'I', 'E', 'N', 'D', 0xAE, 0x42, 0x60, 0x82};
    for (int i = 0; i < 12; i++) q[8 + i] = iend[i];
    *d.png_len = total;
}

// After the block kernels, one launch finishes every image.  A work unit is
// one of `parts` slices of one block.  Its CTA sums the output lengths of
// the image's blocks (the block's stream offset and the stream length) and
// moves its slice of the block's compressed bytes from the scratch slot to
// the PNG; the unit of an image's first block, slice 0, also writes that
// image's checksums and chunks.  No unit waits on another: every unit
// derives the same offsets and the same fits-the-output decision from the
// per-block lengths.  Slices split at 16-byte steps of the slot, so each
// slice's source stays aligned; stored (level-0) blocks are already in place.
__global__ void __launch_bounds__(kFinishThreads)
k_finish(DevImage* __restrict__ imgs, BlockOut* __restrict__ blocks, int nblocks, int parts,
         const uint8_t* __restrict__ scratch, uint64_t slot_bytes, const uint32_t* __restrict__ xpow)
{
    constexpr int NT = kFinishThreads;
    __shared__ uint64_t sw[NT / 32];
    __shared__ uint64_t red64[NT / 32];
    __shared__ uint32_t red32[NT / 32];
    __shared__ uint32_t tab[4][256];
    bool have_tab = false;
    const int units = nblocks * parts;
    for (int u = blockIdx.x; u < units; u += gridDim.x) {
        const int b = u / parts, part = u - b * parts;
        const int n = (int)blocks[b].out_len;
        DevImage& d = imgs[blocks[b].img];
        BlockOut* B = blocks + d.blk0;
        const int nb = d.nblocks, local = b - d.blk0;
        const int st0 = d.status;
        // one warp sums the image's block lengths: this block's stream
        // offset and the stream length
        if (threadIdx.x < 32) {
            uint64_t before = 0, all = 0;
            for (int i = threadIdx.x; i < nb; i += 32) {
                const uint64_t len = B[i].out_len;
                all += len;
                if (i < local) before += len;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                before += __shfl_xor_sync(0xFFFFFFFFu, before, o);
                all += __shfl_xor_sync(0xFFFFFFFFu, all, o);
            }
            if (threadIdx.x == 0) {
                sw[0] = before;
                sw[1] = all;
            }
        }
        __syncthreads();
        const uint64_t before = sw[0], all = sw[1];
        __syncthreads();                         // sw is reused by the image finish and the next unit
        if (local == 0 && part == 0) {
            if (!have_tab) {
                build_crc_tables(tab);
                have_tab = true;
            }
            finish_image<NT>(d, B, all, xpow, tab, sw, red64, red32);
        }
        if (st0 != 0 || d.level == 0 || output_need(d, all) > d.png_cap) continue;
        const int c0 = (int)(((int64_t)n * part / parts) & ~15ll);
        const int c1 = (part + 1 == parts) ? n : (int)(((int64_t)n * (part + 1) / parts) & ~15ll);
        cta_copy_to_global<NT>(d.png + d.prefix + before + c0, scratch + (size_t)b * slot_bytes + c0, c1 - c0);
    }
}

// ---------------------------------------------------------------------------
// Standalone checksums over arbitrary device data: per-64 KB partials, then
// one combining CTA.
// ---------------------------------------------------------------------------
constexpr int kSumChunk = 65536;

struct SumPart {
    uint32_t crc, s1;
    uint64_t s2;
};

__global__ void __launch_bounds__(kStoredThreads)
k_checksum_parts(const uint8_t* __restrict__ data, uint64_t len, SumPart* parts, int want_adler,
                 const uint32_t* __restrict__ xpow)
{
    extern __shared__ __align__(16) uint8_t sm[];
    uint32_t (*tab)[256] = reinterpret_cast<uint32_t (*)[256]>(sm);
    uint8_t* buf = sm + 4096;
    __shared__ uint64_t red64[kStoredThreads / 32];
    __shared__ uint32_t red32[kStoredThreads / 32];
    build_crc_tables(tab);
    const uint64_t nparts = (len + kSumChunk - 1) / kSumChunk;
    for (uint64_t p = blockIdx.x; p < nparts; p += gridDim.x) {
        const uint64_t o = p * kSumChunk;
        const int n = (int)min((uint64_t)kSumChunk, len - o);
        const uint8_t* src = data + o;
        __syncthreads();
        if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
            for (int i = threadIdx.x; i < (n >> 4); i += kStoredThreads)
                reinterpret_cast<uint4*>(buf)[i] = __ldg(reinterpret_cast<const uint4*>(src) + i);
            for (int i = (n & ~15) + threadIdx.x; i < n; i += kStoredThreads) buf[i] = src[i];
        } else {
            for (int i = threadIdx.x; i < n; i += kStoredThreads) buf[i] = src[i];
        }
        __syncthreads();
        uint32_t crc, s1 = 0;
        uint64_t s2 = 0;
        cta_crc_adler<kStoredThreads>(buf, n, want_adler != 0, tab, xpow, crc, s1, s2, red64, red32);
        if (threadIdx.x == 0) parts[p] = SumPart{crc, s1, s2};
    }
}

__global__ void __launch_bounds__(kFinThreads)
k_checksum_final(const SumPart* __restrict__ parts, uint64_t len, int want_adler, uint32_t* result,
                 const uint32_t* __restrict__ xpow)
{
    __shared__ uint64_t red64[kFinThreads / 32];
    __shared__ uint32_t red32[kFinThreads / 32];
    const uint64_t nparts = (len + kSumChunk - 1) / kSumChunk;
    uint64_t s1 = 0, s2 = 0;
    uint32_t cx = 0;
    for (uint64_t p = threadIdx.x; p < nparts; p += kFinThreads) {
        const uint64_t o = p * kSumChunk;
        const uint64_t n = min((uint64_t)kSumChunk, len - o);
        const uint64_t after = len - o - n;
        if (want_adler) {
            s1 += parts[p].s1;
            s2 = (s2 + parts[p].s2 % kAdlerMod + (after % kAdlerMod) * (parts[p].s1 % kAdlerMod)) % kAdlerMod;
        } else {
            cx ^= gf2_mulmod(parts[p].crc, xpow8n(after, xpow));
        }
    }
    if (want_adler) {
        s1 = cta_sum64<kFinThreads>(s1, red64);
        s2 = cta_sum64<kFinThreads>(s2, red64);
        if (threadIdx.x == 0) *result = adler_from_sums(s1, s2 % kAdlerMod, len);
    } else {
        cx = cta_xor<kFinThreads>(cx, red32);
        // crc32 of empty data is 0; otherwise the XOR of the shifted partials
        if (threadIdx.x == 0) *result = (len == 0) ? 0u : cx;
    }
}

// ---------------------------------------------------------------------------
// launch wrappers
// ---------------------------------------------------------------------------
int stored_smem_bytes(int block_size) { return 4096 + block_size + 16; }

cudaError_t launch_stored(const DevImage* imgs, BlockOut* blocks, int nblocks, int max_block,
                          const uint32_t* xpow, int grid, cudaStream_t s)
{
    const int smem = stored_smem_bytes(max_block);
    cudaError_t e = cudaFuncSetAttribute(k_stored_blocks, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    k_stored_blocks<<<grid, kStoredThreads, smem, s>>>(imgs, blocks, nblocks, xpow);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_finish(DevImage* imgs, BlockOut* blocks, int nblocks, int parts, const uint8_t* scratch,
                          uint64_t slot_bytes, const uint32_t* xpow, int grid, cudaStream_t s)
{
    if (parts < 1 || parts > 64 || nblocks < 1 || grid < 1) return cudaErrorInvalidValue;
    k_finish<<<grid, kFinishThreads, 0, s>>>(imgs, blocks, nblocks, parts, scratch, slot_bytes, xpow);
    note_launch();
    return cudaGetLastError();
}

int finish_parts(int nblocks, int nsm)
{
    // about eight units per SM when blocks are few; one unit per block otherwise
    const int want = (8 * nsm + nblocks - 1) / std::max(nblocks, 1);
    return std::min(8, std::max(1, want));
}

size_t checksum_scratch_bytes(uint64_t len)
{
    return (size_t)((len + kSumChunk - 1) / kSumChunk + 1) * sizeof(SumPart);
}

cudaError_t launch_checksum(const uint8_t* data, uint64_t len, bool adler, uint32_t* result, void* scratch,
                            const uint32_t* xpow, int grid, cudaStream_t s)
{
    const int smem = 4096 + kSumChunk + 16;
    cudaError_t e = cudaFuncSetAttribute(k_checksum_parts, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    SumPart* parts = reinterpret_cast<SumPart*>(scratch);
    if (len > 0) {
        k_checksum_parts<<<grid, kStoredThreads, smem, s>>>(data, len, parts, adler ? 1 : 0, xpow);
        note_launch();
    }
    k_checksum_final<<<1, kFinThreads, 0, s>>>(parts, len, adler ? 1 : 0, result, xpow);
    note_launch();
    return cudaGetLastError();
}

}  // namespace r2p
