// r2p_noalloc.cu -- zlib compression of device data that allocates nothing.
//
// Some callers cannot allocate device memory once they are running: code
// hosted inside a framework that owns all GPU memory and forbids allocation
// after start-up (an imaging viewer's plug-in, a frame pipeline with a fixed
// memory budget), and latency-sensitive callers for which cudaMalloc/cudaFree
// are unacceptable because they can stall or synchronize the device.  For
// them r2p_zlib_compress_noalloc runs the same DEFLATE kernels as
// r2p_zlib_compress_device (stored blocks at level 0, LZ77 + fixed Huffman at
// level 1, dynamic Huffman over a run-length parse at levels 2-9, Adler-32
// trailer) with every piece of scratch -- work descriptors, per-block results,
// the LZ77 block slots and the CRC power table -- in one file-scope
// __device__ array of kNoAllocScratchBytes.  Every GPU that loads the library
// holds that array until the process exits.  The caller passes the input, the
// output and the length word.
//
// Set-up: the first call on a device (with that device current) looks up the
// array's device address with cudaGetSymbolAddress and fills the CRC power
// table with a kernel, then waits for it; make that first call before any
// stream capture.  The set-up is kept for the life of the process: after
// cudaDeviceReset (which clears the array) the entry point must not be used
// again.  All calls share the array, which keeps the previous call's
// contents: each call rewrites every descriptor it reads.  Calls that overlap
// on the GPU race on the array: issue them on one stream, or order them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "k_deflate.cuh"
#include "r2p_kernels.h"

namespace r2p {

constexpr size_t kNoAllocMaxInput = 1u << 20;          // bytes of input per call (1 MiB)
constexpr size_t kNoAllocScratchBytes = 2u << 20;      // static scratch per GPU (2 MiB)

// scratch layout (offsets in bytes)
constexpr size_t kNaImage = 0;                          // DevImage
constexpr size_t kNaXpow = 256;                         // kXpowLevels * 1024 uint32
constexpr size_t kNaBlocks = kNaXpow + kXpowLevels * 1024 * 4;   // BlockOut[]

static_assert(sizeof(DevImage) <= kNaXpow - kNaImage, "the image descriptor overruns the power table");
static_assert(kNaBlocks % alignof(BlockOut) == 0 && kNaXpow % 16 == 0, "scratch regions misaligned");

static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

// x^(8 * j * 2^(10 l)) mod P for every table entry (same values as the
// engine's host-built table).
__global__ void k_noalloc_xpow(uint32_t* tab)
{
    __shared__ uint32_t pow2[64];
    if (threadIdx.x == 0) {
        uint32_t v = 1u << 23;   // x^8
        for (int k = 0; k < 64; k++) {
            pow2[k] = v;
            v = gf2_mulmod(v, v);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kXpowLevels * 1024; i += blockDim.x) {
        const int l = i >> 10, j = i & 1023;
        tab[i] = crc_shift(0x80000000u, (uint64_t)j << (10 * l), pow2);
    }
}

// Rewrite the descriptors of one call: a single "image" whose filtered
// stream is the caller's input and whose output is a bare zlib stream.
__global__ void k_noalloc_plan(DevImage* d, BlockOut* bo, const uint8_t* in, uint64_t len, int level, int bs,
                               uint8_t* out, uint64_t cap, uint64_t* out_len)
{
    const int nb = (int)((len + bs - 1) / bs);
    if (threadIdx.x == 0) {
        DevImage z;
        memset(&z, 0, sizeof(z));
        z.width = 1; z.height = 1; z.channels = 1; z.ib = 1; z.ob = 1; z.bpp = 1;
        z.filt_bytes = len;
        z.req_mode = R2P_WINDOW_NONE;
        z.filt = const_cast<uint8_t*>(in);
        z.level = level;
        z.block_size = bs;
        z.hash_bits = 10;
        z.nblocks = nb;
        z.out_kind = 1;
        z.prefix = 2;
        z.png = out;
        z.png_cap = cap;
        z.png_len = out_len;
        *d = z;
    }
    for (int k = threadIdx.x; k < nb; k += blockDim.x) {
        BlockOut b;
        memset(&b, 0, sizeof(b));
        b.in_off = (uint32_t)((uint64_t)k * bs);
        b.in_len = (uint32_t)min((uint64_t)bs, len - (uint64_t)k * bs);
        bo[k] = b;
    }
}

struct NoAllocDevice {
    bool ready = false;
    uint8_t* scratch = nullptr;
    int nsm = 1;
};

static std::mutex g_na_mu;
static NoAllocDevice g_na_dev[64];

static int na_fail(cudaError_t e, const char* where);
static int na_einval(const char* what);

}  // namespace r2p

// defined in r2p_engine.cu: record a status message for r2p_last_error()
int r2p_internal_set_error(int code, const char* msg);

namespace r2p {

static int na_fail(cudaError_t e, const char* where)
{
    char buf[256];
    snprintf(buf, sizeof(buf), "r2p_zlib_compress_noalloc: %s: %s", where, cudaGetErrorString(e));
    return r2p_internal_set_error(R2P_ECUDA, buf);
}

static int na_einval(const char* what) { return r2p_internal_set_error(R2P_EINVAL, what); }

}  // namespace r2p

using namespace r2p;

extern "C" int r2p_zlib_compress_noalloc(const void* d_in, size_t len, int level, int block_size, void* d_out,
                                         size_t out_cap, uint64_t* d_out_len, void* stream)
{
    if (!d_in || !d_out || !d_out_len) return na_einval("r2p_zlib_compress_noalloc: NULL argument");
    if (len == 0 || len > kNoAllocMaxInput)
        return na_einval("r2p_zlib_compress_noalloc: len must be in [1, 1048576] (1 MiB static scratch limit)");
    if (level < 0 || level > 9) return na_einval("r2p_zlib_compress_noalloc: level must be 0..9");
    const int bs = block_size ? block_size : kBlock64;
    if (bs < 1024 || bs > kBlock64 || (bs & 15))
        return na_einval("r2p_zlib_compress_noalloc: block_size must be a multiple of 16 in [1024, 65520]");
    const size_t nb = (len + bs - 1) / bs;
    const uint64_t slot = lz77_slot_bytes(bs);
    const size_t blocks_end = (kNaBlocks + nb * sizeof(BlockOut) + 255) & ~(size_t)255;
    const size_t need = blocks_end + (level > 0 ? nb * slot : 0);
    if (need > kNoAllocScratchBytes)
        return na_einval("r2p_zlib_compress_noalloc: input needs more than the 2 MiB static scratch");
    if (out_cap < 2 + len + (size_t)kStoredHdr * (nb + 1) + 4)
        return r2p_internal_set_error(R2P_ENOSPC, "r2p_zlib_compress_noalloc: out_cap below r2p_zlib_bound()");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64) return na_einval("r2p_zlib_compress_noalloc: device index above 63");
    NoAllocDevice nd;
    {
        std::lock_guard<std::mutex> lk(g_na_mu);
        NoAllocDevice& st = g_na_dev[dev];
        if (!st.ready) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return na_fail(e, "cudaGetSymbolAddress");
            e = cudaDeviceGetAttribute(&st.nsm, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return na_fail(e, "cudaDeviceGetAttribute");
            st.scratch = static_cast<uint8_t*>(p);
            k_noalloc_xpow<<<1, 256, 0, s>>>(reinterpret_cast<uint32_t*>(st.scratch + kNaXpow));
            note_launch();
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return na_fail(e, "power-table set-up");
            st.ready = true;
        }
        nd = st;
    }
    uint8_t* S = nd.scratch;
    DevImage* dimg = reinterpret_cast<DevImage*>(S + kNaImage);
    const uint32_t* xpow = reinterpret_cast<const uint32_t*>(S + kNaXpow);
    BlockOut* dblk = reinterpret_cast<BlockOut*>(S + kNaBlocks);
    uint8_t* slots = S + blocks_end;
    k_noalloc_plan<<<1, 256, 0, s>>>(dimg, dblk, static_cast<const uint8_t*>(d_in), len, level, bs,
                                     static_cast<uint8_t*>(d_out), out_cap, d_out_len);
    note_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return na_fail(e, "k_noalloc_plan");
    const int grid = (int)std::min<size_t>(nb, (size_t)nd.nsm * 8);
    if (level == 0) e = launch_stored(dimg, dblk, (int)nb, bs, xpow, grid, s);
    else if (level == 1) e = launch_lz77(dimg, dblk, (int)nb, bs, slots, slot, xpow, grid, 10, s);
    else e = launch_dyn(dimg, dblk, (int)nb, bs, slots, slot, xpow, nd.nsm, s);
    if (e != cudaSuccess) return na_fail(e, "DEFLATE blocks");
    const int parts = finish_parts((int)nb, nd.nsm);
    const int fgrid = (int)std::min<size_t>(nb * (size_t)parts, (size_t)nd.nsm * 8);
    e = launch_finish(dimg, dblk, (int)nb, parts, slots, slot, xpow, fgrid, s);
    if (e != cudaSuccess) return na_fail(e, "k_finish");
    return R2P_OK;
}
