// r2p_kernels.h -- host-side launch wrappers of the CUDA kernels.
#pragma once
#include <cuda_runtime.h>

#include "r2p_device.h"

namespace r2p {

// count of kernels this library launched (all streams)
void note_launch();

// k_filter.cu
cudaError_t launch_prepare_window(DevImage* imgs, int n, cudaStream_t s);
// The bounded barrier wait on a barrier nothing completes (arrive = 0) or
// one arrival completes (arrive = 1); writes R2P_ETIMEOUT or R2P_OK.
cudaError_t launch_wait_probe(int arrive, uint64_t limit_ns, int* d_status, cudaStream_t s);
// BMP files of n images (max_words: 4-byte words of the largest file).
cudaError_t launch_bmp(DevImage* imgs, int n, uint32_t max_words, int nsm, cudaStream_t s);
cudaError_t launch_window_filter(DevImage* imgs, const BandItem* items, int nitems, int grid,
                                 int smem, cudaStream_t s);
int filter_smem_bytes(int rb, int in_pitch, int mode, int lut_entries, int lut_esize);
int filter_tile_rows(int rb, int in_pitch, int smem, int lut_region);
int filter_lut_region(int mode, int lut_entries, int lut_esize);
int filter_ctas_per_sm(int smem);

// k_filter_reg.cu: rows of up to 8 KB held in registers by groups of warps
// (the engine sends it the rows narrower than the warp-per-row kernel's)
int reg_filter_warps(int rb);
bool reg_filter_eligible(int rb, int in_pitch, int lut_bytes);
int reg_filter_cta_warps(int max_w);
int reg_filter_smem(int rb, int in_pitch, int lut_bytes, int nw);
int reg_filter_ctas_per_sm(int nw, int smem);
cudaError_t launch_window_filter_reg(DevImage* imgs, const BandItem* items, int nitems, int grid, int nw, int smem,
                                     cudaStream_t s);

// k_filter_rows.cu: wide rows, one warp per row; k_window_lut builds the
// tables of the images whose fpath is kFiltRows, then k_filter_rows runs
// over items of rows_filter_rows_per_item() rows
bool rows_filter_eligible(int in_pitch, int lut_bytes);
int rows_filter_rows_per_item();
int rows_filter_stash(int rb, int lut_bytes);       // per-warp stash bytes for such rows (0: none)
int rows_filter_smem(int lut_bytes, int stash);
int rows_filter_ctas_per_sm(int smem);
cudaError_t launch_filter_rows(DevImage* imgs, int n, int lut_bytes, int stash, const BandItem* items, int nitems,
                               int grid, cudaStream_t s);

// k_deflate.cu
int stored_smem_bytes(int block_size);
cudaError_t launch_stored(const DevImage* imgs, BlockOut* blocks, int nblocks, int max_block,
                          const uint32_t* xpow, int grid, cudaStream_t s);
// k_finish over nblocks * parts units (slices of blocks) on `grid` CTAs
cudaError_t launch_finish(DevImage* imgs, BlockOut* blocks, int nblocks, int parts, const uint8_t* scratch,
                          uint64_t slot_bytes, const uint32_t* xpow, int grid, cudaStream_t s);
int finish_parts(int nblocks, int nsm);   // slices per block for a launch of nblocks blocks
size_t checksum_scratch_bytes(uint64_t len);
cudaError_t launch_checksum(const uint8_t* data, uint64_t len, bool adler, uint32_t* result, void* scratch,
                            const uint32_t* xpow, int grid, cudaStream_t s);

// k_lz77.cu
uint64_t lz77_slot_bytes(int block_size);
cudaError_t launch_lz77(const DevImage* imgs, BlockOut* blocks, int nblocks, int max_block, uint8_t* scratch,
                        uint64_t slot_bytes, const uint32_t* xpow, int grid, int hash_bits, cudaStream_t s);
// levels 2-9: dynamic-Huffman blocks over a run-length parse (same slots as
// LZ77); picks its CTA size and grid from the block count and SM count
cudaError_t launch_dyn(const DevImage* imgs, BlockOut* blocks, int nblocks, int max_block, uint8_t* scratch,
                       uint64_t slot_bytes, const uint32_t* xpow, int nsm, cudaStream_t s);

}  // namespace r2p
