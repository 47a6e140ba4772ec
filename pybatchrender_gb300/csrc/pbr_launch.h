// pbr_launch.h -- host-side launchers exported by the .cu translation units to
// the C ABI layer (pbr_capi.cu).
#pragma once

#include <cuda_runtime.h>

#include "pbr_kernels.cuh"

namespace pbr {

// Hard raster (pbr_hard.cu).  threads in {128, 256, 512}; plain selects the
// per-node variant that reads/writes the global depth/colour buffer.
cudaError_t hard_set_smem_limit(int threads, bool plain, bool winner, bool tex, int bytes);
cudaError_t hard_occupancy(int threads, bool plain, bool winner, bool tex, int smem_bytes, int* blocks_per_sm);
// the textured instantiation of the tile kernel (pbr_hard_tex.cu); null for an unsupported combination
const void* hard_tex_fn(int threads, bool plain, bool winner);
cudaError_t hard_launch(int threads, bool plain, bool winner, const SceneParams& P, const RasterArgs& A,
                        int grid, int smem_bytes, cudaStream_t stream);
// Scene-per-warp raster (pbr_small.cu); blocks of 1..small_max_warps() warps, small_warps() by default.
int small_warps();
int small_max_warps();
int small_smem_per_warp(const RasterArgs& A, int W, int H);  // -1: image has more than 64 bins
cudaError_t small_set_smem_limit(bool plain, bool winner, int shade, int bytes);  // shade 0 flat, 1 smooth, 2 textured
cudaError_t small_occupancy(bool plain, bool winner, int shade, int warps, int smem_bytes, int* blocks_per_sm);
cudaError_t small_launch(bool plain, bool winner, const SceneParams& P, const RasterArgs& A, int warps, int grid,
                         int smem_bytes, cudaStream_t stream);
// Soft coverage (pbr_soft.cu); threads in {128, 256}.
int soft_smem_bytes(const SoftArgs& a, int threads);
cudaError_t soft_set_smem_limit(int threads, bool backward, int bytes);
cudaError_t soft_launch(int threads, bool backward, const SceneParams& P, const SoftArgs& A, int grid, int smem_bytes,
                        cudaStream_t stream);
// Scene-per-warp soft coverage (pbr_soft_small.cu); blocks of soft_small_warps() warps.
int soft_small_warps();
int soft_small_smem_per_warp(const SoftArgs& a, int W, int H);
cudaError_t soft_small_set_smem_limit(bool backward, int bytes);
cudaError_t soft_small_launch(bool backward, const SceneParams& P, const SoftArgs& A, int grid, int smem_bytes,
                              cudaStream_t stream);
// Binned soft coverage for large scenes (pbr_soft_large.cu); soft_large_threads() threads per CTA.
int soft_large_threads();
int soft_large_smem_bytes(const SoftArgs& a);
long long soft_large_slab_float4(int cap, int nblocks);
cudaError_t soft_large_set_smem_limit(bool backward, int bytes);
cudaError_t soft_large_occupancy(bool backward, int smem_bytes, int* blocks_per_sm);
cudaError_t soft_large_launch(bool backward, const SceneParams& P, const SoftArgs& A, int grid, int smem_bytes,
                              cudaStream_t stream);
cudaError_t plain_clear_launch(const SceneParams& P, float* zbuf, uint32_t* cbuf, cudaStream_t stream);
cudaError_t plain_resolve_launch(const SceneParams& P, const float* zbuf, const uint32_t* cbuf, uint8_t* out,
                                 float* depth, cudaStream_t stream);
cudaError_t debug_transforms_launch(const NodeDesc& node, long long rows, float* out, cudaStream_t stream);

}  // namespace pbr
