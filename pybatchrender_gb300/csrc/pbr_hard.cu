// pbr_hard.cu -- hard rasteriser for sm_103a.
//
// One CTA processes one work item = (scene k, pixel region r), where a region
// is threads*16 consecutive pixels of the scene's W x H image (the whole image
// for 64x64 at 256 threads).  Per item the CTA runs the whole pipeline in
// shared memory, with no global scratch:
//
//   K1  instance stage: per instance M = [R(hpr)*s | t]
//       (renderer/shader_context.py:47-84, renderer/node.py:116-126), in
//       batches of up to icap instances; instances whose bounding sphere
//       projects outside the region are dropped, and for meshes with clusters
//       (groups of 32 triangles, pbr_mesh_set_clusters) so are the (instance,
//       cluster) pairs that face away from the eye or hold no pixel centre
//   K2  one source triangle per thread: its three vertices clip = VP[k] * M * v
//       (shaders/basic.vert:29-53; one per-instance VP * M for meshes of 128+
//       triangles), near-plane clip, GL viewport transform into the scene's own
//       image (basic.vert:45-52 + the atlas flip of
//       renderer/frame_grabber.py:105), back-face cull, bbox, and in dense
//       scenes an exact coverage-and-depth test against the pixels' current
//       keys; the kept triangles are counted in draw order (warp prefix sums +
//       per-warp totals, one barrier per round), which fixes their slots in a
//       shared-memory triangle list ("chunk"), wait in their warp's queue and
//       are set up 32 at a time: world normal(s), watertight FP32 edge
//       functions with the top-left rule, depth plane and flat shading
//       + warp-ballot binner: one __ballot_sync per (32 triangles, bin) builds
//       the per-bin triangle bit masks
//   K3  raster of the chunk, (bin, mask word) items spread over the warps: the
//       candidates' (triangle, pixel) pairs inside the bin are packed 32 per
//       pass (prefix sum of the clipped bbox areas), so tiny triangles cost a
//       few instructions each; every covered pixel does a 64-bit atomicMin of
//       (window depth, emit order + 1) into the region's key array in shared
//       memory -- strict-less depth, ties to the earlier drawn triangle, across
//       chunks; then each lane resolves the colours of its 16 pixels that the
//       chunk won (basic.frag:20-39) and, after the last chunk, writes each
//       channel with one 128-bit store straight into the [N,C,H,W] output (no
//       framebuffer, no readback, no rearrange copy).
//
// Scenes whose triangles overflow the chunk are processed chunk by chunk; the
// key array and the per-lane colours carry over between chunks.
#include <cstdio>

#include "pbr_hard.cuh"
#include "pbr_launch.h"

namespace pbr {

// ---------------------------------------------------------------------------
// plain-mode helpers

__global__ void plain_clear_kernel(long long total, float* zbuf, uint32_t* cbuf, uint32_t bg) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    zbuf[i] = 1.f;
    cbuf[i] = bg;
  }
}

__global__ void plain_resolve_kernel(int N, int C, int HW, const float* zbuf, const uint32_t* cbuf, uint8_t* out,
                                     float* depth) {
  const long long total = (long long)N * HW;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long k = i / HW, q = i - k * HW;
    const uint32_t c = cbuf[i];
    for (int ch = 0; ch < C; ++ch) out[(k * C + ch) * HW + q] = (uint8_t)((c >> (8 * ch)) & 0xffu);
    if (depth) depth[i] = zbuf[i];
  }
}

__global__ void debug_transforms_kernel(const NodeDesc nd, long long rows, float* out) {
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < rows;
       id += (long long)gridDim.x * blockDim.x) {
    float m[12];
    build_model(nd, id, m);
    for (int i = 0; i < 12; ++i) out[id * 16 + i] = m[i];
    out[id * 16 + 12] = 0.f;
    out[id * 16 + 13] = 0.f;
    out[id * 16 + 14] = 0.f;
    out[id * 16 + 15] = 1.f;
  }
}

// ---------------------------------------------------------------------------
// host launchers

template <int T, bool PL, bool WN>
static const void* hard_fn() {
  return reinterpret_cast<const void*>(&hard_kernel<T, PL, WN, false>);
}

static const void* pick_hard(int threads, bool plain, bool winner, bool tex) {
  if (tex) return hard_tex_fn(threads, plain, winner);
  if (plain) {
    if (winner) return nullptr;
    switch (threads) {
      case 128: return hard_fn<128, true, false>();
      case 256: return hard_fn<256, true, false>();
      case 512: return hard_fn<512, true, false>();
    }
    return nullptr;
  }
  switch (threads) {
    case 128: return winner ? hard_fn<128, false, true>() : hard_fn<128, false, false>();
    case 256: return winner ? hard_fn<256, false, true>() : hard_fn<256, false, false>();
    case 512: return winner ? hard_fn<512, false, true>() : hard_fn<512, false, false>();
  }
  return nullptr;
}

cudaError_t hard_set_smem_limit(int threads, bool plain, bool winner, bool tex, int bytes) {
  const void* f = pick_hard(threads, plain, winner, tex);
  if (!f) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

cudaError_t hard_occupancy(int threads, bool plain, bool winner, bool tex, int smem_bytes, int* blocks_per_sm) {
  const void* f = pick_hard(threads, plain, winner, tex);
  if (!f) return cudaErrorInvalidValue;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, threads, smem_bytes);
}

cudaError_t hard_launch(int threads, bool plain, bool winner, const SceneParams& P, const RasterArgs& A, int grid,
                        int smem_bytes, cudaStream_t stream) {
  const void* f = pick_hard(threads, plain, winner, A.tex_any != 0);
  if (!f) return cudaErrorInvalidValue;
  void* args[] = {const_cast<SceneParams*>(&P), const_cast<RasterArgs*>(&A)};
  return cudaLaunchKernel(f, dim3(grid), dim3(threads), args, (size_t)smem_bytes, stream);
}

cudaError_t plain_clear_launch(const SceneParams& P, float* zbuf, uint32_t* cbuf, cudaStream_t stream) {
  const long long total = (long long)P.N * P.W * P.H;
  const int grid = (int)min((total + 255) / 256, (long long)152 * 8);
  plain_clear_kernel<<<grid, 256, 0, stream>>>(total, zbuf, cbuf, P.bg_packed);
  return cudaGetLastError();
}

cudaError_t plain_resolve_launch(const SceneParams& P, const float* zbuf, const uint32_t* cbuf, uint8_t* out,
                                 float* depth, cudaStream_t stream) {
  const long long total = (long long)P.N * P.W * P.H;
  const int grid = (int)min((total + 255) / 256, (long long)152 * 8);
  plain_resolve_kernel<<<grid, 256, 0, stream>>>(P.N, P.C, P.W * P.H, zbuf, cbuf, out, depth);
  return cudaGetLastError();
}

cudaError_t debug_transforms_launch(const NodeDesc& node, long long rows, float* out, cudaStream_t stream) {
  const int grid = (int)min((rows + 255) / 256, (long long)152 * 4);
  debug_transforms_kernel<<<max(grid, 1), 256, 0, stream>>>(node, rows, out);
  return cudaGetLastError();
}

}  // namespace pbr
