// pbr_kernels.cuh -- device-side scene description shared by the raster kernels
// and the C ABI (pbr_capi.cu).
//
// Everything a launch needs travels by value in the kernel parameters
// (SceneParams + RasterArgs, < 4 KB), so a launch captured into a CUDA graph
// replays with the same buffer addresses and the caller updates the scene by
// writing those buffers in place.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pbr {

constexpr int kMaxNodes = 24;
constexpr int kMaxMeshes = 24;
constexpr int kPx = 16;  // pixels per thread: one 128-bit store per channel
constexpr int kMaxInstBatch = 256;               // instances per batch of the tile kernel (icap)
constexpr int kInstWords = kMaxInstBatch / 32;

enum : int { kModeHpr = 0, kModeRot = 1, kModeMat = 2 };

// Device error flags (RasterArgs::status / SoftArgs::status, OR-ed; read and cleared by pbr_device_status).
// The current kernels raise none of them: the planner rejects scenes whose winner ids would not fit in 31 bits
// before any launch, and the tile kernel sizes its rounds so that a chunk always holds what it places.  The
// values stay reserved for kernels that detect an error only on the device.
enum : int {
  kStatusIdOverflow = 1,   // a winner id did not fit in 31 bits
  kStatusCapacity = 2,     // a chunk could not hold what a round placed
};

constexpr int kClusterTris = 32;    // triangles per cluster (the last cluster of a mesh may hold fewer)
constexpr int kMaxClusterPairs = 2048;  // (instance, cluster) pairs the tile kernel compacts at a time
constexpr int kWarpQueue = 64;    // tile kernel: a warp's queue of kept triangles (drained at 32, one placement adds <= 32)
constexpr int kMvpMinTris = 128;  // tile kernel: meshes this large transform vertices with a per-instance VP * M

struct MeshDesc {
  const float* pos;    // [nv,3]
  const float* nrm;    // [nv,3]
  const int32_t* idx;  // [nt,3]
  const float* uv;     // [nv,2] texture coordinates, or null (all 0)
  int32_t nv, nt, smooth, pad;
  float4 bound;        // bounding sphere (centre, radius) in mesh coordinates; radius <= 0: unknown
  // clusters of kClusterTris consecutive triangles, two float4 each: bounding sphere (centre, radius) and the
  // cone of their face normals (unit axis, cosine of its half-angle; <= 0: no cone); null: none
  const float4* clusters;
  int32_t ncl, pad1, pad2, pad3;
};

struct NodeDesc {
  const int32_t* counts;  // [N] or null
  const float* pos;       // [B,3]
  const float* rot;       // [B,3] | [B,9] | [B,16]
  const float* scale;     // [B]
  const float* color;     // [B,4]
  float* gpos;            // soft-mode gradients, accumulated (may be null)
  float* grot;            // d/d(heading, pitch, roll)
  float* gscale;
  float* gcol;
  // texture (shaders/basic.frag:31-32): [tex_h, tex_w] RGBA8 texels, row 0 at
  // v = 0 (the bottom row of the image); null when the node is untextured
  const uint32_t* tex;
  int32_t mesh, ips, shared, mode;
  int32_t rank_base, tex_w, tex_h, pad0;
  // state binding: position component c (0..2) / HPR angle c (3..5) of buffer
  // row r is src[r * src_stride + src_col[c]] when src is set and src_col[c] >= 0
  const float* src;
  int64_t src_stride;
  int8_t src_col[8];
};

struct SceneParams {
  int32_t N, W, H, C;
  const float* vp;  // [N,16] row-major
  float amb[3];
  float lcol[3];
  float ldir[3];     // normalised direction towards the light
  float ldir_raw[3]; // as given (the soft backward differentiates through the normalisation)
  float strength;    // clamped to [0,1]
  float bg[4];
  uint32_t bg_packed;
  float znear, zfar, sigma, gamma;
  int32_t num_nodes, num_meshes, max_tris, cull;
  MeshDesc meshes[kMaxMeshes];
  NodeDesc nodes[kMaxNodes];
};

struct RasterArgs {
  uint8_t* out;       // [N,C,H,W]
  float* depth;       // [N,H,W] or null
  int32_t* winner;    // [N,H,W] or null
  float* zbuf;        // plain mode: [N*H*W]
  uint32_t* cbuf;     // plain mode: [N*H*W] packed RGBA8
  int32_t* work_counter;  // persistent scheduling
  int32_t* status;
  int32_t node_begin, node_end;
  int32_t bin_px, bins_x;
  int32_t tri_cap, vcap, icap;
  int32_t region_px, regions_per_scene, num_items;
  int32_t max_region_bins;
  int32_t persistent;
  int32_t smooth_any;  // per-pixel shading records S0..S3 (smooth meshes or textured nodes)
  int32_t tex_any;     // texture-coordinate records S4, S5 (textured nodes)
  int32_t multi_chunk;
  int32_t cl_any;      // some node's mesh has clusters: the tile kernel culls (instance, cluster) pairs
  int32_t win_test;    // tile kernel: pre-test small kept triangles against coverage and the keys (count_may_win)
  int32_t mvp_any;     // tile kernel: some node's mesh has kMvpMinTris+ triangles (instances cache VP * M too)
};

// Soft-coverage launch arguments (pbr_soft.cu).
struct SoftArgs {
  float* out;          // forward: [N,3,H,W] output; backward: the forward's output (read)
  float* stats;        // [6*N*H*W]: float4 [N*H*W] (max zs, softmax denominator, coverage code, Cfg - C_r x),
                       // then float2 [N*H*W] (Cfg - C_r y, z)
  const float* gout;   // backward: dL/dout [N,3,H,W]
  float* glight;       // backward: dL/d(normalised light direction) [3], accumulated
  int32_t* status;
  int32_t tri_cap, vcap, icap, iacc_cap;
  int32_t region_px, regions_per_scene, num_items;
  int32_t bin_px, bins_x, max_region_bins;
  int32_t backward;
  int32_t split;  // scene-per-warp soft kernel: warps per scene (each takes every split-th pixel block)
  float4* scratch;          // binned soft kernel: one slab per CTA (records, block masks, accumulators)
  int64_t scratch_stride;   // float4 per slab
};

struct SoftLayout {
  int rec[15];
  int masks, vcache, vidx, icache, state, tacc, iacc, misc, total;
};

// Shared-memory carve-up, identical on host (to size the launch) and device.
struct SmemLayout {
  int t0, t1, t2, t3, t4;  // float4 [tri_cap]: three edges, depth plane + x-box, meta
  int s0, s1, s2, s3;      // float4 [tri_cap]: smooth-shading attributes (if smooth_any)
  int s4, s5;              // float4 [tri_cap]: texture coordinates + node (if tex_any)
  int masks;               // uint32 [max_region_bins * tri_cap/32]
  int vcache;              // float4 [vcap*2]: clip position, world normal
  int icache;              // float4 [icap*4]: model matrix rows, colour
  int state;               // per-pixel depth / emit-order keys of the region [threads*kPx] (uint64)
  int misc;                // per-warp survivor counts (two rounds), VP, work item, instance compaction
  int pairs;               // kept (instance, cluster) pairs [kMaxClusterPairs] and the scene's eye (float4)
  int wq;                  // per-warp queues of kept triangles waiting to be written [threads/32][kWarpQueue] (int2)
  int total;
};

__host__ __device__ inline int align16(int b) { return (b + 15) & ~15; }

__host__ __device__ inline SmemLayout smem_layout(const RasterArgs& a, int threads, bool winner) {
  SmemLayout L;
  int off = 0;
  const int t4 = a.tri_cap * 16;
  L.t0 = off; off += align16(t4);
  L.t1 = off; off += align16(t4);
  L.t2 = off; off += align16(t4);
  L.t3 = off; off += align16(t4);
  L.t4 = off; off += align16(t4);
  if (a.smooth_any) {
    L.s0 = off; off += align16(t4);
    L.s1 = off; off += align16(t4);
    L.s2 = off; off += align16(t4);
    L.s3 = off; off += align16(t4);
  } else {
    L.s0 = L.s1 = L.s2 = L.s3 = 0;
  }
  if (a.tex_any) {
    L.s4 = off; off += align16(t4);
    L.s5 = off; off += align16(t4);
  } else {
    L.s4 = L.s5 = 0;
  }
  L.masks = off; off += align16(a.max_region_bins * (a.tri_cap / 32) * 4);
  L.vcache = off; off += align16(a.vcap * 32);
  L.icache = off; off += align16(a.icap * (a.mvp_any ? 128 : 64));
  L.state = off;  // depth / emit-order keys of the region's pixels, uint64 each
  off += align16(threads * kPx * 8);
  L.misc = off; off += align16((2 * (threads / 32) + 8) * 4 + 16 * 4 + 16 + (kInstWords + kMaxInstBatch) * 4);
  L.pairs = off; off += a.cl_any ? align16(kMaxClusterPairs * 4 + 16) : 0;  // kept pairs; eye position
  L.wq = off; off += align16((threads / 32) * kWarpQueue * 8);
  L.total = off;
  return L;
}

}  // namespace pbr
