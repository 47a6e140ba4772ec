// pbr_capi.cu -- implementation of include/pbr_capi.h.
//
// The context holds the host copy of the kernel parameters (SceneParams) and
// the launch configuration; every render call derives RasterArgs from it and
// enqueues kernels on the caller's stream.  The context owns only scratch: a
// work counter and status word for the persistent schedule, and the colour /
// depth buffer of the plain per-node path.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pbr_capi.h"
#include "pbr_launch.h"

using pbr::MeshDesc;
using pbr::NodeDesc;
using pbr::RasterArgs;
using pbr::SceneParams;

struct pbr_ctx {
  int device = 0;
  int sm_count = 1;
  int max_smem = 48 * 1024;
  int smem_per_sm = 0;       // shared memory of an SM, and what each resident block reserves of it
  int smem_reserved = 0;
  std::string err;
  SceneParams P;
  std::vector<bool> node_ready;
  bool cam_bound = false;
  // launch configuration
  int threads = 256;
  int bin_px = 16;
  int tri_cap_req = 0;
  int persistent = 0;
  int pretest = -1;  // tile kernel's coverage-and-depth pre-test: -1 by scene density, 0 off, 1 on
  int kernel = 0;  // 0 auto, 1 scene-per-warp, 2 tile (CTA per scene region), 3 binned (soft only)
  // scratch
  int32_t* d_counter = nullptr;
  int32_t* d_status = nullptr;
  float* d_zbuf = nullptr;
  uint32_t* d_cbuf = nullptr;
  // cudaFuncSetAttribute cache: [threads idx][plain][winner]
  int smem_set[3][2][2][2] = {};
  int small_smem_set[2][2][3] = {};
  int soft_small_smem_set[2] = {};
  int soft_large_smem_set[2] = {};
  float4* d_soft_scratch = nullptr;  // binned soft kernel slabs, grown on demand
  size_t soft_scratch_bytes = 0;
  int soft_smem_set[2][2] = {};
  int soft_threads = 256;
};

// One launch configuration (what the autotuner searches over).
struct LaunchCfg {
  int kernel;  // 1 scene-per-warp, 2 tile; 0 = pick
  int threads;
  int bin_px;
  int tri_cap;
  int persistent;
};

static thread_local std::string g_create_err;

static int set_err(pbr_ctx* ctx, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx) ctx->err = buf; else g_create_err = buf;
  return code;
}

static int cuda_err(pbr_ctx* ctx, cudaError_t e, const char* what) {
  return set_err(ctx, PBR_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

#define PBR_CHECK_CTX(ctx) \
  do { if (!(ctx)) { g_create_err = "null context"; return PBR_ERR_INVALID; } } while (0)

static int threads_index(int t) { return t == 128 ? 0 : (t == 256 ? 1 : 2); }

static uint32_t pack_bg(const float* c) {
  uint32_t v = 0;
  for (int i = 0; i < 4; ++i) {
    float x = std::min(std::max(c[i], 0.f), 1.f);
    uint32_t b = (uint32_t)std::floor(x * 255.f + 0.5f);
    v |= b << (8 * i);
  }
  return v;
}

// ---------------------------------------------------------------------------
// launch configuration

struct LaunchPlan {
  RasterArgs A;
  int smem = 0;
  int grid = 0;
  int kind = 2;     // 1 scene-per-warp, 2 tile
  int threads = 256;
};

static long long scene_source_tris(const pbr_ctx* ctx, int n0, int n1) {
  long long s = 0;
  for (int n = n0; n < n1; ++n) {
    const NodeDesc& nd = ctx->P.nodes[n];
    s += (long long)nd.ips * ctx->P.meshes[nd.mesh].nt;
  }
  return s;
}

static int plan_tile(pbr_ctx* ctx, int threads, int bin_px, int tri_cap_req, int persistent, bool plain,
                     bool winner, int n0, int n1, LaunchPlan* out) {
  const SceneParams& P = ctx->P;
  RasterArgs A;
  memset(&A, 0, sizeof(A));
  const int HW = P.W * P.H;
  A.node_begin = n0;
  A.node_end = n1;
  A.bin_px = bin_px;
  A.bins_x = (P.W + bin_px - 1) / bin_px;
  A.region_px = threads * pbr::kPx;
  A.regions_per_scene = (HW + A.region_px - 1) / A.region_px;
  A.num_items = P.N * A.regions_per_scene;
  int mrb = 1;
  for (int r = 0; r < A.regions_per_scene; ++r) {
    const int p0 = r * A.region_px, p1 = std::min(p0 + A.region_px, HW);
    const int rb = ((p1 - 1) / P.W) / bin_px - (p0 / P.W) / bin_px + 1;
    mrb = std::max(mrb, rb);
  }
  A.max_region_bins = mrb * A.bins_x;
  int max_nv = 1;
  long long max_inst_verts = 1;
  for (int n = n0; n < n1; ++n) {
    const NodeDesc& nd = P.nodes[n];
    const MeshDesc& me = P.meshes[nd.mesh];
    max_nv = std::max(max_nv, me.nv);
    max_inst_verts = std::max(max_inst_verts, (long long)nd.ips * me.nv);
    if (me.smooth) A.smooth_any = 1;
    if (nd.tex) A.smooth_any = A.tex_any = 1;  // textured triangles are shaded per pixel
  }
  // no vertex cache: each thread transforms its own triangle's vertices
  A.vcap = 0;
  for (int n = n0; n < n1; ++n)
    if (P.meshes[P.nodes[n].mesh].clusters) A.cl_any = 1;
  for (int n = n0; n < n1; ++n)
    if (P.meshes[P.nodes[n].mesh].nt >= pbr::kMvpMinTris) A.mvp_any = 1;
  int icap = 1;
  for (int n = n0; n < n1; ++n) icap = std::max(icap, P.nodes[n].ips);
  A.icap = std::min(icap, 256);
  const long long need = 2 * scene_source_tris(ctx, n0, n1);
  // the coverage-and-depth pre-test pays where scenes hold at least as many source triangles as pixels (many
  // small, overlapping triangles); in sparser scenes it costs more than it saves
  A.win_test = ctx->pretest >= 0 ? ctx->pretest : (need / 2 >= (long long)HW ? 1 : 0);
  int cap = tri_cap_req > 0 ? tri_cap_req : (int)std::min<long long>(std::max<long long>(need, 64), 1024);
  cap = std::max(64, (cap + 31) & ~31);
  A.persistent = persistent;
  A.out = nullptr;
  A.work_counter = ctx->d_counter;
  A.status = ctx->d_status;
  // shrink the chunk until the layout fits in shared memory
  for (;;) {
    A.tri_cap = cap;
    A.multi_chunk = need > cap ? 1 : 0;
    const pbr::SmemLayout L = pbr::smem_layout(A, threads, winner);
    if (L.total <= ctx->max_smem) {
      out->smem = L.total;
      break;
    }
    if (cap > 64) {
      cap = std::max(64, (cap / 2 + 31) & ~31);
      continue;
    }
    if (A.icap > 32) {
      A.icap = std::max(32, A.icap / 2);
      continue;
    }
    return set_err(ctx, PBR_ERR_CAPACITY,
                   "scene does not fit in shared memory (%d bytes needed, %d available); "
                   "reduce mesh size or threads", L.total, ctx->max_smem);
  }
  // A smaller instance batch (down to 64) when that lets more blocks share an SM: its shared memory is the
  // usual limit (register use allows 2 blocks of 256 threads).
  if (ctx->smem_per_sm > 0) {
    auto blocks = [&](int bytes) { return ctx->smem_per_sm / (bytes + ctx->smem_reserved); };
    int best_icap = A.icap, best_smem = out->smem;
    for (int ic = A.icap / 2; ic >= 64; ic /= 2) {
      RasterArgs B = A;
      B.icap = ic;
      const int bytes = pbr::smem_layout(B, threads, winner).total;
      if (blocks(bytes) > blocks(best_smem)) {
        best_icap = ic;
        best_smem = bytes;
      }
    }
    A.icap = best_icap;
    out->smem = best_smem;
  }
  // kernel attribute + occupancy
  int& cached = ctx->smem_set[threads_index(threads)][plain ? 1 : 0][winner ? 1 : 0][A.tex_any ? 1 : 0];
  if (out->smem > 48 * 1024 && out->smem > cached) {
    cudaError_t e = pbr::hard_set_smem_limit(threads, plain, winner, A.tex_any != 0, out->smem);
    if (e != cudaSuccess) return cuda_err(ctx, e, "cudaFuncSetAttribute");
    cached = out->smem;
  }
  if (persistent) {
    int bps = 0;
    cudaError_t e = pbr::hard_occupancy(threads, plain, winner, A.tex_any != 0, out->smem, &bps);
    if (e != cudaSuccess) return cuda_err(ctx, e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    out->grid = std::max(1, std::min(A.num_items, ctx->sm_count * std::max(1, bps)));
  } else {
    out->grid = A.num_items;
  }
  out->A = A;
  out->kind = 2;
  out->threads = threads;
  return PBR_OK;
}

// Scene-per-warp plan with blocks of `warps` warps; returns PBR_ERR_CAPACITY
// when the scene is not small or the block does not fit in shared memory.
static int plan_small(pbr_ctx* ctx, bool plain, bool winner, int n0, int n1, LaunchPlan* out,
                      int warps = pbr::small_warps()) {
  const SceneParams& P = ctx->P;
  if (P.W % 16 != 0) return set_err(ctx, PBR_ERR_CAPACITY, "scene-per-warp kernel needs width %% 16 == 0");
  const long long need = 2 * scene_source_tris(ctx, n0, n1);  // a near-plane clip can split a triangle in two
  if (need > 128) return set_err(ctx, PBR_ERR_CAPACITY, "scene too large for the scene-per-warp kernel");
  RasterArgs A;
  memset(&A, 0, sizeof(A));
  A.node_begin = n0;
  A.node_end = n1;
  A.tri_cap = std::max(16, (int)((need + 15) & ~15LL));
  long long insts = 0, verts = 0;
  for (int n = n0; n < n1; ++n) {
    const NodeDesc& nd = P.nodes[n];
    const MeshDesc& me = P.meshes[nd.mesh];
    insts += nd.ips;
    verts += (long long)nd.ips * me.nv;
    if (me.smooth) A.smooth_any = 1;
    if (nd.tex) A.smooth_any = A.tex_any = 1;  // textured triangles are shaded per pixel
  }
  if (insts > 32 || verts > 256)
    return set_err(ctx, PBR_ERR_CAPACITY, "scene too large for the scene-per-warp kernel");
  A.icap = std::max(1, (int)insts);
  A.vcap = std::max(1, (int)verts);
  A.num_items = P.N;
  A.status = ctx->d_status;
  const int per_warp = pbr::small_smem_per_warp(A, P.W, P.H);
  if (per_warp < 0) return set_err(ctx, PBR_ERR_CAPACITY, "image too large for the scene-per-warp kernel");
  const int smem = per_warp * warps;
  if (smem > ctx->max_smem) return set_err(ctx, PBR_ERR_CAPACITY, "scene-per-warp layout exceeds shared memory");
  const int shade = A.tex_any ? 2 : (A.smooth_any ? 1 : 0);
  int& cached = ctx->small_smem_set[plain ? 1 : 0][winner ? 1 : 0][shade];
  if (smem > 48 * 1024 && smem > cached) {
    cudaError_t e = pbr::small_set_smem_limit(plain, winner, shade, smem);
    if (e != cudaSuccess) return cuda_err(ctx, e, "cudaFuncSetAttribute");
    cached = smem;
  }
  out->A = A;
  out->smem = smem;
  out->grid = (P.N + warps - 1) / warps;
  out->kind = 1;
  out->threads = warps * 32;
  return PBR_OK;
}

// Warps per block of the scene-per-warp kernel for a launch configuration:
// its thread count when the configuration names that kernel, else the default.
static int small_warps_of(const LaunchCfg& c) {
  return (c.kernel == 1 && c.threads % 32 == 0 && c.threads / 32 <= pbr::small_max_warps()) ? c.threads / 32
                                                                                              : pbr::small_warps();
}

static int plan_any(pbr_ctx* ctx, const LaunchCfg& c, bool plain, bool winner, int n0, int n1, LaunchPlan* out) {
  if (c.kernel == 1) return plan_small(ctx, plain, winner, n0, n1, out, small_warps_of(c));
  if (c.kernel == 0) {
    if (plan_small(ctx, plain, winner, n0, n1, out) == PBR_OK) return PBR_OK;
    ctx->err.clear();
  }
  return plan_tile(ctx, c.threads, c.bin_px, c.tri_cap, c.persistent, plain, winner, n0, n1, out);
}

static cudaError_t launch_plan(pbr_ctx* ctx, const LaunchPlan& lp, bool plain, bool winner, cudaStream_t s) {
  if (lp.kind == 1) return pbr::small_launch(plain, winner, ctx->P, lp.A, lp.threads / 32, lp.grid, lp.smem, s);
  return pbr::hard_launch(lp.threads, plain, winner, ctx->P, lp.A, lp.grid, lp.smem, s);
}

static LaunchCfg ctx_cfg(const pbr_ctx* ctx) {
  return LaunchCfg{ctx->kernel, ctx->threads, ctx->bin_px, ctx->tri_cap_req, ctx->persistent};
}

static int check_ready(pbr_ctx* ctx, int n0, int n1) {
  if (!ctx->cam_bound) return set_err(ctx, PBR_ERR_STATE, "no camera bound (pbr_camera_bind)");
  for (int n = n0; n < n1; ++n)
    if (!ctx->node_ready[n]) return set_err(ctx, PBR_ERR_STATE, "node %d has no buffers bound", n);
  long long ranks = 0;
  for (int n = 0; n < ctx->P.num_nodes; ++n) ranks += ctx->P.nodes[n].ips;
  if (ranks * (long long)ctx->P.max_tris >= (1LL << 31))
    return set_err(ctx, PBR_ERR_CAPACITY, "instances per scene x triangles per mesh exceeds 2^31");
  return PBR_OK;
}

// ---------------------------------------------------------------------------
// C ABI

extern "C" {

int pbr_version(void) { return 100; }

const char* pbr_last_error(const pbr_ctx* ctx) {
  if (!ctx) return g_create_err.c_str();
  return ctx->err.c_str();
}

int pbr_create(pbr_ctx** out_ctx, int num_scenes, int width, int height, int channels, int flags) {
  if (!out_ctx) return set_err(nullptr, PBR_ERR_INVALID, "out_ctx is null");
  *out_ctx = nullptr;
  if (num_scenes <= 0 || width <= 0 || height <= 0)
    return set_err(nullptr, PBR_ERR_INVALID, "num_scenes, width and height must be positive (got %d, %d, %d)",
                   num_scenes, width, height);
  if (width > 65535 || height > 65535)
    return set_err(nullptr, PBR_ERR_INVALID, "width and height must be at most 65535");
  if ((long long)width * height > (1LL << 30) || (long long)num_scenes * width * height * 4 > (1LL << 62))
    return set_err(nullptr, PBR_ERR_INVALID, "image too large");
  if (channels < 1 || channels > 4) return set_err(nullptr, PBR_ERR_INVALID, "channels must be 1..4 (got %d)", channels);
  if (flags != 0) return set_err(nullptr, PBR_ERR_INVALID, "flags must be 0");
  pbr_ctx* ctx = new pbr_ctx();
  memset(&ctx->P, 0, sizeof(ctx->P));
  cudaError_t e = cudaGetDevice(&ctx->device);
  if (e != cudaSuccess) {
    delete ctx;
    return set_err(nullptr, PBR_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  }
  cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->device);
  cudaDeviceGetAttribute(&ctx->max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
  cudaDeviceGetAttribute(&ctx->smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device);
  cudaDeviceGetAttribute(&ctx->smem_reserved, cudaDevAttrReservedSharedMemoryPerBlock, ctx->device);
  ctx->P.N = num_scenes;
  ctx->P.W = width;
  ctx->P.H = height;
  ctx->P.C = channels;
  ctx->P.cull = 1;
  ctx->P.bg[3] = 1.f;
  ctx->P.bg_packed = pack_bg(ctx->P.bg);
  ctx->P.ldir[2] = 1.f;
  ctx->P.ldir_raw[2] = 1.f;
  ctx->P.znear = 0.05f;
  ctx->P.zfar = 100.f;
  ctx->P.sigma = 0.5f / (2.f * std::log(9.f));
  ctx->P.gamma = 1e-3f;
  ctx->P.max_tris = 1;
  e = cudaMalloc(&ctx->d_counter, 2 * sizeof(int32_t));
  if (e != cudaSuccess) {
    delete ctx;
    return set_err(nullptr, PBR_ERR_CUDA, "cudaMalloc: %s", cudaGetErrorString(e));
  }
  ctx->d_status = ctx->d_counter + 1;
  e = cudaMemset(ctx->d_counter, 0, 2 * sizeof(int32_t));
  if (e != cudaSuccess) {
    cudaFree(ctx->d_counter);
    delete ctx;
    return set_err(nullptr, PBR_ERR_CUDA, "cudaMemset: %s", cudaGetErrorString(e));
  }
  *out_ctx = ctx;
  return PBR_OK;
}

int pbr_destroy(pbr_ctx* ctx) {
  if (!ctx) return PBR_OK;
  cudaFree(ctx->d_counter);
  cudaFree(ctx->d_zbuf);
  cudaFree(ctx->d_cbuf);
  cudaFree(ctx->d_soft_scratch);
  delete ctx;
  return PBR_OK;
}

int pbr_mesh_register(pbr_ctx* ctx, const float* d_pos, const float* d_nrm, const int32_t* d_idx, int nv, int nt,
                      int smooth, int* out_mesh_id) {
  PBR_CHECK_CTX(ctx);
  if (!out_mesh_id) return set_err(ctx, PBR_ERR_INVALID, "out_mesh_id is null");
  if (ctx->P.num_meshes >= pbr::kMaxMeshes)
    return set_err(ctx, PBR_ERR_CAPACITY, "at most %d meshes per renderer", pbr::kMaxMeshes);
  if (nv <= 0 || nt < 0) return set_err(ctx, PBR_ERR_INVALID, "mesh needs nv > 0 and nt >= 0");
  if (!d_pos || !d_nrm || (nt > 0 && !d_idx)) return set_err(ctx, PBR_ERR_INVALID, "mesh pointers must be non-null");
  MeshDesc& m = ctx->P.meshes[ctx->P.num_meshes];
  m.pos = d_pos;
  m.nrm = d_nrm;
  m.idx = d_idx;
  m.nv = nv;
  m.nt = nt;
  m.smooth = smooth ? 1 : 0;
  ctx->P.max_tris = std::max(ctx->P.max_tris, nt);
  *out_mesh_id = ctx->P.num_meshes++;
  return PBR_OK;
}

int pbr_mesh_set_bounds(pbr_ctx* ctx, int mesh_id, float cx, float cy, float cz, float radius) {
  PBR_CHECK_CTX(ctx);
  if (mesh_id < 0 || mesh_id >= ctx->P.num_meshes) return set_err(ctx, PBR_ERR_INVALID, "unknown mesh id %d", mesh_id);
  if (!(radius >= 0.f) || !std::isfinite(cx) || !std::isfinite(cy) || !std::isfinite(cz) || !std::isfinite(radius))
    return set_err(ctx, PBR_ERR_INVALID, "mesh bounds must be finite with radius >= 0");
  ctx->P.meshes[mesh_id].bound = make_float4(cx, cy, cz, radius);
  return PBR_OK;
}

int pbr_mesh_set_clusters(pbr_ctx* ctx, int mesh_id, const float* d_clusters, int num_clusters,
                          int cluster_triangles) {
  PBR_CHECK_CTX(ctx);
  if (mesh_id < 0 || mesh_id >= ctx->P.num_meshes) return set_err(ctx, PBR_ERR_INVALID, "unknown mesh id %d", mesh_id);
  MeshDesc& m = ctx->P.meshes[mesh_id];
  if (!d_clusters) {
    m.clusters = nullptr;
    m.ncl = 0;
    return PBR_OK;
  }
  if (cluster_triangles != pbr::kClusterTris)
    return set_err(ctx, PBR_ERR_INVALID, "clusters must hold %d triangles (got %d)", pbr::kClusterTris,
                   cluster_triangles);
  const int need = (m.nt + pbr::kClusterTris - 1) / pbr::kClusterTris;
  if (num_clusters != need || need > 65535)
    return set_err(ctx, PBR_ERR_INVALID, "mesh %d needs %d clusters (at most 65535), got %d", mesh_id, need,
                   num_clusters);
  if (((uintptr_t)d_clusters & 15u) != 0) return set_err(ctx, PBR_ERR_INVALID, "d_clusters must be 16-byte aligned");
  m.clusters = reinterpret_cast<const float4*>(d_clusters);
  m.ncl = num_clusters;
  return PBR_OK;
}

int pbr_mesh_set_uv(pbr_ctx* ctx, int mesh_id, const float* d_uv) {
  PBR_CHECK_CTX(ctx);
  if (mesh_id < 0 || mesh_id >= ctx->P.num_meshes) return set_err(ctx, PBR_ERR_INVALID, "unknown mesh id %d", mesh_id);
  if (((uintptr_t)d_uv & 7u) != 0) return set_err(ctx, PBR_ERR_INVALID, "d_uv must be 8-byte aligned");
  ctx->P.meshes[mesh_id].uv = d_uv;
  return PBR_OK;
}

int pbr_node_set_texture(pbr_ctx* ctx, int node_id, const uint8_t* d_rgba, int width, int height) {
  PBR_CHECK_CTX(ctx);
  if (node_id < 0 || node_id >= ctx->P.num_nodes) return set_err(ctx, PBR_ERR_INVALID, "unknown node id %d", node_id);
  NodeDesc& nd = ctx->P.nodes[node_id];
  if (!d_rgba) {
    nd.tex = nullptr;
    nd.tex_w = nd.tex_h = 0;
    return PBR_OK;
  }
  if (width <= 0 || height <= 0 || width > 16384 || height > 16384)
    return set_err(ctx, PBR_ERR_INVALID, "texture size must be 1..16384 in each dimension (got %d x %d)", width, height);
  if (((uintptr_t)d_rgba & 3u) != 0) return set_err(ctx, PBR_ERR_INVALID, "d_rgba must be 4-byte aligned");
  nd.tex = reinterpret_cast<const uint32_t*>(d_rgba);
  nd.tex_w = width;
  nd.tex_h = height;
  return PBR_OK;
}

int pbr_node_add(pbr_ctx* ctx, int mesh_id, int instances_per_scene, int shared, int* out_node_id) {
  PBR_CHECK_CTX(ctx);
  if (!out_node_id) return set_err(ctx, PBR_ERR_INVALID, "out_node_id is null");
  if (ctx->P.num_nodes >= pbr::kMaxNodes)
    return set_err(ctx, PBR_ERR_CAPACITY, "at most %d nodes per renderer", pbr::kMaxNodes);
  if (mesh_id < 0 || mesh_id >= ctx->P.num_meshes) return set_err(ctx, PBR_ERR_INVALID, "unknown mesh id %d", mesh_id);
  if (instances_per_scene < 0) return set_err(ctx, PBR_ERR_INVALID, "instances_per_scene must be >= 0");
  const int n = ctx->P.num_nodes;
  NodeDesc& nd = ctx->P.nodes[n];
  memset(&nd, 0, sizeof(nd));
  nd.mesh = mesh_id;
  nd.ips = instances_per_scene;
  nd.shared = shared ? 1 : 0;
  nd.mode = pbr::kModeHpr;
  for (int c = 0; c < 8; ++c) nd.src_col[c] = -1;
  int rank = 0;
  for (int i = 0; i < n; ++i) rank += ctx->P.nodes[i].ips;
  nd.rank_base = rank;
  ctx->P.num_nodes++;
  ctx->node_ready.push_back(false);
  *out_node_id = n;
  return PBR_OK;
}

int pbr_node_set_buffers(pbr_ctx* ctx, int node_id, int mode, const float* d_pos, const float* d_rot,
                         const float* d_scale, const float* d_color, const int32_t* d_counts) {
  PBR_CHECK_CTX(ctx);
  if (node_id < 0 || node_id >= ctx->P.num_nodes) return set_err(ctx, PBR_ERR_INVALID, "unknown node id %d", node_id);
  if (mode != pbr::kModeHpr && mode != pbr::kModeRot && mode != pbr::kModeMat)
    return set_err(ctx, PBR_ERR_INVALID, "unknown rotation mode %d", mode);
  if (!d_rot || !d_color) return set_err(ctx, PBR_ERR_INVALID, "rotation and colour buffers must be non-null");
  if (mode != pbr::kModeMat && (!d_pos || !d_scale))
    return set_err(ctx, PBR_ERR_INVALID, "position and scale buffers must be non-null");
  if (((uintptr_t)d_color & 15u) != 0) return set_err(ctx, PBR_ERR_INVALID, "d_color must be 16-byte aligned");
  NodeDesc& nd = ctx->P.nodes[node_id];
  nd.mode = mode;
  nd.pos = d_pos;
  nd.rot = d_rot;
  nd.scale = d_scale;
  nd.color = d_color;
  nd.counts = d_counts;
  ctx->node_ready[node_id] = true;
  return PBR_OK;
}

int pbr_node_bind_state(pbr_ctx* ctx, int node_id, int component, int column) {
  PBR_CHECK_CTX(ctx);
  if (node_id < 0 || node_id >= ctx->P.num_nodes) return set_err(ctx, PBR_ERR_INVALID, "unknown node id %d", node_id);
  if (component < 0 || component > 5)
    return set_err(ctx, PBR_ERR_INVALID, "component must be 0..2 (position) or 3..5 (heading, pitch, roll)");
  if (column > 127) return set_err(ctx, PBR_ERR_INVALID, "state column must be < 128");
  ctx->P.nodes[node_id].src_col[component] = (int8_t)(column < 0 ? -1 : column);
  return PBR_OK;
}

int pbr_state_source(pbr_ctx* ctx, const float* d_state, long long rows, int cols, long long row_stride) {
  PBR_CHECK_CTX(ctx);
  SceneParams& P = ctx->P;
  if (d_state) {
    if (rows < 0 || cols < 0 || row_stride < cols)
      return set_err(ctx, PBR_ERR_INVALID, "state matrix needs rows >= 0 and row_stride >= cols >= 0");
    for (int n = 0; n < P.num_nodes; ++n) {
      const NodeDesc& nd = P.nodes[n];
      const long long need = nd.shared ? (long long)nd.ips : (long long)nd.ips * P.N;
      for (int c = 0; c < 6; ++c) {
        if (nd.src_col[c] < 0) continue;
        if (nd.src_col[c] >= cols)
          return set_err(ctx, PBR_ERR_INVALID, "node %d binds column %d of a %d-column state", n, nd.src_col[c], cols);
        if (need > rows)
          return set_err(ctx, PBR_ERR_INVALID, "node %d needs %lld state rows, got %lld", n, need, rows);
        if (c >= 3 && nd.mode != pbr::kModeHpr)
          return set_err(ctx, PBR_ERR_STATE, "node %d binds an angle but is not in HPR mode", n);
      }
    }
  }
  for (int n = 0; n < P.num_nodes; ++n) {
    NodeDesc& nd = P.nodes[n];
    bool any = false;
    for (int c = 0; c < 6; ++c) any = any || nd.src_col[c] >= 0;
    nd.src = (d_state && any) ? d_state : nullptr;
    nd.src_stride = row_stride;
  }
  return PBR_OK;
}

int pbr_camera_bind(pbr_ctx* ctx, const float* d_vp, float z_near, float z_far) {
  PBR_CHECK_CTX(ctx);
  if (!d_vp) return set_err(ctx, PBR_ERR_INVALID, "d_vp is null");
  if (!(z_far > z_near)) return set_err(ctx, PBR_ERR_INVALID, "z_far must be greater than z_near");
  ctx->P.vp = d_vp;
  ctx->P.znear = z_near;
  ctx->P.zfar = z_far;
  ctx->cam_bound = true;
  return PBR_OK;
}

int pbr_light_set(pbr_ctx* ctx, const float ambient[3], const float direction[3], const float color[3],
                  float strength) {
  PBR_CHECK_CTX(ctx);
  if (!ambient || !direction || !color) return set_err(ctx, PBR_ERR_INVALID, "light arrays must be non-null");
  const double l = std::sqrt((double)direction[0] * direction[0] + (double)direction[1] * direction[1] +
                             (double)direction[2] * direction[2]);
  for (int i = 0; i < 3; ++i) {
    ctx->P.amb[i] = ambient[i];
    ctx->P.lcol[i] = color[i];
    ctx->P.ldir_raw[i] = direction[i];
    ctx->P.ldir[i] = l > 0 ? (float)(direction[i] / l) : 0.f;
  }
  ctx->P.strength = std::min(std::max(strength, 0.f), 1.f);
  return PBR_OK;
}

int pbr_background_set(pbr_ctx* ctx, const float rgba[4]) {
  PBR_CHECK_CTX(ctx);
  if (!rgba) return set_err(ctx, PBR_ERR_INVALID, "rgba is null");
  for (int i = 0; i < 4; ++i) ctx->P.bg[i] = rgba[i];
  ctx->P.bg_packed = pack_bg(ctx->P.bg);
  return PBR_OK;
}

int pbr_raster_config(pbr_ctx* ctx, int kernel, int threads, int bin_px, int tri_cap, int persistent) {
  PBR_CHECK_CTX(ctx);
  if (kernel < 0 || kernel > 3)
    return set_err(ctx, PBR_ERR_INVALID, "kernel must be 0 (auto), 1, 2 or 3 (got %d)", kernel);
  // the tile kernel has 128-, 256- and 512-thread instantiations; the scene-per-warp kernel (kernel 1)
  // also takes blocks of 7 or 14 warps
  const bool small_only = kernel == 1 && (threads == 224 || threads == 448);
  if (threads != 128 && threads != 256 && threads != 512 && !small_only)
    return set_err(ctx, PBR_ERR_INVALID, "threads must be 128, 256 or 512, or 224 or 448 with kernel 1 (got %d)",
                   threads);
  if (bin_px != 8 && bin_px != 16 && bin_px != 32)
    return set_err(ctx, PBR_ERR_INVALID, "bin_px must be 8, 16 or 32 (got %d)", bin_px);
  if (tri_cap != 0 && (tri_cap < 64 || tri_cap > 4096 || (tri_cap % 32) != 0))
    return set_err(ctx, PBR_ERR_INVALID, "tri_cap must be 0 or a multiple of 32 in [64, 4096]");
  ctx->threads = threads;
  ctx->bin_px = bin_px;
  ctx->tri_cap_req = tri_cap;
  ctx->persistent = persistent ? 1 : 0;
  ctx->kernel = kernel;
  return PBR_OK;
}

int pbr_tile_pretest(pbr_ctx* ctx, int mode) {
  PBR_CHECK_CTX(ctx);
  if (mode < -1 || mode > 1) return set_err(ctx, PBR_ERR_INVALID, "mode must be -1 (by density), 0 or 1 (got %d)", mode);
  ctx->pretest = mode;
  return PBR_OK;
}

static int render_with(pbr_ctx* ctx, const LaunchCfg& cfg, uint8_t* d_out, float* d_depth, int32_t* d_winner,
                       cudaStream_t s) {
  LaunchPlan lp;
  const bool winner = d_winner != nullptr;
  int rc = plan_any(ctx, cfg, false, winner, 0, ctx->P.num_nodes, &lp);
  if (rc) return rc;
  lp.A.out = d_out;
  lp.A.depth = d_depth;
  lp.A.winner = d_winner;
  if (lp.kind == 2 && lp.A.persistent) {
    cudaError_t e = cudaMemsetAsync(ctx->d_counter, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) return cuda_err(ctx, e, "cudaMemsetAsync");
  }
  cudaError_t e = launch_plan(ctx, lp, false, winner, s);
  if (e != cudaSuccess) return cuda_err(ctx, e, "raster launch");
  return PBR_OK;
}

static bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

int pbr_render(pbr_ctx* ctx, uint8_t* d_out, float* d_depth, int32_t* d_winner, void* stream) {
  PBR_CHECK_CTX(ctx);
  if (!d_out) return set_err(ctx, PBR_ERR_INVALID, "d_out is null");
  if (!aligned16(d_out) || !aligned16(d_depth) || !aligned16(d_winner))
    return set_err(ctx, PBR_ERR_INVALID, "output buffers must be 16-byte aligned");
  int rc = check_ready(ctx, 0, ctx->P.num_nodes);
  if (rc) return rc;
  return render_with(ctx, ctx_cfg(ctx), d_out, d_depth, d_winner, (cudaStream_t)stream);
}

int pbr_render_state(pbr_ctx* ctx, const float* d_state, long long rows, int cols, long long row_stride,
                     uint8_t* d_out, float* d_depth, int32_t* d_winner, void* stream) {
  PBR_CHECK_CTX(ctx);
  if (!d_state) return set_err(ctx, PBR_ERR_INVALID, "d_state is null");
  int rc = pbr_state_source(ctx, d_state, rows, cols, row_stride);
  if (rc) return rc;
  rc = pbr_render(ctx, d_out, d_depth, d_winner, stream);
  pbr_state_source(ctx, nullptr, 0, 0, 0);  // the launch has its copy of the parameters
  return rc;
}

int pbr_autotune(pbr_ctx* ctx, uint8_t* d_out, void* stream, int* out_kernel, int* out_threads, int* out_bin_px,
                 int* out_tri_cap, int* out_persistent, float* out_ms) {
  PBR_CHECK_CTX(ctx);
  if (!d_out) return set_err(ctx, PBR_ERR_INVALID, "d_out is null");
  int rc = check_ready(ctx, 0, ctx->P.num_nodes);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  std::vector<LaunchCfg> cands;
  {
    LaunchPlan probe;
    for (int w : {4, 7, 14}) {  // blocks of 4, 7 or 14 warps, where they fit in shared memory
      if (plan_small(ctx, false, false, 0, ctx->P.num_nodes, &probe, w) == PBR_OK) cands.push_back({1, w * 32, 16, 0, 0});
      ctx->err.clear();
    }
    const long long need = 2 * scene_source_tris(ctx, 0, ctx->P.num_nodes);
    std::vector<int> caps = {0};
    if (need > 256) { caps.push_back(256); caps.push_back(384); caps.push_back(512); }
    for (int t : {128, 256, 512})
      for (int b : {8, 16, 32})
        for (int p : {0, 1})
          for (int cap : caps) cands.push_back({2, t, b, cap, p});
  }
  float best = 1e30f;
  LaunchCfg bestc = ctx_cfg(ctx);
  int status = PBR_OK;
  for (const LaunchCfg& c : cands) {
    int r = render_with(ctx, c, d_out, nullptr, nullptr, s);  // warm-up
    if (r == PBR_ERR_CAPACITY) { ctx->err.clear(); continue; }
    if (r) { status = r; break; }
    cudaEventRecord(e0, s);
    for (int rep = 0; rep < 3; ++rep) render_with(ctx, c, d_out, nullptr, nullptr, s);
    cudaEventRecord(e1, s);
    cudaError_t ce = cudaEventSynchronize(e1);
    if (ce != cudaSuccess) { status = cuda_err(ctx, ce, "autotune"); break; }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= 3.f;
    if (ms < best) { best = ms; bestc = c; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (status) return status;
  ctx->kernel = bestc.kernel;
  ctx->threads = bestc.threads;
  ctx->bin_px = bestc.bin_px;
  ctx->persistent = bestc.persistent;
  ctx->tri_cap_req = bestc.tri_cap;
  if (out_kernel) *out_kernel = bestc.kernel;
  if (out_threads) *out_threads = bestc.threads;
  if (out_bin_px) *out_bin_px = bestc.bin_px;
  if (out_tri_cap) *out_tri_cap = bestc.tri_cap;
  if (out_persistent) *out_persistent = bestc.persistent;
  if (out_ms) *out_ms = best;
  return PBR_OK;
}

static int ensure_plain_buffers(pbr_ctx* ctx) {
  if (ctx->d_zbuf) return PBR_OK;
  const size_t n = (size_t)ctx->P.N * ctx->P.W * ctx->P.H;
  cudaError_t e = cudaMalloc(&ctx->d_zbuf, n * sizeof(float));
  if (e != cudaSuccess) return cuda_err(ctx, e, "cudaMalloc (plain depth buffer)");
  e = cudaMalloc(&ctx->d_cbuf, n * sizeof(uint32_t));
  if (e != cudaSuccess) {
    cudaFree(ctx->d_zbuf);
    ctx->d_zbuf = nullptr;
    return cuda_err(ctx, e, "cudaMalloc (plain colour buffer)");
  }
  return PBR_OK;
}

int pbr_plain_clear(pbr_ctx* ctx, void* stream) {
  PBR_CHECK_CTX(ctx);
  int rc = ensure_plain_buffers(ctx);
  if (rc) return rc;
  cudaError_t e = pbr::plain_clear_launch(ctx->P, ctx->d_zbuf, ctx->d_cbuf, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_err(ctx, e, "plain clear launch");
  return PBR_OK;
}

int pbr_plain_draw(pbr_ctx* ctx, int node_id, void* stream) {
  PBR_CHECK_CTX(ctx);
  if (node_id < 0 || node_id >= ctx->P.num_nodes) return set_err(ctx, PBR_ERR_INVALID, "unknown node id %d", node_id);
  if (!ctx->d_zbuf) return set_err(ctx, PBR_ERR_STATE, "pbr_plain_clear must run first");
  int rc = check_ready(ctx, node_id, node_id + 1);
  if (rc) return rc;
  LaunchPlan lp;
  LaunchCfg c = ctx_cfg(ctx);
  c.persistent = 0;
  rc = plan_any(ctx, c, true, false, node_id, node_id + 1, &lp);
  if (rc) return rc;
  lp.A.zbuf = ctx->d_zbuf;
  lp.A.cbuf = ctx->d_cbuf;
  cudaError_t e = launch_plan(ctx, lp, true, false, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_err(ctx, e, "plain draw launch");
  return PBR_OK;
}

int pbr_plain_resolve(pbr_ctx* ctx, uint8_t* d_out, float* d_depth, void* stream) {
  PBR_CHECK_CTX(ctx);
  if (!d_out) return set_err(ctx, PBR_ERR_INVALID, "d_out is null");
  if (!ctx->d_zbuf) return set_err(ctx, PBR_ERR_STATE, "pbr_plain_clear must run first");
  cudaError_t e = pbr::plain_resolve_launch(ctx->P, ctx->d_zbuf, ctx->d_cbuf, d_out, d_depth, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_err(ctx, e, "plain resolve launch");
  return PBR_OK;
}

// ---------------------------------------------------------------------------
// soft coverage

static int plan_soft(pbr_ctx* ctx, int threads, bool backward, pbr::SoftArgs* out, int* smem_out, int* grid_out) {
  const SceneParams& P = ctx->P;
  pbr::SoftArgs A;
  memset(&A, 0, sizeof(A));
  const int HW = P.W * P.H;
  const int bin_px = ctx->bin_px;
  A.backward = backward ? 1 : 0;
  A.region_px = threads * 8;
  A.regions_per_scene = (HW + A.region_px - 1) / A.region_px;
  A.num_items = P.N * A.regions_per_scene;
  A.bin_px = bin_px;
  A.bins_x = (P.W + bin_px - 1) / bin_px;
  int mrb = 1;
  for (int r = 0; r < A.regions_per_scene; ++r) {
    const int p0 = r * A.region_px, p1 = std::min(p0 + A.region_px, HW);
    mrb = std::max(mrb, ((p1 - 1) / P.W) / bin_px - (p0 / P.W) / bin_px + 1);
  }
  A.max_region_bins = mrb * A.bins_x;
  int max_nv = 1;
  long long max_inst_verts = 1, tris = 0, insts = 0;
  for (int n = 0; n < P.num_nodes; ++n) {
    const NodeDesc& nd = P.nodes[n];
    const MeshDesc& me = P.meshes[nd.mesh];
    max_nv = std::max(max_nv, me.nv);
    max_inst_verts = std::max(max_inst_verts, (long long)nd.ips * me.nv);
    tris += (long long)nd.ips * me.nt;
    insts += nd.ips;
  }
  if (backward && insts > 1024)
    return set_err(ctx, PBR_ERR_CAPACITY, "soft backward supports at most 1024 instances per scene (got %lld)", insts);
  A.iacc_cap = backward ? (int)std::max<long long>(insts, 1) : 0;
  A.vcap = (std::max(max_nv, (int)std::min<long long>(max_inst_verts, 512)) + 31) & ~31;
  int icap = 1;
  for (int n = 0; n < P.num_nodes; ++n) {
    const NodeDesc& nd = P.nodes[n];
    icap = std::max(icap, std::min(nd.ips, A.vcap / std::max(1, P.meshes[nd.mesh].nv)));
  }
  A.icap = std::min(icap, 128);
  int cap = (int)std::min<long long>(std::max<long long>((tris + 31) & ~31LL, 32), 512);
  A.status = ctx->d_status;
  for (;;) {
    A.tri_cap = cap;
    const int bytes = pbr::soft_smem_bytes(A, threads);
    if (bytes <= ctx->max_smem) {
      *smem_out = bytes;
      break;
    }
    if (cap > 32) {
      cap = std::max(32, (cap / 2 + 31) & ~31);
      continue;
    }
    if (A.vcap > max_nv) {
      A.vcap = std::max((max_nv + 31) & ~31, A.vcap / 2);
      A.icap = std::max(1, std::min(A.icap, A.vcap / max_nv));
      continue;
    }
    return set_err(ctx, PBR_ERR_CAPACITY, "soft scene does not fit in shared memory (%d bytes needed)", bytes);
  }
  int& cached = ctx->soft_smem_set[threads == 256 ? 1 : 0][backward ? 1 : 0];
  if (*smem_out > 48 * 1024 && *smem_out > cached) {
    cudaError_t e = pbr::soft_set_smem_limit(threads, backward, *smem_out);
    if (e != cudaSuccess) return cuda_err(ctx, e, "cudaFuncSetAttribute");
    cached = *smem_out;
  }
  *grid_out = A.num_items;
  *out = A;
  return PBR_OK;
}

// Scene-per-warp soft plan, used for both passes so that the forward and the
// adjoint always agree on the kernel (the warp forward writes statistics only
// where the adjoint reads them).  Sized by the adjoint's layout.
static int plan_soft_small(pbr_ctx* ctx, bool backward, pbr::SoftArgs* out, int* smem_out, int* grid_out) {
  const SceneParams& P = ctx->P;
  long long tris = 0, insts = 0, verts = 0;
  for (int n = 0; n < P.num_nodes; ++n) {
    const NodeDesc& nd = P.nodes[n];
    const MeshDesc& me = P.meshes[nd.mesh];
    tris += (long long)nd.ips * me.nt;
    insts += nd.ips;
    verts += (long long)nd.ips * me.nv;
  }
  if (tris > 128 || insts > 32 || verts > 256)
    return set_err(ctx, PBR_ERR_CAPACITY, "scene too large for the scene-per-warp soft kernel");
  if ((P.W * P.H) % 4 != 0)  // the background is written with float4 stores per plane
    return set_err(ctx, PBR_ERR_CAPACITY, "scene-per-warp soft kernel needs W*H %% 4 == 0");
  pbr::SoftArgs A;
  memset(&A, 0, sizeof(A));
  A.tri_cap = std::max(16, (int)((tris + 15) & ~15LL));
  A.vcap = std::max(1, (int)verts);
  A.icap = std::max(1, (int)insts);
  A.iacc_cap = A.icap;
  A.num_items = P.N;
  A.status = ctx->d_status;
  A.backward = 1;
  const int warps = pbr::soft_small_warps();
  const int smem_bwd = pbr::soft_small_smem_per_warp(A, P.W, P.H) * warps;
  if (smem_bwd > ctx->max_smem)
    return set_err(ctx, PBR_ERR_CAPACITY, "scene-per-warp soft layout exceeds shared memory");
  A.backward = backward ? 1 : 0;
  // few scenes: several warps per scene (each takes every split-th pixel block) so that ~16 warps per SM work
  const long long want = (long long)ctx->sm_count * 16;
  A.split = (int)std::min<long long>(4, std::max<long long>(1, (want + P.N - 1) / std::max(1, P.N)));
  const int smem = pbr::soft_small_smem_per_warp(A, P.W, P.H) * warps;
  int& cached = ctx->soft_small_smem_set[backward ? 1 : 0];
  if (smem > 48 * 1024 && smem > cached) {
    cudaError_t e = pbr::soft_small_set_smem_limit(backward, smem);
    if (e != cudaSuccess) return cuda_err(ctx, e, "cudaFuncSetAttribute");
    cached = smem;
  }
  *out = A;
  *smem_out = smem;
  *grid_out = (int)(((long long)P.N * A.split + warps - 1) / warps);
  return PBR_OK;
}

// Binned soft plan (both passes): persistent CTAs, one slab of scratch each,
// sized for the scene's source triangles.  Allocates the slabs on first use
// (and when a larger scene needs more).
static int plan_soft_large(pbr_ctx* ctx, bool backward, pbr::SoftArgs* out, int* smem_out, int* grid_out) {
  const SceneParams& P = ctx->P;
  long long tris = 0, insts = 0;
  int max_ips = 1;
  for (int n = 0; n < P.num_nodes; ++n) {
    const NodeDesc& nd = P.nodes[n];
    tris += (long long)nd.ips * P.meshes[nd.mesh].nt;
    insts += nd.ips;
    max_ips = std::max(max_ips, nd.ips);
  }
  if (tris > (1 << 22)) return set_err(ctx, PBR_ERR_CAPACITY, "binned soft kernel: at most 4M triangles per scene");
  if (insts > 1024)
    return set_err(ctx, PBR_ERR_CAPACITY, "soft mode supports at most 1024 instances per scene (got %lld)", insts);
  pbr::SoftArgs A;
  memset(&A, 0, sizeof(A));
  A.tri_cap = (int)std::max<long long>(32, (tris + 31) & ~31LL);
  A.icap = std::min(max_ips, 256);
  A.iacc_cap = (int)std::max<long long>(1, insts);
  A.backward = backward ? 1 : 0;
  A.num_items = P.N;
  A.status = ctx->d_status;
  const int smem = pbr::soft_large_smem_bytes(A);
  // both passes share the slabs (one per CTA): size them for the larger grid of the two
  int grid = 1, grid_max = 1;
  for (int pass = 0; pass < 2; ++pass) {
    pbr::SoftArgs Ap = A;
    Ap.backward = pass;
    const int smem_p = pbr::soft_large_smem_bytes(Ap);
    if (smem_p > ctx->max_smem) return set_err(ctx, PBR_ERR_CAPACITY, "binned soft layout exceeds shared memory");
    int& cached = ctx->soft_large_smem_set[pass];
    if (smem_p > 48 * 1024 && smem_p > cached) {
      cudaError_t ea = pbr::soft_large_set_smem_limit(pass == 1, smem_p);
      if (ea != cudaSuccess) return cuda_err(ctx, ea, "cudaFuncSetAttribute");
      cached = smem_p;
    }
    int bps = 1;
    cudaError_t e = pbr::soft_large_occupancy(pass == 1, smem_p, &bps);
    if (e != cudaSuccess) return cuda_err(ctx, e, "occupancy");
    const int g = std::max(1, std::min(P.N, ctx->sm_count * std::max(1, bps)));
    grid_max = std::max(grid_max, g);
    if ((pass == 1) == backward) grid = g;
  }
  const int nblocks = ((P.W + 7) / 8) * ((P.H + 3) / 4);
  const long long slab = pbr::soft_large_slab_float4(A.tri_cap, nblocks);
  const size_t need = (size_t)slab * 16 * (size_t)grid_max;
  cudaError_t e;
  if (need > ctx->soft_scratch_bytes) {
    if (ctx->d_soft_scratch) cudaFree(ctx->d_soft_scratch);
    ctx->d_soft_scratch = nullptr;
    ctx->soft_scratch_bytes = 0;
    e = cudaMalloc(&ctx->d_soft_scratch, need);
    if (e != cudaSuccess) return cuda_err(ctx, e, "cudaMalloc (binned soft scratch)");
    ctx->soft_scratch_bytes = need;
  }
  A.scratch = ctx->d_soft_scratch;
  A.scratch_stride = slab;
  *out = A;
  *smem_out = smem;
  *grid_out = grid;
  return PBR_OK;
}

// Soft kernel choice, identical for both passes: 1 = scene per warp, 2 = tile, 3 = binned.
static int soft_kind(pbr_ctx* ctx) {
  if (ctx->kernel == 2) return 2;
  if (ctx->kernel == 3) return 3;
  pbr::SoftArgs A;
  int smem = 0, grid = 0;
  if (plan_soft_small(ctx, true, &A, &smem, &grid) == PBR_OK) return 1;
  if (ctx->kernel == 1) return -1;
  ctx->err.clear();
  return 3;
}

int pbr_soft_config(pbr_ctx* ctx, float sigma, float gamma, int threads) {
  PBR_CHECK_CTX(ctx);
  if (!(sigma > 0.f) || !(gamma > 0.f)) return set_err(ctx, PBR_ERR_INVALID, "sigma and gamma must be positive");
  if (threads != 128 && threads != 256) return set_err(ctx, PBR_ERR_INVALID, "soft threads must be 128 or 256");
  ctx->P.sigma = sigma;
  ctx->P.gamma = gamma;
  ctx->soft_threads = threads;
  return PBR_OK;
}

int pbr_node_set_grads(pbr_ctx* ctx, int node_id, float* d_gpos, float* d_ghpr, float* d_gscale, float* d_gcol) {
  PBR_CHECK_CTX(ctx);
  if (node_id < 0 || node_id >= ctx->P.num_nodes) return set_err(ctx, PBR_ERR_INVALID, "unknown node id %d", node_id);
  NodeDesc& nd = ctx->P.nodes[node_id];
  nd.gpos = d_gpos;
  nd.grot = d_ghpr;
  nd.gscale = d_gscale;
  nd.gcol = d_gcol;
  return PBR_OK;
}

static int reject_textures(pbr_ctx* ctx) {
  for (int n = 0; n < ctx->P.num_nodes; ++n)
    if (ctx->P.nodes[n].tex)
      return set_err(ctx, PBR_ERR_INVALID, "node %d is textured: the soft mode draws untextured nodes only", n);
  return PBR_OK;
}

int pbr_render_soft(pbr_ctx* ctx, float* d_out, float* d_stats, void* stream) {
  PBR_CHECK_CTX(ctx);
  if (!d_out) return set_err(ctx, PBR_ERR_INVALID, "d_out is null");
  if (reject_textures(ctx)) return PBR_ERR_INVALID;
  if (((uintptr_t)d_stats & 15u) != 0) return set_err(ctx, PBR_ERR_INVALID, "d_stats must be 16-byte aligned");
  int rc = check_ready(ctx, 0, ctx->P.num_nodes);
  if (rc) return rc;
  pbr::SoftArgs A;
  int smem = 0, grid = 0;
  const int kind = soft_kind(ctx);
  if (kind < 0) return PBR_ERR_CAPACITY;
  if (kind == 1 && ((uintptr_t)d_out & 15u) != 0)
    return set_err(ctx, PBR_ERR_INVALID, "d_out must be 16-byte aligned");
  rc = kind == 1   ? plan_soft_small(ctx, false, &A, &smem, &grid)
       : kind == 3 ? plan_soft_large(ctx, false, &A, &smem, &grid)
                   : plan_soft(ctx, ctx->soft_threads, false, &A, &smem, &grid);
  if (rc) return rc;
  A.out = d_out;
  A.stats = d_stats;
  cudaError_t e = kind == 1   ? pbr::soft_small_launch(false, ctx->P, A, grid, smem, (cudaStream_t)stream)
                  : kind == 3 ? pbr::soft_large_launch(false, ctx->P, A, grid, smem, (cudaStream_t)stream)
                              : pbr::soft_launch(ctx->soft_threads, false, ctx->P, A, grid, smem, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_err(ctx, e, "soft forward launch");
  return PBR_OK;
}

int pbr_backward_soft(pbr_ctx* ctx, const float* d_out, const float* d_stats, const float* d_grad_out,
                      float* d_grad_light, void* stream) {
  PBR_CHECK_CTX(ctx);
  if (!d_out || !d_stats || !d_grad_out) return set_err(ctx, PBR_ERR_INVALID, "d_out, d_stats and d_grad_out are required");
  if (reject_textures(ctx)) return PBR_ERR_INVALID;
  if (((uintptr_t)d_stats & 15u) != 0) return set_err(ctx, PBR_ERR_INVALID, "d_stats must be 16-byte aligned");
  int rc = check_ready(ctx, 0, ctx->P.num_nodes);
  if (rc) return rc;
  for (int n = 0; n < ctx->P.num_nodes; ++n)
    if (ctx->P.nodes[n].mode != pbr::kModeHpr)
      return set_err(ctx, PBR_ERR_STATE, "soft backward needs every node in HPR mode (node %d is not)", n);
  pbr::SoftArgs A;
  int smem = 0, grid = 0;
  const int kind = soft_kind(ctx);
  if (kind < 0) return PBR_ERR_CAPACITY;
  // the tile adjoint keeps 15 values per pixel in shared memory: 128-thread CTAs
  rc = kind == 1   ? plan_soft_small(ctx, true, &A, &smem, &grid)
       : kind == 3 ? plan_soft_large(ctx, true, &A, &smem, &grid)
                   : plan_soft(ctx, 128, true, &A, &smem, &grid);
  if (rc) return rc;
  A.out = const_cast<float*>(d_out);
  A.stats = const_cast<float*>(d_stats);
  A.gout = d_grad_out;
  A.glight = d_grad_light;
  cudaError_t e = kind == 1   ? pbr::soft_small_launch(true, ctx->P, A, grid, smem, (cudaStream_t)stream)
                  : kind == 3 ? pbr::soft_large_launch(true, ctx->P, A, grid, smem, (cudaStream_t)stream)
                              : pbr::soft_launch(128, true, ctx->P, A, grid, smem, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_err(ctx, e, "soft backward launch");
  return PBR_OK;
}

int pbr_debug_transforms(pbr_ctx* ctx, int node_id, float* d_out, void* stream) {
  PBR_CHECK_CTX(ctx);
  if (node_id < 0 || node_id >= ctx->P.num_nodes) return set_err(ctx, PBR_ERR_INVALID, "unknown node id %d", node_id);
  if (!ctx->node_ready[node_id]) return set_err(ctx, PBR_ERR_STATE, "node %d has no buffers bound", node_id);
  if (!d_out) return set_err(ctx, PBR_ERR_INVALID, "d_out is null");
  const NodeDesc& nd = ctx->P.nodes[node_id];
  const long long rows = nd.shared ? (long long)nd.ips : (long long)nd.ips * ctx->P.N;
  cudaError_t e = pbr::debug_transforms_launch(nd, rows, d_out, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_err(ctx, e, "debug transforms launch");
  return PBR_OK;
}

int pbr_device_status(pbr_ctx* ctx, int32_t* out_flags) {
  PBR_CHECK_CTX(ctx);
  if (!out_flags) return set_err(ctx, PBR_ERR_INVALID, "out_flags is null");
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_err(ctx, e, "cudaDeviceSynchronize");
  int32_t v = 0;
  e = cudaMemcpy(&v, ctx->d_status, sizeof(v), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_err(ctx, e, "cudaMemcpy");
  e = cudaMemset(ctx->d_status, 0, sizeof(int32_t));
  if (e != cudaSuccess) return cuda_err(ctx, e, "cudaMemset");
  *out_flags = v;
  return PBR_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Plain per-node render without any allocation.
//
// pbr_plain_clear allocates the plain path's depth/colour buffer with
// cudaMalloc on first use.  Callers that may not allocate device memory at
// render time -- a render issued while a CUDA stream is being captured (an
// allocation there invalidates the capture), or a host framework whose
// allocator has already reserved the device memory and forbids raw
// cudaMalloc -- use pbr_plain_render_noalloc instead.  Its scratch is a
// file-scope device array.  CUDA loads a library's device code lazily, per
// device, so the array's 16 MiB are reserved by the driver when the first call
// on a device looks up its address (cudaGetSymbolAddress loads this file's
// module); from then on the device holds it until the process exits, and
// later calls allocate nothing.
#include <mutex>

#define PBR_NOALLOC_SCRATCH_BYTES (16u << 20)  // 16 MiB: N*H*W*8 bytes (plus alignment) must fit

static __device__ __align__(256) unsigned char g_noalloc_scratch[PBR_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mutex;
static void* g_noalloc_base[256];  // device address of g_noalloc_scratch, per device ordinal

extern "C" int pbr_plain_render_noalloc(pbr_ctx* ctx, uint8_t* d_out, float* d_depth, void* stream) {
  PBR_CHECK_CTX(ctx);
  if (!d_out) return set_err(ctx, PBR_ERR_INVALID, "d_out is null");
  int rc = check_ready(ctx, 0, ctx->P.num_nodes);
  if (rc) return rc;
  const size_t px = (size_t)ctx->P.N * ctx->P.W * ctx->P.H;
  const size_t cofs = (px * sizeof(float) + 255) & ~(size_t)255;  // colour buffer after the depth buffer
  const size_t need = cofs + px * sizeof(uint32_t);
  if (need > PBR_NOALLOC_SCRATCH_BYTES)
    return set_err(ctx, PBR_ERR_CAPACITY,
                   "pbr_plain_render_noalloc needs %zu bytes of scratch for %zu pixels; its static buffer holds %u "
                   "bytes (at most about %u pixels: num_scenes * width * height)",
                   need, px, (unsigned)PBR_NOALLOC_SCRATCH_BYTES, (unsigned)(PBR_NOALLOC_SCRATCH_BYTES / 8));
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_err(ctx, e, "cudaGetDevice");
  if (dev != ctx->device)
    return set_err(ctx, PBR_ERR_STATE, "the context's device (%d) must be current (current: %d)", ctx->device, dev);
  if (dev < 0 || dev >= 256) return set_err(ctx, PBR_ERR_INVALID, "device ordinal %d out of range", dev);
  void* base = nullptr;
  {
    // first call on this device: load the module that holds the array and look
    // up its device address (a host reference to g_noalloc_scratch is only a
    // stand-in, not a device address)
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_base[dev]) {
      e = cudaGetSymbolAddress(&g_noalloc_base[dev], g_noalloc_scratch);
      if (e != cudaSuccess) {
        g_noalloc_base[dev] = nullptr;
        return cuda_err(ctx, e, "cudaGetSymbolAddress");
      }
    }
    base = g_noalloc_base[dev];
  }
  float* zbuf = reinterpret_cast<float*>(base);
  uint32_t* cbuf = reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(base) + cofs);
  cudaStream_t s = (cudaStream_t)stream;
  // every pixel of the used range is written by the clear: no stale state survives
  e = pbr::plain_clear_launch(ctx->P, zbuf, cbuf, s);
  if (e != cudaSuccess) return cuda_err(ctx, e, "plain clear launch");
  LaunchCfg c = ctx_cfg(ctx);
  c.persistent = 0;
  for (int n = 0; n < ctx->P.num_nodes; ++n) {
    LaunchPlan lp;
    rc = plan_any(ctx, c, true, false, n, n + 1, &lp);
    if (rc) return rc;
    lp.A.zbuf = zbuf;
    lp.A.cbuf = cbuf;
    e = launch_plan(ctx, lp, true, false, s);
    if (e != cudaSuccess) return cuda_err(ctx, e, "plain draw launch");
  }
  e = pbr::plain_resolve_launch(ctx->P, zbuf, cbuf, d_out, d_depth, s);
  if (e != cudaSuccess) return cuda_err(ctx, e, "plain resolve launch");
  return PBR_OK;
}
