// pbr_small.cu -- scene-per-warp hard rasteriser for many small scenes.
//
// The headline workload renders thousands of scenes of a few dozen triangles
// each into small images (4096 x 64x64 CartPole).  There the output bytes are
// the only real cost, so each warp owns one scene at a time and never waits
// on a block barrier:
//
//   K1  the scene's instances of every node, flattened in draw order into one
//       table (lane = instance): model matrix M = [R(hpr)*s | t] and colour;
//       then lane = vertex: clip = VP * M * v, n = normalize(mat3(M) n)
//       (shaders/basic.vert:29-53)
//   K2  lane = triangle: near clip, cull, watertight edges, depth plane, flat
//       shading; compacted in draw order with a warp prefix sum (__shfl_up);
//       then the warp-ballot binner: for each 32x16-pixel bin one
//       __ballot_sync over the lanes (= triangles) is the bin's mask
//   K3  per bin: an empty bin is written as background with 128-bit stores;
//       otherwise the warp walks the bin's triangles in draw order and, per
//       triangle, maps its bbox-in-bin pixels onto the lanes (edge test,
//       strict-less depth test, colour of basic.frag:20-39) against a per-warp
//       shared-memory depth/colour tile; then each lane owns one 16-pixel row
//       segment, transposes RGBA to planes with byte permutes and stores
//       each channel with one st.global.v4.
//
// Shared memory per warp: the triangle list plus one region that holds the
// vertex cache / instance table during K1-K2 and the bin's depth / colour /
// winner tile during K3.  The host picks this kernel when a scene has at most
// 64 source triangles, 32 instances and 256 vertices, and W % 16 == 0.
#include "pbr_device.cuh"
#include "pbr_launch.h"

namespace pbr {

constexpr int kBinW = 32;  // bin = 32 x 16 pixels = 32 lanes x 16-pixel row segments
constexpr int kBinH = 16;
constexpr int kBinPx = kBinW * kBinH;

struct SmallLayout {
  int t0, t1, t2, t3, t4, s0, s1, s2, s3, masks, vp, uni;
  int vcache, itab;          // inside uni (setup)
  int zbuf, cbuf, wbuf;      // inside uni (raster)
  int per_warp;
};

__host__ __device__ inline SmallLayout small_layout(int tri_cap, int vcap, int icap, int nbins, int smooth) {
  SmallLayout L;
  int off = 0;
  const int t4 = tri_cap * 16;
  L.t0 = off; off += align16(t4);
  L.t1 = off; off += align16(t4);
  L.t2 = off; off += align16(t4);
  L.t3 = off; off += align16(t4);
  L.t4 = off; off += align16(t4);
  if (smooth) {
    L.s0 = off; off += align16(t4);
    L.s1 = off; off += align16(t4);
    L.s2 = off; off += align16(t4);
    L.s3 = off; off += align16(t4);
  } else {
    L.s0 = L.s1 = L.s2 = L.s3 = 0;
  }
  L.masks = off; off += align16(nbins * (tri_cap / 32) * 4);
  L.vp = off; off += 64;
  L.uni = off;
  const int setup = align16(vcap * 32) + align16(icap * 80);
  const int raster = kBinPx * 4 + kBinPx * 4 + kBinPx;
  L.vcache = off;
  L.itab = off + align16(vcap * 32);
  L.zbuf = off;
  L.cbuf = off + kBinPx * 4;
  L.wbuf = off + kBinPx * 8;
  off += align16(setup > raster ? setup : raster);
  L.per_warp = align16(off);
  return L;
}

int small_smem_per_warp(const RasterArgs& A, int W, int H) {
  const int nbins = ((W + kBinW - 1) / kBinW) * ((H + kBinH - 1) / kBinH);
  return small_layout(A.tri_cap, A.vcap, A.icap, nbins, A.smooth_any).per_warp;
}

// RGBA words of pixels p0..p3 -> channel-planar words (4 pixels per word).
__device__ __forceinline__ void rgba_to_planes(uint32_t p0, uint32_t p1, uint32_t p2, uint32_t p3, uint32_t& r,
                                               uint32_t& g, uint32_t& b, uint32_t& a) {
  const uint32_t t0 = __byte_perm(p0, p1, 0x5140), t1 = __byte_perm(p2, p3, 0x5140);
  const uint32_t t2 = __byte_perm(p0, p1, 0x7362), t3 = __byte_perm(p2, p3, 0x7362);
  r = __byte_perm(t0, t1, 0x5410);
  g = __byte_perm(t0, t1, 0x7632);
  b = __byte_perm(t2, t3, 0x5410);
  a = __byte_perm(t2, t3, 0x7632);
}

template <int WARPS, bool PLAIN, bool WINNER>
__global__ void __launch_bounds__(WARPS * 32, 24 / WARPS) small_kernel(const __grid_constant__ SceneParams P,
                                                                          const __grid_constant__ RasterArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int W = P.W, H = P.H, HW = W * H;
  const int bins_x = (W + kBinW - 1) / kBinW, bins_y = (H + kBinH - 1) / kBinH;
  const int nbins = bins_x * bins_y;
  const int words = A.tri_cap >> 5;
  const SmallLayout L = small_layout(A.tri_cap, A.vcap, A.icap, nbins, A.smooth_any);
  unsigned char* base = smem + warp * L.per_warp;
  SetupCtx S;
  S.T0 = reinterpret_cast<float4*>(base + L.t0);
  S.T1 = reinterpret_cast<float4*>(base + L.t1);
  S.T2 = reinterpret_cast<float4*>(base + L.t2);
  S.T3 = reinterpret_cast<float4*>(base + L.t3);
  S.T4 = reinterpret_cast<float4*>(base + L.t4);
  S.S0 = reinterpret_cast<float4*>(base + L.s0);
  S.S1 = reinterpret_cast<float4*>(base + L.s1);
  S.S2 = reinterpret_cast<float4*>(base + L.s2);
  S.S3 = reinterpret_cast<float4*>(base + L.s3);
  S.W = (float)W;
  S.H = (float)H;
  S.ry0 = 0.f;
  S.ry1 = (float)(H - 1);
  S.cull = P.cull;
  uint32_t* masks = reinterpret_cast<uint32_t*>(base + L.masks);
  float* s_vp = reinterpret_cast<float*>(base + L.vp);
  float4* vcache = reinterpret_cast<float4*>(base + L.vcache);
  float4* itab = reinterpret_cast<float4*>(base + L.itab);  // per instance: 3 matrix rows, colour, meta
  float* zb = reinterpret_cast<float*>(base + L.zbuf);       // [16][32]: pixel j of lane l at j*32 + l
  uint32_t* cb = reinterpret_cast<uint32_t*>(base + L.cbuf);
  uint8_t* wb = base + L.wbuf;

  const int seg_r = lane >> 1, seg_x = (lane & 1) * 16;
  const uint32_t bg = P.bg_packed;
  uint32_t bgw[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) bgw[c] = ((bg >> (8 * c)) & 0xffu) * 0x01010101u;

  for (int k = blockIdx.x * WARPS + warp; k < P.N; k += gridDim.x * WARPS) {
    if (lane < 16) s_vp[lane] = P.vp[(long long)k * 16 + lane];

    // ---- K1: instance table, flattened over nodes in draw order ---------
    // node-level counts are uniform across the warp
    int total_inst = 0, total_verts = 0, total_tris = 0;
    for (int n = A.node_begin; n < A.node_end; ++n) {
      const NodeDesc& nd = P.nodes[n];
      int cnt = nd.counts ? nd.counts[k] : nd.ips;
      cnt = max(0, min(cnt, nd.ips));
      const MeshDesc& me = P.meshes[nd.mesh];
      for (int i = lane; i < cnt; i += 32) {
        const long long id = nd.shared ? (long long)i : (long long)k * nd.ips + i;
        float m[12];
        build_model(nd, id, m);
        float4* e = itab + (total_inst + i) * 5;
        e[0] = make_float4(m[0], m[1], m[2], m[3]);
        e[1] = make_float4(m[4], m[5], m[6], m[7]);
        e[2] = make_float4(m[8], m[9], m[10], m[11]);
        const float4 cc = *reinterpret_cast<const float4*>(nd.color + id * 4);
        e[3] = cc;
        // meta: node, first vertex, draw id of triangle 0, first triangle
        e[4] = make_float4(__int_as_float(n), __int_as_float(total_verts + i * me.nv),
                           __int_as_float((nd.rank_base + i) * P.max_tris), __int_as_float(total_tris + i * me.nt));
      }
      total_inst += cnt;
      total_verts += cnt * me.nv;
      total_tris += cnt * me.nt;
    }
    __syncwarp();

    // ---- K1: vertices ------------------------------------------------------
    for (int v = lane; v < total_verts; v += 32) {
      // find the instance holding flat vertex v (instances are few: linear scan)
      int inst = 0;
      while (inst + 1 < total_inst && __float_as_int(itab[(inst + 1) * 5 + 4].y) <= v) ++inst;
      const float4 meta = itab[inst * 5 + 4];
      const MeshDesc& me = P.meshes[P.nodes[__float_as_int(meta.x)].mesh];
      const int vi = v - __float_as_int(meta.y);
      const float4 r0 = itab[inst * 5 + 0], r1 = itab[inst * 5 + 1], r2 = itab[inst * 5 + 2];
      const float ox = me.pos[3 * vi], oy = me.pos[3 * vi + 1], oz = me.pos[3 * vi + 2];
      const float wx = r0.x * ox + r0.y * oy + r0.z * oz + r0.w;
      const float wy = r1.x * ox + r1.y * oy + r1.z * oz + r1.w;
      const float wz = r2.x * ox + r2.y * oy + r2.z * oz + r2.w;
      const float4 q0 = *reinterpret_cast<const float4*>(s_vp), q1 = *reinterpret_cast<const float4*>(s_vp + 4);
      const float4 q2 = *reinterpret_cast<const float4*>(s_vp + 8), q3 = *reinterpret_cast<const float4*>(s_vp + 12);
      float4 c;
      c.x = q0.x * wx + q0.y * wy + q0.z * wz + q0.w;
      c.y = q1.x * wx + q1.y * wy + q1.z * wz + q1.w;
      c.z = q2.x * wx + q2.y * wy + q2.z * wz + q2.w;
      c.w = q3.x * wx + q3.y * wy + q3.z * wz + q3.w;
      const float ax = me.nrm[3 * vi], ay = me.nrm[3 * vi + 1], az = me.nrm[3 * vi + 2];
      const float nx = r0.x * ax + r0.y * ay + r0.z * az;
      const float ny = r1.x * ax + r1.y * ay + r1.z * az;
      const float nz = r2.x * ax + r2.y * ay + r2.z * az;
      const float l2 = nx * nx + ny * ny + nz * nz;
      const float inv = l2 > 0.f ? rsqrtf(l2) : 0.f;
      vcache[2 * v] = c;
      vcache[2 * v + 1] = make_float4(nx * inv, ny * inv, nz * inv, 0.f);
    }
    __syncwarp();

    // ---- K2: triangles, compacted in draw order -------------------------
    int tri_count = 0;
    for (int t0 = 0; t0 < total_tris; t0 += 32) {
      const int t = t0 + lane;
      int c = 0, inst = 0, ti = 0, vbase = 0, i0 = 0, i1 = 0, i2 = 0;
      float4 col = make_float4(0.f, 0.f, 0.f, 0.f);
      bool smooth = false;
      int dbase = 0;
      if (t < total_tris) {
        // instance holding flat triangle t (instances are few: linear scan)
        while (inst + 1 < total_inst && __float_as_int(itab[(inst + 1) * 5 + 4].w) <= t) ++inst;
        const float4 meta = itab[inst * 5 + 4];
        const MeshDesc& me = P.meshes[P.nodes[__float_as_int(meta.x)].mesh];
        ti = t - __float_as_int(meta.w);
        vbase = __float_as_int(meta.y);
        dbase = __float_as_int(meta.z);
        smooth = me.smooth != 0;
        col = itab[inst * 5 + 3];
        i0 = me.idx[3 * ti];
        i1 = me.idx[3 * ti + 1];
        i2 = me.idx[3 * ti + 2];
        c = process_tri<false>(P, S, vcache, vbase, i0, i1, i2, 0, col, 0, smooth);
      }
      int incl = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      if (c > 0) process_tri<true>(P, S, vcache, vbase, i0, i1, i2, tri_count + incl - c, col, dbase + ti, smooth);
      tri_count += total;
    }
    __syncwarp();

    // ---- warp-ballot binner ----------------------------------------------
    const int T = tri_count;
    const int nw = (T + 31) >> 5;
    for (int w = 0; w < nw; ++w) {
      const int t = w * 32 + lane;
      int bx0 = 1 << 20, bx1 = -1, by0 = 1 << 20, by1 = -1;
      if (t < T) {
        const uint32_t xb = __float_as_uint(S.T3[t].w), yb = __float_as_uint(S.T4[t].x);
        bx0 = (int)(xb & 0xffffu) / kBinW;
        bx1 = (int)(xb >> 16) / kBinW;
        by0 = (int)(yb & 0xffffu) / kBinH;
        by1 = (int)(yb >> 16) / kBinH;
      }
      for (int b = 0; b < nbins; ++b) {
        const int by = b / bins_x, bx = b - by * bins_x;
        const uint32_t m = __ballot_sync(0xffffffffu, (bx >= bx0) && (bx <= bx1) && (by >= by0) && (by <= by1));
        if (lane == 0) masks[b * words + w] = m;
      }
    }
    __syncwarp();

    // ---- K3: bin by bin ----------------------------------------------------
    for (int b = 0; b < nbins; ++b) {
      const int by = b / bins_x, bx = b - by * bins_x;
      const int row0 = by * kBinH, col0 = bx * kBinW;
      const int y = row0 + seg_r, x0 = col0 + seg_x;
      const bool active = (y < H) && (x0 < W);
      const long long pix0 = (long long)k * HW + (long long)y * W + x0;
      uint8_t* out0 = A.out + (long long)k * P.C * HW + (long long)y * W + x0;
      uint32_t any = 0u;
      for (int w = 0; w < nw; ++w) any |= masks[b * words + w];
      if (any == 0u) {
        if (!PLAIN && active) {
          for (int c = 0; c < P.C; ++c)
            *reinterpret_cast<uint4*>(out0 + (long long)c * HW) = make_uint4(bgw[c], bgw[c], bgw[c], bgw[c]);
          if (A.depth) {
            float4* d = reinterpret_cast<float4*>(A.depth + pix0);
            const float4 one = make_float4(1.f, 1.f, 1.f, 1.f);
            d[0] = one; d[1] = one; d[2] = one; d[3] = one;
          }
          if (WINNER) {
            int4* d = reinterpret_cast<int4*>(A.winner + pix0);
            const int4 none = make_int4(-1, -1, -1, -1);
            d[0] = none; d[1] = none; d[2] = none; d[3] = none;
          }
        }
        continue;
      }
      // this bin's depth / colour / winner tile
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        float z0 = 1.f;
        uint32_t c0 = bg;
        if (PLAIN && active) {
          z0 = A.zbuf[pix0 + j];
          c0 = A.cbuf[pix0 + j];
        }
        zb[j * 32 + lane] = z0;
        cb[j * 32 + lane] = c0;
        if (WINNER) wb[j * 32 + lane] = 0xffu;
      }
      __syncwarp();
      for (int w = 0; w < nw; ++w) {
        uint32_t m = masks[b * words + w];
        while (m) {
          const int t = w * 32 + __ffs(m) - 1;
          m &= m - 1u;
          const float4 zp = S.T3[t];
          const float4 meta = S.T4[t];
          const uint32_t xb = __float_as_uint(zp.w), yb = __float_as_uint(meta.x);
          const int ax0 = max((int)(xb & 0xffffu), col0), ax1 = min((int)(xb >> 16), col0 + kBinW - 1);
          const int ay0 = max((int)(yb & 0xffffu), row0), ay1 = min((int)(yb >> 16), row0 + kBinH - 1);
          const int bw = ax1 - ax0 + 1, bh = ay1 - ay0 + 1;
          if (bw <= 0 || bh <= 0) continue;
          const float4 e0 = S.T0[t], e1 = S.T1[t], e2 = S.T2[t];
          const uint32_t fl = __float_as_uint(meta.y);
          const uint32_t flat_col = __float_as_uint(meta.z);
          const float inv_bw = 1.f / (float)bw;
          const int npx = bw * bh;
          for (int i = lane; i < npx; i += 32) {
            const int ry = (int)(((float)i + 0.5f) * inv_bw);
            const int xx = ax0 + i - ry * bw, yy = ay0 + ry;
            const float px = (float)xx + 0.5f, py = (float)yy + 0.5f;
            const float E0 = fmaf(e0.x, px - e0.z, e0.y * (py - e0.w));
            const float E1 = fmaf(e1.x, px - e1.z, e1.y * (py - e1.w));
            const float E2 = fmaf(e2.x, px - e2.z, e2.y * (py - e2.w));
            const bool in0 = (fl & 1u) ? (E0 >= 0.f) : (E0 > 0.f);
            const bool in1 = (fl & 2u) ? (E1 >= 0.f) : (E1 > 0.f);
            const bool in2 = (fl & 4u) ? (E2 >= 0.f) : (E2 > 0.f);
            if (in0 && in1 && in2) {
              const float z = fmaxf(fmaf(zp.x, px, fmaf(zp.y, py, zp.z)), 0.f);
              const int p = (yy - row0) * kBinW + (xx - col0);
              const int idx = (p & 15) * 32 + (p >> 4);
              if (z < zb[idx]) {
                zb[idx] = z;
                cb[idx] = (fl & 8u) ? shade_smooth(P, S, t, px, py) : flat_col;
                if (WINNER) wb[idx] = (uint8_t)t;
              }
            }
          }
          __syncwarp();
        }
      }
      // each lane stores its 16-pixel row segment
      if (active) {
        if (PLAIN) {
          uint4* cd = reinterpret_cast<uint4*>(A.cbuf + pix0);
          float4* zd = reinterpret_cast<float4*>(A.zbuf + pix0);
#pragma unroll
          for (int g = 0; g < 4; ++g) {
            cd[g] = make_uint4(cb[(4 * g) * 32 + lane], cb[(4 * g + 1) * 32 + lane], cb[(4 * g + 2) * 32 + lane],
                               cb[(4 * g + 3) * 32 + lane]);
            zd[g] = make_float4(zb[(4 * g) * 32 + lane], zb[(4 * g + 1) * 32 + lane], zb[(4 * g + 2) * 32 + lane],
                                zb[(4 * g + 3) * 32 + lane]);
          }
        } else {
          uint32_t pr[4], pg[4], pb[4], pa[4];
#pragma unroll
          for (int g = 0; g < 4; ++g)
            rgba_to_planes(cb[(4 * g) * 32 + lane], cb[(4 * g + 1) * 32 + lane], cb[(4 * g + 2) * 32 + lane],
                           cb[(4 * g + 3) * 32 + lane], pr[g], pg[g], pb[g], pa[g]);
          *reinterpret_cast<uint4*>(out0) = make_uint4(pr[0], pr[1], pr[2], pr[3]);
          if (P.C > 1) *reinterpret_cast<uint4*>(out0 + HW) = make_uint4(pg[0], pg[1], pg[2], pg[3]);
          if (P.C > 2) *reinterpret_cast<uint4*>(out0 + 2LL * HW) = make_uint4(pb[0], pb[1], pb[2], pb[3]);
          if (P.C > 3) *reinterpret_cast<uint4*>(out0 + 3LL * HW) = make_uint4(pa[0], pa[1], pa[2], pa[3]);
          if (A.depth) {
            float4* d = reinterpret_cast<float4*>(A.depth + pix0);
#pragma unroll
            for (int g = 0; g < 4; ++g)
              d[g] = make_float4(zb[(4 * g) * 32 + lane], zb[(4 * g + 1) * 32 + lane], zb[(4 * g + 2) * 32 + lane],
                                 zb[(4 * g + 3) * 32 + lane]);
          }
          if (WINNER) {
            int wi[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const int t = wb[j * 32 + lane];
              wi[j] = (t != 0xff) ? __float_as_int(S.T4[t].w) : -1;
            }
            int4* d = reinterpret_cast<int4*>(A.winner + pix0);
#pragma unroll
            for (int g = 0; g < 4; ++g) d[g] = make_int4(wi[4 * g], wi[4 * g + 1], wi[4 * g + 2], wi[4 * g + 3]);
          }
        }
      }
      __syncwarp();
    }
    __syncwarp();  // the next scene's K1 reuses the raster tile as vertex cache
  }
}

// ---------------------------------------------------------------------------

template <int WP, bool PL, bool WN>
static const void* small_fn() {
  return reinterpret_cast<const void*>(&small_kernel<WP, PL, WN>);
}

static const void* pick_small(int warps, bool plain, bool winner) {
  if (plain && winner) return nullptr;
  if (warps == 4) return plain ? small_fn<4, true, false>() : (winner ? small_fn<4, false, true>() : small_fn<4, false, false>());
  if (warps == 8) return plain ? small_fn<8, true, false>() : (winner ? small_fn<8, false, true>() : small_fn<8, false, false>());
  return nullptr;
}

cudaError_t small_set_smem_limit(int warps, bool plain, bool winner, int bytes) {
  const void* f = pick_small(warps, plain, winner);
  if (!f) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

cudaError_t small_occupancy(int warps, bool plain, bool winner, int smem_bytes, int* blocks_per_sm) {
  const void* f = pick_small(warps, plain, winner);
  if (!f) return cudaErrorInvalidValue;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, warps * 32, smem_bytes);
}

cudaError_t small_launch(int warps, bool plain, bool winner, const SceneParams& P, const RasterArgs& A, int grid,
                         int smem_bytes, cudaStream_t stream) {
  const void* f = pick_small(warps, plain, winner);
  if (!f) return cudaErrorInvalidValue;
  void* args[] = {const_cast<SceneParams*>(&P), const_cast<RasterArgs*>(&A)};
  return cudaLaunchKernel(f, dim3(grid), dim3(warps * 32), args, (size_t)smem_bytes, stream);
}

}  // namespace pbr
