// pbr_small.cu -- scene-per-warp hard rasteriser for many small scenes.
//
// The headline workload renders thousands of scenes of a few dozen triangles
// each into small images (4096 x 64x64 CartPole).  There the output bytes are
// the only real cost, so each warp owns one scene at a time and never waits
// on a block barrier:
//
//   K1  the scene's instances of every node, flattened in draw order into one
//       table (lane = instance, so all pose loads are in flight together):
//       model matrix M = [R(hpr)*s | t] and colour; then lane = vertex:
//       clip = VP * M * v and its screen position (shaders/basic.vert:29-53;
//       smooth meshes also n = normalize(mat3(M) n))
//   K2  lane = triangle: near clip, cull, watertight edges, depth plane, flat
//       shading (a flat mesh's provoking normal is transformed here, for
//       survivors only), written at the triangle's two fixed slots (2t, 2t+1:
//       draw order, room for a near-plane split; unused slots are empty);
//       then the warp-ballot binner: for each 32x16-pixel bin one
//       __ballot_sync over the lanes (= triangles) is the bin's mask
//   K3  per bin: a bin without candidates is written as background with
//       128-bit stores.
//       Otherwise the bin's candidate triangles and the pixels of their
//       bbox-in-bin are laid out end to end (warp prefix sum of the areas) and
//       dealt 32 per pass to the lanes, so many tiny triangles share a pass.
//       Each covered pixel does a 64-bit atomicMin of (window depth, draw
//       order + 1) into a shared-memory tile: strict-less depth with ties to
//       the earlier draw, independent of lane order.  Then every lane resolves
//       its own 16-pixel row segment (shaders/basic.frag:20-39, once per
//       pixel), transposes RGBA to planes with byte permutes and stores each
//       channel with one st.global.v4.
//
// Shared memory per warp: the triangle list plus one region that holds the
// vertex cache / instance table during K1-K2 and the bin's key tile during K3.
// The host picks this kernel when a scene has at most 64 source triangles,
// 32 instances, 256 vertices and 64 bins, and W % 16 == 0.
#include "pbr_device.cuh"
#include "pbr_launch.h"

namespace pbr {

constexpr int kBinW = 32;  // bin = 32 x 16 pixels = 32 lanes x 16-pixel row segments
constexpr int kBinH = 16;
constexpr int kBinPx = kBinW * kBinH;
constexpr int kWarps = 4;        // default warps per block
constexpr int kMaxWarps = 14;    // launch bound: blocks of up to 14 warps, two per SM (the same 72-register
constexpr int kMinBlocks = 2;    // budget as seven blocks of 4 warps); the block size is chosen at launch

struct SmallLayout {
  int t0, t1, t2, t3, bgrec, t4, s0, s1, s2, s3, s4, s5, masks, vp, uni;
  int vcache, itab;  // inside uni (setup)
  int keys;          // inside uni (raster): uint64 [16][32]
  int per_warp;
};

// Per-warp shared memory.  Triangle records T0..T4 (S0..S3 for per-pixel
// shading, S4..S5 for texture coordinates); bgrec is a T4-shaped record just before T4[0] holding the
// background colour (.z) and winner -1 (.w), so that draw order + 1 indexes
// both.  The setup stage's vertex cache (3 float4 per vertex: clip position;
// normal with .w = z + w; screen position), instance table (5 float4 per
// instance: 3 model-matrix rows, colour, meta) and view-projection matrix
// share one region with the raster stage's key tile.  Cartpole-sized scenes
// need 8016 bytes a warp, which keeps 28 warps on an SM (7 blocks of 4 warps
// or 2 blocks of 14).
__host__ __device__ inline SmallLayout small_layout(int tri_cap, int vcap, int icap, int nbins, int smooth,
                                                    int tex) {
  SmallLayout L;
  int off = 0;
  const int t4 = tri_cap * 16;
  L.t0 = off; off += align16(t4);
  L.t1 = off; off += align16(t4);
  L.t2 = off; off += align16(t4);
  L.t3 = off; off += align16(t4);
  L.bgrec = off; off += 16;
  L.t4 = off; off += align16(t4);
  if (smooth) {
    L.s0 = off; off += align16(t4);
    L.s1 = off; off += align16(t4);
    L.s2 = off; off += align16(t4);
    L.s3 = off; off += align16(t4);
  } else {
    L.s0 = L.s1 = L.s2 = L.s3 = 0;
  }
  if (smooth && tex) {
    L.s4 = off; off += align16(t4);
    L.s5 = off; off += align16(t4);
  } else {
    L.s4 = L.s5 = 0;
  }
  L.masks = off; off += align16(nbins * ((tri_cap + 31) / 32) * 4);
  L.uni = off;
  const int setup = align16(vcap * 48) + align16(icap * 80) + 64;
  const int raster = kBinPx * 8;
  L.vcache = off;
  L.itab = off + align16(vcap * 48);
  L.vp = L.itab + align16(icap * 80);
  L.keys = off;
  off += align16(setup > raster ? setup : raster);
  L.per_warp = align16(off);
  return L;
}

int small_smem_per_warp(const RasterArgs& A, int W, int H) {
  const int nbins = ((W + kBinW - 1) / kBinW) * ((H + kBinH - 1) / kBinH);
  if (nbins > 64) return -1;  // the non-empty bins of a scene are one 64-bit mask
  return small_layout(A.tri_cap, A.vcap, A.icap, nbins, A.smooth_any, A.tex_any).per_warp;
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

__device__ __forceinline__ int node_count(const NodeDesc& nd, int k) {
  const int c = nd.counts ? nd.counts[k] : nd.ips;
  return max(0, min(c, nd.ips));
}

// Triangle t of the flattened scene: count (WRITE = false) or set up at slot.
// Smooth meshes take the vertex normals from the vertex cache; a flat mesh's
// triangle is lit with its first vertex's normal (all three are identical),
// transformed here, only for triangles that survive culling.
template <bool WRITE, bool SMOOTH, bool TEX>
__device__ __forceinline__ int small_tri(const SceneParams& P, const SetupCtx& S, const float4* vcache,
                                         const float4* itab, int total_inst, int t, int slot) {
  int inst = 0;
  while (inst + 1 < total_inst && __float_as_int(itab[(inst + 1) * 5 + 4].w) <= t) ++inst;
  const float4 meta = itab[inst * 5 + 4];
  const MeshDesc& me = P.meshes[P.nodes[__float_as_int(meta.x)].mesh];
  const int ti = (int)PBR_IX(t - __float_as_int(meta.w), me.nt, 20);
  const int vbase = __float_as_int(meta.y);
  const int i0 = (int)PBR_IX(me.idx[3 * ti], me.nv, 21), i1 = (int)PBR_IX(me.idx[3 * ti + 1], me.nv, 21);
  const int i2 = (int)PBR_IX(me.idx[3 * ti + 2], me.nv, 21);
  float4 n0 = vcache[3 * (vbase + i0) + 1], n1 = vcache[3 * (vbase + i1) + 1], n2 = vcache[3 * (vbase + i2) + 1];
  const bool front = n0.w >= 0.f && n1.w >= 0.f && n2.w >= 0.f;
  if (!front && n0.w < 0.f && n1.w < 0.f && n2.w < 0.f) return 0;
  const float4 col = itab[inst * 5 + 3];
  const int draw_id = __float_as_int(meta.z) + ti;
  const int node = __float_as_int(meta.x);
  const bool textured = TEX && P.nodes[node].tex != nullptr;  // shaded per pixel like smooth meshes
  const bool smooth = SMOOTH && (me.smooth != 0 || textured);
  TexIn tx;
  if (WRITE && textured) {
    tx.t0 = mesh_uv(me, i0);
    tx.t1 = mesh_uv(me, i1);
    tx.t2 = mesh_uv(me, i2);
    tx.node = node;
  }
  if (WRITE && !SMOOTH) {
    const float4 r0 = itab[inst * 5 + 0], r1 = itab[inst * 5 + 1], r2 = itab[inst * 5 + 2];
    const float ax = me.nrm[3 * i0], ay = me.nrm[3 * i0 + 1], az = me.nrm[3 * i0 + 2];
    const float nx = r0.x * ax + r0.y * ay + r0.z * az;
    const float ny = r1.x * ax + r1.y * ay + r1.z * az;
    const float nz = r2.x * ax + r2.y * ay + r2.z * az;
    const float l2 = nx * nx + ny * ny + nz * nz;
    const float inv = l2 > 0.f ? rsqrtf(l2) : 0.f;
    n0 = make_float4(nx * inv, ny * inv, nz * inv, 0.f);
    n1 = n0;
    n2 = n0;
  }
  if (front) {
    const float4 a = vcache[3 * (vbase + i0) + 2], b = vcache[3 * (vbase + i1) + 2], c = vcache[3 * (vbase + i2) + 2];
    return setup_tri_sv<WRITE>(P, S, SV{a.x, a.y, a.z, a.w}, n0, SV{b.x, b.y, b.z, b.w}, n1, SV{c.x, c.y, c.z, c.w},
                               n2, slot, col, draw_id, smooth, tx);
  }
  return clip_tri<WRITE>(P, S, vcache[3 * (vbase + i0)], n0, vcache[3 * (vbase + i1)], n1, vcache[3 * (vbase + i2)],
                         n2, i0, i1, i2, slot, col, draw_id, smooth, tx);
}

// SHADE: 0 = flat meshes only, 1 = smooth meshes (per-pixel normals), 2 = smooth and textured
template <bool PLAIN, bool WINNER, int SHADE>
__global__ void __launch_bounds__(kMaxWarps * 32, kMinBlocks) small_kernel(const __grid_constant__ SceneParams P,
                                                                         const __grid_constant__ RasterArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr bool SMOOTH = SHADE >= 1, TEX = SHADE == 2;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int W = P.W, H = P.H, HW = W * H, C = P.C;
  const int bins_x = (W + kBinW - 1) / kBinW, bins_y = (H + kBinH - 1) / kBinH;
  const int nbins = bins_x * bins_y;
  const int words = (A.tri_cap + 31) >> 5;
  const SmallLayout L = small_layout(A.tri_cap, A.vcap, A.icap, nbins, SMOOTH ? 1 : 0, TEX ? 1 : 0);
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
  S.S4 = reinterpret_cast<float4*>(base + L.s4);
  S.S5 = reinterpret_cast<float4*>(base + L.s5);
  S.W = (float)W;
  S.H = (float)H;
  S.ry0 = 0.f;
  S.ry1 = (float)(H - 1);
  S.cull = P.cull;
  uint32_t* masks = reinterpret_cast<uint32_t*>(base + L.masks);
  float* s_vp = reinterpret_cast<float*>(base + L.vp);
  float4* vcache = reinterpret_cast<float4*>(base + L.vcache);
  float4* itab = reinterpret_cast<float4*>(base + L.itab);
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(base + L.keys);  // [16][32]
  // T4 record r - 1 for r = draw order + 1 (r = 0: the background record)
  const unsigned char* rec4 = base + L.bgrec;

  const uint32_t bg = P.bg_packed;
  if (lane == 0) *reinterpret_cast<float4*>(base + L.bgrec) = make_float4(0.f, 0.f, __uint_as_float(bg), __int_as_float(-1));
  const uint32_t bg0 = (bg & 0xffu) * 0x01010101u, bg1 = ((bg >> 8) & 0xffu) * 0x01010101u;
  const uint32_t bg2 = ((bg >> 16) & 0xffu) * 0x01010101u, bg3 = (bg >> 24) * 0x01010101u;
  // this lane's 16-pixel row segment of a bin: row lane / 2, columns (lane % 2) * 16 .. + 15
  const int seg_r = lane >> 1, seg_x = (lane & 1) * 16;
  const int lane_off = seg_r * W + seg_x;
  // key of an untouched pixel: depth 1.0 (the clear), draw order 0 (before every triangle)
  const unsigned long long clear_key = (unsigned long long)__float_as_uint(1.f) << 32;

  const int nwarps = blockDim.x >> 5;
  for (int k = blockIdx.x * nwarps + warp; k < P.N; k += gridDim.x * nwarps) {
    if (lane < 16) s_vp[lane] = P.vp[(long long)k * 16 + lane];

    // ---- K1: instance table, flattened over nodes in draw order ---------
    int total_inst = 0, total_verts = 0, total_tris = 0;
    for (int n = A.node_begin; n < A.node_end; ++n) {
      const NodeDesc& nd = P.nodes[n];
      const int cnt = node_count(nd, k);
      const MeshDesc& me = P.meshes[nd.mesh];
      total_inst += cnt;
      total_verts += cnt * me.nv;
      total_tris += cnt * me.nt;
    }
    for (int i = lane; i < total_inst; i += 32) {
      int n = A.node_begin, ai = 0, av = 0, at = 0;
      for (; n < A.node_end; ++n) {
        const int cnt = node_count(P.nodes[n], k);
        if (i < ai + cnt) break;
        const MeshDesc& me = P.meshes[P.nodes[n].mesh];
        ai += cnt;
        av += cnt * me.nv;
        at += cnt * me.nt;
      }
      const NodeDesc& nd = P.nodes[n];
      const MeshDesc& me = P.meshes[nd.mesh];
      const int li = i - ai;
      const long long id = nd.shared ? (long long)li : (long long)k * nd.ips + li;
      // the colour first: issued with the pose loads, before the write-back stores it cannot be moved past
      const float4 col = *reinterpret_cast<const float4*>(nd.color + id * 4);
      float m[12];
      build_model(nd, id, m);
      write_back_bound(nd, id);
      float4* e = itab + i * 5;
      e[0] = make_float4(m[0], m[1], m[2], m[3]);
      e[1] = make_float4(m[4], m[5], m[6], m[7]);
      e[2] = make_float4(m[8], m[9], m[10], m[11]);
      e[3] = col;
      // meta: node, first vertex, draw id of triangle 0, first triangle
      e[4] = make_float4(__int_as_float(n), __int_as_float(av + li * me.nv),
                         __int_as_float((nd.rank_base + li) * P.max_tris), __int_as_float(at + li * me.nt));
    }
    __syncwarp();

    // ---- K1: vertices ------------------------------------------------------
    // two vertices per lane and pass (v and v + 32), so that the mesh loads of
    // both are in flight together
    for (int v0 = lane; v0 < total_verts; v0 += 64) {
      int vv[2], inst[2];
      float o[2][3], a[2][3];
      const MeshDesc* mp[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int v = min(v0 + 32 * u, total_verts - 1);  // a lane past the end repeats a vertex, unstored
        int in = 0;
        while (in + 1 < total_inst && __float_as_int(itab[(in + 1) * 5 + 4].y) <= v) ++in;
        const float4 meta = itab[in * 5 + 4];
        mp[u] = &P.meshes[P.nodes[__float_as_int(meta.x)].mesh];
        const int vi = v - __float_as_int(meta.y);
        vv[u] = vi;
        inst[u] = in;
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const float* pp = mp[u]->pos + 3 * vv[u];
        o[u][0] = pp[0];
        o[u][1] = pp[1];
        o[u][2] = pp[2];
        if (SMOOTH) {
          const float* np = mp[u]->nrm + 3 * vv[u];
          a[u][0] = np[0];
          a[u][1] = np[1];
          a[u][2] = np[2];
        }
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int v = v0 + 32 * u;
        if (v >= total_verts) continue;
        const int in = inst[u];
        const float4 r0 = itab[in * 5 + 0], r1 = itab[in * 5 + 1], r2 = itab[in * 5 + 2];
        const float ox = o[u][0], oy = o[u][1], oz = o[u][2];
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
        float4 nv = make_float4(0.f, 0.f, 0.f, c.z + c.w);
        if (SMOOTH) {
          const float ax = a[u][0], ay = a[u][1], az = a[u][2];
          const float nx = r0.x * ax + r0.y * ay + r0.z * az;
          const float ny = r1.x * ax + r1.y * ay + r1.z * az;
          const float nz = r2.x * ax + r2.y * ay + r2.z * az;
          const float l2 = nx * nx + ny * ny + nz * nz;
          const float inv = l2 > 0.f ? rsqrtf(l2) : 0.f;
          nv.x = nx * inv;
          nv.y = ny * inv;
          nv.z = nz * inv;
        }
        const SV sv = to_screen(c, S.W, S.H);
        (void)PBR_IX(v, A.vcap, 23);
        vcache[3 * v] = c;
        vcache[3 * v + 1] = nv;
        vcache[3 * v + 2] = make_float4(sv.x, sv.y, sv.z, sv.iw);
      }
    }
    __syncwarp();

    // ---- K2: triangles at fixed slots in draw order ------------------------
    // Triangle t owns slots 2t and 2t + 1 (a near-plane clip can split it in
    // two), so each triangle is set up once, with no count pass: a slot that
    // holds no triangle gets an empty row range (first row 0xffff, last row
    // 0), which puts it in no bin.  Slot order is draw order.
    for (int t = lane; t < total_tris; t += 32) {
      (void)PBR_IX(2 * t + 1, A.tri_cap, 22);
      const int c = small_tri<true, SMOOTH, TEX>(P, S, vcache, itab, total_inst, t, 2 * t);
      const float no_rows = __uint_as_float(0xffffu);
      if (c < 1) reinterpret_cast<float*>(&S.T4[2 * t])[0] = no_rows;
      if (c < 2) reinterpret_cast<float*>(&S.T4[2 * t + 1])[0] = no_rows;
    }
    __syncwarp();

    // ---- warp-ballot binner ----------------------------------------------
    const int T = 2 * total_tris;
    const int nw = (T + 31) >> 5;
    unsigned long long ne = 0ull;  // bit b: bin b has candidates
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
      int b = 0;
      for (int by = 0; by < bins_y; ++by) {
        const bool yin = (by >= by0) && (by <= by1);
        for (int bx = 0; bx < bins_x; ++bx, ++b) {
          const uint32_t m = __ballot_sync(0xffffffffu, yin && (bx >= bx0) && (bx <= bx1));
          if (lane == 0) masks[PBR_IX(b * words + w, nbins * words, 24)] = m;
          ne |= (unsigned long long)(m != 0u) << b;
        }
      }
    }
    __syncwarp();

    // ---- K3: background for bins without candidates, raster the others -----
    uint8_t* const lane_out = A.out + (size_t)k * C * HW + lane_off;
    const size_t lane_pix = (size_t)k * HW + lane_off;
    if (!PLAIN) {
      // bins without candidates: background, one 128-bit store per plane (depth 1, no winner)
      const unsigned long long row_bits = (bins_x >= 64) ? ~0ull : ((1ull << bins_x) - 1ull);
      for (int by = 0; by < bins_y; ++by) {
        const int row0 = by * kBinH;
        if (row0 + seg_r >= H) continue;
        for (unsigned long long rem = ~(ne >> (by * bins_x)) & row_bits; rem != 0ull; rem &= rem - 1ull) {
          const int col0 = (__ffsll((long long)rem) - 1) * kBinW;
          if (col0 + seg_x >= W) continue;
          const int boff = row0 * W + col0;
          uint8_t* o = lane_out + boff;
          *reinterpret_cast<uint4*>(o) = make_uint4(bg0, bg0, bg0, bg0);
          if (C > 1) *reinterpret_cast<uint4*>(o + HW) = make_uint4(bg1, bg1, bg1, bg1);
          if (C > 2) *reinterpret_cast<uint4*>(o + 2 * HW) = make_uint4(bg2, bg2, bg2, bg2);
          if (C > 3) *reinterpret_cast<uint4*>(o + 3 * HW) = make_uint4(bg3, bg3, bg3, bg3);
          if (A.depth) {
            float4* d = reinterpret_cast<float4*>(A.depth + lane_pix + boff);
            const float4 one = make_float4(1.f, 1.f, 1.f, 1.f);
            d[0] = one; d[1] = one; d[2] = one; d[3] = one;
          }
          if (WINNER) {
            int4* d = reinterpret_cast<int4*>(A.winner + lane_pix + boff);
            const int4 none = make_int4(-1, -1, -1, -1);
            d[0] = none; d[1] = none; d[2] = none; d[3] = none;
          }
        }
      }
    }
    for (unsigned long long rem = ne; rem != 0ull; rem &= rem - 1ull) {
      const int b = __ffsll((long long)rem) - 1;
      const int by = b / bins_x;
      const int row0 = by * kBinH, col0 = (b - by * bins_x) * kBinW;
      {
        const bool active = (row0 + seg_r < H) && (col0 + seg_x < W);
        const int boff = row0 * W + col0;
        // key tile: depth bits << 32 | (draw order + 1); order 0 = the buffer's previous content
        if (PLAIN) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            unsigned long long k0 = clear_key;
            if (active) k0 = (unsigned long long)(__float_as_uint(A.zbuf[lane_pix + boff + j]) & 0x7fffffffu) << 32;
            keys[j * 32 + lane] = k0;
          }
        } else {
          const uint4 ck = make_uint4(0u, __float_as_uint(1.f), 0u, __float_as_uint(1.f));
#pragma unroll
          for (int j = 0; j < 8; ++j) reinterpret_cast<uint4*>(keys)[j * 32 + lane] = ck;
        }
        __syncwarp();
        for (int w = 0; w < nw; ++w) {
          const uint32_t m = masks[PBR_IX(b * words + w, nbins * words, 24)];
          if (m == 0u) continue;
          // this lane's candidate (triangle w*32+lane if its bit is set) and its bbox-in-bin
          int ax0 = 0, ay0 = 0, bw = 1, npx = 0;
          if ((m >> lane) & 1u) {
            const int t = w * 32 + lane;
            const uint32_t xb = __float_as_uint(S.T3[t].w), yb = __float_as_uint(S.T4[t].x);
            ax0 = max((int)(xb & 0xffffu), col0);
            const int ax1 = min((int)(xb >> 16), col0 + kBinW - 1);
            ay0 = max((int)(yb & 0xffffu), row0);
            const int ay1 = min((int)(yb >> 16), row0 + kBinH - 1);
            const int bh = ay1 - ay0 + 1;
            bw = ax1 - ax0 + 1;
            npx = (bw > 0 && bh > 0) ? bw * bh : 0;
            bw = max(bw, 1);
          }
          const float ibw = __fdividef(1.f, (float)bw);
          int incl = npx;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
          }
          const int total = __shfl_sync(0xffffffffu, incl, 31);
          for (int g0 = 0; g0 < total; g0 += 32) {
            const int g = g0 + lane;
            // owner lane: the first lane whose inclusive area sum exceeds g
            int o = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
              const int probe = __shfl_sync(0xffffffffu, incl, o + step - 1);
              if (probe <= g) o += step;
            }
            const int o_start = __shfl_sync(0xffffffffu, incl - npx, o);
            const int o_ax0 = __shfl_sync(0xffffffffu, ax0, o);
            const int o_ay0 = __shfl_sync(0xffffffffu, ay0, o);
            const int o_bw = __shfl_sync(0xffffffffu, bw, o);
            const float o_ibw = __shfl_sync(0xffffffffu, ibw, o);
            if (g >= total) continue;
            const int t = (int)PBR_IX(w * 32 + o, A.tri_cap, 25);
            const int local = g - o_start;
            // row within the bbox: (local + 0.5) / bw lies at least 0.5 / bw >= 1/64 from an
            // integer, far more than the error of the approximate reciprocal product
            const int ry = (int)(((float)local + 0.5f) * o_ibw);
            const int xx = o_ax0 + local - ry * o_bw, yy = o_ay0 + ry;
            const float px = (float)xx + 0.5f, py = (float)yy + 0.5f;
            const float4 e0 = S.T0[t], e1 = S.T1[t], e2 = S.T2[t], zp = S.T3[t];
            const uint32_t fl = __float_as_uint(S.T4[t].y);
            const float E0 = fmaf(e0.x, px - e0.z, e0.y * (py - e0.w));
            const float E1 = fmaf(e1.x, px - e1.z, e1.y * (py - e1.w));
            const float E2 = fmaf(e2.x, px - e2.z, e2.y * (py - e2.w));
            const bool in0 = (fl & 1u) ? (E0 >= 0.f) : (E0 > 0.f);
            const bool in1 = (fl & 2u) ? (E1 >= 0.f) : (E1 > 0.f);
            const bool in2 = (fl & 4u) ? (E2 >= 0.f) : (E2 > 0.f);
            if (in0 && in1 && in2) {
              const float z = fmaxf(fmaf(zp.x, px, fmaf(zp.y, py, zp.z)), 0.f);
              const int p = (yy - row0) * kBinW + (xx - col0);
              // z >= 0, so its bits order like the values (the mask folds -0 into +0)
              const unsigned long long key =
                  ((unsigned long long)(__float_as_uint(z) & 0x7fffffffu) << 32) | (unsigned)(t + 1);
              atomicMin(&keys[PBR_IX((p & 15) * 32 + (p >> 4), kBinPx, 26)], key);
            }
          }
        }
        __syncwarp();
        // resolve this lane's 16-pixel row segment, four pixels at a time
        if (active) {
          const uint32_t* klo = reinterpret_cast<const uint32_t*>(keys) + 2 * lane;  // low word of key j: klo[64 j]
          uint32_t pr[4], pg[4], pb[4], pa[4];
#pragma unroll
          for (int g = 0; g < 4; ++g) {
            uint32_t col[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const int j = 4 * g + q;
              const uint32_t r = (uint32_t)PBR_IX(klo[64 * j], A.tri_cap + 1, 27);
              const float4* rec = reinterpret_cast<const float4*>(rec4 + 16 * r);
              if (PLAIN && r == 0) {
                col[q] = A.cbuf[lane_pix + boff + j];
              } else if (SMOOTH && (__float_as_uint(rec->y) & 8u)) {
                col[q] = shade_smooth<TEX>(P, S, (int)r - 1, (float)(col0 + seg_x + j) + 0.5f, (float)(row0 + seg_r) + 0.5f);
              } else {
                col[q] = __float_as_uint(rec->z);
              }
            }
            if (PLAIN) {
              reinterpret_cast<uint4*>(A.cbuf + lane_pix + boff)[g] = make_uint4(col[0], col[1], col[2], col[3]);
            } else {
              rgba_to_planes(col[0], col[1], col[2], col[3], pr[g], pg[g], pb[g], pa[g]);
            }
          }
          if (PLAIN || A.depth) {
            float4* zd = reinterpret_cast<float4*>((PLAIN ? A.zbuf : A.depth) + lane_pix + boff);
#pragma unroll
            for (int g = 0; g < 4; ++g) {
              float z4[4];
#pragma unroll
              for (int q = 0; q < 4; ++q) z4[q] = __uint_as_float(klo[64 * (4 * g + q) + 1]);
              zd[g] = make_float4(z4[0], z4[1], z4[2], z4[3]);
            }
          }
          if (!PLAIN) {
            uint8_t* o = lane_out + boff;
            *reinterpret_cast<uint4*>(o) = make_uint4(pr[0], pr[1], pr[2], pr[3]);
            if (C > 1) *reinterpret_cast<uint4*>(o + HW) = make_uint4(pg[0], pg[1], pg[2], pg[3]);
            if (C > 2) *reinterpret_cast<uint4*>(o + 2 * HW) = make_uint4(pb[0], pb[1], pb[2], pb[3]);
            if (C > 3) *reinterpret_cast<uint4*>(o + 3 * HW) = make_uint4(pa[0], pa[1], pa[2], pa[3]);
          }
          if (WINNER) {
            int4* d = reinterpret_cast<int4*>(A.winner + lane_pix + boff);
#pragma unroll
            for (int g = 0; g < 4; ++g) {
              int wi[4];
#pragma unroll
              for (int q = 0; q < 4; ++q)
                wi[q] = __float_as_int(reinterpret_cast<const float4*>(rec4 + 16 * klo[64 * (4 * g + q)])->w);
              d[g] = make_int4(wi[0], wi[1], wi[2], wi[3]);
            }
          }
        }
        __syncwarp();
      }
    }
    __syncwarp();  // the next scene's K1 reuses the key tile as vertex cache
  }
}

// ---------------------------------------------------------------------------

template <bool PL, bool WN, int SH>
static const void* small_fn() {
  return reinterpret_cast<const void*>(&small_kernel<PL, WN, SH>);
}

template <int SH>
static const void* pick_shade(bool plain, bool winner) {
  return plain ? small_fn<true, false, SH>() : (winner ? small_fn<false, true, SH>() : small_fn<false, false, SH>());
}

// shade: 0 = flat meshes only, 1 = smooth meshes, 2 = textured nodes (per-pixel shading)
static const void* pick_small(bool plain, bool winner, int shade) {
  if (plain && winner) return nullptr;
  switch (shade) {
    case 0: return pick_shade<0>(plain, winner);
    case 1: return pick_shade<1>(plain, winner);
    case 2: return pick_shade<2>(plain, winner);
  }
  return nullptr;
}

static int shade_of(const RasterArgs& A) { return A.tex_any ? 2 : (A.smooth_any ? 1 : 0); }

int small_warps() { return kWarps; }

cudaError_t small_set_smem_limit(bool plain, bool winner, int shade, int bytes) {
  const void* f = pick_small(plain, winner, shade);
  if (!f) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

cudaError_t small_occupancy(bool plain, bool winner, int shade, int warps, int smem_bytes, int* blocks_per_sm) {
  const void* f = pick_small(plain, winner, shade);
  if (!f || warps < 1 || warps > kMaxWarps) return cudaErrorInvalidValue;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, warps * 32, smem_bytes);
}

cudaError_t small_launch(bool plain, bool winner, const SceneParams& P, const RasterArgs& A, int warps, int grid,
                         int smem_bytes, cudaStream_t stream) {
  const void* f = pick_small(plain, winner, shade_of(A));
  if (!f || warps < 1 || warps > kMaxWarps) return cudaErrorInvalidValue;
  void* args[] = {const_cast<SceneParams*>(&P), const_cast<RasterArgs*>(&A)};
  return cudaLaunchKernel(f, dim3(grid), dim3(warps * 32), args, (size_t)smem_bytes, stream);
}

int small_max_warps() { return kMaxWarps; }

}  // namespace pbr
