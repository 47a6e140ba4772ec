// pbr_hard.cuh -- the tile kernel (hard rasteriser) template, instantiated
// without texture support in pbr_hard.cu and with it in pbr_hard_tex.cu.
// The pipeline is described at the top of pbr_hard.cu.
#pragma once

#include "pbr_device.cuh"

namespace pbr {

// Whether no triangle of a cluster (bounding sphere cs, normal cone ca) of an
// instance (model matrix rows r0..r2) can be drawn in the rows [ry0, ry1] of
// a W x H image: either every triangle faces away from the eye (HPR poses
// with a positive determinant only: their linear part is a rotation times a
// uniform scale, so normals turn with the axis), or the projection of the
// sphere's box holds no pixel centre of the region.  Conservative: margins
// of 1e-2 of the eye distance on the facing test and 0.01 px on the pixel
// test, and a cluster with a corner behind the eye or a non-finite value is
// kept.
__device__ __forceinline__ bool cluster_culled(float4 cs, float4 ca, float4 r0, float4 r1, float4 r2,
                                               const float* vp, float ex, float ey, float ez, bool eye_ok,
                                               bool hpr, float W, float H, float ry0, float ry1) {
  const float wx = r0.x * cs.x + r0.y * cs.y + r0.z * cs.z + r0.w;
  const float wy = r1.x * cs.x + r1.y * cs.y + r1.z * cs.z + r1.w;
  const float wz = r2.x * cs.x + r2.y * cs.y + r2.z * cs.z + r2.w;
  const float n0 = r0.x * r0.x + r1.x * r1.x + r2.x * r2.x;
  const float n1 = r0.y * r0.y + r1.y * r1.y + r2.y * r2.y;
  const float n2 = r0.z * r0.z + r1.z * r1.z + r2.z * r2.z;
  const float sv2 = hpr ? fmaxf(fmaxf(n0, n1), n2) : n0 + n1 + n2;
  const float R = cs.w * sqrtf(sv2) * 1.0001f + 1e-6f;
  if (eye_ok && hpr && ca.w > 0.f) {
    const float det = r0.x * (r1.y * r2.z - r1.z * r2.y) - r0.y * (r1.x * r2.z - r1.z * r2.x) +
                      r0.z * (r1.x * r2.y - r1.y * r2.x);
    if (det > 0.f) {
      const float ax = r0.x * ca.x + r0.y * ca.y + r0.z * ca.z;
      const float ay = r1.x * ca.x + r1.y * ca.y + r1.z * ca.z;
      const float az = r2.x * ca.x + r2.y * ca.y + r2.z * ca.z;
      const float al = sqrtf(ax * ax + ay * ay + az * az);
      const float ux = wx - ex, uy = wy - ey, uz = wz - ez;
      const float d = sqrtf(ux * ux + uy * uy + uz * uz);
      if (al > 0.f && d > R) {
        // every normal n lies within the cone's half-angle th of the axis, and the directions to the sphere's
        // points within phi of u: dot(n, p - e) >= d cos(phi + th) - R > 0 means every triangle faces away
        const float cphi = (ux * ax + uy * ay + uz * az) / (d * al);
        const float sphi = sqrtf(fmaxf(0.f, 1.f - cphi * cphi));
        const float sth = sqrtf(fmaxf(0.f, 1.f - ca.w * ca.w));
        if (d * (cphi * ca.w - sphi * sth) > R + 1e-2f * d) return true;
      }
    }
  }
  const float cx = vp[0] * wx + vp[1] * wy + vp[2] * wz + vp[3], cy = vp[4] * wx + vp[5] * wy + vp[6] * wz + vp[7];
  const float cw = vp[12] * wx + vp[13] * wy + vp[14] * wz + vp[15];
  float xmin = 3.0e38f, xmax = -3.0e38f, ymin = 3.0e38f, ymax = -3.0e38f;
  bool ok = true;
#pragma unroll
  for (int corner = 0; corner < 8; ++corner) {
    const float sx = (corner & 1) ? R : -R, sy = (corner & 2) ? R : -R, sz = (corner & 4) ? R : -R;
    const float x = cx + vp[0] * sx + vp[1] * sy + vp[2] * sz;
    const float y = cy + vp[4] * sx + vp[5] * sy + vp[6] * sz;
    const float w = cw + vp[12] * sx + vp[13] * sy + vp[14] * sz;
    ok = ok && (w > 1e-6f);
    const float iw = 1.f / w;
    const float px = (x * iw + 1.f) * 0.5f * W, py = (1.f - y * iw) * 0.5f * H;
    xmin = fminf(xmin, px);
    xmax = fmaxf(xmax, px);
    ymin = fminf(ymin, py);
    ymax = fmaxf(ymax, py);
    ok = ok && isfinite(px) && isfinite(py);
  }
  if (!ok) return false;
  // no pixel centre i + 0.5 within [min, max] (0.01 px margin) inside the image's columns and the region's rows
  const float ix0 = fmaxf(ceilf(xmin - 0.51f), 0.f), ix1 = fminf(floorf(xmax - 0.49f), W - 1.f);
  const float iy0 = fmaxf(ceilf(ymin - 0.51f), ry0), iy1 = fminf(floorf(ymax - 0.49f), ry1);
  return ix0 > ix1 || iy0 > iy1;
}

// The count pass for a front triangle in scenes with many small triangles:
// the tests of setup_tri_sv (orientation, box with a pixel centre of the
// region), then, for boxes of at most 16 pixel centres, whether the triangle
// can still take a pixel of the region [p0, p1): it covers a pixel centre there
// (the raster's edge functions and top-left rule) whose key, from the chunks
// drawn so far, holds a larger depth than the triangle's at that centre.  A
// triangle emitted later wins a pixel only with a strictly smaller depth, and
// the arithmetic is the setup's and the raster's, so the triangles this drops
// would not have changed any pixel.  The depth plane (and its division) is
// formed only once a centre is found covered.  Returns 1 to keep, 0 to drop.
__device__ __forceinline__ int count_may_win(const SetupCtx& S, SV v0, SV v1, SV v2,
                                             const unsigned long long* keys, int W, int p0, int p1) {
  float area2 = fmaf(v1.x - v0.x, v2.y - v0.y, -((v2.x - v0.x) * (v1.y - v0.y)));
  if (S.cull) {
    if (!(area2 < 0.f)) return 0;  // back-facing, degenerate or NaN
  } else {
    if (!(area2 < 0.f) && !(area2 > 0.f)) return 0;
  }
  if (area2 < 0.f) {
    SV t = v1; v1 = v2; v2 = t;
    area2 = -area2;
  }
  const float mnx = fminf(fminf(v0.x, v1.x), v2.x), mxx = fmaxf(fmaxf(v0.x, v1.x), v2.x);
  const float mny = fminf(fminf(v0.y, v1.y), v2.y), mxy = fmaxf(fmaxf(v0.y, v1.y), v2.y);
  const float fx0 = fmaxf(ceilf(mnx - 0.501f), 0.f), fx1 = fminf(floorf(mxx - 0.499f), S.W - 1.f);
  const float fy0 = fmaxf(ceilf(mny - 0.501f), S.ry0), fy1 = fminf(floorf(mxy - 0.499f), S.ry1);
  if (!(fx0 <= fx1 && fy0 <= fy1)) return 0;
  const int x0 = (int)fx0, x1 = (int)fx1, y0 = (int)fy0, y1 = (int)fy1;
  if ((x1 - x0 + 1) * (y1 - y0 + 1) > 16) return 1;
  bool tl0, tl1, tl2;
  const float4 e0 = make_edge(v1.x, v1.y, v2.x, v2.y, tl0);
  const float4 e1 = make_edge(v2.x, v2.y, v0.x, v0.y, tl1);
  const float4 e2 = make_edge(v0.x, v0.y, v1.x, v1.y, tl2);
  bool plane = false;
  float zA = 0.f, zB = 0.f, zC = 0.f;
  for (int yy = y0; yy <= y1; ++yy)
    for (int xx = x0; xx <= x1; ++xx) {
      const int q = yy * W + xx;
      if (q < p0 || q >= p1) continue;
      const float px = (float)xx + 0.5f, py = (float)yy + 0.5f;
      const float E0 = fmaf(e0.x, px - e0.z, e0.y * (py - e0.w));
      const float E1 = fmaf(e1.x, px - e1.z, e1.y * (py - e1.w));
      const float E2 = fmaf(e2.x, px - e2.z, e2.y * (py - e2.w));
      const bool in0 = tl0 ? (E0 >= 0.f) : (E0 > 0.f);
      const bool in1 = tl1 ? (E1 >= 0.f) : (E1 > 0.f);
      const bool in2 = tl2 ? (E2 >= 0.f) : (E2 > 0.f);
      if (in0 && in1 && in2) {
        if (!plane) {
          const float ia = 1.f / area2;
          zA = fmaf(e2.x, v2.z, fmaf(e1.x, v1.z, e0.x * v0.z)) * ia;
          zB = fmaf(e2.y, v2.z, fmaf(e1.y, v1.z, e0.y * v0.z)) * ia;
          zC = fmaf(-zB, v0.y, fmaf(-zA, v0.x, v0.z));
          plane = true;
        }
        const float z = fmaxf(fmaf(zA, px, fmaf(zB, py, zC)), 0.f);
        if ((__float_as_uint(z) & 0x7fffffffu) < (uint32_t)(keys[q - p0] >> 32)) return 1;
      }
    }
  return 0;
}

template <int THREADS, bool PLAIN, bool WINNER, bool TEX>
__global__ void __launch_bounds__(THREADS, 512 / THREADS) hard_kernel(const __grid_constant__ SceneParams P,
                                                       const __grid_constant__ RasterArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NW = THREADS / 32;
  const SmemLayout L = smem_layout(A, THREADS, WINNER);
  SetupCtx S;
  S.T0 = reinterpret_cast<float4*>(smem + L.t0);
  S.T1 = reinterpret_cast<float4*>(smem + L.t1);
  S.T2 = reinterpret_cast<float4*>(smem + L.t2);
  S.T3 = reinterpret_cast<float4*>(smem + L.t3);
  S.T4 = reinterpret_cast<float4*>(smem + L.t4);
  S.S0 = reinterpret_cast<float4*>(smem + L.s0);
  S.S1 = reinterpret_cast<float4*>(smem + L.s1);
  S.S2 = reinterpret_cast<float4*>(smem + L.s2);
  S.S3 = reinterpret_cast<float4*>(smem + L.s3);
  S.S4 = reinterpret_cast<float4*>(smem + L.s4);
  S.S5 = reinterpret_cast<float4*>(smem + L.s5);
  S.W = (float)P.W;
  S.H = (float)P.H;
  S.cull = P.cull;
  uint32_t* masks = reinterpret_cast<uint32_t*>(smem + L.masks);
  float4* icache = reinterpret_cast<float4*>(smem + L.icache);
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(smem + L.state);  // [THREADS * kPx]
  int* s_scan = reinterpret_cast<int*>(smem + L.misc);
  float* s_vp = reinterpret_cast<float*>(s_scan + 2 * NW + 8);
  int* s_item = reinterpret_cast<int*>(s_vp + 16);
  uint32_t* s_keep = reinterpret_cast<uint32_t*>(s_item + 4);           // [kInstWords] kept instances of a batch
  int* s_ci = reinterpret_cast<int*>(s_keep + kInstWords);              // [kMaxInstBatch] their batch indices
  int* s_pairs = reinterpret_cast<int*>(smem + L.pairs);  // [kMaxClusterPairs] kept (instance, cluster) pairs
  int2* s_wq = reinterpret_cast<int2*>(smem + L.wq);      // [NW][kWarpQueue] kept triangles waiting to be written

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int2* const wq = s_wq + warp * kWarpQueue;
  int qn = 0;  // this warp's queued kept triangles (the same in every lane)
  const int W = P.W, H = P.H;
  const int HW = W * H;
  const int words = A.tri_cap >> 5;
  const int B = A.bin_px;
  // source triangles per round: one per thread, at most a chunk's records. A round keeps up to 2 * RT records
  // (near-plane splits); one that keeps more than a chunk holds is placed in two halves of at most RT records.
  const int RT = min(THREADS, A.tri_cap);
  const int IS = A.mvp_any ? 8 : 4;  // float4 per cached instance: model rows, colour [, view-projection x model rows]

  for (int it = 0;; ++it) {
    int item;
    if (A.persistent) {
      if (tid == 0) *s_item = atomicAdd(A.work_counter, 1);
      __syncthreads();
      item = *s_item;
      __syncthreads();
    } else {
      item = blockIdx.x + it * gridDim.x;
    }
    if (item >= A.num_items) break;
    const int k = item / A.regions_per_scene;
    const int r = item - k * A.regions_per_scene;
    const int p0 = r * A.region_px;
    const int p1 = min(p0 + A.region_px, HW);
    const int ry0 = p0 / W, ry1 = (p1 - 1) / W;
    S.ry0 = (float)ry0;
    S.ry1 = (float)ry1;
    if (tid < 16) s_vp[tid] = P.vp[(long long)k * 16 + tid];

    // this thread's 16 pixels: flat indices q0 .. q0+15 of the region
    const int q0 = p0 + tid * kPx;
    const int ly = q0 / W, lx = q0 - ly * W;
    const bool active = q0 < p1;

    // Per-pixel state of the region across chunks.  keys[q - p0] (shared
    // memory) = depth bits << 32 | (emit order + 1), where emit order counts
    // the triangles of earlier chunks too: atomicMin keeps the nearest
    // fragment and, for equal depths, the earliest drawn (order 0 = the
    // buffer's previous content).  The colour (and winner id) of each of this
    // lane's 16 pixels stay in registers and are updated after every chunk
    // for the pixels that chunk won.
    uint32_t col[kPx];
    int32_t wid[kPx];
    int tri_count = 0;
    unsigned emit_base = 0;  // triangles emitted by earlier chunks
#pragma unroll
    for (int j = 0; j < kPx; ++j) {
      const int q = q0 + j;
      unsigned long long k0 = (unsigned long long)__float_as_uint(1.f) << 32;
      col[j] = P.bg_packed;
      if (PLAIN && q < p1) {
        k0 = (unsigned long long)(__float_as_uint(A.zbuf[(long long)k * HW + q]) & 0x7fffffffu) << 32;
        col[j] = A.cbuf[(long long)k * HW + q];
      }
      keys[tid * kPx + j] = k0;
      wid[j] = -1;
    }

    // ---- K3: pixel-pair raster of the current chunk, then resolve ---------
    auto flush = [&](bool final_flush) {
      const int T = tri_count;
      const int nw = (T + 31) >> 5;
      const int by_lo = ry0 / B, by_hi = ry1 / B;
      const int nbins = (by_hi - by_lo + 1) * A.bins_x;
      for (int i = tid; i < nbins * words; i += THREADS) masks[i] = 0u;
      __syncthreads();
      // warp-ballot binner
      for (int w = warp; w < nw; w += NW) {
        const int t = w * 32 + lane;
        int bx0 = 1 << 20, bx1 = -1, by0 = 1 << 20, by1 = -1;
        if (t < T) {
          const uint32_t xb = __float_as_uint(S.T3[t].w), yb = __float_as_uint(S.T4[t].x);
          bx0 = (int)(xb & 0xffffu) / B;
          bx1 = (int)(xb >> 16) / B;
          by0 = (int)(yb & 0xffffu) / B - by_lo;
          by1 = (int)(yb >> 16) / B - by_lo;
        }
        const int ux0 = __reduce_min_sync(0xffffffffu, bx0), ux1 = __reduce_max_sync(0xffffffffu, bx1);
        const int uy0 = __reduce_min_sync(0xffffffffu, by0), uy1 = __reduce_max_sync(0xffffffffu, by1);
        for (int by = uy0; by <= uy1; ++by)
          for (int bx = ux0; bx <= ux1; ++bx) {
            const bool bit = (bx >= bx0) && (bx <= bx1) && (by >= by0) && (by <= by1);
            const uint32_t m = __ballot_sync(0xffffffffu, bit);
            if (lane == 0) masks[PBR_IX((by * A.bins_x + bx) * words + w, A.max_region_bins * words, 11)] = m;
          }
      }
      __syncthreads();
      // (bin, mask word) pairs warp-strided, so that a few crowded bins do not hold the other warps idle; per
      // pair, the candidates' (triangle, pixel) pairs inside the bin are packed 32 per pass (prefix sum of the
      // clipped bbox areas).  Fragments of different warps meet only in the atomicMin on the pixel keys.
      for (int bw_item = warp; bw_item < nbins * nw; bw_item += NW) {
        const int b = bw_item / nw, w = bw_item - b * nw;
        {
          const uint32_t m = masks[PBR_IX(b * words + w, A.max_region_bins * words, 11)];
          if (m == 0u) continue;
          const int bry = b / A.bins_x, bcx = b - bry * A.bins_x;
          const int bx0 = bcx * B, bx1 = min(bx0 + B, W) - 1;
          const int by0 = max((by_lo + bry) * B, ry0), by1 = min((by_lo + bry) * B + B - 1, ry1);
          int ax0 = 0, ay0 = 0, bw = 1, npx = 0;
          if ((m >> lane) & 1u) {
            const int t = (int)PBR_IX(w * 32 + lane, A.tri_cap, 9);
            const uint32_t xb = __float_as_uint(S.T3[t].w), yb = __float_as_uint(S.T4[t].x);
            ax0 = max((int)(xb & 0xffffu), bx0);
            const int ax1 = min((int)(xb >> 16), bx1);
            ay0 = max((int)(yb & 0xffffu), by0);
            const int ay1 = min((int)(yb >> 16), by1);
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
            const int t = (int)PBR_IX(w * 32 + o, A.tri_cap, 9);
            const int local = g - o_start;
            // (local + 0.5) / bw lies at least 0.5 / bw >= 1/64 from an integer
            const int ry = (int)(((float)local + 0.5f) * o_ibw);
            const int xx = o_ax0 + local - ry * o_bw, yy = o_ay0 + ry;
            const int q = yy * W + xx;
            if (q < p0 || q >= p1) continue;  // the region starts or ends inside a row
            (void)PBR_IX(q - p0, THREADS * kPx, 13);
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
              // z >= 0, so its bits order like the values (the mask folds -0 into +0)
              const unsigned long long key = ((unsigned long long)(__float_as_uint(z) & 0x7fffffffu) << 32) |
                                             (unsigned)(emit_base + (unsigned)t + 1u);
              atomicMin(&keys[q - p0], key);
            }
          }
        }
      }
      __syncthreads();
      // resolve the pixels this chunk won
      const float py_a = (float)ly + 0.5f;
#pragma unroll
      for (int j = 0; j < kPx; ++j) {
        const uint32_t lo = (uint32_t)keys[tid * kPx + j];
        if (q0 + j < p1 && lo > emit_base) {
          const int t = (int)PBR_IX((int)(lo - emit_base) - 1, A.tri_cap, 10);
          const float4 meta = S.T4[t];
          if (__float_as_uint(meta.y) & 8u) {
            int x = lx + j;
            float py = py_a;
            while (x >= W) { x -= W; py += 1.f; }
            col[j] = shade_smooth<TEX>(P, S, t, (float)x + 0.5f, py);
          } else {
            col[j] = __float_as_uint(meta.z);
          }
          if (WINNER) wid[j] = __float_as_int(meta.w);
        }
      }
      emit_base += (unsigned)T;
      if (final_flush && active) {
        const bool full = (q0 + kPx <= p1);
        float zb[kPx];
#pragma unroll
        for (int j = 0; j < kPx; ++j) zb[j] = __uint_as_float((uint32_t)(keys[tid * kPx + j] >> 32));
        if (PLAIN) {
          float* zdst = A.zbuf + (long long)k * HW + q0;
          uint32_t* cdst = A.cbuf + (long long)k * HW + q0;
#pragma unroll
          for (int j = 0; j < kPx; ++j)
            if (q0 + j < p1) { zdst[j] = zb[j]; cdst[j] = col[j]; }
        } else {
          const bool vec = full && ((HW & 15) == 0);
          for (int c = 0; c < P.C; ++c) {
            uint8_t* dst = A.out + ((long long)k * P.C + c) * HW + q0;
            const int sh = 8 * c;
            if (vec) {
              uint32_t wv[4];
#pragma unroll
              for (int g = 0; g < 4; ++g) {
                wv[g] = ((col[4 * g + 0] >> sh) & 0xffu) | (((col[4 * g + 1] >> sh) & 0xffu) << 8) |
                        (((col[4 * g + 2] >> sh) & 0xffu) << 16) | (((col[4 * g + 3] >> sh) & 0xffu) << 24);
              }
              *reinterpret_cast<uint4*>(dst) = make_uint4(wv[0], wv[1], wv[2], wv[3]);
            } else {
#pragma unroll
              for (int j = 0; j < kPx; ++j)
                if (q0 + j < p1) dst[j] = (uint8_t)((col[j] >> sh) & 0xffu);
            }
          }
          if (A.depth) {
            float* dd = A.depth + (long long)k * HW + q0;
            if (full && ((HW & 3) == 0)) {
#pragma unroll
              for (int g = 0; g < 4; ++g)
                *reinterpret_cast<float4*>(dd + 4 * g) = make_float4(zb[4 * g], zb[4 * g + 1], zb[4 * g + 2], zb[4 * g + 3]);
            } else {
#pragma unroll
              for (int j = 0; j < kPx; ++j)
                if (q0 + j < p1) dd[j] = zb[j];
            }
          }
          if (WINNER) {
            int32_t* wd = A.winner + (long long)k * HW + q0;
#pragma unroll
            for (int j = 0; j < kPx; ++j)
              if (q0 + j < p1) wd[j] = wid[j];
          }
        }
      }
      tri_count = 0;
      __syncthreads();
    };

    // ---- K1 / K2: walk nodes and instances in draw order -----------------
    // Instance batches of up to icap instances (model matrices in shared
    // memory); then rounds of THREADS source triangles, one per thread: the
    // thread transforms its triangle's three vertices itself (no vertex cache,
    // no per-instance barriers), culls and rejects triangles that cover no
    // pixel centre, and the survivors are compacted in draw order with one
    // barrier per round (warp prefix sums + per-warp totals in shared memory).
    __syncthreads();  // s_vp visible
    const float vp0 = s_vp[0], vp1 = s_vp[1], vp2 = s_vp[2], vp3 = s_vp[3];
    const float vp4 = s_vp[4], vp5 = s_vp[5], vp6 = s_vp[6], vp7 = s_vp[7];
    const float vp8 = s_vp[8], vp9 = s_vp[9], vp10 = s_vp[10], vp11 = s_vp[11];
    const float vp12 = s_vp[12], vp13 = s_vp[13], vp14 = s_vp[14], vp15 = s_vp[15];
    // clip coordinates of mesh vertex vi of an instance (model rows r0..r2): world position, then the
    // view-projection (meshes below kMvpMinTris triangles; larger ones use the cached VP * M rows)
    auto clip_of = [&](const MeshDesc& me, int vi, float4 r0, float4 r1, float4 r2) -> float4 {
      vi = (int)PBR_IX(vi, me.nv, 5);
      const float ox = me.pos[3 * vi], oy = me.pos[3 * vi + 1], oz = me.pos[3 * vi + 2];
      const float wx = r0.x * ox + r0.y * oy + r0.z * oz + r0.w;
      const float wy = r1.x * ox + r1.y * oy + r1.z * oz + r1.w;
      const float wz = r2.x * ox + r2.y * oy + r2.z * oz + r2.w;
      float4 o;
      o.x = vp0 * wx + vp1 * wy + vp2 * wz + vp3;
      o.y = vp4 * wx + vp5 * wy + vp6 * wz + vp7;
      o.z = vp8 * wx + vp9 * wy + vp10 * wz + vp11;
      o.w = vp12 * wx + vp13 * wy + vp14 * wz + vp15;
      return o;
    };
    // The eye: the point where rows 0, 1 and 3 of the view-projection vanish (the centre of a perspective
    // projection); for the clusters' facing test.  A singular system (no centre of projection) disables it.
    float ex = 0.f, ey = 0.f, ez = 0.f;
    bool eye_ok = false;
    if (A.cl_any) {
      const float bcx = vp5 * vp14 - vp6 * vp13, bcy = vp6 * vp12 - vp4 * vp14, bcz = vp4 * vp13 - vp5 * vp12;
      const float cax = vp13 * vp2 - vp14 * vp1, cay = vp14 * vp0 - vp12 * vp2, caz = vp12 * vp1 - vp13 * vp0;
      const float abx = vp1 * vp6 - vp2 * vp5, aby = vp2 * vp4 - vp0 * vp6, abz = vp0 * vp5 - vp1 * vp4;
      const float det = vp0 * bcx + vp1 * bcy + vp2 * bcz;
      if (fabsf(det) > 1e-20f) {
        const float id = 1.f / det;
        ex = (-vp3 * bcx - vp7 * cax - vp15 * abx) * id;
        ey = (-vp3 * bcy - vp7 * cay - vp15 * aby) * id;
        ez = (-vp3 * bcz - vp7 * caz - vp15 * abz) * id;
        eye_ok = isfinite(ex) && isfinite(ey) && isfinite(ez);
      }
    }
    int parity = 0;
    for (int n = A.node_begin; n < A.node_end; ++n) {
      const NodeDesc& nd = P.nodes[n];
      const MeshDesc& me = P.meshes[nd.mesh];
      int cnt = nd.counts ? nd.counts[k] : nd.ips;
      cnt = max(0, min(cnt, nd.ips));
      const int nt = me.nt;
      if (cnt == 0 || nt == 0) continue;
      const bool textured = TEX && nd.tex != nullptr;  // textured triangles are shaded per pixel
      const bool smooth = me.smooth != 0 || textured;
      // meshes of kMvpMinTris+ triangles transform their vertices with the instance's VP * M in one step
      const bool use_mvp = A.mvp_any && nt >= kMvpMinTris;
      for (int b0 = 0; b0 < cnt; b0 += A.icap) {
        const int nbc = min(A.icap, cnt - b0);
        __syncthreads();  // the previous batch's triangles are done with icache
        for (int i = tid; i < nbc; i += THREADS) {
          const long long id =
              PBR_IX(nd.shared ? (long long)(b0 + i) : (long long)k * nd.ips + b0 + i,
                     nd.shared ? (long long)nd.ips : (long long)P.N * nd.ips, 12);
          float m[12];
          build_model(nd, id, m);
          if (r == 0) write_back_bound(nd, id);
          (void)PBR_IX(i, A.icap, 1);
          icache[i * IS + 0] = make_float4(m[0], m[1], m[2], m[3]);
          icache[i * IS + 1] = make_float4(m[4], m[5], m[6], m[7]);
          icache[i * IS + 2] = make_float4(m[8], m[9], m[10], m[11]);
          const float* cc = nd.color + id * 4;
          icache[i * IS + 3] = make_float4(cc[0], cc[1], cc[2], cc[3]);
          if (use_mvp) {
            // rows of VP * M (M's last row 0 0 0 1), so that a vertex takes 12 FMAs to clip space
            const float vpr[16] = {vp0, vp1, vp2, vp3, vp4, vp5, vp6, vp7, vp8, vp9, vp10, vp11, vp12, vp13, vp14, vp15};
#pragma unroll
            for (int rr = 0; rr < 4; ++rr) {
              const float a0 = vpr[4 * rr], a1 = vpr[4 * rr + 1], a2 = vpr[4 * rr + 2], a3 = vpr[4 * rr + 3];
              icache[i * IS + 4 + rr] = make_float4(fmaf(a2, m[8], fmaf(a1, m[4], a0 * m[0])),
                                                    fmaf(a2, m[9], fmaf(a1, m[5], a0 * m[1])),
                                                    fmaf(a2, m[10], fmaf(a1, m[6], a0 * m[2])),
                                                    fmaf(a2, m[11], fmaf(a1, m[7], fmaf(a0, m[3], a3))));
            }
          }
        }
        __syncthreads();
        // Instances whose bounding sphere projects entirely above or below this region's rows,
        // or left or right of the image, cannot cover a pixel centre here: the batch is
        // compacted to the others, in draw order.  The projection of the sphere's world-space
        // box (eight corners, all in front of the camera, else the instance is kept) bounds the
        // projection of the mesh.
        const bool can_cull = me.bound.w > 0.f;
        int nb = nbc;
        if (can_cull) {
          for (int i0c = 0; i0c < nbc; i0c += THREADS) {
            const int i = i0c + tid;
            bool keep = false;
            if (i < nbc) {
              const float4 r0 = icache[i * IS + 0], r1 = icache[i * IS + 1], r2 = icache[i * IS + 2];
              const float4 b = me.bound;
              const float wx = r0.x * b.x + r0.y * b.y + r0.z * b.z + r0.w;
              const float wy = r1.x * b.x + r1.y * b.y + r1.z * b.z + r1.w;
              const float wz = r2.x * b.x + r2.y * b.y + r2.z * b.z + r2.w;
              // world radius: mesh radius times the largest singular value of the linear part, which is
              // the (common) column norm of a rotation times a uniform scale (HPR mode); other modes may
              // hold any matrix, bounded by its Frobenius norm
              const float n0 = r0.x * r0.x + r1.x * r1.x + r2.x * r2.x;
              const float n1 = r0.y * r0.y + r1.y * r1.y + r2.y * r2.y;
              const float n2 = r0.z * r0.z + r1.z * r1.z + r2.z * r2.z;
              const float sv2 = nd.mode == kModeHpr ? fmaxf(fmaxf(n0, n1), n2) : n0 + n1 + n2;
              const float R = b.w * sqrtf(sv2) * 1.0001f + 1e-6f;
              const float cx = vp0 * wx + vp1 * wy + vp2 * wz + vp3, cy = vp4 * wx + vp5 * wy + vp6 * wz + vp7;
              const float cw = vp12 * wx + vp13 * wy + vp14 * wz + vp15;
              float xmin = 3.0e38f, xmax = -3.0e38f, ymin = 3.0e38f, ymax = -3.0e38f;
              bool front = true;
#pragma unroll
              for (int corner = 0; corner < 8; ++corner) {
                const float sx = (corner & 1) ? R : -R, sy = (corner & 2) ? R : -R, sz = (corner & 4) ? R : -R;
                const float x = cx + vp0 * sx + vp1 * sy + vp2 * sz;
                const float y = cy + vp4 * sx + vp5 * sy + vp6 * sz;
                const float w = cw + vp12 * sx + vp13 * sy + vp14 * sz;
                front = front && (w > 1e-6f);
                const float iw = 1.f / w;
                const float px = (x * iw + 1.f) * 0.5f * S.W, py = (1.f - y * iw) * 0.5f * S.H;
                xmin = fminf(xmin, px);
                xmax = fmaxf(xmax, px);
                ymin = fminf(ymin, py);
                ymax = fmaxf(ymax, py);
              }
              // two pixels of slack; a NaN anywhere keeps the instance (every comparison is false)
              const bool out = front && (ymax < S.ry0 - 2.f || ymin > S.ry1 + 3.f || xmax < -2.f || xmin > S.W + 2.f);
              keep = !out;
            }
            const uint32_t bal = __ballot_sync(0xffffffffu, keep);
            if (lane == 0 && i0c + warp * 32 < kMaxInstBatch) s_keep[(i0c >> 5) + warp] = bal;
          }
          __syncthreads();
          int total_keep = 0;
          const int words_b = (nbc + 31) >> 5;
          for (int wd = 0; wd < words_b; ++wd) total_keep += __popc(s_keep[wd]);
          for (int i = tid; i < nbc; i += THREADS) {
            const uint32_t word = s_keep[i >> 5];
            if ((word >> (i & 31)) & 1u) {
              int slot = __popc(word & ((1u << (i & 31)) - 1u));
              for (int wd = 0; wd < (i >> 5); ++wd) slot += __popc(s_keep[wd]);
              s_ci[PBR_IX(slot, kMaxInstBatch, 2)] = i;
            }
          }
          nb = total_keep;
          __syncthreads();
        }
        // Meshes with clusters: the kept instances in sub-batches whose (instance, cluster) pairs fit the pair
        // list; each pair is tested (cluster_culled) and the survivors compacted in draw order, then the
        // triangle rounds run over the kept pairs' triangles only.  The culled clusters hold no triangle that
        // would be drawn, so the output is the same as without clusters.
        // clip coordinates of source triangle (i0, i1, i2) of batch instance li
        auto clip3 = [&](int li, int i0, int i1, int i2, float4 cv[3]) {
          if (use_mvp) {
            const float4 m0 = icache[li * IS + 4], m1 = icache[li * IS + 5], m2 = icache[li * IS + 6];
            const float4 m3 = icache[li * IS + 7];
            const int iv[3] = {i0, i1, i2};
#pragma unroll
            for (int q = 0; q < 3; ++q) {
              const int vi = (int)PBR_IX(iv[q], me.nv, 5);
              const float ox = me.pos[3 * vi], oy = me.pos[3 * vi + 1], oz = me.pos[3 * vi + 2];
              cv[q] = make_float4(fmaf(m0.x, ox, fmaf(m0.y, oy, fmaf(m0.z, oz, m0.w))),
                                  fmaf(m1.x, ox, fmaf(m1.y, oy, fmaf(m1.z, oz, m1.w))),
                                  fmaf(m2.x, ox, fmaf(m2.y, oy, fmaf(m2.z, oz, m2.w))),
                                  fmaf(m3.x, ox, fmaf(m3.y, oy, fmaf(m3.z, oz, m3.w))));
            }
          } else {
            const float4 r0 = icache[li * IS + 0], r1 = icache[li * IS + 1], r2 = icache[li * IS + 2];
            cv[0] = clip_of(me, i0, r0, r1, r2);
            cv[1] = clip_of(me, i1, r0, r1, r2);
            cv[2] = clip_of(me, i2, r0, r1, r2);
          }
        };
        // Kept triangles wait in their warp's queue -- (source triangle; instance, slot count, front, slot) -- and
        // are set up 32 at a time, one per lane, when the queue holds 32, before a chunk flush and at the end of
        // the instance batch: a round's few survivors no longer hold most warps in the long write path.  The
        // writer repeats the vertex transform (the same arithmetic, so the same screen coordinates) and fills
        // exactly the slots the count reserved (an empty record where it does not emit the triangle).
        auto write_queued = [&](int2 e) {
          const int ti = (int)PBR_IX(e.x, nt, 4), li = (int)PBR_IX(e.y & 0xff, A.icap, 1);
          const int c = (e.y >> 8) & 3, slot = e.y >> 11;
          const bool front = ((e.y >> 10) & 1) != 0;
          const int i0 = me.idx[3 * ti], i1 = me.idx[3 * ti + 1], i2 = me.idx[3 * ti + 2];
          float4 cv[3];
          clip3(li, i0, i1, i2, cv);
          const float4 r0 = icache[li * IS + 0], r1 = icache[li * IS + 1], r2 = icache[li * IS + 2];
          const float4 col = icache[li * IS + 3];
          const int draw_id = (nd.rank_base + b0 + li) * P.max_tris + ti;
          // world normals: the provoking vertex's for flat meshes (the three are identical), all three if smooth
          float4 nv[3];
          const int iv[3] = {i0, i1, i2};
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            if (q == 0 || smooth) {
              const int vi = (int)PBR_IX(iv[q], me.nv, 6);
              const float ax = me.nrm[3 * vi], ay = me.nrm[3 * vi + 1], az = me.nrm[3 * vi + 2];
              const float nx = r0.x * ax + r0.y * ay + r0.z * az;
              const float ny = r1.x * ax + r1.y * ay + r1.z * az;
              const float nz = r2.x * ax + r2.y * ay + r2.z * az;
              const float l2 = nx * nx + ny * ny + nz * nz;
              const float inv = l2 > 0.f ? rsqrtf(l2) : 0.f;
              nv[q] = make_float4(nx * inv, ny * inv, nz * inv, 0.f);
            } else {
              nv[q] = nv[0];
            }
          }
          TexIn tx;
          if (textured) {
            tx.t0 = mesh_uv(me, i0);
            tx.t1 = mesh_uv(me, i1);
            tx.t2 = mesh_uv(me, i2);
            tx.node = n;
          }
          if (front) {
            SV sv[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) sv[q] = to_screen(cv[q], S.W, S.H);
            if (!setup_tri_sv<true>(P, S, sv[0], nv[0], sv[1], nv[1], sv[2], nv[2], slot, col, draw_id, smooth, tx))
              write_empty(S, slot);
          } else {
            clip_tri<true>(P, S, cv[0], nv[0], cv[1], nv[1], cv[2], nv[2], i0, i1, i2, slot, col, draw_id, smooth, tx,
                           c);
          }
        };
        // the warp's last m queued triangles, one per lane (warp-uniform m <= 32)
        auto drain = [&](int m) {
          __syncwarp();
          if (lane < m) write_queued(wq[qn - m + lane]);
          __syncwarp();
          qn -= m;
        };
        const bool use_cl = A.cl_any && me.clusters != nullptr && me.ncl > 0;
        const int per_sub = use_cl ? max(1, kMaxClusterPairs / me.ncl) : max(nb, 1);
        for (int s0 = 0; s0 < nb; s0 += per_sub) {
        const int ns = min(per_sub, nb - s0);
        int nkept = 0;
        if (use_cl) {
          __syncthreads();  // the previous sub-batch's triangles are done with the pair list
          const float vpa[16] = {vp0, vp1, vp2, vp3, vp4, vp5, vp6, vp7, vp8, vp9, vp10, vp11, vp12, vp13, vp14, vp15};
          for (int p0 = 0; p0 < ns * me.ncl; p0 += THREADS) {
            const int p = p0 + tid;
            bool keep = false;
            int li = 0, c = 0;
            if (p < ns * me.ncl) {
              const int lv = p / me.ncl;
              c = p - lv * me.ncl;
              li = (int)PBR_IX(can_cull ? s_ci[PBR_IX(s0 + lv, kMaxInstBatch, 2)] : s0 + lv, A.icap, 1);
              c = (int)PBR_IX(c, me.ncl, 7);
              keep = !cluster_culled(me.clusters[2 * c], me.clusters[2 * c + 1], icache[li * IS + 0],
                                     icache[li * IS + 1], icache[li * IS + 2], vpa, ex, ey, ez, eye_ok,
                                     nd.mode == kModeHpr, S.W, S.H, S.ry0, S.ry1);
            }
            const uint32_t bal = __ballot_sync(0xffffffffu, keep);
            int* wc = s_scan + parity * NW;
            if (lane == 0) wc[warp] = __popc(bal);
            __syncthreads();
            int before = 0, total = 0;
#pragma unroll
            for (int w = 0; w < NW; ++w) {
              const int v = wc[w];
              before += w < warp ? v : 0;
              total += v;
            }
            parity ^= 1;
            if (keep) s_pairs[PBR_IX(nkept + before + __popc(bal & ((1u << lane) - 1u)), kMaxClusterPairs, 3)] =
                (li << 16) | c;
            nkept += total;
          }
          __syncthreads();
        }
        const int total_t = use_cl ? nkept * kClusterTris : nb * nt;
        for (int t0 = 0; t0 < total_t; t0 += RT) {
          const int rem = min(RT, total_t - t0);
          int c = 0, li = 0, ti = 0, i0 = 0, i1 = 0, i2 = 0;
          float4 cv[3];
          SV sv[3];
          bool front = false;
          bool has = tid < rem;
          if (has) {
            const int t = t0 + tid;
            if (use_cl) {
              const int pr = s_pairs[PBR_IX(t / kClusterTris, kMaxClusterPairs, 3)];
              li = pr >> 16;
              ti = (pr & 0xffff) * kClusterTris + (t & (kClusterTris - 1));
              has = ti < nt;  // the mesh's last cluster may hold fewer triangles
            } else {
              li = t / nt;
              ti = t - li * nt;
              if (can_cull) li = s_ci[PBR_IX(li, kMaxInstBatch, 2)];
            }
            if (has) {
              li = (int)PBR_IX(li, A.icap, 1);
              ti = (int)PBR_IX(ti, nt, 4);
            }
          }
          if (has) {
            i0 = me.idx[3 * ti];
            i1 = me.idx[3 * ti + 1];
            i2 = me.idx[3 * ti + 2];
            clip3(li, i0, i1, i2, cv);
            const float d0 = cv[0].z + cv[0].w, d1 = cv[1].z + cv[1].w, d2 = cv[2].z + cv[2].w;
            front = d0 >= 0.f && d1 >= 0.f && d2 >= 0.f;
            const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
            if (front) {
#pragma unroll
              for (int q = 0; q < 3; ++q) sv[q] = to_screen(cv[q], S.W, S.H);
              c = A.win_test ? count_may_win(S, sv[0], sv[1], sv[2], keys, W, p0, p1)
                             : setup_tri_sv<false>(P, S, sv[0], z4, sv[1], z4, sv[2], z4, 0, z4, 0, smooth);
            } else if (!(d0 < 0.f && d1 < 0.f && d2 < 0.f)) {
              c = clip_tri<false>(P, S, cv[0], z4, cv[1], z4, cv[2], z4, i0, i1, i2, 0, z4, 0, smooth);
            }
          }
          // draw-order compaction: warp prefix sum, then the totals of the warps before this one (one barrier)
          auto compact = [&](int n, int& incl_o, int& before_o, int& total_o) {
            int incl = n;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
              const int y = __shfl_up_sync(0xffffffffu, incl, o);
              if (lane >= o) incl += y;
            }
            int* wcnt = s_scan + parity * NW;
            if (lane == 31) wcnt[warp] = incl;
            __syncthreads();
            int before = 0, total = 0;
#pragma unroll
            for (int w = 0; w < NW; ++w) {
              const int v = wcnt[w];
              before += w < warp ? v : 0;
              total += v;
            }
            parity ^= 1;
            incl_o = incl;
            before_o = before;
            total_o = total;
          };
          // the kept triangles' slots (the chunk flushed first, its queued triangles written, when they do not
          // fit), then into the warp's queue
          auto place = [&](int n, int incl, int before, int total) {
            if (tri_count + total > A.tri_cap) {
              if (qn > 0) drain(qn);
              flush(false);
            }
            const uint32_t kept = __ballot_sync(0xffffffffu, n > 0);
            if (n > 0) {
              const int slot0 = tri_count + before + incl - n, last = slot0 + n - 1;
              const int slot = (int)PBR_IX(last, A.tri_cap, 8) == last ? slot0 : 0;
              const int packed = li | (n << 8) | (front ? 1 << 10 : 0) | (slot << 11);
              wq[qn + __popc(kept & ((1u << lane) - 1u))] = make_int2(ti, packed);
            }
            qn += __popc(kept);
            if (qn >= 32) drain(32);
            tri_count += total;
          };
          int incl, before, total;
          compact(c, incl, before, total);
          // More kept records than a chunk holds (many near-plane splits): the round's two halves in draw order,
          // RT / 2 source triangles each, so at most RT <= tri_cap records each.  One copy of place() serves both
          // cases (it inlines the write pass; more copies cost instruction-cache misses in every launch).
          const int pieces = total <= A.tri_cap ? 1 : 2;
#pragma unroll 1
          for (int h = 0; h < pieces; ++h) {
            int n = c;
            if (pieces == 2) {
              n = ((tid < (RT >> 1)) == (h == 0)) ? c : 0;
              compact(n, incl, before, total);
            }
            place(n, incl, before, total);
          }
        }
        }  // sub-batches
        if (qn > 0) drain(qn);  // before the next batch replaces the instance matrices
      }
    }
    flush(true);
  }
}

}  // namespace pbr
