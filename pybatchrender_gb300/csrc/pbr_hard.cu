// pbr_hard.cu -- hard rasteriser for sm_103a.
//
// One CTA processes one work item = (scene k, pixel region r), where a region
// is threads*16 consecutive pixels of the scene's W x H image (the whole image
// for 64x64 at 256 threads).  Per item the CTA runs the whole pipeline in
// shared memory, with no global scratch:
//
//   K1  instance + vertex stage: per instance M = [R(hpr)*s | t]
//       (renderer/shader_context.py:47-84, renderer/node.py:116-126), then
//       clip = VP[k] * M * v and n = normalize(mat3(M) n)  (shaders/basic.vert:29-53)
//   K2  triangle setup: near-plane clip, GL viewport transform into the scene's
//       own image (basic.vert:45-52 + the atlas flip of renderer/frame_grabber.py:105),
//       back-face cull, bbox, watertight FP32 edge functions with the top-left
//       rule, depth plane, flat shading resolved per triangle; survivors are
//       compacted in draw order with a block prefix sum into a shared-memory
//       triangle list ("chunk")
//       + warp-ballot binner: one __ballot_sync per (32 triangles, bin) builds
//       the per-bin triangle bit masks
//   K3  tile raster: every lane owns 16 consecutive pixels, iterates the set
//       bits of its warp's bins in ascending (= draw) order, depth-tests
//       strict-less, then resolves the winner's colour (basic.frag:20-39) and
//       writes each channel with one 128-bit store straight into the
//       [N,C,H,W] output (no framebuffer, no readback, no rearrange copy).
//
// Scenes whose triangles overflow the chunk are processed chunk by chunk with
// the per-pixel depth/colour kept in shared memory between chunks.
#include <cstdio>

#include "pbr_device.cuh"
#include "pbr_launch.h"

namespace pbr {

template <int THREADS>
__device__ __forceinline__ int block_exclusive_scan(int v, int* s_warp, int& total) {
  constexpr int NW = THREADS / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = lane < NW ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < NW) s_warp[lane] = w;
  }
  __syncthreads();
  const int prefix = warp > 0 ? s_warp[warp - 1] : 0;
  total = s_warp[NW - 1];
  __syncthreads();
  return prefix + x - v;
}

template <int THREADS, bool PLAIN, bool WINNER>
__global__ void __launch_bounds__(THREADS) hard_kernel(const __grid_constant__ SceneParams P,
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
  S.W = (float)P.W;
  S.H = (float)P.H;
  S.cull = P.cull;
  uint32_t* masks = reinterpret_cast<uint32_t*>(smem + L.masks);
  float4* vcache = reinterpret_cast<float4*>(smem + L.vcache);
  float4* icache = reinterpret_cast<float4*>(smem + L.icache);
  float* st_z = reinterpret_cast<float*>(smem + L.state);
  uint32_t* st_c = reinterpret_cast<uint32_t*>(smem + L.state) + THREADS * kPx;
  int32_t* st_w = reinterpret_cast<int32_t*>(smem + L.state) + 2 * THREADS * kPx;
  int* s_scan = reinterpret_cast<int*>(smem + L.misc);
  float* s_vp = reinterpret_cast<float*>(s_scan + NW + 8);
  int* s_item = reinterpret_cast<int*>(s_vp + 16);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int W = P.W, H = P.H;
  const int HW = W * H;
  const int words = A.tri_cap >> 5;
  const int B = A.bin_px;
  const int RT = min(THREADS, A.tri_cap >> 1);

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
    const int lane_y1 = min((q0 + kPx - 1) / W, H - 1);
    const int lane_x0 = (lane_y1 == ly) ? lx : 0;
    const int lane_x1 = (lane_y1 == ly) ? lx + kPx - 1 : W - 1;
    const bool active = q0 < p1;

    float zb[kPx];
    int win[kPx];
    int nflush = 0;
    int tri_count = 0;

    // ---- K3 + resolve for the current chunk ------------------------------
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
            if (lane == 0) masks[(by * A.bins_x + bx) * words + w] = m;
          }
      }
      // pixel state in
#pragma unroll
      for (int j = 0; j < kPx; ++j) {
        win[j] = -1;
        if (nflush == 0) {
          if (PLAIN) {
            const int q = q0 + j;
            zb[j] = (q < p1) ? A.zbuf[(long long)k * HW + q] : 1.f;
          } else {
            zb[j] = 1.f;
          }
        } else {
          zb[j] = st_z[j * THREADS + tid];
        }
      }
      __syncthreads();
      // the warp's bins: rows of its 32*16 pixels, columns it touches
      const int wq0 = p0 + warp * 32 * kPx;
      const int wq1 = min(wq0 + 32 * kPx, p1) - 1;
      int wbx0 = 0, wbx1 = -1, wby0 = 0, wby1 = -1;
      if (wq0 < p1) {
        const int wy0 = wq0 / W, wy1 = wq1 / W;
        wby0 = wy0 / B - by_lo;
        wby1 = wy1 / B - by_lo;
        if (wy0 == wy1) {
          wbx0 = (wq0 - wy0 * W) / B;
          wbx1 = (wq1 - wy1 * W) / B;
        } else {
          wbx0 = 0;
          wbx1 = A.bins_x - 1;
        }
      }
      const int wnbx = wbx1 - wbx0 + 1;
      const int wnb = (wby1 >= wby0) ? (wby1 - wby0 + 1) * wnbx : 0;
      const float py_a = (float)ly + 0.5f;
      for (int w = 0; w < nw; ++w) {
        uint32_t m = 0u;
        for (int b = lane; b < wnb; b += 32) {
          const int by = wby0 + b / wnbx, bx = wbx0 + b % wnbx;
          m |= masks[(by * A.bins_x + bx) * words + w];
        }
        m = __reduce_or_sync(0xffffffffu, m);
        while (m) {
          const int j0 = __ffs(m) - 1;
          m &= m - 1u;
          const int t = w * 32 + j0;
          const float4 zp = S.T3[t];
          const float4 meta = S.T4[t];
          const uint32_t xb = __float_as_uint(zp.w), yb = __float_as_uint(meta.x);
          const int tx0 = (int)(xb & 0xffffu), tx1 = (int)(xb >> 16);
          const int ty0 = (int)(yb & 0xffffu), ty1 = (int)(yb >> 16);
          if (!active || ty1 < ly || ty0 > lane_y1 || tx1 < lane_x0 || tx0 > lane_x1) continue;
          const float4 e0 = S.T0[t], e1 = S.T1[t], e2 = S.T2[t];
          const uint32_t fl = __float_as_uint(meta.y);
          const bool tl0 = fl & 1u, tl1 = fl & 2u, tl2 = fl & 4u;
#pragma unroll
          for (int j = 0; j < kPx; ++j) {
            int x = lx + j;
            float py = py_a;
            if (x >= W) {
              x -= W;
              py += 1.f;
              while (x >= W) { x -= W; py += 1.f; }
            }
            const float px = (float)x + 0.5f;
            const float E0 = fmaf(e0.x, px - e0.z, e0.y * (py - e0.w));
            const float E1 = fmaf(e1.x, px - e1.z, e1.y * (py - e1.w));
            const float E2 = fmaf(e2.x, px - e2.z, e2.y * (py - e2.w));
            const bool in0 = tl0 ? (E0 >= 0.f) : (E0 > 0.f);
            const bool in1 = tl1 ? (E1 >= 0.f) : (E1 > 0.f);
            const bool in2 = tl2 ? (E2 >= 0.f) : (E2 > 0.f);
            const float z = fmaxf(fmaf(zp.x, px, fmaf(zp.y, py, zp.z)), 0.f);
            if (in0 && in1 && in2 && z < zb[j] && q0 + j < p1) {
              zb[j] = z;
              win[j] = t;
            }
          }
        }
      }
      // resolve winners of this chunk
      uint32_t col[kPx];
      int32_t wid[kPx];
#pragma unroll
      for (int j = 0; j < kPx; ++j) {
        if (nflush == 0) {
          if (PLAIN) {
            const int q = q0 + j;
            col[j] = (q < p1) ? A.cbuf[(long long)k * HW + q] : P.bg_packed;
          } else {
            col[j] = P.bg_packed;
          }
          wid[j] = -1;
        } else {
          col[j] = st_c[j * THREADS + tid];
          if (WINNER) wid[j] = st_w[j * THREADS + tid];
        }
        if (win[j] >= 0) {
          const int t = win[j];
          const float4 meta = S.T4[t];
          const uint32_t fl = __float_as_uint(meta.y);
          if (fl & 8u) {
            int x = lx + j;
            float py = py_a;
            while (x >= W) { x -= W; py += 1.f; }
            col[j] = shade_smooth(P, S, t, (float)x + 0.5f, py);
          } else {
            col[j] = __float_as_uint(meta.z);
          }
          if (WINNER) wid[j] = __float_as_int(meta.w);
        }
      }
      if (!final_flush) {
#pragma unroll
        for (int j = 0; j < kPx; ++j) {
          st_z[j * THREADS + tid] = zb[j];
          st_c[j * THREADS + tid] = col[j];
          if (WINNER) st_w[j * THREADS + tid] = wid[j];
        }
      } else if (active) {
        const bool full = (q0 + kPx <= p1);
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
      ++nflush;
      tri_count = 0;
      __syncthreads();
    };

    // ---- K1 / K2: walk nodes and instances in draw order -----------------
    __syncthreads();  // s_vp visible
    const float vp0 = s_vp[0], vp1 = s_vp[1], vp2 = s_vp[2], vp3 = s_vp[3];
    const float vp4 = s_vp[4], vp5 = s_vp[5], vp6 = s_vp[6], vp7 = s_vp[7];
    const float vp8 = s_vp[8], vp9 = s_vp[9], vp10 = s_vp[10], vp11 = s_vp[11];
    const float vp12 = s_vp[12], vp13 = s_vp[13], vp14 = s_vp[14], vp15 = s_vp[15];
    for (int n = A.node_begin; n < A.node_end; ++n) {
      const NodeDesc& nd = P.nodes[n];
      const MeshDesc& me = P.meshes[nd.mesh];
      int cnt = nd.counts ? nd.counts[k] : nd.ips;
      cnt = max(0, min(cnt, nd.ips));
      const int nv = me.nv, nt = me.nt;
      if (cnt == 0 || nt == 0) continue;
      const int nb = max(1, min(A.icap, A.vcap / nv));
      const bool smooth = me.smooth != 0;
      for (int b0 = 0; b0 < cnt; b0 += nb) {
        const int nbc = min(nb, cnt - b0);
        // instance stage
        for (int i = tid; i < nbc; i += THREADS) {
          const long long id = nd.shared ? (long long)(b0 + i) : (long long)k * nd.ips + b0 + i;
          float m[12];
          build_model(nd, id, m);
          if (r == 0) write_back_bound(nd, id);
          icache[i * 4 + 0] = make_float4(m[0], m[1], m[2], m[3]);
          icache[i * 4 + 1] = make_float4(m[4], m[5], m[6], m[7]);
          icache[i * 4 + 2] = make_float4(m[8], m[9], m[10], m[11]);
          const float* cc = nd.color + id * 4;
          icache[i * 4 + 3] = make_float4(cc[0], cc[1], cc[2], cc[3]);
        }
        __syncthreads();
        // vertex stage
        for (int v = tid; v < nbc * nv; v += THREADS) {
          const int li = v / nv, vi = v - li * nv;
          const float4 r0 = icache[li * 4 + 0], r1 = icache[li * 4 + 1], r2 = icache[li * 4 + 2];
          const float ox = me.pos[3 * vi], oy = me.pos[3 * vi + 1], oz = me.pos[3 * vi + 2];
          const float wx = r0.x * ox + r0.y * oy + r0.z * oz + r0.w;
          const float wy = r1.x * ox + r1.y * oy + r1.z * oz + r1.w;
          const float wz = r2.x * ox + r2.y * oy + r2.z * oz + r2.w;
          float4 c;
          c.x = vp0 * wx + vp1 * wy + vp2 * wz + vp3;
          c.y = vp4 * wx + vp5 * wy + vp6 * wz + vp7;
          c.z = vp8 * wx + vp9 * wy + vp10 * wz + vp11;
          c.w = vp12 * wx + vp13 * wy + vp14 * wz + vp15;
          const float ax = me.nrm[3 * vi], ay = me.nrm[3 * vi + 1], az = me.nrm[3 * vi + 2];
          float nx = r0.x * ax + r0.y * ay + r0.z * az;
          float ny = r1.x * ax + r1.y * ay + r1.z * az;
          float nz = r2.x * ax + r2.y * ay + r2.z * az;
          const float l2 = nx * nx + ny * ny + nz * nz;
          const float inv = l2 > 0.f ? rsqrtf(l2) : 0.f;
          vcache[2 * v] = c;
          vcache[2 * v + 1] = make_float4(nx * inv, ny * inv, nz * inv, 0.f);
        }
        __syncthreads();
        // triangle stage, rounds of RT source triangles
        const int total_t = nbc * nt;
        for (int t0 = 0; t0 < total_t; t0 += RT) {
          const int rem = min(RT, total_t - t0);
          if (tri_count + 2 * rem > A.tri_cap) flush(false);
          int c = 0, li = 0, ti = 0;
          const bool mine = tid < rem;
          if (mine) {
            const int t = t0 + tid;
            li = t / nt;
            ti = t - li * nt;
            c = process_tri<false>(P, S, vcache, li * nv, me.idx[3 * ti], me.idx[3 * ti + 1], me.idx[3 * ti + 2], 0,
                                   icache[li * 4 + 3], 0, smooth);
          }
          int total;
          const int off = block_exclusive_scan<THREADS>(c, s_scan, total);
          if (c > 0) {
            const int draw_id = (nd.rank_base + b0 + li) * P.max_tris + ti;
            process_tri<true>(P, S, vcache, li * nv, me.idx[3 * ti], me.idx[3 * ti + 1], me.idx[3 * ti + 2],
                              tri_count + off, icache[li * 4 + 3], draw_id, smooth);
          }
          tri_count += total;
          __syncthreads();
        }
      }
    }
    flush(true);
  }
}

// ---------------------------------------------------------------------------
// plain-mode helpers

__global__ void plain_clear_kernel(int total, float* zbuf, uint32_t* cbuf, uint32_t bg) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
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
  return reinterpret_cast<const void*>(&hard_kernel<T, PL, WN>);
}

static const void* pick_hard(int threads, bool plain, bool winner) {
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

cudaError_t hard_set_smem_limit(int threads, bool plain, bool winner, int bytes) {
  const void* f = pick_hard(threads, plain, winner);
  if (!f) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

cudaError_t hard_occupancy(int threads, bool plain, bool winner, int smem_bytes, int* blocks_per_sm) {
  const void* f = pick_hard(threads, plain, winner);
  if (!f) return cudaErrorInvalidValue;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, threads, smem_bytes);
}

cudaError_t hard_launch(int threads, bool plain, bool winner, const SceneParams& P, const RasterArgs& A, int grid,
                        int smem_bytes, cudaStream_t stream) {
  const void* f = pick_hard(threads, plain, winner);
  if (!f) return cudaErrorInvalidValue;
  void* args[] = {const_cast<SceneParams*>(&P), const_cast<RasterArgs*>(&A)};
  return cudaLaunchKernel(f, dim3(grid), dim3(threads), args, (size_t)smem_bytes, stream);
}

cudaError_t plain_clear_launch(const SceneParams& P, float* zbuf, uint32_t* cbuf, cudaStream_t stream) {
  const int total = P.N * P.W * P.H;
  const int grid = min((total + 255) / 256, 152 * 8);
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
