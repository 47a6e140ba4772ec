// pbr_soft.cu -- soft-coverage rasteriser for scenes of any size (forward K4,
// adjoint K5); the model and its adjoint are in pbr_soft.cuh.  Work item =
// (scene, region of threads*8 pixels), one CTA each.  The adjoint recomputes
// every region's fragment list from the triangle setup (nothing per-fragment
// is stored), accumulates per-triangle gradients with warp reductions, chains
// them through the viewport / projection / model matrix to per-instance
// position, HPR, scale and colour, and to the light direction.
#include "pbr_launch.h"
#include "pbr_soft.cuh"

namespace pbr {

constexpr int kSPx = 8;   // pixels per thread

__host__ __device__ inline SoftLayout soft_layout(const SoftArgs& a, int threads) {
  SoftLayout L;
  int off = 0;
  const int t4 = a.tri_cap * 16;
  for (int i = 0; i < kSoftRecs; ++i) { L.rec[i] = off; off += align16(t4); }
  L.masks = off; off += align16(a.max_region_bins * (a.tri_cap / 32) * 4);
  L.vcache = off; off += align16(a.vcap * 32);
  L.vidx = off; off += align16(a.vcap * 4);
  L.icache = off; off += align16(a.icap * 64);
  L.state = off; off += align16(threads * kSPx * (a.backward ? 15 : 11) * 4);
  if (a.backward) {
    L.tacc = off; off += align16(a.tri_cap * 24 * 4);
    L.iacc = off; off += align16(a.iacc_cap * kIacc * 4);
  } else {
    L.tacc = L.iacc = 0;
  }
  L.misc = off; off += align16((threads / 32 + 8) * 4 + 16 * 4 + 16 + 16);
  L.total = off;
  return L;
}

int soft_smem_bytes(const SoftArgs& a, int threads) { return soft_layout(a, threads).total; }

template <int THREADS>
__device__ __forceinline__ int soft_block_scan(int v, int* s_warp, int& total) {
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

template <int THREADS, bool BACKWARD>
__global__ void __launch_bounds__(THREADS) soft_kernel(const __grid_constant__ SceneParams P,
                                                       const __grid_constant__ SoftArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NW = THREADS / 32;
  const SoftLayout L = soft_layout(A, THREADS);
  SoftCtx S;
#pragma unroll
  for (int i = 0; i < kSoftRecs; ++i) S.R[i] = reinterpret_cast<float4*>(smem + L.rec[i]);
  S.W = (float)P.W;
  S.H = (float)P.H;
  S.cut = kSoftCut * P.sigma;
  uint32_t* masks = reinterpret_cast<uint32_t*>(smem + L.masks);
  float4* vcache = reinterpret_cast<float4*>(smem + L.vcache);
  float4* icache = reinterpret_cast<float4*>(smem + L.icache);
  float* st = reinterpret_cast<float*>(smem + L.state);  // [field][kSPx][THREADS]
  float* tacc = reinterpret_cast<float*>(smem + L.tacc);  // [tri_cap][24]
  float* iacc = reinterpret_cast<float*>(smem + L.iacc);  // [iacc_cap][kIacc]
  int* s_scan = reinterpret_cast<int*>(smem + L.misc);
  float* s_vp = reinterpret_cast<float*>(s_scan + NW + 8);
  float* s_light = s_vp + 16;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int W = P.W, H = P.H, HW = W * H;
  const int words = A.tri_cap >> 5;
  const int Bp = A.bin_px;
  const int RT = min(THREADS, A.tri_cap);
  const float inv_sigma = 1.f / P.sigma;
  const float inv_zr = 1.f / (P.zfar - P.znear);
  const float inv_gamma = 1.f / P.gamma;
  auto ST = [&](int field, int j) -> float& { return st[(field * kSPx + j) * THREADS + tid]; };

  for (int item = blockIdx.x; item < A.num_items; item += gridDim.x) {
    const int k = item / A.regions_per_scene;
    const int r = item - k * A.regions_per_scene;
    const int p0 = r * A.region_px;
    const int p1 = min(p0 + A.region_px, HW);
    const int ry0 = p0 / W, ry1 = (p1 - 1) / W;
    S.ry0 = (float)ry0;
    S.ry1 = (float)ry1;
    if (tid < 16) s_vp[tid] = P.vp[(long long)k * 16 + tid];
    if (tid < 4) s_light[tid] = 0.f;
    const int q0 = p0 + tid * kSPx;
    const int ly = q0 / W, lx = q0 - ly * W;
    const int lane_y1 = min((q0 + kSPx - 1) / W, H - 1);
    const int lane_x0 = (lane_y1 == ly) ? lx : 0;
    const int lane_x1 = (lane_y1 == ly) ? lx + kSPx - 1 : W - 1;
    const bool active = q0 < p1;

    // ---- per-pixel state ---------------------------------------------------
    // forward:  m, S, acc0..2 (relative to C_r), Pnz, nz, C_r0..2, has_ref
    // backward: m, Pnz, nz, dL/dA, Cfg-C_r 0..2, dLdCfg0..2, 1/S, C_r0..2, has_ref
#pragma unroll
    for (int j = 0; j < kSPx; ++j) {
      const int q = q0 + j;
      if (!BACKWARD) {
        ST(0, j) = -1e30f; ST(1, j) = 0.f; ST(2, j) = 0.f; ST(3, j) = 0.f; ST(4, j) = 0.f;
        ST(5, j) = 1.f; ST(6, j) = 0.f; ST(7, j) = 0.f; ST(8, j) = 0.f; ST(9, j) = 0.f; ST(10, j) = 0.f;
      } else {
        float Lv = -1e30f, Sv = 1.f, code = 1.f, Av = 0.f, cf[3] = {0.f, 0.f, 0.f}, g[3] = {0.f, 0.f, 0.f};
        float dl[3] = {0.f, 0.f, 0.f};
        if (active && q < p1) {
          float4 stv;
          float2 stw;
          stats_load(A.stats, (long long)P.N * HW, (long long)k * HW + q, stv, stw);
          Lv = stv.x;
          Sv = stv.y;
          code = stv.z;
          dl[0] = stv.w;
          dl[1] = stw.x;
          dl[2] = stw.y;
          float Pnz, nz;
          if (code >= 0.f) { Pnz = code; nz = 0.f; } else if (code >= -2.f) { Pnz = -1.f - code; nz = 1.f; } else { Pnz = 0.f; nz = 2.f; }
          Av = nz > 0.f ? 1.f : 1.f - Pnz;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const float o = A.out[((long long)k * 3 + c) * HW + q];
            g[c] = A.gout[((long long)k * 3 + c) * HW + q];
            cf[c] = Av > 0.f ? (o - (1.f - Av) * P.bg[c]) / Av : 0.f;
          }
          ST(1, j) = Pnz;
          ST(2, j) = nz;
        } else {
          ST(1, j) = 1.f;
          ST(2, j) = 0.f;
        }
        ST(0, j) = Lv;
        // dL/dA = g . (Cfg - bg); Cfg from the output is accurate enough here
        // (this term is not amplified by 1/gamma)
        ST(3, j) = g[0] * (cf[0] - P.bg[0]) + g[1] * (cf[1] - P.bg[1]) + g[2] * (cf[2] - P.bg[2]);
        ST(10, j) = Sv > 0.f ? 1.f / Sv : 0.f;
        ST(14, j) = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          ST(4 + c, j) = dl[c];
          ST(7 + c, j) = Av * g[c];
        }
      }
    }
    if (BACKWARD) {
      for (int i = tid; i < A.iacc_cap * kIacc; i += THREADS) iacc[i] = 0.f;
    }
    __syncthreads();

    int tri_count = 0;
    // ---- K3 (soft): raster the current chunk --------------------------------
    auto flush = [&]() {
      const int T = tri_count;
      const int nw = (T + 31) >> 5;
      const int by_lo = ry0 / Bp, by_hi = ry1 / Bp;
      const int nbins = (by_hi - by_lo + 1) * A.bins_x;
      for (int i = tid; i < nbins * words; i += THREADS) masks[i] = 0u;
      if (BACKWARD)
        for (int i = tid; i < T * 24; i += THREADS) tacc[i] = 0.f;
      __syncthreads();
      for (int w = warp; w < nw; w += NW) {
        const int t = w * 32 + lane;
        int bx0 = 1 << 20, bx1 = -1, by0 = 1 << 20, by1 = -1;
        if (t < T) {
          const uint32_t xb = __float_as_uint(S.R[4][t].w), yb = __float_as_uint(S.R[5][t].x);
          bx0 = (int)(xb & 0xffffu) / Bp;
          bx1 = (int)(xb >> 16) / Bp;
          by0 = (int)(yb & 0xffffu) / Bp - by_lo;
          by1 = (int)(yb >> 16) / Bp - by_lo;
        }
        const int ux0 = __reduce_min_sync(0xffffffffu, bx0), ux1 = __reduce_max_sync(0xffffffffu, bx1);
        const int uy0 = __reduce_min_sync(0xffffffffu, by0), uy1 = __reduce_max_sync(0xffffffffu, by1);
        for (int by = uy0; by <= uy1; ++by)
          for (int bx = ux0; bx <= ux1; ++bx) {
            const uint32_t m = __ballot_sync(0xffffffffu, (bx >= bx0) && (bx <= bx1) && (by >= by0) && (by <= by1));
            if (lane == 0) masks[(by * A.bins_x + bx) * words + w] = m;
          }
      }
      __syncthreads();
      // the warp's bins
      const int wq0 = p0 + warp * 32 * kSPx;
      const int wq1 = min(wq0 + 32 * kSPx, p1) - 1;
      int wbx0 = 0, wbx1 = -1, wby0 = 0, wby1 = -1;
      if (wq0 < p1) {
        const int wy0 = wq0 / W, wy1 = wq1 / W;
        wby0 = wy0 / Bp - by_lo;
        wby1 = wy1 / Bp - by_lo;
        if (wy0 == wy1) {
          wbx0 = (wq0 - wy0 * W) / Bp;
          wbx1 = (wq1 - wy1 * W) / Bp;
        } else {
          wbx0 = 0;
          wbx1 = A.bins_x - 1;
        }
      }
      const int wnbx = wbx1 - wbx0 + 1;
      const int wnb = (wby1 >= wby0) ? (wby1 - wby0 + 1) * wnbx : 0;
      for (int w = 0; w < nw; ++w) {
        uint32_t m = 0u;
        for (int b = lane; b < wnb; b += 32) {
          const int by = wby0 + b / wnbx, bx = wbx0 + b % wnbx;
          m |= masks[(by * A.bins_x + bx) * words + w];
        }
        m = __reduce_or_sync(0xffffffffu, m);
        while (m) {
          const int t = w * 32 + __ffs(m) - 1;
          m &= m - 1u;
          const uint32_t xb = __float_as_uint(S.R[4][t].w), yb = __float_as_uint(S.R[5][t].x);
          const int tx0 = (int)(xb & 0xffffu), tx1 = (int)(xb >> 16);
          const int ty0 = (int)(yb & 0xffffu), ty1 = (int)(yb >> 16);
          const bool hit = active && !(ty1 < ly || ty0 > lane_y1 || tx1 < lane_x0 || tx0 > lane_x1);
          if (!BACKWARD) {
            if (!hit) continue;
#pragma unroll
            for (int j = 0; j < kSPx; ++j) {
              int x = lx + j;
              float py = (float)ly + 0.5f;
              while (x >= W) { x -= W; py += 1.f; }
              if (q0 + j >= p1) continue;
              Frag f;
              if (!soft_frag(P, S, t, (float)x + 0.5f, py, inv_sigma, inv_zr, f)) continue;
              float m0 = ST(0, j), S0 = ST(1, j);
              if (1.f - f.D == 0.f) ST(6, j) += 1.f;
              else ST(5, j) *= (1.f - f.D);
              if (ST(10, j) == 0.f) {  // first fragment: the colour reference
                ST(7, j) = f.C[0];
                ST(8, j) = f.C[1];
                ST(9, j) = f.C[2];
                ST(10, j) = 1.f;
              }
              const float d0 = f.C[0] - ST(7, j), d1 = f.C[1] - ST(8, j), d2 = f.C[2] - ST(9, j);
              if (f.zs > m0) {
                const float sc = expf((m0 - f.zs) * inv_gamma);
                ST(1, j) = S0 * sc + f.D;
                ST(2, j) = ST(2, j) * sc + f.D * d0;
                ST(3, j) = ST(3, j) * sc + f.D * d1;
                ST(4, j) = ST(4, j) * sc + f.D * d2;
                ST(0, j) = f.zs;
              } else {
                const float wv = f.D * expf((f.zs - m0) * inv_gamma);
                ST(1, j) = S0 + wv;
                ST(2, j) += wv * d0;
                ST(3, j) += wv * d1;
                ST(4, j) += wv * d2;
              }
            }
          } else {
            // per-lane gradient accumulators of triangle t
            float acc[24];
#pragma unroll
            for (int i = 0; i < 24; ++i) acc[i] = 0.f;
            if (hit) {
              // screen vertices of t
              float vx[3], vy[3];
#pragma unroll
              for (int v = 0; v < 3; ++v) {
                const float4 cv = S.R[10 + v][t];
                const float iwv = 1.f / cv.z;
                vx[v] = (cv.x * iwv + 1.f) * 0.5f * S.W;
                vy[v] = (1.f - cv.y * iwv) * 0.5f * S.H;
              }
              const float4 iwr = S.R[4][t];
              const float iwk[3] = {iwr.x, iwr.y, iwr.z};
              const float4 n0 = S.R[7][t], n1 = S.R[8][t], n2 = S.R[9][t];
              const float4 col = S.R[6][t];
              const bool smooth = (__float_as_uint(S.R[5][t].y) & 8u) != 0u;
              const float4 il = S.R[3][t];
              const float invL[3] = {il.x, il.y, il.z};
#pragma unroll
              for (int j = 0; j < kSPx; ++j) {
                int x = lx + j;
                float py = (float)ly + 0.5f;
                while (x >= W) { x -= W; py += 1.f; }
                if (q0 + j >= p1) continue;
                const float px = (float)x + 0.5f;
                Frag f;
                if (!soft_frag(P, S, t, px, py, inv_sigma, inv_zr, f)) continue;
                SoftPixB pb;
                pb.m = ST(0, j);
                pb.Pnz = ST(1, j);
                pb.nz = ST(2, j);
                pb.dLdA = ST(3, j);
                pb.invS = ST(10, j);
                pb.ref = ST(14, j);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                  pb.dl[c] = ST(4 + c, j);
                  pb.dc[c] = ST(7 + c, j);
                  pb.Cr[c] = ST(11 + c, j);
                }
                soft_grad(P, f, pb, px, py, vx, vy, iwk, invL, n0, n1, n2, col, smooth, inv_sigma, inv_zr, inv_gamma,
                          acc);
                if (ST(14, j) == 0.f) {  // first fragment: the colour reference of the forward
                  ST(11, j) = pb.Cr[0];
                  ST(12, j) = pb.Cr[1];
                  ST(13, j) = pb.Cr[2];
                  ST(14, j) = 1.f;
                }
              }
            }
            if (__any_sync(0xffffffffu, hit)) {
#pragma unroll
              for (int i = 0; i < 24; ++i) {
                const float v = warp_sum(acc[i]);
                if (lane == 0 && v != 0.f) atomicAdd(&tacc[t * 24 + i], v);
              }
            }
          }
        }
      }
      __syncthreads();
      if (BACKWARD) {
        // per triangle: chain to clip -> world -> model matrix, per instance
        for (int t = tid; t < T; t += THREADS) {
          soft_tri_chain(P, S, t, tacc + t * 24, s_vp, iacc, A.iacc_cap, s_light);
        }
        __syncthreads();
      }
      tri_count = 0;
    };

    // ---- K1 / K2 ------------------------------------------------------------
    __syncthreads();
    for (int n = 0; n < P.num_nodes; ++n) {
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
        for (int i = tid; i < nbc; i += THREADS) {
          const long long id = nd.shared ? (long long)(b0 + i) : (long long)k * nd.ips + b0 + i;
          float m[12];
          build_model(nd, id, m);
          icache[i * 4 + 0] = make_float4(m[0], m[1], m[2], m[3]);
          icache[i * 4 + 1] = make_float4(m[4], m[5], m[6], m[7]);
          icache[i * 4 + 2] = make_float4(m[8], m[9], m[10], m[11]);
          icache[i * 4 + 3] = *reinterpret_cast<const float4*>(nd.color + id * 4);
        }
        __syncthreads();
        for (int v = tid; v < nbc * nv; v += THREADS) {
          const int li = v / nv, vi = v - li * nv;
          const float4 r0 = icache[li * 4 + 0], r1 = icache[li * 4 + 1], r2 = icache[li * 4 + 2];
          const float ox = me.pos[3 * vi], oy = me.pos[3 * vi + 1], oz = me.pos[3 * vi + 2];
          const float wx = r0.x * ox + r0.y * oy + r0.z * oz + r0.w;
          const float wy = r1.x * ox + r1.y * oy + r1.z * oz + r1.w;
          const float wz = r2.x * ox + r2.y * oy + r2.z * oz + r2.w;
          float4 c;
          c.x = s_vp[0] * wx + s_vp[1] * wy + s_vp[2] * wz + s_vp[3];
          c.y = s_vp[4] * wx + s_vp[5] * wy + s_vp[6] * wz + s_vp[7];
          c.z = s_vp[8] * wx + s_vp[9] * wy + s_vp[10] * wz + s_vp[11];
          c.w = s_vp[12] * wx + s_vp[13] * wy + s_vp[14] * wz + s_vp[15];
          const float ax = me.nrm[3 * vi], ay = me.nrm[3 * vi + 1], az = me.nrm[3 * vi + 2];
          const float nx = r0.x * ax + r0.y * ay + r0.z * az;
          const float ny = r1.x * ax + r1.y * ay + r1.z * az;
          const float nz = r2.x * ax + r2.y * ay + r2.z * az;
          const float l2 = nx * nx + ny * ny + nz * nz;
          const float inv = l2 > 0.f ? rsqrtf(l2) : 0.f;
          vcache[2 * v] = c;
          // depth offset from the scene reference w_ref = VP[15] (clip w of the world origin), computed
          // without the large constant term so that it keeps its relative precision
          const float dw = s_vp[12] * wx + s_vp[13] * wy + s_vp[14] * wz;
          vcache[2 * v + 1] = make_float4(nx * inv, ny * inv, nz * inv, dw);
        }
        __syncthreads();
        const int total_t = nbc * nt;
        for (int t0 = 0; t0 < total_t; t0 += RT) {
          const int rem = min(RT, total_t - t0);
          if (tri_count + rem > A.tri_cap) flush();
          int c = 0, li = 0, ti = 0;
          int i0 = 0, i1 = 0, i2 = 0;
          if (tid < rem) {
            const int t = t0 + tid;
            li = t / nt;
            ti = t - li * nt;
            i0 = me.idx[3 * ti];
            i1 = me.idx[3 * ti + 1];
            i2 = me.idx[3 * ti + 2];
            const int vb = li * nv;
            c = soft_setup<false>(P, S, vcache[2 * (vb + i0)], vcache[2 * (vb + i0) + 1], i0, vcache[2 * (vb + i1)],
                                  vcache[2 * (vb + i1) + 1], i1, vcache[2 * (vb + i2)], vcache[2 * (vb + i2) + 1], i2,
                                  0, icache[li * 4 + 3], 0, smooth);
          }
          int total;
          const int off = soft_block_scan<THREADS>(c, s_scan, total);
          if (c > 0) {
            const int vb = li * nv;
            soft_setup<true>(P, S, vcache[2 * (vb + i0)], vcache[2 * (vb + i0) + 1], i0, vcache[2 * (vb + i1)],
                             vcache[2 * (vb + i1) + 1], i1, vcache[2 * (vb + i2)], vcache[2 * (vb + i2) + 1], i2,
                             tri_count + off, icache[li * 4 + 3], nd.rank_base + b0 + li, smooth);
          }
          tri_count += total;
          __syncthreads();
        }
      }
    }
    flush();
    __syncthreads();

    if (!BACKWARD) {
      if (active) {
#pragma unroll
        for (int j = 0; j < kSPx; ++j) {
          const int q = q0 + j;
          if (q >= p1) continue;
          const float m0 = ST(0, j), S0 = ST(1, j), Pv = ST(5, j), nz = ST(6, j);
          const float Av = 1.f - (nz > 0.f ? 0.f : Pv);
          float dl[3];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            dl[c] = S0 > 0.f ? ST(2 + c, j) / S0 : 0.f;  // Cfg - C_r
            const float fg = ST(7 + c, j) + dl[c];
            A.out[((long long)k * 3 + c) * HW + q] = Av * fg + (1.f - Av) * P.bg[c];
          }
          if (A.stats) {
            // coverage code: prod over non-zero (1 - D), folded with the count of zero factors
            const float code = nz == 0.f ? Pv : (nz == 1.f ? -1.f - Pv : -3.f);
            stats_store(A.stats, (long long)P.N * HW, (long long)k * HW + q, make_float4(m0, S0, code, dl[0]),
                        make_float2(dl[1], dl[2]));
          }
        }
      }
    } else {
      // per instance of this scene: dM3 -> d(hpr), d(scale); dt -> d(pos)
      int ninst = 0;
      for (int n = 0; n < P.num_nodes; ++n) ninst = max(ninst, P.nodes[n].rank_base + P.nodes[n].ips);
      for (int s = tid; s < ninst; s += THREADS) {
        soft_instance_grads(P, k, s, iacc + s * kIacc);
      }
      if (tid < 3 && A.glight) atomicAdd(&A.glight[tid], s_light[tid]);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------

static const void* pick_soft(int threads, bool backward) {
  if (threads == 128) return backward ? (const void*)&soft_kernel<128, true> : (const void*)&soft_kernel<128, false>;
  if (threads == 256) return backward ? (const void*)&soft_kernel<256, true> : (const void*)&soft_kernel<256, false>;
  return nullptr;
}

cudaError_t soft_set_smem_limit(int threads, bool backward, int bytes) {
  const void* f = pick_soft(threads, backward);
  if (!f) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

cudaError_t soft_launch(int threads, bool backward, const SceneParams& P, const SoftArgs& A, int grid, int smem_bytes,
                        cudaStream_t stream) {
  const void* f = pick_soft(threads, backward);
  if (!f) return cudaErrorInvalidValue;
  void* args[] = {const_cast<SceneParams*>(&P), const_cast<SoftArgs*>(&A)};
  return cudaLaunchKernel(f, dim3(grid), dim3(threads), args, (size_t)smem_bytes, stream);
}

}  // namespace pbr
