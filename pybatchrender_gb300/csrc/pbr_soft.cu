// pbr_soft.cu -- differentiable soft-coverage rasteriser (forward K4, adjoint K5).
//
// Soft model, per pixel p and front-facing triangle j fully in front of the
// near plane (nothing here exists in the reference; it sits beside the hard
// raster and shares its setup):
//   e_k  = E_k(p) / |(A_k, B_k)|            signed distance to edge line k (px)
//   D_j  = prod_k sigmoid(e_k / sigma) T(d),  d = distance from p to the triangle (0 inside),
//          T = smootherstep((16 sigma - d) / (4 sigma)): C1 everywhere, exactly 0 at 16 sigma
//   w    = area2 / sum_k E_k iw_k           perspective-correct clip w
//   zs_j = (zfar - w) / (zfar - znear)      nearer = larger
//   C_j  = shading of shaders/basic.frag:33-38 (unclamped) with the
//          perspective-correct normal
//   w_j  = D_j exp((zs_j - max zs) / gamma),   A = 1 - prod_j (1 - D_j)
//   out  = A sum_j w_j C_j / sum_j w_j + (1 - A) bg
//
// Colours are accumulated relative to the first fragment's colour C_r, so that
// C_j - Cfg, which the adjoint multiplies by 1/gamma, is exactly 0 where all
// fragments share a colour (the faces of a flat-shaded mesh).  The forward
// stores per-pixel statistics (the running max m of zs, the softmax
// denominator S relative to it -- kept apart because m + gamma ln S in float32
// would lose m's precision 1/gamma-fold --, a code for prod(1 - D), and
// Cfg - C_r) so the adjoint needs a single sweep: it
// recomputes every tile's fragment list from the triangle setup (nothing
// per-fragment is stored), accumulates per-triangle gradients with warp
// reductions, chains them through the viewport / projection / model matrix
// to per-instance position, HPR, scale and colour, and to the light
// direction.  Work item = (scene, region of threads*8 pixels), one CTA each.
#include "pbr_device.cuh"
#include "pbr_launch.h"

namespace pbr {

constexpr float kSoftCut = 16.f;    // coverage is 0 at 16 sigma or more from the triangle
constexpr float kSoftTaper = 4.f;   // tapered to 0 over the last 4 sigma
constexpr int kSPx = 8;   // pixels per thread
constexpr int kSoftRecs = 15;
constexpr int kIacc = 24; // per-instance gradient accumulator: dM3 (9), dt (3), dcol (3), dM3 normal chain (9)

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

struct SoftCtx {
  float4* R[15];
  float W, H, ry0, ry1, cut;
};

// Soft triangle setup: no near clipping (triangles that are not fully in
// front of the near plane are dropped), back faces culled, bbox widened by
// the coverage cutoff.  Records:
//   R0..R2  edge k: (A, B, x_ref, y_ref)      R3 (1/L0, 1/L1, 1/L2, area2)
//   R4      (iw0, iw1, iw2, x-box)            R5 (y-box, flags, instance slot, d2)
//   R6      instance colour                   R7..R9 (n_k, flat shaded colour channel k)
//   R10..R12 (clip x, clip y, clip w, mesh vertex index) of vertex k
//   R13, R14 screen vertices (x0, y0, x1, y1), (x2, y2, d0, d1); R5.w = d2, where
//            d_k = w_k - w_ref is vertex k's depth offset from the scene reference
template <bool WRITE>
__device__ __forceinline__ int soft_setup(const SceneParams& P, const SoftCtx& S, float4 c0, float4 n0, int v0,
                                          float4 c1, float4 n1, int v1, float4 c2, float4 n2, int v2, int slot,
                                          float4 col, int inst_slot, bool smooth) {
  if (!(c0.z + c0.w >= 0.f && c1.z + c1.w >= 0.f && c2.z + c2.w >= 0.f)) return 0;
  SV s0 = to_screen(c0, S.W, S.H), s1 = to_screen(c1, S.W, S.H), s2 = to_screen(c2, S.W, S.H);
  float area2 = (s1.x - s0.x) * (s2.y - s0.y) - (s2.x - s0.x) * (s1.y - s0.y);
  if (!(area2 < 0.f)) return 0;  // back-facing, degenerate or NaN
  { SV t = s1; s1 = s2; s2 = t; }
  { float4 t = n1; n1 = n2; n2 = t; }
  { float4 t = c1; c1 = c2; c2 = t; }
  { int t = v1; v1 = v2; v2 = t; }
  area2 = -area2;
  const float r = S.cut + 1.f;
  const float mnx = fminf(fminf(s0.x, s1.x), s2.x) - r, mxx = fmaxf(fmaxf(s0.x, s1.x), s2.x) + r;
  const float mny = fminf(fminf(s0.y, s1.y), s2.y) - r, mxy = fmaxf(fmaxf(s0.y, s1.y), s2.y) + r;
  const float fx0 = fmaxf(floorf(mnx), 0.f), fx1 = fminf(ceilf(mxx), S.W - 1.f);
  const float fy0 = fmaxf(floorf(mny), S.ry0), fy1 = fminf(ceilf(mxy), S.ry1);
  if (!(fx0 <= fx1 && fy0 <= fy1)) return 0;
  if (!WRITE) return 1;
  bool tl0, tl1, tl2;
  const float4 e0 = make_edge(s1.x, s1.y, s2.x, s2.y, tl0);
  const float4 e1 = make_edge(s2.x, s2.y, s0.x, s0.y, tl1);
  const float4 e2 = make_edge(s0.x, s0.y, s1.x, s1.y, tl2);
  S.R[0][slot] = e0;
  S.R[1][slot] = e1;
  S.R[2][slot] = e2;
  S.R[3][slot] = make_float4(1.f / sqrtf(e0.x * e0.x + e0.y * e0.y), 1.f / sqrtf(e1.x * e1.x + e1.y * e1.y),
                             1.f / sqrtf(e2.x * e2.x + e2.y * e2.y), area2);
  const uint32_t xbox = (uint32_t)fx0 | ((uint32_t)fx1 << 16), ybox = (uint32_t)fy0 | ((uint32_t)fy1 << 16);
  S.R[4][slot] = make_float4(s0.iw, s1.iw, s2.iw, __uint_as_float(xbox));
  S.R[5][slot] = make_float4(__uint_as_float(ybox), __uint_as_float(smooth ? 8u : 0u), __int_as_float(inst_slot), n2.w);
  S.R[6][slot] = col;
  float rgb[3] = {0.f, 0.f, 0.f};
  if (!smooth) shade_rgb(P, n0.x, n0.y, n0.z, col, rgb);
  S.R[7][slot] = make_float4(n0.x, n0.y, n0.z, rgb[0]);
  S.R[8][slot] = make_float4(n1.x, n1.y, n1.z, rgb[1]);
  S.R[9][slot] = make_float4(n2.x, n2.y, n2.z, rgb[2]);
  S.R[10][slot] = make_float4(c0.x, c0.y, c0.w, __int_as_float(v0));
  S.R[11][slot] = make_float4(c1.x, c1.y, c1.w, __int_as_float(v1));
  S.R[12][slot] = make_float4(c2.x, c2.y, c2.w, __int_as_float(v2));
  S.R[13][slot] = make_float4(s0.x, s0.y, s1.x, s1.y);
  S.R[14][slot] = make_float4(s2.x, s2.y, n0.w, n1.w);
  return 1;
}

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

// acc[2v], acc[2v+1] += (gx, gy) for a vertex index known only at run time,
// written with constant indices so the accumulators stay in registers
__device__ __forceinline__ void vgrad_add(float* acc, int v, float gx, float gy) {
  acc[0] += v == 0 ? gx : 0.f;
  acc[1] += v == 0 ? gy : 0.f;
  acc[2] += v == 1 ? gx : 0.f;
  acc[3] += v == 1 ? gy : 0.f;
  acc[4] += v == 2 ? gx : 0.f;
  acc[5] += v == 2 ? gy : 0.f;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Fragment of chunk triangle t at pixel centre (px, py).  Returns false when
// the pixel is beyond the cutoff or behind the eye.
struct Frag {
  float E[3], e[3], sg[3], D, Ds, dTdd, Q, w, zs;  // sg = sigmoid per edge, Ds = prod sg, D = Ds * T(d)
  int seg_a, seg_b;                                 // closest segment (vertex indices) when T' != 0
  float seg_t, ux, uy;                              // its parameter and the unit vector from it to p
  float C[3], l[3], ndl, un[3], ulen;  // shaded colour, light factor, normal (u = unnormalised)
};

__device__ __forceinline__ bool soft_frag(const SceneParams& P, const SoftCtx& S, int t, float px, float py,
                                          float inv_sigma, float inv_zr, Frag& f) {
  const float4 e0 = S.R[0][t], e1 = S.R[1][t], e2 = S.R[2][t], il = S.R[3][t], iw = S.R[4][t];
  f.E[0] = fmaf(e0.x, px - e0.z, e0.y * (py - e0.w));
  f.E[1] = fmaf(e1.x, px - e1.z, e1.y * (py - e1.w));
  f.E[2] = fmaf(e2.x, px - e2.z, e2.y * (py - e2.w));
  f.e[0] = f.E[0] * il.x;
  f.e[1] = f.E[1] * il.y;
  f.e[2] = f.E[2] * il.z;
  const float emin = fminf(fminf(f.e[0], f.e[1]), f.e[2]);
  if (!(emin > -S.cut)) return false;
  f.Q = f.E[0] * iw.x + f.E[1] * iw.y + f.E[2] * iw.z;
  if (!(f.Q > 0.f)) return false;
#pragma unroll
  for (int k = 0; k < 3; ++k) f.sg[k] = 1.f / (1.f + expf(-f.e[k] * inv_sigma));
  f.Ds = f.sg[0] * f.sg[1] * f.sg[2];
  float T = 1.f;
  f.dTdd = 0.f;
  f.seg_a = 0;
  f.seg_b = 0;
  f.seg_t = 0.f;
  f.ux = 0.f;
  f.uy = 0.f;
  if (emin < 0.f) {
    // distance to the triangle = distance to the closest edge segment
    const float4 v01 = S.R[13][t], v2 = S.R[14][t];
    const float vx[3] = {v01.x, v01.z, v2.x}, vy[3] = {v01.y, v01.w, v2.y};
    float best = 1e30f, bt = 0.f, bdx = 0.f, bdy = 0.f;
    int ba = 0, bb = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int a = (k + 1) % 3, b = (k + 2) % 3;
      const float ux = vx[b] - vx[a], uy = vy[b] - vy[a];
      const float l2 = ux * ux + uy * uy;
      float tt = l2 > 0.f ? ((px - vx[a]) * ux + (py - vy[a]) * uy) / l2 : 0.f;
      tt = fminf(fmaxf(tt, 0.f), 1.f);
      const float dx = px - (vx[a] + tt * ux), dy = py - (vy[a] + tt * uy);
      const float d2 = dx * dx + dy * dy;
      if (d2 < best) { best = d2; bt = tt; bdx = dx; bdy = dy; ba = a; bb = b; }
    }
    const float d = sqrtf(best);
    const float inv_tw = inv_sigma * (1.f / kSoftTaper);
    const float x = (S.cut - d) * inv_tw;
    if (!(x > 0.f)) return false;
    if (x < 1.f) {
      T = x * x * x * (x * (x * 6.f - 15.f) + 10.f);
      f.dTdd = -30.f * x * x * (x - 1.f) * (x - 1.f) * inv_tw;
      const float id = d > 0.f ? 1.f / d : 0.f;
      f.seg_a = ba;
      f.seg_b = bb;
      f.seg_t = bt;
      f.ux = bdx * id;
      f.uy = bdy * id;
    }
  }
  f.D = f.Ds * T;
  if (!(f.D > 0.f)) return false;
  f.w = il.w / f.Q;
  // normalised depth relative to the scene reference: zs - (zfar - w_ref)/(zfar - znear).  The softmax only
  // sees differences, and this form keeps ~7 significant digits of them where (zfar - w) / (zfar - znear)
  // would keep ~1 after the 1/gamma amplification
  {
    const float4 r14 = S.R[14][t];
    const float d2 = S.R[5][t].w;
    f.zs = -((f.E[0] * iw.x * r14.z + f.E[1] * iw.y * r14.w + f.E[2] * iw.z * d2) / f.Q) * inv_zr;
  }
  const float4 n0 = S.R[7][t], n1 = S.R[8][t], n2 = S.R[9][t];
  const float4 col = S.R[6][t];
  const uint32_t fl = __float_as_uint(S.R[5][t].y);
  if (fl & 8u) {
    const float q0 = f.E[0] * iw.x, q1 = f.E[1] * iw.y, q2 = f.E[2] * iw.z;
    f.un[0] = q0 * n0.x + q1 * n1.x + q2 * n2.x;
    f.un[1] = q0 * n0.y + q1 * n1.y + q2 * n2.y;
    f.un[2] = q0 * n0.z + q1 * n1.z + q2 * n2.z;
  } else {
    f.un[0] = n0.x;
    f.un[1] = n0.y;
    f.un[2] = n0.z;
  }
  const float l2 = f.un[0] * f.un[0] + f.un[1] * f.un[1] + f.un[2] * f.un[2];
  f.ulen = sqrtf(l2);
  const float inv = f.ulen > 0.f ? 1.f / f.ulen : 0.f;
  float ndl = (f.un[0] * P.ldir[0] + f.un[1] * P.ldir[1] + f.un[2] * P.ldir[2]) * inv;
  f.ndl = ndl > 0.f ? ndl : 0.f;
  const float s = P.strength;
  f.l[0] = (1.f - s) + (P.amb[0] + f.ndl * P.lcol[0]) * s;
  f.l[1] = (1.f - s) + (P.amb[1] + f.ndl * P.lcol[1]) * s;
  f.l[2] = (1.f - s) + (P.amb[2] + f.ndl * P.lcol[2]) * s;
  if (fl & 8u) {
    f.C[0] = col.x * f.l[0];
    f.C[1] = col.y * f.l[1];
    f.C[2] = col.z * f.l[2];
  } else {
    f.C[0] = n0.w;
    f.C[1] = n1.w;
    f.C[2] = n2.w;
  }
  return true;
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
          const float4 stv = *reinterpret_cast<const float4*>(A.stats + 8 * ((long long)k * HW + q));
          const float4 stw = *reinterpret_cast<const float4*>(A.stats + 8 * ((long long)k * HW + q) + 4);
          Lv = stv.x;
          Sv = stv.y;
          code = stv.z;
          dl[0] = stw.x;
          dl[1] = stw.y;
          dl[2] = stw.z;
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
#pragma unroll
              for (int j = 0; j < kSPx; ++j) {
                int x = lx + j;
                float py = (float)ly + 0.5f;
                while (x >= W) { x -= W; py += 1.f; }
                if (q0 + j >= p1) continue;
                const float px = (float)x + 0.5f;
                Frag f;
                if (!soft_frag(P, S, t, px, py, inv_sigma, inv_zr, f)) continue;
                const float Lp = ST(0, j), Pnz = ST(1, j), nz = ST(2, j);
                if (ST(14, j) == 0.f) {  // first fragment: the colour reference of the forward
                  ST(11, j) = f.C[0];
                  ST(12, j) = f.C[1];
                  ST(13, j) = f.C[2];
                  ST(14, j) = 1.f;
                }
                const float dc0 = ST(7, j), dc1 = ST(8, j), dc2 = ST(9, j);
                const float dLdA = ST(3, j);
                const float ewn = expf((f.zs - Lp) * inv_gamma) * ST(10, j);
                const float wn = f.D * ewn;
                const float dCx = wn * dc0, dCy = wn * dc1, dCz = wn * dc2;
                // C_j - Cfg = (C_j - C_r) - (Cfg - C_r)
                const float dws = dc0 * ((f.C[0] - ST(11, j)) - ST(4, j)) + dc1 * ((f.C[1] - ST(12, j)) - ST(5, j)) +
                                  dc2 * ((f.C[2] - ST(13, j)) - ST(6, j));
                const float omd = 1.f - f.D;
                float dAdD = 0.f;
                if (nz == 0.f) dAdD = Pnz / omd;
                else if (nz == 1.f && omd == 0.f) dAdD = Pnz;
                const float dLdD = dLdA * dAdD + dws * ewn;
                const float dLdzs = dws * wn * inv_gamma;
                // colour / shading
                const float s = P.strength;
                acc[18] += dCx * f.l[0];
                acc[19] += dCy * f.l[1];
                acc[20] += dCz * f.l[2];
                float dE[3], diw[3] = {0.f, 0.f, 0.f};
                float dndl = 0.f;
                if (f.ndl > 0.f) dndl = s * (dCx * col.x * P.lcol[0] + dCy * col.y * P.lcol[1] + dCz * col.z * P.lcol[2]);
                float du[3] = {0.f, 0.f, 0.f};
                if (dndl != 0.f && f.ulen > 0.f) {
                  const float inv = 1.f / f.ulen;
                  const float nh[3] = {f.un[0] * inv, f.un[1] * inv, f.un[2] * inv};
#pragma unroll
                  for (int c = 0; c < 3; ++c) {
                    du[c] = dndl * (P.ldir[c] - f.ndl * nh[c]) * inv;
                    acc[21 + c] += dndl * nh[c];
                  }
                }
                // depth: zs(w), w = area2 / Q
                const float dLdw = -dLdzs * inv_zr;
                const float dLdQ = -dLdw * f.w / f.Q;
                const float dLdarea = dLdw / f.Q;
#pragma unroll
                for (int e = 0; e < 3; ++e) {
                  dE[e] = dLdD * f.D * (1.f - f.sg[e]) * inv_sigma;  // dL/de_e for now
                  diw[e] += dLdQ * f.E[e];
                }
                if (f.dTdd != 0.f) {
                  // d = |p - c|, c on segment (a,b) at parameter t: dd/da = -(1-t) u, dd/db = -t u
                  const float dLdd = dLdD * f.Ds * f.dTdd;
                  const float ga = -dLdd * (1.f - f.seg_t), gb = -dLdd * f.seg_t;
                  vgrad_add(acc, f.seg_a, ga * f.ux, ga * f.uy);
                  vgrad_add(acc, f.seg_b, gb * f.ux, gb * f.uy);
                }
                const float4 il = S.R[3][t];
                const float invL[3] = {il.x, il.y, il.z};
                float dLk[3];
#pragma unroll
                for (int e = 0; e < 3; ++e) {
                  dLk[e] = -dE[e] * f.e[e] * invL[e];  // dL/dL_e
                  dE[e] = dE[e] * invL[e] + dLdQ * iwk[e];
                }
                if (smooth) {
                  const float4 nn[3] = {n0, n1, n2};
#pragma unroll
                  for (int e = 0; e < 3; ++e) {
                    const float ndu = nn[e].x * du[0] + nn[e].y * du[1] + nn[e].z * du[2];
                    dE[e] += iwk[e] * ndu;
                    diw[e] += f.E[e] * ndu;
                    const float q = f.E[e] * iwk[e];
                    acc[9 + 3 * e + 0] += q * du[0];
                    acc[9 + 3 * e + 1] += q * du[1];
                    acc[9 + 3 * e + 2] += q * du[2];
                  }
                } else {
                  acc[9] += du[0];
                  acc[10] += du[1];
                  acc[11] += du[2];
                }
                // edge e from vertex a=(e+1)%3 to b=(e+2)%3
#pragma unroll
                for (int e = 0; e < 3; ++e) {
                  const int a = (e + 1) % 3, b = (e + 2) % 3;
                  const float Ae = vy[a] - vy[b], Be = vx[b] - vx[a];
                  const float ex = dE[e], el = dLk[e] * invL[e];
                  acc[2 * a] += ex * (vy[b] - py) - el * Be;
                  acc[2 * a + 1] += ex * (px - vx[b]) + el * Ae;
                  acc[2 * b] += ex * (py - vy[a]) + el * Be;
                  acc[2 * b + 1] += ex * (vx[a] - px) - el * Ae;
                }
                acc[0] += dLdarea * (vy[1] - vy[2]);
                acc[1] += dLdarea * (vx[2] - vx[1]);
                acc[2] += dLdarea * (vy[2] - vy[0]);
                acc[3] += dLdarea * (vx[0] - vx[2]);
                acc[4] += dLdarea * (vy[0] - vy[1]);
                acc[5] += dLdarea * (vx[1] - vx[0]);
                acc[6] += diw[0];
                acc[7] += diw[1];
                acc[8] += diw[2];
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
          const float* ta = tacc + t * 24;
          const int slot = __float_as_int(S.R[5][t].z);
          float* ia = iacc + slot * kIacc;
          // instance slot -> node
          int n = 0;
          for (int nn = 0; nn < P.num_nodes; ++nn)
            if (P.nodes[nn].rank_base <= slot) n = nn;
          const MeshDesc& me = P.meshes[P.nodes[n].mesh];
          const bool smooth = (__float_as_uint(S.R[5][t].y) & 8u) != 0u;
          float dM[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, dt[3] = {0.f, 0.f, 0.f};
          float dMn[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
          for (int v = 0; v < 3; ++v) {
            const float4 cv = S.R[10 + v][t];
            const int vi = __float_as_int(cv.w);
            const float cw = cv.z, icw = 1.f / cw;
            const float dsx = ta[2 * v], dsy = ta[2 * v + 1], diw = ta[6 + v];
            const float dcx = dsx * 0.5f * S.W * icw;
            const float dcy = -dsy * 0.5f * S.H * icw;
            const float dcw = (-dsx * 0.5f * S.W * cv.x + dsy * 0.5f * S.H * cv.y) * icw * icw - diw * icw * icw;
            float dw[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) dw[c] = s_vp[c] * dcx + s_vp[4 + c] * dcy + s_vp[12 + c] * dcw;
            const float ox = me.pos[3 * vi], oy = me.pos[3 * vi + 1], oz = me.pos[3 * vi + 2];
#pragma unroll
            for (int rr = 0; rr < 3; ++rr) {
              dt[rr] += dw[rr];
              dM[rr * 3 + 0] += dw[rr] * ox;
              dM[rr * 3 + 1] += dw[rr] * oy;
              dM[rr * 3 + 2] += dw[rr] * oz;
            }
            // normal chain: n = normalize(u), u = M3 n_obj; dL/du = (dn - (dn.n) n) / |u| with
            // |u| = |s| for HPR poses and unit mesh normals, applied per instance
            if (smooth || v == 0) {
              const float4 nv = S.R[7 + v][t];
              const float dn[3] = {ta[9 + 3 * v], ta[10 + 3 * v], ta[11 + 3 * v]};
              const float dd = dn[0] * nv.x + dn[1] * nv.y + dn[2] * nv.z;
              const float nobj[3] = {me.nrm[3 * vi], me.nrm[3 * vi + 1], me.nrm[3 * vi + 2]};
              const float nvv[3] = {nv.x, nv.y, nv.z};
#pragma unroll
              for (int rr = 0; rr < 3; ++rr) {
                const float g = dn[rr] - dd * nvv[rr];
#pragma unroll
                for (int cc = 0; cc < 3; ++cc) dMn[rr * 3 + cc] += g * nobj[cc];
              }
            }
          }
#pragma unroll
          for (int i = 0; i < 9; ++i) atomicAdd(&ia[15 + i], dMn[i]);
#pragma unroll
          for (int i = 0; i < 9; ++i) atomicAdd(&ia[i], dM[i]);
          atomicAdd(&ia[9], dt[0]);
          atomicAdd(&ia[10], dt[1]);
          atomicAdd(&ia[11], dt[2]);
          atomicAdd(&ia[12], ta[18]);
          atomicAdd(&ia[13], ta[19]);
          atomicAdd(&ia[14], ta[20]);
          atomicAdd(&s_light[0], ta[21]);
          atomicAdd(&s_light[1], ta[22]);
          atomicAdd(&s_light[2], ta[23]);
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
            float4* so = reinterpret_cast<float4*>(A.stats + 8 * ((long long)k * HW + q));
            so[0] = make_float4(m0, S0, code, 0.f);
            so[1] = make_float4(dl[0], dl[1], dl[2], 0.f);
          }
        }
      }
    } else {
      // per instance of this scene: dM3 -> d(hpr), d(scale); dt -> d(pos)
      int ninst = 0;
      for (int n = 0; n < P.num_nodes; ++n) ninst = max(ninst, P.nodes[n].rank_base + P.nodes[n].ips);
      for (int s = tid; s < ninst; s += THREADS) {
        float* ia = iacc + s * kIacc;
        int n = 0;
        for (int nn = 0; nn < P.num_nodes; ++nn)
          if (P.nodes[nn].rank_base <= s) n = nn;
        const NodeDesc& nd = P.nodes[n];
        const int li = s - nd.rank_base;
        if (li >= nd.ips) continue;
        const long long id = nd.shared ? (long long)li : (long long)k * nd.ips + li;
        const float* a = nd.rot + id * 3;
        float sh, ch, sp, cp, sr, cr;
        sincosf(a[0], &sh, &ch);
        sincosf(a[1], &sp, &cp);
        sincosf(a[2], &sr, &cr);
        const float sc = nd.scale[id];
        const float Rz[9] = {ch, -sh, 0.f, sh, ch, 0.f, 0.f, 0.f, 1.f};
        const float Ry[9] = {cp, 0.f, sp, 0.f, 1.f, 0.f, -sp, 0.f, cp};
        const float Rx[9] = {1.f, 0.f, 0.f, 0.f, cr, -sr, 0.f, sr, cr};
        const float dRz[9] = {-sh, -ch, 0.f, ch, -sh, 0.f, 0.f, 0.f, 0.f};
        const float dRy[9] = {-sp, 0.f, cp, 0.f, 0.f, 0.f, -cp, 0.f, -sp};
        const float dRx[9] = {0.f, 0.f, 0.f, 0.f, -sr, -cr, 0.f, cr, -sr};
        auto mul = [](const float* X, const float* Y, float* Z) {
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) Z[i * 3 + j] = X[i * 3] * Y[j] + X[i * 3 + 1] * Y[3 + j] + X[i * 3 + 2] * Y[6 + j];
        };
        float T0[9], R[9], Gh[9], Gp[9], Gr[9];
        mul(Rz, Ry, T0);
        mul(T0, Rx, R);
        float T1[9];
        mul(dRz, Ry, T1);
        mul(T1, Rx, Gh);
        mul(Rz, dRy, T1);
        mul(T1, Rx, Gp);
        mul(T0, dRx, Gr);
        float dh = 0.f, dp = 0.f, dr = 0.f, ds = 0.f;
        const float inv_abs_s = sc != 0.f ? 1.f / fabsf(sc) : 0.f;
#pragma unroll
        for (int i = 0; i < 9; ++i) {
          const float g = ia[i] + ia[15 + i] * inv_abs_s;
          dh += g * sc * Gh[i];
          dp += g * sc * Gp[i];
          dr += g * sc * Gr[i];
          ds += g * R[i];
        }
        if (nd.gpos) {
          atomicAdd(&nd.gpos[id * 3 + 0], ia[9]);
          atomicAdd(&nd.gpos[id * 3 + 1], ia[10]);
          atomicAdd(&nd.gpos[id * 3 + 2], ia[11]);
        }
        if (nd.grot) {
          atomicAdd(&nd.grot[id * 3 + 0], dh);
          atomicAdd(&nd.grot[id * 3 + 1], dp);
          atomicAdd(&nd.grot[id * 3 + 2], dr);
        }
        if (nd.gscale) atomicAdd(&nd.gscale[id], ds);
        if (nd.gcol) {
          atomicAdd(&nd.gcol[id * 4 + 0], ia[12]);
          atomicAdd(&nd.gcol[id * 4 + 1], ia[13]);
          atomicAdd(&nd.gcol[id * 4 + 2], ia[14]);
        }
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
