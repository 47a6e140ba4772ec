// pbr_soft.cuh -- the soft-coverage model shared by the soft kernels: triangle
// setup, fragment evaluation, the per-fragment adjoint and the chain from
// per-triangle gradients to per-instance pose, scale, colour and light.
//
// Soft model, per pixel p and front-facing triangle j fully in front of the
// near plane (nothing here exists in the reference; it sits beside the hard
// raster and shares its setup):
//   e_k  = E_k(p) / |(A_k, B_k)|            signed distance to edge line k (px)
//   D_j  = prod_k sigmoid(e_k / sigma) T(d),  d = distance from p to the triangle (0 inside),
//          T = smootherstep((16 sigma - d) / (4 sigma)): C1 everywhere, exactly 0 at 16 sigma
//   w    = sat(area2 / Q),  Q = sum_k E_k iw_k: the perspective-correct clip w of the triangle's
//          plane; sat(x) = x up to the triangle's farthest vertex depth w_hi = max_k w_k, and
//          w_hi + s (1 - exp(-(x - w_hi) / s)) beyond it, s = (zfar - znear) / 8; w_hi + s where
//          Q <= 0.  Inside the triangle nothing changes; outside, the extended plane's depth would
//          run off to infinity near the vanishing line of a face seen nearly edge-on (Q changes sign
//          there, inside the soft footprint), and sat keeps it bounded and smooth in the pose (C1
//          at w_hi, C-infinity across Q = 0)
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
// Cfg - C_r) so the adjoint needs a single sweep over the recomputed fragments.
#pragma once

#include "pbr_device.cuh"

namespace pbr {

constexpr float kSoftCut = 16.f;    // coverage is 0 at 16 sigma or more from the triangle
constexpr float kSoftTaper = 4.f;   // tapered to 0 over the last 4 sigma
constexpr float kSoftDepthSat = 0.125f;  // saturation depth s of the extended plane, / (zfar - znear)
constexpr int kSoftRecs = 15;
constexpr int kIacc = 24; // per-instance gradient accumulator: dM3 (9), dt (3), dcol (3), dM3 normal chain (9)

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
  // one explicit fused multiply-add, so that every kernel that inlines this rounds the same way
  float area2 = fmaf(s1.x - s0.x, s2.y - s0.y, -((s2.x - s0.x) * (s1.y - s0.y)));
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
// the pixel is beyond the cutoff.
struct Frag {
  float E[3], e[3], sg[3], D, Ds, dTdd, Q, w, zs;  // sg = sigmoid per edge, Ds = prod sg, D = Ds * T(d)
  float qsgn;                                       // sign of Q (orients the interpolated normal)
  float zsat;                                       // d sat / dx where saturated (0 where Q <= 0)
  int zk;                                           // saturated beyond vertex zk's depth (-1: not)
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
  f.qsgn = f.Q < 0.f ? -1.f : 1.f;
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
  // normalised depth relative to the scene reference: zs - (zfar - w_ref)/(zfar - znear).  The softmax only
  // sees differences, and this form keeps ~7 significant digits of them where (zfar - w) / (zfar - znear)
  // would keep ~1 after the 1/gamma amplification.  w - w_ref = sum_k q_k d_k / Q with d_k = w_k - w_ref,
  // saturated beyond d_hi = max_k d_k
  {
    const float4 r14 = S.R[14][t];
    const float dd[3] = {r14.z, r14.w, S.R[5][t].w};
    const int hi = dd[1] > dd[0] ? (dd[2] > dd[1] ? 2 : 1) : (dd[2] > dd[0] ? 2 : 0);
    const float sat = kSoftDepthSat * (P.zfar - P.znear);
    float dq;
    f.zk = -1;
    f.zsat = 0.f;
    f.w = 0.f;
    if (f.Q > 0.f) {
      f.w = il.w / f.Q;
      dq = (f.E[0] * iw.x * dd[0] + f.E[1] * iw.y * dd[1] + f.E[2] * iw.z * dd[2]) / f.Q;
      if (dq > dd[hi]) {
        f.zk = hi;
        f.zsat = __expf(-(dq - dd[hi]) / sat);  // the saturated tail needs no more than the fast exponential
        dq = dd[hi] + sat * (1.f - f.zsat);
      }
    } else {
      f.zk = hi;
      dq = dd[hi] + sat;
    }
    f.zs = -dq * inv_zr;
  }
  const float4 n0 = S.R[7][t], n1 = S.R[8][t], n2 = S.R[9][t];
  const float4 col = S.R[6][t];
  const uint32_t fl = __float_as_uint(S.R[5][t].y);
  if (fl & 8u) {
    // perspective-correct normal, oriented by the sign of Q (beyond the plane's vanishing line Q < 0)
    const float q0 = f.E[0] * iw.x * f.qsgn, q1 = f.E[1] * iw.y * f.qsgn, q2 = f.E[2] * iw.z * f.qsgn;
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

// Per-pixel adjoint state: max zs, prod(1 - D) over non-unit factors and their
// count, dL/dA, Cfg - C_r from the forward, dL/dCfg = A dL/dout, 1/S, and the
// colour reference C_r of the first fragment (set on the first call).
// The soft forward's per-pixel statistics for its adjoint, 24 bytes a pixel in
// one [6 * npx] float32 buffer (npx = N * H * W): first a float4 per pixel (the
// largest depth logit m, the softmax sum, the coverage code, dl[0]), then a
// float2 per pixel (dl[1], dl[2]), where dl = (foreground colour) - (colour
// reference); both accesses aligned.
__device__ __forceinline__ void stats_store(float* stats, long long npx, long long q, float4 a, float2 b) {
  reinterpret_cast<float4*>(stats)[q] = a;
  reinterpret_cast<float2*>(stats + 4 * npx)[q] = b;
}

__device__ __forceinline__ void stats_load(const float* stats, long long npx, long long q, float4& a, float2& b) {
  a = reinterpret_cast<const float4*>(stats)[q];
  b = reinterpret_cast<const float2*>(stats + 4 * npx)[q];
}

struct SoftPixB {
  float m, Pnz, nz, dLdA, dl[3], dc[3], invS, Cr[3], ref;
};

// Adjoint of one fragment: adds dL/d(screen x, y of the 3 vertices) [0..5],
// dL/d(iw_k) [6..8], dL/d(normals) [9..17] (flat: [9..11]), dL/d(instance
// colour) [18..20] and dL/d(normalised light direction) [21..23] to acc.
__device__ __forceinline__ void soft_grad(const SceneParams& P, const Frag& f, SoftPixB& pb, float px, float py,
                                          const float vx[3], const float vy[3], const float iwk[3],
                                          const float invL[3], float4 n0, float4 n1, float4 n2, float4 col,
                                          bool smooth, float inv_sigma, float inv_zr, float inv_gamma, float acc[24]) {
  const float Lp = pb.m, Pnz = pb.Pnz, nz = pb.nz;
  if (pb.ref == 0.f) {  // first fragment: the colour reference of the forward
    pb.Cr[0] = f.C[0];
    pb.Cr[1] = f.C[1];
    pb.Cr[2] = f.C[2];
    pb.ref = 1.f;
  }
  const float dc0 = pb.dc[0], dc1 = pb.dc[1], dc2 = pb.dc[2];
  const float dLdA = pb.dLdA;
  const float ewn = expf((f.zs - Lp) * inv_gamma) * pb.invS;
  const float wn = f.D * ewn;
  const float dCx = wn * dc0, dCy = wn * dc1, dCz = wn * dc2;
  // C_j - Cfg = (C_j - C_r) - (Cfg - C_r)
  const float dws = dc0 * ((f.C[0] - pb.Cr[0]) - pb.dl[0]) + dc1 * ((f.C[1] - pb.Cr[1]) - pb.dl[1]) +
                    dc2 * ((f.C[2] - pb.Cr[2]) - pb.dl[2]);
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
  // depth: zs(w), w = area2 / Q; where saturated, w = w_hi + s (1 - e) with e = exp(-(area2 / Q - w_hi) / s)
  // (e = 0 where Q <= 0): dw / d(area2 / Q) = e, dw / dw_hi = 1 - e, w_hi = 1 / iw_zk
  float dLdw = -dLdzs * inv_zr;
  if (f.zk >= 0) {
    const float wh = 1.f / (f.zk == 0 ? iwk[0] : (f.zk == 1 ? iwk[1] : iwk[2]));
    const float g = -dLdw * (1.f - f.zsat) * wh * wh;
    diw[0] += f.zk == 0 ? g : 0.f;
    diw[1] += f.zk == 1 ? g : 0.f;
    diw[2] += f.zk == 2 ? g : 0.f;
    dLdw *= f.zsat;
  }
  const float dLdQ = f.Q > 0.f ? -dLdw * f.w / f.Q : 0.f;
  const float dLdarea = f.Q > 0.f ? dLdw / f.Q : 0.f;
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
  float dLk[3];
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    dLk[e] = -dE[e] * f.e[e] * invL[e];  // dL/dL_e
    dE[e] = dE[e] * invL[e] + dLdQ * iwk[e];
  }
  if (smooth) {
    // u = sign(Q) sum_k q_k n_k
    const float4 nn[3] = {n0, n1, n2};
#pragma unroll
    for (int c = 0; c < 3; ++c) du[c] *= f.qsgn;
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

// Chain triangle t's accumulated gradient ta[24] through the viewport, the
// projection (view-projection vp[16]) and the model matrix into the
// per-instance accumulators iacc[slot][kIacc] and the light gradient
// light[3] (shared-memory atomics).
__device__ __forceinline__ void soft_tri_chain(const SceneParams& P, const SoftCtx& S, int t, const float* ta,
                                               const float* s_vp, float* iacc, int iacc_cap, float* s_light) {
  const int slot = (int)PBR_IX(__float_as_int(S.R[5][t].z), iacc_cap, 35);
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

// Instance slot s of scene k: dM3 -> d(hpr), d(scale); dt -> d(pos); colour.
// Adds into the node's gradient buffers (global atomics).
__device__ __forceinline__ void soft_instance_grads(const SceneParams& P, int k, int s, const float* ia) {
  int n = 0;
  for (int nn = 0; nn < P.num_nodes; ++nn)
    if (P.nodes[nn].rank_base <= s) n = nn;
  const NodeDesc& nd = P.nodes[n];
  const int li = s - nd.rank_base;
  if (li >= nd.ips) return;
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

// Sums v[0..23] over the warp in 27 shuffles (halving the values and the
// lanes each step).  Lane l returns the total of index
// 12*b4 + 6*b3 + 3*b2 + (l & 3), where b_i is bit i of l; lanes with
// (l & 3) == 3 return 0 and hold no index.
__device__ __forceinline__ float warp_reduce24(const float v[24], int lane, int& index) {
  float a[12], b[6], c[3];
  const bool h16 = lane & 16, h8 = lane & 8, h4 = lane & 4;
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    const float send = h16 ? v[i] : v[12 + i], keep = h16 ? v[12 + i] : v[i];
    a[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const float send = h8 ? a[i] : a[6 + i], keep = h8 ? a[6 + i] : a[i];
    b[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float send = h4 ? b[i] : b[3 + i], keep = h4 ? b[3 + i] : b[i];
    c[i] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    c[i] += __shfl_xor_sync(0xffffffffu, c[i], 2);
    c[i] += __shfl_xor_sync(0xffffffffu, c[i], 1);
  }
  const int j = lane & 3;
  index = (h16 ? 12 : 0) + (h8 ? 6 : 0) + (h4 ? 3 : 0) + j;
  return j == 0 ? c[0] : (j == 1 ? c[1] : (j == 2 ? c[2] : 0.f));
}

}  // namespace pbr
