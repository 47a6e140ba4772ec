// pbr_device.cuh -- device helpers shared by the raster kernels: model
// matrices (renderer/shader_context.py:47-84, renderer/node.py:116-126),
// vertex/clip transforms (shaders/basic.vert:29-53), triangle setup with
// watertight FP32 edge functions and the top-left rule, and the shading of
// shaders/basic.frag:20-39.
#pragma once

#include "pbr_kernels.cuh"
#ifdef PBR_SELFCHECK
#include <cstdio>
#endif

namespace pbr {

// Self-checks, compiled in with -DPBR_SELFCHECK only (a debugging build): every
// index wrapped in PBR_IX is checked against the length of the buffer it addresses; a bad
// one is printed (the first 32 per process) and replaced by 0, so that the
// access stays inside the buffer.  Without the macro PBR_IX is the index.
#ifdef PBR_SELFCHECK
static __device__ int g_selfcheck_reports;
static __device__ __noinline__ long long selfcheck_index(long long i, long long n, int site) {
  if (i >= 0 && i < n) return i;
  if (atomicAdd(&g_selfcheck_reports, 1) < 32)
    printf("pbr selfcheck: site %d block %d thread %d index %lld of %lld\n", site, (int)blockIdx.x,
           (int)threadIdx.x, i, n);
  return 0;
}
#define PBR_IX(i, n, site) selfcheck_index((long long)(i), (long long)(n), (site))
#else
#define PBR_IX(i, n, site) (i)
#endif


__device__ __forceinline__ float clamp01f(float v) { return fminf(fmaxf(v, 0.f), 1.f); }

__device__ __forceinline__ uint32_t unorm8(float v) {
  return (uint32_t)floorf(clamp01f(v) * 255.f + 0.5f);
}

__device__ __forceinline__ uint32_t pack_rgba(float r, float g, float b, float a) {
  return unorm8(r) | (unorm8(g) << 8) | (unorm8(b) << 16) | (unorm8(a) << 24);
}

// shaders/basic.frag:33-38 with base = 1 (no texture); n need not be unit length.
__device__ __forceinline__ uint32_t shade_pack(const SceneParams& P, float nx, float ny, float nz, float4 col) {
  float l2 = nx * nx + ny * ny + nz * nz;
  float inv = l2 > 0.f ? rsqrtf(l2) : 0.f;
  float ndl = (nx * P.ldir[0] + ny * P.ldir[1] + nz * P.ldir[2]) * inv;
  ndl = fmaxf(ndl, 0.f);
  const float s = P.strength;
  float r = col.x * ((1.f - s) + (P.amb[0] + ndl * P.lcol[0]) * s);
  float g = col.y * ((1.f - s) + (P.amb[1] + ndl * P.lcol[1]) * s);
  float b = col.z * ((1.f - s) + (P.amb[2] + ndl * P.lcol[2]) * s);
  return pack_rgba(r, g, b, col.w);
}

// shaders/basic.frag:33-38 without the UNORM8 clamp (soft mode: float output).
__device__ __forceinline__ void shade_rgb(const SceneParams& P, float nx, float ny, float nz, float4 col, float out[3]) {
  float l2 = nx * nx + ny * ny + nz * nz;
  float inv = l2 > 0.f ? 1.f / sqrtf(l2) : 0.f;
  float ndl = (nx * P.ldir[0] + ny * P.ldir[1] + nz * P.ldir[2]) * inv;
  ndl = ndl > 0.f ? ndl : 0.f;
  const float s = P.strength;
  out[0] = col.x * ((1.f - s) + (P.amb[0] + ndl * P.lcol[0]) * s);
  out[1] = col.y * ((1.f - s) + (P.amb[1] + ndl * P.lcol[1]) * s);
  out[2] = col.z * ((1.f - s) + (P.amb[2] + ndl * P.lcol[2]) * s);
}

// Model matrix rows (3x4, row-major) of buffer row `id` of a node.  All
// loads are issued before any of them is used (the bound state's values
// replace the node's own afterwards), so their latencies overlap.
__device__ __forceinline__ void build_model(const NodeDesc& nd, long long id, float m[12]) {
  if (nd.mode == kModeMat) {
    const float* s = nd.rot + id * 16;
#pragma unroll
    for (int i = 0; i < 12; ++i) m[i] = s[i];
    return;
  }
  const float* pp = nd.pos + id * 3;
  float t[3] = {pp[0], pp[1], pp[2]};
  const float s = nd.scale[id];
  float R[9];
  if (nd.mode == kModeHpr) {
    const float* rp = nd.rot + id * 3;
    float a[3] = {rp[0], rp[1], rp[2]};
    if (nd.src) {
      const float* sp = nd.src + id * nd.src_stride;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (nd.src_col[c] >= 0) t[c] = sp[nd.src_col[c]];
        if (nd.src_col[3 + c] >= 0) a[c] = sp[nd.src_col[3 + c]];
      }
    }
    float sh, ch, sp, cp, sr, cr;
    sincosf(a[0], &sh, &ch);
    sincosf(a[1], &sp, &cp);
    sincosf(a[2], &sr, &cr);
    // Rz(H) @ Ry(P) @ Rx(R)
    R[0] = ch * cp; R[1] = ch * sp * sr - sh * cr; R[2] = ch * sp * cr + sh * sr;
    R[3] = sh * cp; R[4] = sh * sp * sr + ch * cr; R[5] = sh * sp * cr - ch * sr;
    R[6] = -sp;     R[7] = cp * sr;                R[8] = cp * cr;
  } else {
    const float* a = nd.rot + id * 9;
#pragma unroll
    for (int i = 0; i < 9; ++i) R[i] = a[i];
    if (nd.src) {
      const float* sp = nd.src + id * nd.src_stride;
#pragma unroll
      for (int c = 0; c < 3; ++c)
        if (nd.src_col[c] >= 0) t[c] = sp[nd.src_col[c]];
    }
  }
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    m[r * 4 + 0] = R[r * 3 + 0] * s;
    m[r * 4 + 1] = R[r * 3 + 1] * s;
    m[r * 4 + 2] = R[r * 3 + 2] * s;
    m[r * 4 + 3] = t[r];
  }
}

// Copy the state-bound pose components of buffer row `id` into the node's own
// pose buffers, so that they hold what an explicit per-step copy would.
__device__ __forceinline__ void write_back_bound(const NodeDesc& nd, long long id) {
  if (!nd.src) return;
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    if (nd.src_col[c] >= 0) {
      float* dst = const_cast<float*>(c < 3 ? nd.pos + id * 3 + c : nd.rot + id * 3 + (c - 3));
      *dst = nd.src[id * nd.src_stride + nd.src_col[c]];
    }
  }
}

struct SV {
  float x, y, z, iw;
};

__device__ __forceinline__ SV to_screen(float4 c, float W, float H) {
  SV s;
  s.iw = 1.f / c.w;
  s.x = (c.x * s.iw + 1.f) * 0.5f * W;
  s.y = (1.f - c.y * s.iw) * 0.5f * H;
  s.z = c.z * s.iw * 0.5f + 0.5f;
  // The screen coordinates leave here as opaque values: no multiply of this
  // function may be fused with an add or subtract of the caller (the setup's
  // v1.x - v0.x, say), so every setup of the same vertices rounds alike,
  // wherever it is inlined.
  asm("" : "+f"(s.x), "+f"(s.y), "+f"(s.z), "+f"(s.iw));
  return s;
}

// Per-item context for the triangle setup.
struct SetupCtx {
  float4* T0;
  float4* T1;
  float4* T2;
  float4* T3;
  float4* T4;
  float4* S0;
  float4* S1;
  float4* S2;
  float4* S3;
  float4* S4;
  float4* S5;
  float W, H;
  float ry0, ry1;  // region rows (inclusive)
  int cull;
};

// Edge k of (v0,v1,v2) runs from v[(k+1)%3] to v[(k+2)%3].  Its function is
// evaluated from the lexicographically smaller endpoint so that the two
// triangles sharing an edge compute exactly negated values (watertight).
__device__ __forceinline__ float4 make_edge(float xa, float ya, float xb, float yb, bool& tl) {
  const bool a_first = (xa < xb) || (xa == xb && ya < yb);
  const float xf = a_first ? xa : xb, yf = a_first ? ya : yb;
  const float xs = a_first ? xb : xa, ys = a_first ? yb : ya;
  float A = yf - ys, B = xs - xf;
  if (!a_first) { A = -A; B = -B; }
  tl = (A > 0.f) || (A == 0.f && B > 0.f);
  return make_float4(A, B, xf, yf);
}

// Texture input of one triangle: its vertices' texture coordinates and the
// node whose texture it samples (node < 0: untextured).
struct TexIn {
  float2 t0 = {0.f, 0.f}, t1 = {0.f, 0.f}, t2 = {0.f, 0.f};
  int node = -1;
};

__device__ __forceinline__ float2 mesh_uv(const MeshDesc& me, int i) {
  return me.uv ? make_float2(me.uv[2 * i], me.uv[2 * i + 1]) : make_float2(0.f, 0.f);
}

// Triangle setup from screen-space vertices (to_screen of the clip
// coordinates).  Returns 1 when the triangle is kept (and, if WRITE, its
// records are written at slot), 0 when it is culled or covers no pixel centre.
// A textured triangle (tx.node >= 0) is shaded per pixel: pass smooth = true.
template <bool WRITE>
__device__ __forceinline__ int setup_tri_sv(const SceneParams& P, const SetupCtx& S, SV v0, float4 n0, SV v1,
                                            float4 n1, SV v2, float4 n2, int slot, float4 col, int draw_id,
                                            bool smooth, TexIn tx = TexIn()) {
  // one explicit fused multiply-add, so that every kernel that inlines this rounds the same way
  float area2 = fmaf(v1.x - v0.x, v2.y - v0.y, -((v2.x - v0.x) * (v1.y - v0.y)));
  if (S.cull) {
    if (!(area2 < 0.f)) return 0;  // back-facing, degenerate or NaN
  } else {
    if (!(area2 < 0.f) && !(area2 > 0.f)) return 0;
  }
  if (area2 < 0.f) {
    SV t = v1; v1 = v2; v2 = t;
    float4 tn = n1; n1 = n2; n2 = tn;
    float2 tt = tx.t1; tx.t1 = tx.t2; tx.t2 = tt;
    area2 = -area2;
  }
  const float mnx = fminf(fminf(v0.x, v1.x), v2.x), mxx = fmaxf(fmaxf(v0.x, v1.x), v2.x);
  const float mny = fminf(fminf(v0.y, v1.y), v2.y), mxy = fmaxf(fmaxf(v0.y, v1.y), v2.y);
  // pixels whose centre can lie inside, widened by 1e-3 px (the edge test decides)
  float fx0 = fmaxf(ceilf(mnx - 0.501f), 0.f), fx1 = fminf(floorf(mxx - 0.499f), S.W - 1.f);
  float fy0 = fmaxf(ceilf(mny - 0.501f), S.ry0), fy1 = fminf(floorf(mxy - 0.499f), S.ry1);
  if (!(fx0 <= fx1 && fy0 <= fy1)) return 0;
  if (!WRITE) return 1;

  bool tl0, tl1, tl2;
  const float4 e0 = make_edge(v1.x, v1.y, v2.x, v2.y, tl0);
  const float4 e1 = make_edge(v2.x, v2.y, v0.x, v0.y, tl1);
  const float4 e2 = make_edge(v0.x, v0.y, v1.x, v1.y, tl2);
  const float ia = 1.f / area2;
  const float zA = fmaf(e2.x, v2.z, fmaf(e1.x, v1.z, e0.x * v0.z)) * ia;
  const float zB = fmaf(e2.y, v2.z, fmaf(e1.y, v1.z, e0.y * v0.z)) * ia;
  const float zC = fmaf(-zB, v0.y, fmaf(-zA, v0.x, v0.z));
  const uint32_t xbox = (uint32_t)fx0 | ((uint32_t)fx1 << 16);
  const uint32_t ybox = (uint32_t)fy0 | ((uint32_t)fy1 << 16);
  const bool textured = smooth && tx.node >= 0;
  const uint32_t flags =
      (tl0 ? 1u : 0u) | (tl1 ? 2u : 0u) | (tl2 ? 4u : 0u) | (smooth ? 8u : 0u) | (textured ? 16u : 0u);
  const uint32_t color = smooth ? 0u : shade_pack(P, n0.x, n0.y, n0.z, col);
  S.T0[slot] = e0;
  S.T1[slot] = e1;
  S.T2[slot] = e2;
  S.T3[slot] = make_float4(zA, zB, zC, __uint_as_float(xbox));
  S.T4[slot] = make_float4(__uint_as_float(ybox), __uint_as_float(flags), __uint_as_float(color),
                           __int_as_float(draw_id));
  if (smooth) {
    S.S0[slot] = make_float4(n0.x, n0.y, n0.z, v0.iw);
    S.S1[slot] = make_float4(n1.x, n1.y, n1.z, v1.iw);
    S.S2[slot] = make_float4(n2.x, n2.y, n2.z, v2.iw);
    S.S3[slot] = col;
    if (textured) {
      S.S4[slot] = make_float4(tx.t0.x, tx.t0.y, tx.t1.x, tx.t1.y);
      S.S5[slot] = make_float4(tx.t2.x, tx.t2.y, __int_as_float(tx.node), 0.f);
    }
  }
  return 1;
}

// A record that covers no pixel: empty x and y ranges (low end above the high
// end), so that the binner gives it no bin.  The tile kernel fills a slot it
// reserved with one when the write pass does not emit the triangle it counted.
__device__ __forceinline__ void write_empty(const SetupCtx& S, int slot) {
  S.T3[slot].w = __uint_as_float(1u);       // x: [1, 0]
  S.T4[slot].x = __uint_as_float(0xffffu);  // y: [65535, 0]
}

template <bool WRITE>
__device__ __forceinline__ int setup_tri(const SceneParams& P, const SetupCtx& S, float4 c0, float4 n0, float4 c1,
                                         float4 n1, float4 c2, float4 n2, int slot, float4 col, int draw_id,
                                         bool smooth, const TexIn& tx) {
  const SV v0 = to_screen(c0, S.W, S.H), v1 = to_screen(c1, S.W, S.H), v2 = to_screen(c2, S.W, S.H);
  return setup_tri_sv<WRITE>(P, S, v0, n0, v1, n1, v2, n2, slot, col, draw_id, smooth, tx);
}

__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float t) {
  return make_float4(a.x + t * (b.x - a.x), a.y + t * (b.y - a.y), a.z + t * (b.z - a.z), a.w + t * (b.w - a.w));
}

__device__ __forceinline__ float2 lerp2(float2 a, float2 b, float t) {
  return make_float2(a.x + t * (b.x - a.x), a.y + t * (b.y - a.y));
}

// Near-plane clip (Sutherland-Hodgman against z + w >= 0: at most 4
// vertices) and fan emission of a triangle that crosses the plane.  Crossing
// points are interpolated from the endpoint with the smaller mesh index so
// that neighbouring triangles produce identical vertices.  Its arrays live in
// local memory, touched only on this rare path.  With WRITE and limit >= 0
// exactly `limit` records are written from slot on (the kept fan triangles,
// at most limit of them, then empty records), for callers that reserved
// slots from an earlier count.
template <bool WRITE>
__device__ __forceinline__ int clip_tri(const SceneParams& P, const SetupCtx& S, float4 c0, float4 n0, float4 c1,
                                     float4 n1, float4 c2, float4 n2, int i0, int i1, int i2, int slot, float4 col,
                                     int draw_id, bool smooth, const TexIn& tx = TexIn(), int limit = -1) {
  const float4 c[3] = {c0, c1, c2};
  const float4 n[3] = {n0, n1, n2};
  const float2 uv[3] = {tx.t0, tx.t1, tx.t2};
  const int id[3] = {i0, i1, i2};
  const float d[3] = {c0.z + c0.w, c1.z + c1.w, c2.z + c2.w};
  float4 pc[4], pn[4];
  float2 pt[4];
  int np = 0;
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    const int a = e, b = (e + 1) % 3;
    const bool ina = d[a] >= 0.f, inb = d[b] >= 0.f;
    if (ina) { pc[np] = c[a]; pn[np] = n[a]; pt[np] = uv[a]; ++np; }
    if (ina != inb) {
      const int f = id[a] < id[b] ? a : b, s = id[a] < id[b] ? b : a;
      const float t = d[f] / (d[f] - d[s]);
      pc[np] = lerp4(c[f], c[s], t);
      pn[np] = lerp4(n[f], n[s], t);
      pt[np] = lerp2(uv[f], uv[s], t);
      ++np;
    }
  }
  int cnt = 0;
  for (int f = 1; f + 1 < np; ++f) {
    if (WRITE && limit >= 0 && cnt >= limit) break;
    TexIn ft;
    ft.t0 = pt[0];
    ft.t1 = pt[f];
    ft.t2 = pt[f + 1];
    ft.node = tx.node;
    cnt += setup_tri<WRITE>(P, S, pc[0], pn[0], pc[f], pn[f], pc[f + 1], pn[f + 1], slot + cnt, col, draw_id, smooth,
                            ft);
  }
  if (WRITE && limit >= 0)
    for (; cnt < limit; ++cnt) write_empty(S, slot + cnt);
  return cnt;
}

// GL bilinear sample with repeat wrap (the sampler Panda3D gives a loaded
// texture: linear filtering, no mipmaps) at texture coordinates (u, v):
// texel centres at (i + 0.5) / w, RGBA8 texels read as c / 255.  Every index
// is wrapped into [0, w) x [0, h), also for infinite or NaN coordinates.
__device__ __forceinline__ float3 sample_texture(const NodeDesc& nd, float u, float v) {
  const int w = nd.tex_w, h = nd.tex_h;
  if (!nd.tex || w <= 0 || h <= 0) return make_float3(1.f, 1.f, 1.f);
  const float x = fmaf(u - floorf(u), (float)w, -0.5f), y = fmaf(v - floorf(v), (float)h, -0.5f);
  const float fx = floorf(x), fy = floorf(y);
  const float ax = x - fx, ay = y - fy;
  // fx lies in [-1, w - 1]; -1 wraps to w - 1 (fmaxf maps a NaN to -1 as well)
  int x0 = (int)fminf(fmaxf(fx, -1.f), (float)(w - 1));
  int y0 = (int)fminf(fmaxf(fy, -1.f), (float)(h - 1));
  x0 = x0 < 0 ? w - 1 : x0;
  y0 = y0 < 0 ? h - 1 : y0;
  const int x1 = x0 + 1 == w ? 0 : x0 + 1, y1 = y0 + 1 == h ? 0 : y0 + 1;
  const uint32_t* row0 = nd.tex + (long long)y0 * w;
  const uint32_t* row1 = nd.tex + (long long)y1 * w;
  const uint32_t t00 = __ldg(row0 + x0), t10 = __ldg(row0 + x1), t01 = __ldg(row1 + x0), t11 = __ldg(row1 + x1);
  float out[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int sh = 8 * c;
    const float c00 = (float)((t00 >> sh) & 255u) / 255.f, c10 = (float)((t10 >> sh) & 255u) / 255.f;
    const float c01 = (float)((t01 >> sh) & 255u) / 255.f, c11 = (float)((t11 >> sh) & 255u) / 255.f;
    const float top = (1.f - ax) * c00 + ax * c10, bot = (1.f - ax) * c01 + ax * c11;
    out[c] = (1.f - ay) * top + ay * bot;
  }
  return make_float3(out[0], out[1], out[2]);
}

// Per-pixel shading of chunk triangle t at pixel centre (px, py): smooth
// normals and, for textured triangles (flag 16; only when TEX), base = texture(v_uv).
template <bool TEX = true>
__device__ __forceinline__ uint32_t shade_smooth(const SceneParams& P, const SetupCtx& S, int t, float px, float py) {
  const float4 e0 = S.T0[t], e1 = S.T1[t], e2 = S.T2[t];
  const float E0 = fmaf(e0.x, px - e0.z, e0.y * (py - e0.w));
  const float E1 = fmaf(e1.x, px - e1.z, e1.y * (py - e1.w));
  const float E2 = fmaf(e2.x, px - e2.z, e2.y * (py - e2.w));
  const float4 a0 = S.S0[t], a1 = S.S1[t], a2 = S.S2[t];
  // perspective-correct interpolation; the common 1/area2 and 1/sum factors
  // cancel in the normalisation of shade_pack
  const float q0 = E0 * a0.w, q1 = E1 * a1.w, q2 = E2 * a2.w;
  const float nx = q0 * a0.x + q1 * a1.x + q2 * a2.x;
  const float ny = q0 * a0.y + q1 * a1.y + q2 * a2.y;
  const float nz = q0 * a0.z + q1 * a1.z + q2 * a2.z;
  float4 col = S.S3[t];
  if (TEX && (__float_as_uint(S.T4[t].y) & 16u)) {
    // basic.frag:31-32,38: base * v_color.rgb, v_uv interpolated perspective-correct
    const float4 u01 = S.S4[t], u2n = S.S5[t];
    const float qs = q0 + q1 + q2;
    const float iq = qs != 0.f ? 1.f / qs : 0.f;
    const float u = (q0 * u01.x + q1 * u01.z + q2 * u2n.x) * iq;
    const float v = (q0 * u01.y + q1 * u01.w + q2 * u2n.y) * iq;
    const float3 base = sample_texture(P.nodes[__float_as_int(u2n.z)], u, v);
    col.x = base.x * col.x;
    col.y = base.y * col.y;
    col.z = base.z * col.z;
  }
  return shade_pack(P, nx, ny, nz, col);
}

}  // namespace pbr
