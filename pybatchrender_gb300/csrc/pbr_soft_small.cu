// pbr_soft_small.cu -- scene-per-warp soft-coverage forward and adjoint for
// small scenes (the differentiable CartPole renders thousands of 64x64 scenes
// of a few dozen triangles).  The model and its adjoint are in pbr_soft.cuh;
// this kernel only changes how the work is laid out:
//
//   K1  instances flattened over nodes (lane = instance), then lane = vertex:
//       clip position, world normal and the depth offset from the scene
//       reference (shaders/basic.vert:29-53)
//   K2  lane = triangle: soft setup (cull, drop triangles crossing the near
//       plane, bbox widened by the coverage cutoff), compacted in draw order
//   K3  8x4-pixel blocks, one pixel per lane: each triangle marks the blocks
//       its widened bbox touches (shared-memory atomicOr on per-block masks),
//       then every block with candidates evaluates them in draw order.
//       Forward: online softmax per pixel, output and statistics written for
//       that block only (the rest of the scene is written as background first).
//       Adjoint: per (block, triangle) the lanes' 24 gradient terms are summed
//       by a halving warp reduction into the triangle's accumulator.
//   K4  adjoint only: lane = triangle, chain to the instance accumulators;
//       lane = instance, chain to pose / scale / colour (global atomics).
//
// Statistics are written only for pixels of blocks with candidates; the
// adjoint reads them only there (it recomputes the same block masks).
#include "pbr_launch.h"
#include "pbr_soft.cuh"

namespace pbr {

constexpr int kSoftWarps = 4;  // warps per block
constexpr int kBlkW = 8, kBlkH = 4;

struct SoftSmallLayout {
  int rec[15];
  int vcache, itab, vp, bmask, tacc, iacc, light, per_warp;
};

__host__ __device__ inline SoftSmallLayout soft_small_layout(int tri_cap, int vcap, int icap, int nblocks,
                                                             bool backward) {
  SoftSmallLayout L;
  int off = 0;
  for (int i = 0; i < kSoftRecs; ++i) { L.rec[i] = off; off += align16(tri_cap * 16); }
  L.vcache = off; off += align16(vcap * 32);
  L.itab = off; off += align16(icap * 80);
  L.vp = off; off += 64;
  L.bmask = off; off += align16(nblocks * ((tri_cap + 31) / 32) * 4);
  if (backward) {
    L.tacc = off; off += align16(tri_cap * 24 * 4);
    L.iacc = off; off += align16(icap * kIacc * 4);
    L.light = off; off += 16;
  } else {
    L.tacc = L.iacc = L.light = 0;
  }
  L.per_warp = align16(off);
  return L;
}

int soft_small_warps() { return kSoftWarps; }

int soft_small_smem_per_warp(const SoftArgs& a, int W, int H) {
  const int nblocks = ((W + kBlkW - 1) / kBlkW) * ((H + kBlkH - 1) / kBlkH);
  return soft_small_layout(a.tri_cap, a.vcap, a.icap, nblocks, a.backward != 0).per_warp;
}

__device__ __forceinline__ int soft_node_count(const NodeDesc& nd, int k) {
  const int c = nd.counts ? nd.counts[k] : nd.ips;
  return max(0, min(c, nd.ips));
}

template <bool BACKWARD>
__global__ void __launch_bounds__(kSoftWarps * 32) soft_small_kernel(const __grid_constant__ SceneParams P,
                                                                     const __grid_constant__ SoftArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int W = P.W, H = P.H, HW = W * H;
  const int nbx = (W + kBlkW - 1) / kBlkW, nby = (H + kBlkH - 1) / kBlkH;
  const int nblocks = nbx * nby;
  const int words = (A.tri_cap + 31) >> 5;
  const SoftSmallLayout L = soft_small_layout(A.tri_cap, A.vcap, A.icap, nblocks, BACKWARD);
  unsigned char* base = smem + warp * L.per_warp;
  SoftCtx S;
#pragma unroll
  for (int i = 0; i < kSoftRecs; ++i) S.R[i] = reinterpret_cast<float4*>(base + L.rec[i]);
  S.W = (float)W;
  S.H = (float)H;
  S.ry0 = 0.f;
  S.ry1 = (float)(H - 1);
  S.cut = kSoftCut * P.sigma;
  float4* vcache = reinterpret_cast<float4*>(base + L.vcache);
  float4* itab = reinterpret_cast<float4*>(base + L.itab);  // per instance: 3 matrix rows, colour, meta
  float* s_vp = reinterpret_cast<float*>(base + L.vp);
  uint32_t* bmask = reinterpret_cast<uint32_t*>(base + L.bmask);  // [nblocks][words]
  float* tacc = reinterpret_cast<float*>(base + L.tacc);          // [tri_cap][24]
  float* iacc = reinterpret_cast<float*>(base + L.iacc);          // [icap][kIacc]
  float* s_light = reinterpret_cast<float*>(base + L.light);
  const float inv_sigma = 1.f / P.sigma;
  const float inv_zr = 1.f / (P.zfar - P.znear);
  const float inv_gamma = 1.f / P.gamma;
  const int lx = lane & (kBlkW - 1), ly = lane / kBlkW;

  const int split = max(1, A.split);
  for (int gw = blockIdx.x * kSoftWarps + warp; gw / split < P.N; gw += gridDim.x * kSoftWarps) {
    // scene k; this warp takes the pixel blocks b with b % split == sub (all of them when split == 1)
    const int k = gw / split, sub = gw - k * split;
    if (lane < 16) s_vp[lane] = P.vp[(long long)k * 16 + lane];

    // ---- K1: instance table, flattened over nodes in draw order ---------
    int total_inst = 0, total_verts = 0, total_tris = 0;
    for (int n = 0; n < P.num_nodes; ++n) {
      const NodeDesc& nd = P.nodes[n];
      const int cnt = soft_node_count(nd, k);
      const MeshDesc& me = P.meshes[nd.mesh];
      total_inst += cnt;
      total_verts += cnt * me.nv;
      total_tris += cnt * me.nt;
    }
    for (int i = lane; i < total_inst; i += 32) {
      int n = 0, ai = 0, av = 0, at = 0;
      for (; n < P.num_nodes; ++n) {
        const int cnt = soft_node_count(P.nodes[n], k);
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
      float m[12];
      build_model(nd, id, m);
      float4* e = itab + i * 5;
      e[0] = make_float4(m[0], m[1], m[2], m[3]);
      e[1] = make_float4(m[4], m[5], m[6], m[7]);
      e[2] = make_float4(m[8], m[9], m[10], m[11]);
      e[3] = *reinterpret_cast<const float4*>(nd.color + id * 4);
      // meta: node, first vertex, instance slot (gradient accumulator), first triangle
      e[4] = make_float4(__int_as_float(n), __int_as_float(av + li * me.nv), __int_as_float(nd.rank_base + li),
                         __int_as_float(at + li * me.nt));
    }
    if (BACKWARD) {
      for (int i = lane; i < A.icap * kIacc; i += 32) iacc[i] = 0.f;
      if (lane < 4) s_light[lane] = 0.f;
    }
    __syncwarp();

    // ---- K1: vertices ------------------------------------------------------
    for (int v = lane; v < total_verts; v += 32) {
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
    __syncwarp();

    // ---- K2: triangles, compacted in draw order -------------------------
    int T = 0;
    for (int t0 = 0; t0 < total_tris; t0 += 32) {
      const int t = t0 + lane;
      int c = 0, inst = 0, i0 = 0, i1 = 0, i2 = 0, vb = 0;
      bool smooth = false;
      if (t < total_tris) {
        while (inst + 1 < total_inst && __float_as_int(itab[(inst + 1) * 5 + 4].w) <= t) ++inst;
        const float4 meta = itab[inst * 5 + 4];
        const MeshDesc& me = P.meshes[P.nodes[__float_as_int(meta.x)].mesh];
        const int ti = t - __float_as_int(meta.w);
        vb = __float_as_int(meta.y);
        smooth = me.smooth != 0;
        i0 = me.idx[3 * ti];
        i1 = me.idx[3 * ti + 1];
        i2 = me.idx[3 * ti + 2];
        c = soft_setup<false>(P, S, vcache[2 * (vb + i0)], vcache[2 * (vb + i0) + 1], i0, vcache[2 * (vb + i1)],
                              vcache[2 * (vb + i1) + 1], i1, vcache[2 * (vb + i2)], vcache[2 * (vb + i2) + 1], i2, 0,
                              itab[inst * 5 + 3], 0, smooth);
      }
      int incl = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      if (c > 0)
        soft_setup<true>(P, S, vcache[2 * (vb + i0)], vcache[2 * (vb + i0) + 1], i0, vcache[2 * (vb + i1)],
                         vcache[2 * (vb + i1) + 1], i1, vcache[2 * (vb + i2)], vcache[2 * (vb + i2) + 1], i2,
                         T + incl - c, itab[inst * 5 + 3], __float_as_int(itab[inst * 5 + 4].z), smooth);
      T += total;
    }
    __syncwarp();

    // ---- K3: block masks ----------------------------------------------------
    for (int i = lane; i < nblocks * words; i += 32) bmask[i] = 0u;
    if (BACKWARD)
      for (int i = lane; i < T * 24; i += 32) tacc[i] = 0.f;
    __syncwarp();
    for (int t = 0; t < T; ++t) {
      const uint32_t xb = __float_as_uint(S.R[4][t].w), yb = __float_as_uint(S.R[5][t].x);
      const int bx0 = (int)(xb & 0xffffu) / kBlkW, bx1 = (int)(xb >> 16) / kBlkW;
      const int by0 = (int)(yb & 0xffffu) / kBlkH, by1 = (int)(yb >> 16) / kBlkH;
      const uint32_t bit = 1u << (t & 31);
      for (int by = by0; by <= by1; ++by)
        for (int bx = bx0 + lane; bx <= bx1; bx += 32) atomicOr(&bmask[(by * nbx + bx) * words + (t >> 5)], bit);
    }
    __syncwarp();

    if (!BACKWARD && split == 1) {
      // the whole scene as background: float4 stores per plane
      const int n4 = HW >> 2;
      float4* o4 = reinterpret_cast<float4*>(A.out + (long long)k * 3 * HW);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float4 v = make_float4(P.bg[c], P.bg[c], P.bg[c], P.bg[c]);
        for (int i = lane; i < n4; i += 32) o4[c * n4 + i] = v;
      }
      __syncwarp();
    }

    // ---- K3: the blocks with candidates, one pixel per lane ----------------
    for (int b0 = 0; b0 < nblocks; b0 += 32) {
      uint32_t any = 0u;
      const bool mine = (b0 + lane < nblocks) && ((b0 + lane) % split == sub);
      if (mine)
        for (int w = 0; w < words; ++w) any |= bmask[(b0 + lane) * words + w];
      uint32_t todo = __ballot_sync(0xffffffffu, mine && any != 0u);
      if (!BACKWARD && split > 1) {
        // background for this warp's blocks without candidates, one pixel per lane
        uint32_t empty = __ballot_sync(0xffffffffu, mine && any == 0u);
        while (empty) {
          const int b = b0 + __ffs(empty) - 1;
          empty &= empty - 1u;
          const int by = b / nbx, bx = b - by * nbx;
          const int x = bx * kBlkW + lx, y = by * kBlkH + ly;
          if (x < W && y < H) {
            float* o = A.out + (long long)k * 3 * HW + y * W + x;
            o[0] = P.bg[0];
            o[HW] = P.bg[1];
            o[2 * HW] = P.bg[2];
          }
        }
      }
      while (todo) {
        const int b = b0 + __ffs(todo) - 1;
        todo &= todo - 1u;
        const int by = b / nbx, bx = b - by * nbx;
        const int x = bx * kBlkW + lx, y = by * kBlkH + ly;
        const bool active = x < W && y < H;
        const float px = (float)x + 0.5f, py = (float)y + 0.5f;
        const long long q = (long long)k * HW + y * W + x;
        if (!BACKWARD) {
          float m = -1e30f, Ssum = 0.f, acc0 = 0.f, acc1 = 0.f, acc2 = 0.f, Pv = 1.f, nz = 0.f;
          float cr0 = 0.f, cr1 = 0.f, cr2 = 0.f, ref = 0.f;
          for (int w = 0; w < words; ++w) {
            uint32_t mk = bmask[b * words + w];
            while (mk) {
              const int t = w * 32 + __ffs(mk) - 1;
              mk &= mk - 1u;
              Frag f;
              if (!active || !soft_frag(P, S, t, px, py, inv_sigma, inv_zr, f)) continue;
              if (1.f - f.D == 0.f) nz += 1.f;
              else Pv *= (1.f - f.D);
              if (ref == 0.f) {  // first fragment: the colour reference
                cr0 = f.C[0];
                cr1 = f.C[1];
                cr2 = f.C[2];
                ref = 1.f;
              }
              const float d0 = f.C[0] - cr0, d1 = f.C[1] - cr1, d2 = f.C[2] - cr2;
              if (f.zs > m) {
                const float sc = expf((m - f.zs) * inv_gamma);
                Ssum = Ssum * sc + f.D;
                acc0 = acc0 * sc + f.D * d0;
                acc1 = acc1 * sc + f.D * d1;
                acc2 = acc2 * sc + f.D * d2;
                m = f.zs;
              } else {
                const float wv = f.D * expf((f.zs - m) * inv_gamma);
                Ssum += wv;
                acc0 += wv * d0;
                acc1 += wv * d1;
                acc2 += wv * d2;
              }
            }
          }
          if (active) {
            const float Av = 1.f - (nz > 0.f ? 0.f : Pv);
            const float dl0 = Ssum > 0.f ? acc0 / Ssum : 0.f;  // Cfg - C_r
            const float dl1 = Ssum > 0.f ? acc1 / Ssum : 0.f;
            const float dl2 = Ssum > 0.f ? acc2 / Ssum : 0.f;
            float* o = A.out + (long long)k * 3 * HW + y * W + x;
            o[0] = Av * (cr0 + dl0) + (1.f - Av) * P.bg[0];
            o[HW] = Av * (cr1 + dl1) + (1.f - Av) * P.bg[1];
            o[2 * HW] = Av * (cr2 + dl2) + (1.f - Av) * P.bg[2];
            if (A.stats) {
              // coverage code: prod over non-zero (1 - D), folded with the count of zero factors
              const float code = nz == 0.f ? Pv : (nz == 1.f ? -1.f - Pv : -3.f);
              stats_store(A.stats, (long long)P.N * HW, q, make_float4(m, Ssum, code, dl0), make_float2(dl1, dl2));
            }
          }
        } else {
          SoftPixB pb;
          pb.m = -1e30f;
          pb.Pnz = 1.f;
          pb.nz = 0.f;
          pb.dLdA = 0.f;
          pb.invS = 0.f;
          pb.ref = 0.f;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            pb.dl[c] = 0.f;
            pb.dc[c] = 0.f;
            pb.Cr[c] = 0.f;
          }
          if (active) {
            float4 stv;
            float2 stw;
            stats_load(A.stats, (long long)P.N * HW, q, stv, stw);
            const float code = stv.z;
            float Pnz, nzv;
            if (code >= 0.f) { Pnz = code; nzv = 0.f; } else if (code >= -2.f) { Pnz = -1.f - code; nzv = 1.f; } else { Pnz = 0.f; nzv = 2.f; }
            const float Av = nzv > 0.f ? 1.f : 1.f - Pnz;
            float g[3], cf[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const long long oi = ((long long)k * 3 + c) * HW + y * W + x;
              g[c] = A.gout[oi];
              cf[c] = Av > 0.f ? (A.out[oi] - (1.f - Av) * P.bg[c]) / Av : 0.f;
            }
            pb.m = stv.x;
            pb.Pnz = Pnz;
            pb.nz = nzv;
            // dL/dA = g . (Cfg - bg); Cfg from the output is accurate enough here
            // (this term is not amplified by 1/gamma)
            pb.dLdA = g[0] * (cf[0] - P.bg[0]) + g[1] * (cf[1] - P.bg[1]) + g[2] * (cf[2] - P.bg[2]);
            pb.invS = stv.y > 0.f ? 1.f / stv.y : 0.f;
            pb.dl[0] = stv.w;
            pb.dl[1] = stw.x;
            pb.dl[2] = stw.y;
#pragma unroll
            for (int c = 0; c < 3; ++c) pb.dc[c] = Av * g[c];
          }
          for (int w = 0; w < words; ++w) {
            uint32_t mk = bmask[b * words + w];
            while (mk) {
              const int t = w * 32 + __ffs(mk) - 1;
              mk &= mk - 1u;
              float acc[24];
#pragma unroll
              for (int i = 0; i < 24; ++i) acc[i] = 0.f;
              Frag f;
              const bool hit = active && soft_frag(P, S, t, px, py, inv_sigma, inv_zr, f);
              if (hit) {
                const float4 v01 = S.R[13][t], v2 = S.R[14][t];
                const float vx[3] = {v01.x, v01.z, v2.x}, vy[3] = {v01.y, v01.w, v2.y};
                const float4 iwr = S.R[4][t], il = S.R[3][t];
                const float iwk[3] = {iwr.x, iwr.y, iwr.z}, invL[3] = {il.x, il.y, il.z};
                const bool smooth = (__float_as_uint(S.R[5][t].y) & 8u) != 0u;
                soft_grad(P, f, pb, px, py, vx, vy, iwk, invL, S.R[7][t], S.R[8][t], S.R[9][t], S.R[6][t], smooth,
                          inv_sigma, inv_zr, inv_gamma, acc);
              }
              if (__any_sync(0xffffffffu, hit)) {
                int idx;
                const float v = warp_reduce24(acc, lane, idx);
                if ((lane & 3) != 3) tacc[t * 24 + idx] += v;
              }
            }
          }
        }
      }
    }

    if (BACKWARD) {
      __syncwarp();
      // ---- K4: triangle -> instance -> pose, scale, colour ------------------
      for (int t = lane; t < T; t += 32) soft_tri_chain(P, S, t, tacc + t * 24, s_vp, iacc, A.iacc_cap, s_light);
      __syncwarp();
      for (int s = lane; s < total_inst; s += 32) {
        // this scene's instance s is the instance slot stored in its meta
        const int slot = __float_as_int(itab[s * 5 + 4].z);
        soft_instance_grads(P, k, slot, iacc + slot * kIacc);
      }
      if (lane < 3 && A.glight) atomicAdd(&A.glight[lane], s_light[lane]);
      __syncwarp();
    }
  }
}

// ---------------------------------------------------------------------------

static const void* pick_soft_small(bool backward) {
  return backward ? (const void*)&soft_small_kernel<true> : (const void*)&soft_small_kernel<false>;
}

cudaError_t soft_small_set_smem_limit(bool backward, int bytes) {
  return cudaFuncSetAttribute(pick_soft_small(backward), cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

cudaError_t soft_small_launch(bool backward, const SceneParams& P, const SoftArgs& A, int grid, int smem_bytes,
                              cudaStream_t stream) {
  void* args[] = {const_cast<SceneParams*>(&P), const_cast<SoftArgs*>(&A)};
  return cudaLaunchKernel(pick_soft_small(backward), dim3(grid), dim3(kSoftWarps * 32), args, (size_t)smem_bytes,
                          stream);
}

}  // namespace pbr
