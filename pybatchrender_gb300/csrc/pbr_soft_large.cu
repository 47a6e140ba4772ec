// pbr_soft_large.cu -- binned soft-coverage forward and adjoint for scenes of
// thousands of triangles (e.g. 128 instances of 320- and 12-triangle meshes
// per 128x128 scene).  The model and its adjoint are in pbr_soft.cuh.
//
// Persistent CTAs, one scene at a time, each with its own slab of global
// scratch (sized for the scene's source triangles, allocated once):
//
//   A  instance batches (model matrices in shared memory); rounds of THREADS
//      source triangles, one per thread: vertex transform, soft setup (cull,
//      drop triangles crossing the near plane, bbox widened by the cutoff).
//      Survivors are compacted in draw order (warp prefix sums + per-warp
//      totals, one barrier per round), their records written to the slab,
//      and the bit of each survivor is set in the masks of the 8x4-pixel
//      blocks that hold a pixel centre within the coverage cutoff of its
//      vertices' bbox (atomicOr): per block one bit per survivor, so a
//      block's candidates are read back in draw order.
//   B  warps take blocks in turn, one pixel per lane: the block's mask words
//      are read 32 at a time (coalesced), and the set bits give the
//      candidates in draw order.  Forward: online softmax per pixel in
//      registers, output + statistics for blocks with candidates,
//      background otherwise.  Adjoint: per (block, candidate) the lanes' 24
//      gradient terms are summed by the halving warp reduction into the
//      candidate's accumulator in the slab (global atomics).
//   C  adjoint only: thread per survivor, chain to the instance
//      accumulators (shared memory); thread per instance, chain to pose,
//      scale and colour (global atomics).
#include "pbr_launch.h"
#include "pbr_soft.cuh"

namespace pbr {

constexpr int kLargeThreads = 256;
constexpr int kLBlkW = 8, kLBlkH = 4;

struct SoftLargeLayout {
  int icache, wcnt, vp, iacc, light, total;
};

__host__ __device__ inline SoftLargeLayout soft_large_layout(int icap, int inst_total, bool backward) {
  SoftLargeLayout L;
  int off = 0;
  L.icache = off; off += align16(icap * 64);
  L.wcnt = off; off += align16(2 * (kLargeThreads / 32) * 4);
  L.vp = off; off += 64;
  if (backward) {
    L.iacc = off; off += align16(inst_total * kIacc * 4);
    L.light = off; off += 16;
  } else {
    L.iacc = L.light = 0;
  }
  L.total = off;
  return L;
}

int soft_large_threads() { return kLargeThreads; }

int soft_large_smem_bytes(const SoftArgs& a) { return soft_large_layout(a.icap, a.iacc_cap, a.backward != 0).total; }

// float4 slots of one CTA's slab: 15 record arrays of cap, the block masks
// (nblocks * words uint32), the adjoint's accumulators (cap * 24 floats)
long long soft_large_slab_float4(int cap, int nblocks) {
  const long long words = (cap + 31) / 32;
  return 15LL * cap + (nblocks * words + 3) / 4 + (24LL * cap + 3) / 4;
}

// The next candidate's record lines, fetched into L1 while the warp evaluates
// the current one (lane i < kSoftRecs asks for record array i, which starts
// at slab + i * cap): the slab is
// larger than L2 in total, and each candidate's first loads otherwise wait on
// DRAM.  A prefetch changes no value.
__device__ __forceinline__ void prefetch_record(const float4* slab, int cap, int t, int lane) {
  if (lane < kSoftRecs) asm volatile("prefetch.global.L1 [%0];" ::"l"(slab + (long long)lane * cap + t));
}

template <bool BACKWARD>
__global__ void __launch_bounds__(kLargeThreads, 2) soft_large_kernel(const __grid_constant__ SceneParams P,
                                                                   const __grid_constant__ SoftArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NW = kLargeThreads / 32;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int W = P.W, H = P.H, HW = W * H;
  const int nbx = (W + kLBlkW - 1) / kLBlkW, nby = (H + kLBlkH - 1) / kLBlkH;
  const int nblocks = nbx * nby;
  const int cap = A.tri_cap;
  const int words = (cap + 31) >> 5;
  const SoftLargeLayout L = soft_large_layout(A.icap, A.iacc_cap, BACKWARD);
  float4* icache = reinterpret_cast<float4*>(smem + L.icache);
  int* wcnt = reinterpret_cast<int*>(smem + L.wcnt);
  float* s_vp = reinterpret_cast<float*>(smem + L.vp);
  float* iacc = reinterpret_cast<float*>(smem + L.iacc);
  float* s_light = reinterpret_cast<float*>(smem + L.light);

  float4* slab = A.scratch + (long long)blockIdx.x * A.scratch_stride;
  SoftCtx S;
#pragma unroll
  for (int i = 0; i < kSoftRecs; ++i) S.R[i] = slab + (long long)i * cap;
  uint32_t* bmask = reinterpret_cast<uint32_t*>(slab + 15LL * cap);  // [nblocks][words]
  float* tacc = reinterpret_cast<float*>(slab + 15LL * cap + ((long long)nblocks * words + 3) / 4);  // [cap][24]
  S.W = (float)W;
  S.H = (float)H;
  S.ry0 = 0.f;
  S.ry1 = (float)(H - 1);
  S.cut = kSoftCut * P.sigma;
  const float inv_sigma = 1.f / P.sigma;
  const float inv_zr = 1.f / (P.zfar - P.znear);
  const float inv_gamma = 1.f / P.gamma;

  for (int k = blockIdx.x; k < P.N; k += gridDim.x) {
    if (tid < 16) s_vp[tid] = P.vp[(long long)k * 16 + tid];
    for (long long i = tid; i < (long long)nblocks * words; i += kLargeThreads) bmask[i] = 0u;
    if (BACKWARD) {
      for (int i = tid; i < A.iacc_cap * kIacc; i += kLargeThreads) iacc[i] = 0.f;
      if (tid < 4) s_light[tid] = 0.f;
    }
    __syncthreads();
    const float vp0 = s_vp[0], vp1 = s_vp[1], vp2 = s_vp[2], vp3 = s_vp[3];
    const float vp4 = s_vp[4], vp5 = s_vp[5], vp6 = s_vp[6], vp7 = s_vp[7];
    const float vp8 = s_vp[8], vp9 = s_vp[9], vp10 = s_vp[10], vp11 = s_vp[11];
    const float vp12 = s_vp[12], vp13 = s_vp[13], vp14 = s_vp[14], vp15 = s_vp[15];

    // ---- A: setup in draw order ------------------------------------------------
    int T = 0, parity = 0;
    for (int n = 0; n < P.num_nodes; ++n) {
      const NodeDesc& nd = P.nodes[n];
      const MeshDesc& me = P.meshes[nd.mesh];
      int cnt = nd.counts ? nd.counts[k] : nd.ips;
      cnt = max(0, min(cnt, nd.ips));
      const int nt = me.nt;
      if (cnt == 0 || nt == 0) continue;
      const bool smooth = me.smooth != 0;
      for (int b0 = 0; b0 < cnt; b0 += A.icap) {
        const int nbc = min(A.icap, cnt - b0);
        __syncthreads();  // the previous batch is done with icache
        for (int i = tid; i < nbc; i += kLargeThreads) {
          const long long id = nd.shared ? (long long)(b0 + i) : (long long)k * nd.ips + b0 + i;
          float m[12];
          build_model(nd, id, m);
          icache[i * 4 + 0] = make_float4(m[0], m[1], m[2], m[3]);
          icache[i * 4 + 1] = make_float4(m[4], m[5], m[6], m[7]);
          icache[i * 4 + 2] = make_float4(m[8], m[9], m[10], m[11]);
          icache[i * 4 + 3] = *reinterpret_cast<const float4*>(nd.color + id * 4);
        }
        __syncthreads();
        const int total_t = nbc * nt;
        for (int t0 = 0; t0 < total_t; t0 += kLargeThreads) {
          int c = 0, li = 0, iv[3] = {0, 0, 0};
          float4 cv[3], nv[3];
          if (t0 + tid < total_t) {
            const int t = t0 + tid;
            li = (int)PBR_IX(t / nt, A.icap, 34);
            const int ti = t - (t / nt) * nt;
            iv[0] = me.idx[3 * ti];
            iv[1] = me.idx[3 * ti + 1];
            iv[2] = me.idx[3 * ti + 2];
            const float4 r0 = icache[li * 4 + 0], r1 = icache[li * 4 + 1], r2 = icache[li * 4 + 2];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
              const int vi = iv[q];
              const float ox = me.pos[3 * vi], oy = me.pos[3 * vi + 1], oz = me.pos[3 * vi + 2];
              const float wx = r0.x * ox + r0.y * oy + r0.z * oz + r0.w;
              const float wy = r1.x * ox + r1.y * oy + r1.z * oz + r1.w;
              const float wz = r2.x * ox + r2.y * oy + r2.z * oz + r2.w;
              cv[q].x = vp0 * wx + vp1 * wy + vp2 * wz + vp3;
              cv[q].y = vp4 * wx + vp5 * wy + vp6 * wz + vp7;
              cv[q].z = vp8 * wx + vp9 * wy + vp10 * wz + vp11;
              cv[q].w = vp12 * wx + vp13 * wy + vp14 * wz + vp15;
              // depth offset from the scene reference w_ref = VP[15], without the constant term
              nv[q] = make_float4(0.f, 0.f, 0.f, vp12 * wx + vp13 * wy + vp14 * wz);
            }
            c = soft_setup<false>(P, S, cv[0], nv[0], iv[0], cv[1], nv[1], iv[1], cv[2], nv[2], iv[2], 0,
                                  icache[li * 4 + 3], 0, smooth);
          }
          int incl = c;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
          }
          int* wc = wcnt + parity * NW;
          if (lane == 31) wc[warp] = incl;
          __syncthreads();
          int before = 0, total = 0;
#pragma unroll
          for (int w = 0; w < NW; ++w) {
            const int v = wc[w];
            before += w < warp ? v : 0;
            total += v;
          }
          parity ^= 1;
          if (c > 0) {
            const int slot = (int)PBR_IX(T + before + incl - c, cap, 30);
            const float4 r0 = icache[li * 4 + 0], r1 = icache[li * 4 + 1], r2 = icache[li * 4 + 2];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
              const int vi = iv[q];
              const float ax = me.nrm[3 * vi], ay = me.nrm[3 * vi + 1], az = me.nrm[3 * vi + 2];
              const float nx = r0.x * ax + r0.y * ay + r0.z * az;
              const float ny = r1.x * ax + r1.y * ay + r1.z * az;
              const float nz = r2.x * ax + r2.y * ay + r2.z * az;
              const float l2 = nx * nx + ny * ny + nz * nz;
              const float inv = l2 > 0.f ? rsqrtf(l2) : 0.f;
              nv[q] = make_float4(nx * inv, ny * inv, nz * inv, nv[q].w);
            }
            soft_setup<true>(P, S, cv[0], nv[0], iv[0], cv[1], nv[1], iv[1], cv[2], nv[2], iv[2], slot,
                             icache[li * 4 + 3], nd.rank_base + b0 + li, smooth);
            // this survivor's bit in the masks of the blocks holding a pixel centre within the cutoff of its
            // vertices' bbox (a superset of the pixels it can cover: the distance to the triangle is at least
            // the distance to that bbox), widened by 1e-3 px; clamped as floats first, since vertices of
            // near-plane triangles can be far outside the image
            const float4 s01 = S.R[13][slot], s2 = S.R[14][slot];
            const float mnx = fminf(fminf(s01.x, s01.z), s2.x), mxx = fmaxf(fmaxf(s01.x, s01.z), s2.x);
            const float mny = fminf(fminf(s01.y, s01.w), s2.y), mxy = fmaxf(fmaxf(s01.y, s01.w), s2.y);
            const int px0 = (int)fmaxf(0.f, ceilf(mnx - S.cut - 0.501f));
            const int px1 = (int)fminf((float)(W - 1), floorf(mxx + S.cut - 0.499f));
            const int py0 = (int)fmaxf(0.f, ceilf(mny - S.cut - 0.501f));
            const int py1 = (int)fminf((float)(H - 1), floorf(mxy + S.cut - 0.499f));
            const int bx0 = px0 / kLBlkW, bx1 = px1 / kLBlkW;
            const int by0 = py0 / kLBlkH, by1 = py1 / kLBlkH;
            const uint32_t bit = 1u << (slot & 31);
            if (px0 <= px1 && py0 <= py1)
              for (int by = by0; by <= by1; ++by)
                for (int bx = bx0; bx <= bx1; ++bx)
                  atomicOr(&bmask[PBR_IX((long long)(by * nbx + bx) * words + (slot >> 5), (long long)nblocks * words, 31)],
                           bit);
          }
          T += total;
        }
      }
    }
    if (BACKWARD)
      for (long long i = tid; i < (long long)T * 24; i += kLargeThreads) tacc[i] = 0.f;
    __syncthreads();

    // ---- B: blocks, one pixel per lane -------------------------------------------
    const int lx = lane & (kLBlkW - 1), ly = lane / kLBlkW;
    const int used = (T + 31) >> 5;  // mask words that can hold a bit
    for (int b = warp; b < nblocks; b += NW) {
      const int by = b / nbx, bx = b - by * nbx;
      const int x = bx * kLBlkW + lx, y = by * kLBlkH + ly;
      const bool active = x < W && y < H;
      const float px = (float)x + 0.5f, py = (float)y + 0.5f;
      const long long q = (long long)k * HW + (long long)y * W + x;
      const uint32_t* bm = bmask + (long long)b * words;
      if (!BACKWARD) {
        float m = -1e30f, Ssum = 0.f, acc0 = 0.f, acc1 = 0.f, acc2 = 0.f, Pv = 1.f, nz = 0.f;
        float cr0 = 0.f, cr1 = 0.f, cr2 = 0.f, ref = 0.f;
        for (int w0 = 0; w0 < used; w0 += 32) {
          const uint32_t mine = (w0 + lane < used) ? bm[w0 + lane] : 0u;
          uint32_t nzw = __ballot_sync(0xffffffffu, mine != 0u);
          while (nzw) {
            const int j = __ffs(nzw) - 1;
            nzw &= nzw - 1u;
            uint32_t mk = __shfl_sync(0xffffffffu, mine, j);
            while (mk) {
              const int t = (int)PBR_IX((w0 + j) * 32 + __ffs(mk) - 1, cap, 32);
              mk &= mk - 1u;
              if (mk) prefetch_record(slab, cap, (w0 + j) * 32 + __ffs(mk) - 1, lane);
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
        }
        if (active) {
          const float Av = 1.f - (nz > 0.f ? 0.f : Pv);
          const float dl0 = Ssum > 0.f ? acc0 / Ssum : 0.f;  // Cfg - C_r
          const float dl1 = Ssum > 0.f ? acc1 / Ssum : 0.f;
          const float dl2 = Ssum > 0.f ? acc2 / Ssum : 0.f;
          float* o = A.out + (long long)k * 3 * HW + (long long)y * W + x;
          o[0] = Av * (cr0 + dl0) + (1.f - Av) * P.bg[0];
          o[HW] = Av * (cr1 + dl1) + (1.f - Av) * P.bg[1];
          o[2 * HW] = Av * (cr2 + dl2) + (1.f - Av) * P.bg[2];
          if (A.stats) {
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
            const long long oi = ((long long)k * 3 + c) * HW + (long long)y * W + x;
            g[c] = A.gout[oi];
            cf[c] = Av > 0.f ? (A.out[oi] - (1.f - Av) * P.bg[c]) / Av : 0.f;
          }
          pb.m = stv.x;
          pb.Pnz = Pnz;
          pb.nz = nzv;
          pb.dLdA = g[0] * (cf[0] - P.bg[0]) + g[1] * (cf[1] - P.bg[1]) + g[2] * (cf[2] - P.bg[2]);
          pb.invS = stv.y > 0.f ? 1.f / stv.y : 0.f;
          pb.dl[0] = stv.w;
          pb.dl[1] = stw.x;
          pb.dl[2] = stw.y;
#pragma unroll
          for (int c = 0; c < 3; ++c) pb.dc[c] = Av * g[c];
        }
        for (int w0 = 0; w0 < used; w0 += 32) {
          const uint32_t mine = (w0 + lane < used) ? bm[w0 + lane] : 0u;
          uint32_t nzw = __ballot_sync(0xffffffffu, mine != 0u);
          while (nzw) {
            const int j = __ffs(nzw) - 1;
            nzw &= nzw - 1u;
            uint32_t mk = __shfl_sync(0xffffffffu, mine, j);
            while (mk) {
              const int t = (int)PBR_IX((w0 + j) * 32 + __ffs(mk) - 1, cap, 32);
              mk &= mk - 1u;
              if (mk) prefetch_record(slab, cap, (w0 + j) * 32 + __ffs(mk) - 1, lane);
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
                if ((lane & 3) != 3 && v != 0.f) atomicAdd(&tacc[PBR_IX((long long)t * 24 + idx, (long long)cap * 24, 33)], v);
              }
            }
          }
        }
      }
    }

    if (BACKWARD) {
      __syncthreads();
      // ---- C: survivor -> instance -> pose, scale, colour ------------------------
      for (int t = tid; t < T; t += kLargeThreads)
        soft_tri_chain(P, S, t, tacc + (long long)t * 24, s_vp, iacc, A.iacc_cap, s_light);
      __syncthreads();
      for (int s = tid; s < A.iacc_cap; s += kLargeThreads) soft_instance_grads(P, k, s, iacc + s * kIacc);
      if (tid < 3 && A.glight) atomicAdd(&A.glight[tid], s_light[tid]);
    }
    __syncthreads();  // the slab and shared memory are reused by the next scene
  }
}

// ---------------------------------------------------------------------------

static const void* pick_soft_large(bool backward) {
  return backward ? (const void*)&soft_large_kernel<true> : (const void*)&soft_large_kernel<false>;
}

cudaError_t soft_large_set_smem_limit(bool backward, int bytes) {
  return cudaFuncSetAttribute(pick_soft_large(backward), cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

cudaError_t soft_large_occupancy(bool backward, int smem_bytes, int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, pick_soft_large(backward), kLargeThreads,
                                                       smem_bytes);
}

cudaError_t soft_large_launch(bool backward, const SceneParams& P, const SoftArgs& A, int grid, int smem_bytes,
                              cudaStream_t stream) {
  void* args[] = {const_cast<SceneParams*>(&P), const_cast<SoftArgs*>(&A)};
  return cudaLaunchKernel(pick_soft_large(backward), dim3(grid), dim3(kLargeThreads), args, (size_t)smem_bytes,
                          stream);
}

}  // namespace pbr
