// pbr_camera.cu -- per-scene camera matrices on the device in one launch: the
// view of renderer/camera.py:201-240 (rows s, u, -f with s = normalize(f x up),
// u = s x f, translation (-s.e, -u.e, f.e)) and VP = P V of camera.py:252-262,
// in place of the dozen elementwise, reduction and batched-GEMM launches the
// same float32 math takes as tensor operations.
#include <cuda_runtime.h>

#include "pbr_capi.h"

namespace pbr {

struct CamArgs {
  const float* eye;  // [K,3] or null: keep the translation
  const float* fwd;  // [K,3] or null: keep the basis (unless up is given)
  const float* up;   // [K,3] or null: the current up row
  float* V;          // [K,16] row-major, updated in place
  float* VP;         // [K,16] or null
  float P[16];       // projection, row-major
  int K;
};

__device__ __forceinline__ void normalize3(float v[3]) {
  const float n = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  const float d = fmaxf(n, 1e-8f);
  v[0] = v[0] / d;
  v[1] = v[1] / d;
  v[2] = v[2] / d;
}

__device__ __forceinline__ void cross3(const float a[3], const float b[3], float c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

__global__ void camera_update_kernel(const __grid_constant__ CamArgs a) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.K) return;
  float* v = a.V + (long long)k * 16;
  float s[3], u[3], f[3];
  if (a.fwd || a.up) {
    float up_in[3];
    if (a.fwd) {
      f[0] = a.fwd[3 * k]; f[1] = a.fwd[3 * k + 1]; f[2] = a.fwd[3 * k + 2];
      normalize3(f);
    } else {
      f[0] = -v[8]; f[1] = -v[9]; f[2] = -v[10];
    }
    if (a.up) {
      up_in[0] = a.up[3 * k]; up_in[1] = a.up[3 * k + 1]; up_in[2] = a.up[3 * k + 2];
      normalize3(up_in);
    } else {
      up_in[0] = v[4]; up_in[1] = v[5]; up_in[2] = v[6];
    }
    cross3(f, up_in, s);
    normalize3(s);
    cross3(s, f, u);
    v[0] = s[0]; v[1] = s[1]; v[2] = s[2];
    v[4] = u[0]; v[5] = u[1]; v[6] = u[2];
    v[8] = -f[0]; v[9] = -f[1]; v[10] = -f[2];
  } else {
    s[0] = v[0]; s[1] = v[1]; s[2] = v[2];
    u[0] = v[4]; u[1] = v[5]; u[2] = v[6];
    f[0] = -v[8]; f[1] = -v[9]; f[2] = -v[10];
  }
  if (a.eye) {
    const float e[3] = {a.eye[3 * k], a.eye[3 * k + 1], a.eye[3 * k + 2]};
    v[3] = -(s[0] * e[0] + s[1] * e[1] + s[2] * e[2]);
    v[7] = -(u[0] * e[0] + u[1] * e[1] + u[2] * e[2]);
    v[11] = f[0] * e[0] + f[1] * e[1] + f[2] * e[2];
  }
  if (a.VP) {
    float m[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) m[i] = v[i];
    float* o = a.VP + (long long)k * 16;
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c)
        o[r * 4 + c] = a.P[r * 4 + 0] * m[c] + a.P[r * 4 + 1] * m[4 + c] + a.P[r * 4 + 2] * m[8 + c] +
                       a.P[r * 4 + 3] * m[12 + c];
  }
}

}  // namespace pbr

extern "C" int pbr_camera_update(const float* d_eye, const float* d_forward, const float* d_up, float* d_view,
                                 const float projection[16], float* d_vp, int num_scenes, void* stream) {
  if (num_scenes < 0 || !d_view || (d_vp && !projection)) return PBR_ERR_INVALID;
  if (num_scenes == 0) return PBR_OK;
  pbr::CamArgs a;
  a.eye = d_eye;
  a.fwd = d_forward;
  a.up = d_up;
  a.V = d_view;
  a.VP = d_vp;
  for (int i = 0; i < 16; ++i) a.P[i] = projection ? projection[i] : 0.f;
  a.K = num_scenes;
  const int threads = 128;
  pbr::camera_update_kernel<<<(num_scenes + threads - 1) / threads, threads, 0, (cudaStream_t)stream>>>(a);
  return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}
