// pbr_envs.cu -- fused on-device environment steps.
//
// CartPole-v0 (envs/cartpole/env.py:111-218): Euler-integrated cart-pole
// dynamics, termination, survival reward and auto-reset for every scene in
// one launch, replacing the ~40 elementwise kernels the same step costs as
// separate tensor operations.  The arithmetic follows those tensor operations
// one rounding at a time (explicit round-to-nearest multiplies and adds, no
// contraction into fused multiply-adds; a division by a Python scalar is a
// multiply by its float reciprocal, as the tensor library computes it), so the
// fused step reproduces the unfused one.
#include <cstdint>

#include <cuda_runtime.h>

#include "pbr_capi.h"

namespace {

struct CartPoleConsts {
  float force_mag, polemass_length, inv_total_mass, gravity, masspole, length, four_thirds, tau;
  float x_threshold, theta_threshold;
  long long last_step;  // max_steps - 1
  int auto_reset;
};

__global__ void cartpole_step_kernel(const float4* __restrict__ obs, const int64_t* __restrict__ action,
                                     const int64_t* __restrict__ step_count, const float* __restrict__ r0,
                                     const float* __restrict__ r1, const float* __restrict__ r2,
                                     const float* __restrict__ r3, float4* __restrict__ next_raw,
                                     float4* __restrict__ next_obs, float* __restrict__ reward,
                                     bool* __restrict__ done, int64_t* __restrict__ next_step_count,
                                     const CartPoleConsts c, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float4 s = obs[i];
    const float x = s.x, x_dot = s.y, theta = s.z, theta_dot = s.w;
    const float force = action[i] == 1 ? c.force_mag : -c.force_mag;
    const float costheta = cosf(theta), sintheta = sinf(theta);
    // temp = (force + polemass_length * theta_dot^2 * sintheta) / total_mass
    const float td2 = __fmul_rn(theta_dot, theta_dot);
    const float temp = __fmul_rn(__fadd_rn(force, __fmul_rn(__fmul_rn(c.polemass_length, td2), sintheta)),
                                 c.inv_total_mass);
    // thetaacc = (gravity * sintheta - costheta * temp)
    //            / (length * (4/3 - masspole * costheta^2 / total_mass))
    const float num = __fsub_rn(__fmul_rn(c.gravity, sintheta), __fmul_rn(costheta, temp));
    const float c2 = __fmul_rn(costheta, costheta);
    const float den = __fmul_rn(c.length, __fsub_rn(c.four_thirds, __fmul_rn(__fmul_rn(c.masspole, c2),
                                                                            c.inv_total_mass)));
    const float thetaacc = __fdiv_rn(num, den);
    // xacc = temp - polemass_length * thetaacc * costheta / total_mass
    const float xacc = __fsub_rn(temp, __fmul_rn(__fmul_rn(__fmul_rn(c.polemass_length, thetaacc), costheta),
                                                 c.inv_total_mass));
    float4 raw;
    raw.x = __fadd_rn(x, __fmul_rn(c.tau, x_dot));
    raw.y = __fadd_rn(x_dot, __fmul_rn(c.tau, xacc));
    raw.z = __fadd_rn(theta, __fmul_rn(c.tau, theta_dot));
    raw.w = __fadd_rn(theta_dot, __fmul_rn(c.tau, thetaacc));
    next_raw[i] = raw;
    const long long sc = step_count ? (long long)step_count[i] : 0;
    const bool d = (fabsf(raw.x) > c.x_threshold) || (fabsf(raw.z) > c.theta_threshold) || (sc >= c.last_step);
    done[i] = d;
    reward[i] = 1.f;
    if (c.auto_reset) {
      next_obs[i] = d ? make_float4(r0[i], r1[i], r2[i], r3[i]) : raw;
      next_step_count[i] = d ? 0 : sc + 1;
    } else {
      next_obs[i] = raw;
      next_step_count[i] = sc + 1;
    }
  }
}

}  // namespace

extern "C" int pbr_cartpole_step(const float* d_obs, const int64_t* d_action, const int64_t* d_step_count,
                                 const float* d_reset_x, const float* d_reset_x_dot, const float* d_reset_theta,
                                 const float* d_reset_theta_dot, float* d_next_raw, float* d_next_obs,
                                 float* d_reward, uint8_t* d_done, int64_t* d_next_step_count, long long n,
                                 const double* consts, int auto_reset, void* stream) {
  if (n < 0 || !consts) return PBR_ERR_INVALID;
  if (n == 0) return PBR_OK;
  if (!d_obs || !d_action || !d_next_raw || !d_next_obs || !d_reward || !d_done || !d_next_step_count)
    return PBR_ERR_INVALID;
  if (auto_reset && (!d_reset_x || !d_reset_x_dot || !d_reset_theta || !d_reset_theta_dot)) return PBR_ERR_INVALID;
  if ((((uintptr_t)d_obs) | ((uintptr_t)d_next_raw) | ((uintptr_t)d_next_obs)) & 15u) return PBR_ERR_INVALID;
  // consts: gravity, masscart, masspole, length, force_mag, tau, x_threshold, theta_threshold, max_steps
  const double gravity = consts[0], masscart = consts[1], masspole = consts[2], length = consts[3];
  const double total_mass = masscart + masspole, polemass_length = masspole * length;
  CartPoleConsts c;
  c.force_mag = (float)consts[4];
  c.polemass_length = (float)polemass_length;
  c.inv_total_mass = 1.0f / (float)total_mass;
  c.gravity = (float)gravity;
  c.masspole = (float)masspole;
  c.length = (float)length;
  c.four_thirds = (float)(4.0 / 3.0);
  c.tau = (float)consts[5];
  c.x_threshold = (float)consts[6];
  c.theta_threshold = (float)consts[7];
  c.last_step = (long long)consts[8] - 1;
  c.auto_reset = auto_reset ? 1 : 0;
  const int threads = 256;
  const long long blocks = (n + threads - 1) / threads;
  const int grid = (int)(blocks < 152 * 16 ? blocks : 152 * 16);
  cartpole_step_kernel<<<grid, threads, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float4*>(d_obs), d_action, d_step_count, d_reset_x, d_reset_x_dot, d_reset_theta,
      d_reset_theta_dot, reinterpret_cast<float4*>(d_next_raw), reinterpret_cast<float4*>(d_next_obs), d_reward,
      reinterpret_cast<bool*>(d_done), d_next_step_count, c, n);
  return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}
