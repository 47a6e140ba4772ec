"""CartPole environment (``envs/cartpole/env.py``): Euler-integrated
dynamics, termination, survival reward and auto-reset, all on the env's
device; pixels come from ``render_pixels`` each step.

On a CUDA device the step's arithmetic is one fused launch
(``pbr_cartpole_step``) instead of about forty elementwise tensor operations;
it follows those operations rounding by rounding, and the initial states of
the auto-reset are drawn by the same tensor RNG calls in the same order.
``fused_step=False`` keeps the tensor-operation step."""
import ctypes
import math

import torch

from ...env import PBREnv, TensorDict
from .config import CartPoleConfig
from .renderer import CartPoleRenderer


class CartPoleEnv(PBREnv):
    def __init__(self, renderer: CartPoleRenderer, cfg: CartPoleConfig | dict | None = None, **cfg_overrides):
        if cfg is None:
            cfg = renderer.cfg
        super().__init__(renderer=renderer, cfg=cfg, device=torch.device(cfg.device),
                         batch_size=torch.Size([cfg.num_scenes]))
        self.gravity = float(cfg.gravity)
        self.masscart = float(cfg.masscart)
        self.masspole = float(cfg.masspole)
        self.total_mass = self.masscart + self.masspole
        self.length = float(cfg.length)
        self.polemass_length = self.masspole * self.length
        self.force_mag = float(cfg.force_mag)
        self.tau = float(cfg.tau)
        self.theta_threshold = float(cfg.theta_threshold_deg * 2 * math.pi / 360.0)
        self.x_threshold = float(cfg.x_threshold)
        self.max_steps = int(cfg.max_steps)
        self.auto_reset = bool(cfg.auto_reset)
        self.fused_step = bool(getattr(cfg, "fused_step", True))
        self._consts = (ctypes.c_double * 9)(self.gravity, self.masscart, self.masspole, self.length, self.force_mag,
                                             self.tau, self.x_threshold, self.theta_threshold, self.max_steps)
        self.seed = int(cfg.seed)
        self.render = bool(cfg.render)
        th0_lo, th0_hi = float(cfg.init_theta_range_deg[0]), float(cfg.init_theta_range_deg[1])
        thd_lo, thd_hi = float(cfg.init_theta_dot_range_deg[0]), float(cfg.init_theta_dot_range_deg[1])
        self._init_theta_range_rad = (math.radians(min(th0_lo, th0_hi)), math.radians(max(th0_lo, th0_hi)))
        self._init_theta_dot_range_rad = (math.radians(min(thd_lo, thd_hi)), math.radians(max(thd_lo, thd_hi)))
        self.set_default_specs(direct_obs_dim=4, actions=2, with_pixels=self.render, pixels_only=False,
                               discrete_actions=True)
        if self.seed is not None:
            self.set_seed(self.seed)

    def _sample_initial_columns(self, batch_shape: torch.Size) -> list[torch.Tensor]:
        def u(lo_hi):
            return torch.empty(*batch_shape, 1, dtype=torch.float32, device=self.device).uniform_(*lo_hi)
        return [u(self.cfg.init_x_range), u(self.cfg.init_x_dot_range), u(self._init_theta_range_rad),
                u(self._init_theta_dot_range_rad)]

    def _sample_initial_state(self, batch_shape: torch.Size) -> torch.Tensor:
        return torch.cat(self._sample_initial_columns(batch_shape), dim=-1)

    def _dynamics(self, obs: torch.Tensor, action: torch.Tensor) -> torch.Tensor:
        """``envs/cartpole/env.py:111-129``."""
        x, x_dot, theta, theta_dot = obs.unbind(-1)
        force = torch.where(action == 1, self.force_mag, -self.force_mag).to(torch.float32)
        costheta = torch.cos(theta)
        sintheta = torch.sin(theta)
        temp = (force + self.polemass_length * theta_dot.pow(2) * sintheta) / self.total_mass
        thetaacc = (self.gravity * sintheta - costheta * temp) / (
            self.length * (4.0 / 3.0 - self.masspole * costheta.pow(2) / self.total_mass))
        xacc = temp - self.polemass_length * thetaacc * costheta / self.total_mass
        x = x + self.tau * x_dot
        x_dot = x_dot + self.tau * xacc
        theta = theta + self.tau * theta_dot
        theta_dot = theta_dot + self.tau * thetaacc
        return torch.stack([x, x_dot, theta, theta_dot], dim=-1)

    def _termination(self, obs: torch.Tensor, step_count: torch.Tensor) -> torch.Tensor:
        x, x_dot, theta, theta_dot = obs.unbind(-1)
        return ((x.abs() > self.x_threshold) | (theta.abs() > self.theta_threshold)
                | (step_count >= (self.max_steps - 1))).unsqueeze(-1)

    def _reward(self, obs: torch.Tensor, done: torch.Tensor) -> torch.Tensor:
        return torch.ones_like(done, dtype=torch.float32, device=self.device)

    def _set_seed(self, seed: int) -> None:
        torch.manual_seed(int(seed))

    def _reset(self, tensordict=None):
        bs = self.batch_size if self.batch_size != torch.Size([]) else torch.Size([1])
        state = self._sample_initial_state(bs)
        fields = {"observation": state,
                  "step_count": torch.zeros(*bs, dtype=torch.long, device=self.device),
                  "done": torch.zeros(*bs, 1, dtype=torch.bool, device=self.device)}
        if self.render:
            fields["pixels"] = self.render_pixels(state)
        return TensorDict(fields, batch_size=self.batch_size)

    @torch.no_grad()
    def _step(self, tensordict):
        obs = tensordict.get("observation", None)
        if obs is None:
            td0 = self._reset()
            obs, step_count = td0["observation"], td0["step_count"]
        else:
            step_count = tensordict.get("step_count", None)
            if step_count is None:
                step_count = torch.zeros_like(obs[..., 0], dtype=torch.long, device=self.device)
        action = tensordict["action"].to(self.device)
        if self.fused_step and obs.is_cuda:
            return self._fused_step(obs, action, step_count)
        next_obs_raw = self._dynamics(obs, action)
        done = self._termination(next_obs_raw, step_count)
        reward = self._reward(next_obs_raw, done)
        pixels = self.render_pixels(next_obs_raw) if self.render else None
        if self.auto_reset:
            reset_state = self._sample_initial_state(next_obs_raw.shape[:-1])
            next_obs = torch.where(done, reset_state, next_obs_raw)
            next_step_count = torch.where(done.squeeze(-1), torch.zeros_like(step_count), step_count + 1)
        else:
            next_obs, next_step_count = next_obs_raw, step_count + 1
        out = {"observation": next_obs, "reward": reward, "done": done, "step_count": next_step_count}
        if pixels is not None:
            out["pixels"] = pixels
        return TensorDict(out, batch_size=self.batch_size)

    def _fused_step(self, obs: torch.Tensor, action: torch.Tensor, step_count: torch.Tensor):
        """The step above as one ``pbr_cartpole_step`` launch (graph-capturable:
        no host synchronisation, outputs from the caching allocator)."""
        from ... import _capi
        lib = _capi.load()
        obs = obs.to(torch.float32).contiguous()
        bs = obs.shape[:-1]
        n = obs.numel() // 4
        act = action.reshape(bs).to(torch.int64).contiguous()
        sc = step_count.reshape(bs).to(torch.int64).contiguous()
        resets = [None] * 4
        if self.auto_reset:
            resets = self._sample_initial_columns(bs)  # the tensor path's RNG calls, in its order
        raw = torch.empty_like(obs)
        nxt = torch.empty_like(obs)
        reward = torch.empty(*bs, 1, dtype=torch.float32, device=obs.device)
        done = torch.empty(*bs, 1, dtype=torch.bool, device=obs.device)
        nsc = torch.empty(*bs, dtype=torch.int64, device=obs.device)
        stream = torch.cuda.current_stream(obs.device).cuda_stream
        rc = lib.pbr_cartpole_step(_capi.ptr(obs), _capi.ptr(act), _capi.ptr(sc), *[_capi.ptr(t) for t in resets],
                                   _capi.ptr(raw), _capi.ptr(nxt), _capi.ptr(reward), _capi.ptr(done), _capi.ptr(nsc),
                                   n, self._consts, int(self.auto_reset), ctypes.c_void_p(stream))
        if rc != 0:
            raise _capi.PBRError("pbr_cartpole_step", rc, "invalid arguments or launch failure")
        out = {"observation": nxt, "reward": reward, "done": done, "step_count": nsc}
        if self.render:
            out["pixels"] = self.render_pixels(raw)
        return TensorDict(out, batch_size=self.batch_size)
