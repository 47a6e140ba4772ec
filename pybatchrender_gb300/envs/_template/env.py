"""Template environment (``envs/_template/env.py``): reset, dynamics,
termination, reward and auto-reset as batched tensor operations on the env's
device; pixels from ``render_pixels``."""
import torch

from ...env import PBREnv, TensorDict
from .config import MyEnvConfig
from .renderer import MyEnvRenderer


class MyEnv(PBREnv):
    def __init__(self, renderer: MyEnvRenderer, cfg: MyEnvConfig | dict | None = None, **cfg_overrides):
        if cfg is None:
            cfg = renderer.cfg
        super().__init__(renderer=renderer, cfg=cfg, device=torch.device(cfg.device),
                         batch_size=torch.Size([cfg.num_scenes]))
        self.max_steps = int(cfg.max_steps)
        self.auto_reset = bool(cfg.auto_reset)
        self.render = bool(cfg.render)
        self.set_default_specs(direct_obs_dim=int(cfg.direct_obs_dim), actions=int(cfg.action_n),
                               with_pixels=self.render, pixels_only=False, discrete_actions=True)
        torch.manual_seed(int(cfg.seed))

    def _sample_initial_state(self, batch_shape: torch.Size) -> torch.Tensor:
        x = torch.empty(*batch_shape, 1, device=self.device).uniform_(*self.cfg.init_x_range)
        return torch.cat([x, torch.zeros_like(x)], dim=-1)

    def _dynamics(self, obs: torch.Tensor, action: torch.Tensor) -> torch.Tensor:
        x, v = obs.unbind(-1)
        v = v + torch.where(action == 1, self.cfg.push, -self.cfg.push)
        return torch.stack([x + self.cfg.dt * v, v], dim=-1)

    def _termination(self, obs: torch.Tensor, step_count: torch.Tensor) -> torch.Tensor:
        return ((obs[..., 0].abs() > self.cfg.limit) | (step_count >= self.max_steps - 1)).unsqueeze(-1)

    def _reward(self, obs: torch.Tensor, done: torch.Tensor) -> torch.Tensor:
        return 1.0 - (obs[..., :1].abs() / self.cfg.limit)

    def _reset(self, tensordict=None):
        bs = self.batch_size
        state = self._sample_initial_state(bs)
        fields = {"observation": state, "step_count": torch.zeros(*bs, dtype=torch.long, device=self.device),
                  "done": torch.zeros(*bs, 1, dtype=torch.bool, device=self.device)}
        if self.render:
            fields["pixels"] = self.render_pixels(state)
        return TensorDict(fields, batch_size=bs)

    @torch.no_grad()
    def _step(self, tensordict):
        obs = tensordict["observation"]
        step_count = tensordict.get("step_count", None)
        if step_count is None:
            step_count = torch.zeros(obs.shape[:-1], dtype=torch.long, device=self.device)
        nxt = self._dynamics(obs, tensordict["action"].to(self.device))
        done = self._termination(nxt, step_count)
        reward = self._reward(nxt, done)
        out = {"reward": reward, "done": done}
        if self.render:
            out["pixels"] = self.render_pixels(nxt)
        if self.auto_reset:
            nxt = torch.where(done, self._sample_initial_state(nxt.shape[:-1]), nxt)
            step_count = torch.where(done.squeeze(-1), torch.zeros_like(step_count), step_count + 1)
        else:
            step_count = step_count + 1
        out.update({"observation": nxt, "step_count": step_count})
        return TensorDict(out, batch_size=self.batch_size)
