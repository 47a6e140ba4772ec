"""Steering environment (``envs/steering/env.py:18-471``): a vehicle drives
forward along a lane at a speed that grows with every obstacle passed and
drops on a collision; the continuous action steers it sideways.  All state
is on the env's device.

Observation ``[B, 6]``: player x, player y, forward speed, grace active
(1 while recovering from a collision), next obstacle x, next obstacle y.
Reward: ``collision_penalty`` per collision outside the grace period, else
0.  Done at the track end (``terminate_on_track_end``), on a collision
(``terminate_on_collision``) or after ``max_steps``.  As in the reference,
auto-reset only restarts the step counter of finished scenes; their
observation is kept (``env.py:441-450`` re-reads the current observation
instead of resetting)."""
from __future__ import annotations

import random

import torch

from ...env import PBREnv, TensorDict
from .config import SteeringConfig
from .renderer import SteeringRenderer


class SteeringEnv(PBREnv):
    def __init__(self, renderer: SteeringRenderer, cfg: SteeringConfig | dict | None = None, **cfg_overrides):
        if cfg is None:
            cfg = renderer.cfg
        super().__init__(renderer=renderer, cfg=cfg, device=torch.device(cfg.device),
                         batch_size=torch.Size([cfg.num_scenes]))
        c = cfg
        self.speed_initial = float(c.speed_initial)
        self.minimal_speed = float(c.minimal_speed)
        self.speed_increment = float(c.speed_increment)
        self.speed_decrement = float(c.speed_decrement)
        self.grace_period = float(c.grace_period)
        self.steering_speed = float(c.steering_speed)
        self.tau = float(c.tau)
        self.lane_width = float(c.lane_width)
        self.player_half_width = float(c.player_dimensions[0]) * 0.5
        self.obstacle_half_width = float(c.obstacle_dimensions[0]) * 0.5
        self.collision_threshold = self.player_half_width + self.obstacle_half_width
        self.rail_half_width = float(c.rail_dimensions[0]) * 0.5
        limit = self.lane_width * 0.5 - self.player_half_width - self.rail_half_width
        self.x_min, self.x_max = -limit, limit
        self.obstacle_seed = c.obstacle_seed
        self.prob_gold = float(c.prob_gold)
        self.prob_cone = float(c.prob_cone)
        self.distance_to_first_obstacle = float(c.distance_to_first_obstacle)
        self.number_of_obstacles = int(c.number_of_obstacles)
        self.obstacle_y_spacing = float(c.obstacle_y_spacing)
        self.obstacle_x_positions = list(c.obstacle_x_position)
        self.max_steps = int(c.max_steps)
        self.auto_reset = bool(c.auto_reset)
        self.wheel_sensitivity = float(c.wheel_sensitivity)
        self.collision_penalty = float(c.collision_penalty)
        self.terminate_on_collision = bool(c.terminate_on_collision)
        self.terminate_on_track_end = bool(c.terminate_on_track_end)
        self.action_low = float(c.action_low)
        self.action_high = float(c.action_high)
        self.seed_val = int(c.seed) if c.seed is not None else 0
        self.render_enabled = bool(c.render)

        self._obstacles = None
        self._player_x = self._player_y = self._forward_speed = None
        self._grace_remaining = self._next_obstacle_idx = None
        self._prev_player_x = self._prev_player_y = None

        discrete = c.action_type == "discrete"
        self.set_default_specs(direct_obs_dim=int(c.direct_obs_dim), actions=int(c.action_n),
                               with_pixels=self.render_enabled, pixels_only=False, discrete_actions=discrete,
                               action_low=None if discrete else self.action_low,
                               action_high=None if discrete else self.action_high)
        self.set_seed(self.seed_val)

    # ------------------------------------------------------------------ world
    def _generate_obstacles(self) -> torch.Tensor:
        """``[B, n, 4]``: x from the allowed lane positions, y evenly spaced
        from the first-obstacle distance, gold and cone flags (``env.py:165-196``)."""
        B, n = int(self.cfg.num_scenes), self.number_of_obstacles
        dev = self.device
        ob = torch.zeros(B, n, 4, dtype=torch.float32, device=dev)
        xs = torch.tensor(self.obstacle_x_positions, dtype=torch.float32, device=dev)
        ob[:, :, 0] = xs[torch.randint(0, len(xs), (B, n), device=dev)]
        ob[:, :, 1] = torch.arange(n, dtype=torch.float32, device=dev) * self.obstacle_y_spacing \
            + self.distance_to_first_obstacle
        ob[:, :, 2] = (torch.rand(B, n, device=dev) < self.prob_gold).float()
        ob[:, :, 3] = (torch.rand(B, n, device=dev) < self.prob_cone).float()
        return ob

    def _get_observation(self) -> torch.Tensor:
        B = int(self.cfg.num_scenes)
        dev = self.device
        nx = torch.zeros(B, device=dev)
        ny = torch.zeros(B, device=dev)
        if self._obstacles is not None:
            m = self._obstacles.shape[1]
            valid = self._next_obstacle_idx < m
            idx = torch.clamp(self._next_obstacle_idx, max=m - 1)
            nxt = self._obstacles[torch.arange(B, device=dev), idx]
            nx = torch.where(valid, nxt[:, 0], torch.zeros_like(nx))
            ny = torch.where(valid, nxt[:, 1], self._player_y + 1000.0)
        grace = (self._grace_remaining > 0).float()
        return torch.stack([self._player_x, self._player_y, self._forward_speed, grace, nx, ny], dim=-1)

    def _check_collisions(self) -> tuple[torch.Tensor, torch.Tensor]:
        """Obstacles the player passed since the last step: passages, and
        hits where the player's x interpolated at the obstacle's y is within
        the collision distance (``env.py:230-285``)."""
        B = int(self.cfg.num_scenes)
        dev = self.device
        collisions = torch.zeros(B, dtype=torch.int32, device=dev)
        passages = torch.zeros(B, dtype=torch.int32, device=dev)
        if self._obstacles is None or self._obstacles.numel() == 0:
            return collisions, passages
        m = self._obstacles.shape[1]
        rows = torch.arange(B, device=dev)
        for _ in range(m):  # bounded: one obstacle per scene per pass
            idx = torch.clamp(self._next_obstacle_idx, max=m - 1)
            ob = self._obstacles[rows, idx]
            passed = (self._next_obstacle_idx < m) & (ob[:, 1] <= self._player_y)
            if not bool(passed.any()):
                break
            denom = self._player_y - self._prev_player_y
            denom = torch.where(denom.abs() < 1e-6, torch.ones_like(denom), denom)
            t = (ob[:, 1] - self._prev_player_y) / denom
            x_at = self._prev_player_x + (self._player_x - self._prev_player_x) * t
            hit = passed & ((x_at - ob[:, 0]).abs() <= self.collision_threshold)
            self._next_obstacle_idx = self._next_obstacle_idx + passed.long()
            passages = passages + passed.int()
            collisions = collisions + hit.int()
        return collisions, passages

    def _dynamics(self, action: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
        self._prev_player_x = self._player_x.clone()
        self._prev_player_y = self._player_y.clone()
        self._grace_remaining = torch.clamp(self._grace_remaining - self.tau, min=0.0)
        self._player_y = self._player_y + self._forward_speed * self.tau
        steer = action.float() if action.dim() == 1 else action.squeeze(-1).float()
        dx = steer * self._forward_speed / self.wheel_sensitivity * self.tau
        self._player_x = torch.clamp(self._player_x + dx, self.x_min, self.x_max)
        collisions, passages = self._check_collisions()
        crashes = (collisions > 0) & (self._grace_remaining <= 0)
        self._grace_remaining = torch.where(crashes, torch.full_like(self._grace_remaining, self.grace_period),
                                            self._grace_remaining)
        speed = self._forward_speed + passages.float() * self.speed_increment - crashes.float() * self.speed_decrement
        self._forward_speed = torch.clamp(speed, min=self.minimal_speed)
        reached_end = self._next_obstacle_idx >= self.number_of_obstacles
        return crashes, reached_end

    def _termination(self, crashes, reached_end, step_count) -> torch.Tensor:
        done = torch.zeros_like(step_count, dtype=torch.bool)
        if self.terminate_on_collision:
            done = done | crashes
        if self.terminate_on_track_end:
            done = done | reached_end
        return (done | (step_count >= self.max_steps - 1)).unsqueeze(-1)

    def _reward(self, crashes, done) -> torch.Tensor:
        return (crashes.float() * self.collision_penalty).unsqueeze(-1)

    def _set_seed(self, seed: int) -> None:
        torch.manual_seed(int(seed))
        random.seed(int(seed))

    # -------------------------------------------------------------------- API
    def _reset(self, tensordict=None):
        bs = self.batch_size if self.batch_size != torch.Size([]) else torch.Size([1])
        B = int(bs[0]) if len(bs) else 1
        dev = self.device
        self._obstacles = self._generate_obstacles()
        self._renderer.build_obstacles(self._obstacles)
        self._player_x = torch.empty(B, device=dev).uniform_(self.x_min, self.x_max)
        self._player_y = torch.zeros(B, device=dev)
        self._prev_player_x = torch.zeros(B, device=dev)
        self._prev_player_y = torch.zeros(B, device=dev)
        self._forward_speed = torch.full((B,), self.speed_initial, device=dev)
        self._grace_remaining = torch.zeros(B, device=dev)
        self._next_obstacle_idx = torch.zeros(B, dtype=torch.long, device=dev)
        obs = self._get_observation()
        fields = {"observation": obs, "step_count": torch.zeros(*bs, dtype=torch.long, device=dev),
                  "done": torch.zeros(*bs, 1, dtype=torch.bool, device=dev)}
        if self.render_enabled:
            fields["pixels"] = self.render_pixels(obs)
        return TensorDict(fields, batch_size=self.batch_size)

    @torch.no_grad()
    def _step(self, tensordict):
        obs = tensordict.get("observation", None)
        if obs is None or self._player_x is None:
            td0 = self._reset()
            step_count = td0["step_count"]
        else:
            step_count = tensordict.get("step_count", None)
            if step_count is None:
                step_count = torch.zeros_like(obs[..., 0], dtype=torch.long, device=self.device)
        action = tensordict["action"].to(self.device)
        crashes, reached_end = self._dynamics(action)
        next_obs = self._get_observation()
        done = self._termination(crashes, reached_end, step_count)
        reward = self._reward(crashes, done)
        pixels = self.render_pixels(next_obs) if self.render_enabled else None
        if self.auto_reset:
            next_step_count = torch.where(done.squeeze(-1), torch.zeros_like(step_count), step_count + 1)
        else:
            next_step_count = step_count + 1
        out = {"observation": next_obs, "reward": reward, "done": done, "step_count": next_step_count}
        if pixels is not None:
            out["pixels"] = pixels
        return TensorDict(out, batch_size=self.batch_size)
