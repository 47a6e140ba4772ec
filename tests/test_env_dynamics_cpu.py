"""Environment dynamics against trajectories recorded from the reference's
own CartPole and Steering environments (``tests/golden/make_golden.py``):
the same seeded states, obstacles and actions stepped through this package's
``_step`` give bit-identical observations, rewards, done flags and step
counters (CPU, float32, no rendering, no auto-reset)."""
import os

import numpy as np
import pytest
import torch

from pybatchrender_gb300.envs.cartpole import CartPoleConfig, CartPoleEnv, CartPoleRenderer
from pybatchrender_gb300.envs.steering import SteeringConfig, SteeringEnv, SteeringRenderer

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_env_dynamics.npz")


@pytest.fixture(scope="module")
def ref():
    return np.load(GOLDEN)


def test_cartpole_matches_reference_trajectory(ref):
    B = ref["cp_obs0"].shape[0]
    cfg = CartPoleConfig(num_scenes=B, device="cpu", render=False, auto_reset=False)
    env = CartPoleEnv(CartPoleRenderer(cfg), cfg)
    obs, sc = torch.from_numpy(ref["cp_obs0"]), torch.from_numpy(ref["cp_sc0"])
    for t in range(ref["cp_actions"].shape[0]):
        td = env._step({"observation": obs, "step_count": sc, "action": torch.from_numpy(ref["cp_actions"][t])})
        for k in ("observation", "reward", "done", "step_count"):
            assert np.array_equal(td[k].numpy(), ref[f"cp_{k}"][t]), (t, k)
        obs, sc = td["observation"], td["step_count"]
    # the trajectory exercises every termination: cart out of bounds, pole past 12 degrees, the step limit
    last = ref["cp_observation"][-1]
    assert (np.abs(last[:, 0]) > 2.4).any() and (np.abs(last[:, 2]) > np.radians(12)).any()
    assert (ref["cp_done"][0, :, 0] & (ref["cp_sc0"] >= 499)).any()


def test_steering_matches_reference_trajectory(ref):
    B = ref["st_obs0"].shape[0]
    cfg = SteeringConfig(num_scenes=B, device="cpu", render=False, auto_reset=False, number_of_obstacles=20,
                         max_steps=300)
    env = SteeringEnv(SteeringRenderer(cfg), cfg)
    env._obstacles = torch.from_numpy(ref["st_obstacles"]).clone()
    env._player_x = torch.from_numpy(ref["st_player_x0"]).clone()
    env._player_y = torch.zeros(B)
    env._prev_player_x = torch.zeros(B)
    env._prev_player_y = torch.zeros(B)
    env._forward_speed = torch.full((B,), env.speed_initial)
    env._grace_remaining = torch.zeros(B)
    env._next_obstacle_idx = torch.zeros(B, dtype=torch.long)
    obs = env._get_observation()
    assert np.array_equal(obs.numpy(), ref["st_obs0"])
    sc = torch.from_numpy(ref["st_sc0"])
    for t in range(ref["st_actions"].shape[0]):
        td = env._step({"observation": obs, "step_count": sc, "action": torch.from_numpy(ref["st_actions"][t])})
        for k in ("observation", "reward", "done", "step_count"):
            assert np.array_equal(td[k].numpy(), ref[f"st_{k}"][t]), (t, k)
        assert np.array_equal(env._grace_remaining.numpy(), ref["st_grace"][t]), t
        assert np.array_equal(env._next_obstacle_idx.numpy(), ref["st_next_idx"][t]), t
        obs, sc = td["observation"], td["step_count"]
    # collisions (penalty and grace period), the track end and the step limit all occur
    assert (ref["st_reward"] < 0).sum() > 10 and ref["st_next_idx"].max() == 20
    assert (ref["st_done"][:, :, 0] & (ref["st_next_idx"] < 20)).any()
