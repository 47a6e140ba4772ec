"""The CartPole env step (dynamics, termination, reward, auto-reset and the
state-bound render) replayed as one CUDA graph (``GraphedEnvStep``): same
results as the eager ``_step``."""
import pytest
import torch

import pybatchrender_gb300 as pbr

pytestmark = pytest.mark.gpu


def _env(n, auto_reset):
    return pbr.envs.make("CartPole-v0", num_scenes=n, auto_reset=auto_reset)


def test_graphed_env_step_matches_eager(cuda):
    n = 64
    eager, graphed = _env(n, False), _env(n, False)
    g = pbr.GraphedEnvStep(graphed)
    td = eager.reset()
    obs, sc = td["observation"].clone(), td["step_count"].clone()
    gen = torch.Generator(device="cuda").manual_seed(3)
    ob_e, sc_e, ob_g, sc_g = obs, sc, obs.clone(), sc.clone()
    for _ in range(6):
        act = torch.randint(0, 2, (n,), generator=gen, device="cuda")
        e = eager._step(pbr.env.TensorDict({"observation": ob_e, "action": act, "step_count": sc_e}, batch_size=[n]))
        o = g({"observation": ob_g, "action": act, "step_count": sc_g})
        for key in ("observation", "reward", "done", "step_count", "pixels"):
            assert torch.equal(e[key], o[key]), key
        ob_e, sc_e = e["observation"], e["step_count"]
        ob_g, sc_g = o["observation"].clone(), o["step_count"].clone()
    assert e["pixels"].float().mean() > 0


def test_graphed_env_step_auto_reset(cuda):
    """Scenes that terminate are reset to states inside the initial ranges."""
    n = 256
    env = _env(n, True)
    g = pbr.GraphedEnvStep(env)
    td = env.reset()
    obs, sc = td["observation"].clone(), td["step_count"].clone()
    obs[: n // 2, 0] = 3.0  # beyond the x threshold: these terminate on the next step
    act = torch.zeros(n, dtype=torch.long, device=cuda)
    o = g({"observation": obs, "action": act, "step_count": sc})
    done = o["done"].squeeze(-1)
    assert done[: n // 2].all()
    x = o["observation"][: n // 2, 0]
    assert (x.abs() <= 2.0).all() and torch.equal(o["step_count"][: n // 2], torch.zeros_like(sc[: n // 2]))
    assert o["pixels"].shape == (n, 3, 64, 64)
