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


@pytest.mark.parametrize("auto_reset", [True, False])
def test_fused_cartpole_step_matches_tensor_ops(cuda, auto_reset):
    """pbr_cartpole_step (one launch) against the step written as tensor
    operations: identical observations, rewards, done flags and step counts
    over 300 random-action steps, resets included (the same RNG calls draw the
    initial states)."""
    n = 2048
    fused = pbr.envs.make("CartPole-v0", num_scenes=n, render=False, auto_reset=auto_reset)
    ops = pbr.envs.make("CartPole-v0", num_scenes=n, render=False, auto_reset=auto_reset, fused_step=False)
    assert fused.fused_step and not ops.fused_step
    torch.manual_seed(11)
    td = fused.reset()
    obs, sc = td["observation"], td["step_count"]
    # start some scenes near the thresholds so that done flips in the first steps
    obs[:64, 0] = torch.linspace(-2.45, 2.45, 64, device="cuda")
    obs[64:128, 2] = torch.linspace(-1.6, 1.6, 64, device="cuda")
    sc[128:192] = 498
    gen = torch.Generator(device="cuda").manual_seed(4)
    ob_f, sc_f, ob_o, sc_o = obs.clone(), sc.clone(), obs.clone(), sc.clone()
    resets = 0
    for t in range(300):
        act = torch.randint(0, 2, (n,), generator=gen, device="cuda")
        torch.manual_seed(1000 + t)
        f = fused._step(pbr.env.TensorDict({"observation": ob_f, "action": act, "step_count": sc_f}, batch_size=[n]))
        torch.manual_seed(1000 + t)
        o = ops._step(pbr.env.TensorDict({"observation": ob_o, "action": act, "step_count": sc_o}, batch_size=[n]))
        for key in ("observation", "reward", "done", "step_count"):
            assert torch.equal(f[key], o[key]), (t, key, (f[key] != o[key]).sum().item())
        resets += int(f["done"].sum())
        ob_f, sc_f, ob_o, sc_o = f["observation"], f["step_count"], o["observation"], o["step_count"]
    assert resets > 100


def test_fused_step_in_graph_with_render(cuda):
    """GraphedEnvStep over the fused step: pixels equal an eager render of the
    raw next state."""
    n = 128
    env = pbr.envs.make("CartPole-v0", num_scenes=n)
    g = pbr.GraphedEnvStep(env)
    td = env.reset()
    obs, sc = td["observation"].clone(), td["step_count"].clone()
    for _ in range(4):
        act = torch.randint(0, 2, (n,), device="cuda")
        o = g({"observation": obs, "action": act, "step_count": sc})
        raw = env._dynamics(obs, act)
        ref = env._renderer.step(raw)
        assert torch.equal(o["pixels"], ref)
        obs, sc = o["observation"].clone(), o["step_count"].clone()


def test_template_env_renders(cuda, oracle):
    """The template environment on the GPU: state-bound render, parity with the
    oracle, and the box follows the state."""
    from pybatchrender_gb300.envs._template import MyEnv, MyEnvConfig, MyEnvRenderer
    from tests.test_gpu_render import check_parity
    cfg = MyEnvConfig(num_scenes=32, device="cuda")
    env = MyEnv(MyEnvRenderer(cfg), cfg)
    td = env.reset()
    assert td["pixels"].shape == (32, 3, 64, 64)
    td["action"] = torch.ones(32, dtype=torch.long, device="cuda")
    nxt = env.step(td)["next"]
    assert not torch.equal(nxt["pixels"], td["pixels"])
    check_parity(env._renderer, oracle)


def test_template_env_in_graph(cuda):
    """GraphedEnvStep over the template environment: same observations and
    pixels as the eager step (no auto-reset, so no random draws)."""
    from pybatchrender_gb300.envs._template import MyEnv, MyEnvConfig, MyEnvRenderer
    def make():
        cfg = MyEnvConfig(num_scenes=64, device="cuda", auto_reset=False)
        return MyEnv(MyEnvRenderer(cfg), cfg)
    eager, graphed = make(), make()
    g = pbr.GraphedEnvStep(graphed)
    td = eager.reset()
    obs, sc = td["observation"].clone(), td["step_count"].clone()
    ob_e, sc_e, ob_g, sc_g = obs, sc, obs.clone(), sc.clone()
    for i in range(5):
        act = (torch.arange(64, device="cuda") + i) % 2
        e = eager._step(pbr.env.TensorDict({"observation": ob_e, "action": act, "step_count": sc_e}, batch_size=[64]))
        o = g({"observation": ob_g, "action": act, "step_count": sc_g})
        for key in ("observation", "reward", "done", "step_count", "pixels"):
            assert torch.equal(e[key], o[key]), key
        ob_e, sc_e = e["observation"], e["step_count"]
        ob_g, sc_g = o["observation"].clone(), o["step_count"].clone()
