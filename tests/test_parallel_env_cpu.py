"""``envs.make_parallel`` without TorchRL: spawned process replicas, each with
its own env and renderer, seen as one env of batch ``[num_workers,
num_scenes]`` (``envs/__init__.py:127-164`` and ``env.py:360-440`` of the
reference).  Two CPU workers of CartPole-v0 (dynamics only, no pixels: the
renderer needs a GPU) must produce exactly what two single envs built with the
workers' seeds (seed + worker index) produce from the same actions."""
import pytest
import torch

import pybatchrender_gb300 as pbr
from pybatchrender_gb300.env import HAVE_TORCHRL

pytestmark = pytest.mark.skipif(HAVE_TORCHRL, reason="TorchRL installed: make_parallel returns TorchRL's ParallelEnv")

KW = dict(num_scenes=6, render=False, device="cpu", seed=3)


def _actions(steps, W, B):
    g = torch.Generator().manual_seed(11)
    return [torch.randint(0, 2, (W, B), generator=g) for _ in range(steps)]


def _single_rollouts(W, acts):
    """What worker i computes: its own env (seed 3 + i) reset, then stepped."""
    out = []
    for i in range(W):
        env = pbr.envs.make("CartPole-v0", **dict(KW, seed=KW["seed"] + i, worker_index=i, num_workers=W))
        td = env.reset()
        rec = [td["observation"].clone()]
        for a in acts:
            td["action"] = a[i]
            td = env.step(td)["next"]
            rec += [td["observation"].clone(), td["reward"].clone(), td["done"].clone(), td["step_count"].clone()]
        out.append(rec)
    return out


@pytest.mark.parametrize("shared_memory", [True, False])
def test_make_parallel_matches_single_envs(shared_memory):
    W, B, steps = 2, KW["num_scenes"], 25
    acts = _actions(steps, W, B)
    want = _single_rollouts(W, acts)
    env = pbr.envs.make_parallel("CartPole-v0", num_workers=W, shared_memory=shared_memory, **KW)
    try:
        assert env.batch_size == torch.Size([W, B])
        assert env.action_spec.rand().shape == (W, B)
        td = env.reset()
        assert td["observation"].shape == (W, B, 4)
        got = [[td["observation"][i].clone()] for i in range(W)]
        for a in acts:
            td = td.clone()
            td["action"] = a
            td = env.step(td)
            assert td["next", "reward"].shape == (W, B, 1)
            td = td["next"]
            for i in range(W):
                got[i] += [td["observation"][i].clone(), td["reward"][i].clone(), td["done"][i].clone(),
                           td["step_count"][i].clone()]
        for i in range(W):
            for g, w in zip(got[i], want[i]):
                assert torch.equal(g, w)
        # the returned tensors are copies: the next step does not change them
        obs = td["observation"].clone()
        td["action"] = acts[0]
        env.step(td)
        assert torch.equal(td["observation"], obs)
    finally:
        env.close()
    assert env.is_closed


class FailingRenderer:
    """A renderer whose construction fails inside the worker process."""

    def __init__(self, cfg):
        raise ValueError("renderer construction fails here")


def test_worker_errors_surface_in_the_main_process():
    from pybatchrender_gb300.envs.cartpole import CartPoleConfig, CartPoleEnv
    with pytest.raises(RuntimeError, match="(?s)worker 0 failed.*renderer construction fails here"):
        CartPoleEnv.make_parallel_env(config=CartPoleConfig(**KW), renderer_cls=FailingRenderer, num_workers=1)


def test_devices_need_one_entry_per_worker():
    with pytest.raises(ValueError):
        pbr.envs.make_parallel("CartPole-v0", num_workers=2, devices=["cpu"], **KW)
