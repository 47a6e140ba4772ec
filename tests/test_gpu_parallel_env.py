"""``envs.make_parallel`` on the GPU without TorchRL: two CartPole-v0 workers in
spawned processes render on cuda:0 (independent CUDA contexts, no work waits
on another process) and write observations, rewards and pixels into buffers
shared with the main process through CUDA IPC.  Every tensor must equal what
a single env built with the worker's seed produces from the same actions."""
import pytest
import torch

import pybatchrender_gb300 as pbr
from pybatchrender_gb300.env import HAVE_TORCHRL

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(HAVE_TORCHRL, reason="TorchRL installed: make_parallel returns TorchRL's ParallelEnv")]


def test_make_parallel_cuda_workers_match_single_envs(cuda):
    W, B, steps = 2, 64, 6
    kw = dict(num_scenes=B, device="cuda", seed=5, tile_resolution=(64, 64))
    g = torch.Generator().manual_seed(12)
    acts = [torch.randint(0, 2, (W, B), generator=g) for _ in range(steps)]
    want = []
    for i in range(W):
        env = pbr.envs.make("CartPole-v0", **dict(kw, seed=kw["seed"] + i, worker_index=i, num_workers=W))
        td = env.reset()
        rec = [td["observation"].clone(), td["pixels"].clone()]
        for a in acts:
            td["action"] = a[i].to(cuda)
            td = env.step(td)["next"]
            rec += [td["observation"].clone(), td["reward"].clone(), td["pixels"].clone()]
        want.append(rec)
        del env
    env = pbr.envs.make_parallel("CartPole-v0", num_workers=W, **kw)
    try:
        assert env.batch_size == torch.Size([W, B]) and env.device == cuda
        td = env.reset()
        assert td["pixels"].shape == (W, B, 3, 64, 64) and td["pixels"].is_cuda
        got = [[td["observation"][i].clone(), td["pixels"][i].clone()] for i in range(W)]
        for a in acts:
            td = td.clone()
            td["action"] = a.to(cuda)
            td = env.step(td)["next"]
            for i in range(W):
                got[i] += [td["observation"][i].clone(), td["reward"][i].clone(), td["pixels"][i].clone()]
        for i in range(W):
            for j, (x, y) in enumerate(zip(got[i], want[i])):
                assert torch.equal(x, y), (i, j)
        assert want[0][-1].float().mean() > 0  # frames are not empty
    finally:
        env.close()
