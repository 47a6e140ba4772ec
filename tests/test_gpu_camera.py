"""Per-scene cameras on the GPU: ``pbr_camera_update`` (one launch per camera
update) against the same float32 formulas as tensor operations on the CPU
(``renderer/camera.py:150-291``: lookAt basis, eye translation, GL
perspective with the window aspect, VP = P V), for every setter, plus the
reference's own CartPole cameras (``ref_cartpole_N64.npz``, the
view-projection matrices recorded from the reference).  Both
sides round in float32 in slightly different orders, so the bar is a few
units in the last place (4e-6 relative to the matrix's largest entry)."""
import os

import numpy as np
import pytest
import torch

import pybatchrender_gb300 as pbr
from pybatchrender_gb300.envs.cartpole import CartPoleConfig, CartPoleRenderer

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _cams(K, device):
    r = pbr.PBRRenderer(num_scenes=K, tile_resolution=(64, 48), device=device, report_fps=False)
    return r.add_camera(fov_y_deg=47.0, z_near=0.1, z_far=80.0)


def _close(a, b, rel=4e-6):
    a, b = a.detach().cpu().double(), b.detach().cpu().double()
    scale = b.abs().amax(dim=(-2, -1), keepdim=True).clamp_min(1e-30)
    return float(((a - b).abs() / scale).max())


def test_camera_kernel_matches_tensor_math(cuda):
    K = 37
    g = torch.Generator().manual_seed(50)
    eye = torch.randn((K, 3), generator=g) * 5
    target = torch.randn((K, 3), generator=g)
    hpr = torch.rand((K, 3), generator=g) * 6.2 - 3.1
    up = torch.randn((K, 3), generator=g)
    fwd = torch.randn((K, 3), generator=g)
    gpu, cpu = _cams(K, "cuda"), _cams(K, "cpu")
    steps = [("set_positions_and_lookat", (eye, target)), ("set_eye", (eye * 0.5,)), ("set_hprs", (hpr,)),
             ("set_up", (up,)), ("set_forward", (fwd,)), ("look_at", (target * 2,)),
             ("set_eye", (torch.tensor([1.0, -9.0, 2.0]),))]
    for name, args in steps:
        getattr(gpu, name)(*[a.to(cuda) for a in args])
        getattr(cpu, name)(*args)
        torch.cuda.synchronize()
        assert _close(gpu.V_k44, cpu.V_k44) <= 4e-6, (name, _close(gpu.V_k44, cpu.V_k44))
        assert _close(gpu.VP_k44, cpu.VP_k44) <= 4e-6, (name, _close(gpu.VP_k44, cpu.VP_k44))
    # lazy: the view changes, the view-projection follows at the next non-lazy update
    before = gpu.VP_k44.clone()
    gpu.set_eye(eye.to(cuda), lazy=True)
    cpu.set_eye(eye, lazy=True)
    assert torch.equal(gpu.VP_k44, before)
    gpu.set_projection(fov_y_deg=33.0)
    cpu.set_projection(fov_y_deg=33.0)
    assert _close(gpu.VP_k44, cpu.VP_k44) <= 4e-6


def test_reference_cartpole_cameras(cuda):
    """The reference's CartPole renderer cameras (its view-projection matrices,
    recorded from the reference itself), computed by the kernel."""
    ref = np.load(os.path.join(GOLDEN, "ref_cartpole_N64.npz"))
    r = CartPoleRenderer(CartPoleConfig(num_scenes=64, report_fps=False))
    got = r._pbr_cam.VP_k44.cpu().numpy()
    want = np.asarray(ref["VP"], np.float32)  # per-scene view-projection the reference builds (row-major)
    err = np.abs(got - want).max() / np.abs(want).max()
    assert err <= 4e-6, err


def test_camera_update_is_one_launch(cuda):
    """A per-step eye update (Steering's following camera) is a single launch
    of the library's camera kernel."""
    cam = _cams(512, "cuda")
    eye = torch.randn((512, 3), device=cuda)
    cam.set_eye(eye)
    torch.cuda.synchronize()
    from torch.profiler import ProfilerActivity, profile
    with profile(activities=[ProfilerActivity.CUDA]) as prof:
        cam.set_eye(eye)
        torch.cuda.synchronize()
    kernels = [e.name for e in prof.events() if e.device_type == torch.autograd.DeviceType.CUDA]
    if not kernels:
        pytest.skip("the profiler recorded no CUDA activity here")
    assert len(kernels) == 1 and "camera_update_kernel" in kernels[0], kernels
