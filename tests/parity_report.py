"""Parity report: the CUDA renderer against the FP64 oracle on the standard
scenes, one table row per scene (run on a CUDA machine:
``python -m tests.parity_report``).  The pytest suite asserts the bars; this
prints the measured margins."""
import numpy as np
import torch

import pybatchrender_gb300 as pbr
from oracle import oracle
from pybatchrender_gb300 import workloads
from pybatchrender_gb300.envs.cartpole import CartPoleConfig, CartPoleRenderer


def measure(r):
    pix, depth, win = r.render(return_depth=True, return_winner=True)
    torch.cuda.synchronize()
    sc, me, no = r.export_scene()
    ref = oracle.render_hard(sc, me, no, want_depth=True, want_winner=True, want_ambiguous=True, nthreads=8)
    gpu = {"pixels": pix.cpu().numpy(), "winner": win.cpu().numpy(), "depth": depth.cpu().numpy()}
    cmp = oracle.compare_hard(gpu, ref)
    cov = (ref["winner"] >= 0) & ~ref["ambiguous"]
    dz = float(np.abs(gpu["depth"] - ref["depth"])[cov].max()) if cov.any() else 0.0
    return cmp, dz, float(cov.mean())


def scenes():
    yield "CartPole bench scene, 256 x 64x64", lambda: _with_states(workloads.cartpole_bench(num_scenes=256, seed=1))
    yield "reference CartPole scene, 256 x 64x64", lambda: _with_states(
        CartPoleRenderer(CartPoleConfig(num_scenes=256, device="cuda")))
    yield "many cubes, 64 x 128x128", lambda: workloads.many_cubes(num_scenes=64, seed=2)
    yield "uneven mixed meshes, 64 x 84x84", lambda: workloads.uneven(num_scenes=64, max_instances=128, seed=3)
    yield "Steering-v0, 16 x 64x64", _steering
    yield "textured CartPole-sized scenes, 256 x 64x64", _textured


def _with_states(r):
    r._step(workloads.cartpole_states(r.num_scenes, seed=5, device="cuda"))
    return r


def _textured():
    from tests.test_gpu_textures import _small_textured
    return _small_textured("auto")


def _steering():
    env = pbr.envs.make("Steering-v0", num_scenes=16)
    env.reset()
    return env._renderer


def main():
    print("| scene | pixels | ambiguous | winner mismatches | colour max diff (unambiguous) | exact | within 1/255 | "
          "depth max diff (covered, unambiguous) | covered |")
    print("|---|---|---|---|---|---|---|---|---|")
    for name, make in scenes():
        cmp, dz, cov = measure(make())
        print(f"| {name} | {cmp['pixels']} | {cmp['ambiguous']} | {cmp['winner_mismatch']} | "
              f"{cmp['color_max_diff_unambiguous']} | {100 * cmp['color_exact']:.3f} % | "
              f"{100 * cmp['color_within_1']:.3f} % | {dz:.2e} | {100 * cov:.2f} % |", flush=True)


if __name__ == "__main__":
    main()
