"""The many-cubes and uneven configurations at their full sizes: the whole
batch is rendered on the GPU in one launch, and scenes spread over the batch
(first, last, and the scenes with the most instances) are checked against
the FP64 oracle with the parity bar of test_gpu_render.py.  Scenes are
independent, so a subset check covers the batch's layout and scheduling."""
import numpy as np
import pytest
import torch

from pybatchrender_gb300 import workloads

pytestmark = pytest.mark.gpu


def _check_scenes(r, oracle, scenes, depth_tol=1e-5, measured=None):
    pix, depth, win = r.render(return_depth=True, return_winner=True)
    torch.cuda.synchronize()
    sc, me, no = r.export_scene()
    for k in scenes:
        ref = oracle.render_hard(sc, me, no, k, k + 1, want_depth=True, want_winner=True, want_ambiguous=True,
                                 nthreads=8)
        gpu = {"pixels": pix[k:k + 1].cpu().numpy(), "winner": win[k:k + 1].cpu().numpy(),
               "depth": depth[k:k + 1].cpu().numpy()}
        cmp = oracle.compare_hard(gpu, ref)
        assert cmp["winner_mismatch"] == 0, (k, cmp)
        assert cmp["color_max_diff_unambiguous"] <= 1, (k, cmp)
        assert cmp["color_within_1"] >= 0.995, (k, cmp)
        covered = (ref["winner"] >= 0) & ~ref["ambiguous"]
        derr = float(np.abs(gpu["depth"] - ref["depth"])[covered].max()) if covered.any() else 0.0
        if measured is not None:
            measured(f"scene {k}", dict(cmp, depth_max_err=f"{derr:.2e}"))
        assert derr <= depth_tol, (k, cmp)


def test_many_cubes_full_config(cuda, oracle, measured):
    """1024 scenes x 128x128, 64 cubes per scene (+ depth output)."""
    r = workloads.many_cubes(num_scenes=1024, res=128, instances=64, seed=0)
    _check_scenes(r, oracle, [0, 1, 511, 1023], measured=measured)


def test_uneven_full_config(cuda, oracle, measured):
    """4096 scenes x 84x84, 1..512 instances of cube / cylinder-64 /
    icosphere-3 per scene, per-scene cameras, persistent launch.  Winners
    (coverage and depth order) are exact; the window depth bar is 1e-4: the
    busiest scenes hold sub-pixel, nearly edge-on triangles whose depth
    planes are steep, and their float32 plane evaluation differs from the
    FP64 one by up to 2.3e-5 (measured)."""
    r = workloads.uneven(num_scenes=4096, res=84, max_instances=512, seed=0, persistent=True)
    counts = r.total_counts
    busiest = torch.argsort(counts, descending=True)[:2].tolist()
    _check_scenes(r, oracle, [0, 4095] + busiest, depth_tol=1e-4, measured=measured)
