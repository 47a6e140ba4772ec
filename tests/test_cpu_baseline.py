"""The timed CPU baseline is the oracle's FP32 build (``precision="f32"``, all
host threads).  These CPU tests check that it renders the same frames as the
FP64 oracle, so that its frames/s counts the same work: identical winners on
every unambiguous pixel, colour within 1/255, and output independent of the
thread count."""
import numpy as np
import pytest

from tests import kat_scenes as K


@pytest.fixture(scope="module")
def cartpole_scene():
    from pybatchrender_gb300 import workloads
    r = workloads.cartpole_bench(num_scenes=64, res=64, seed=0, device="cpu")
    r._step(workloads.cartpole_states(64, seed=1000))
    return r.export_scene()


def test_fp32_baseline_matches_fp64_oracle(oracle, cartpole_scene):
    sc, me, no = cartpole_scene
    ref = oracle.render_hard(sc, me, no, want_winner=True, want_ambiguous=True)
    got = oracle.render_hard(sc, me, no, want_winner=True, precision="f32", nthreads=4)
    ok = ~ref["ambiguous"]
    assert np.array_equal(got["winner"][ok], ref["winner"][ok])
    diff = np.abs(got["pixels"].astype(np.int16) - ref["pixels"].astype(np.int16))
    assert diff.max(initial=0) <= 1
    assert np.all(diff.max(axis=1)[ok] <= 1)
    assert (ref["winner"] >= 0).sum() > 1000  # the scene covers pixels at all


def test_fp32_baseline_is_independent_of_thread_count(oracle, cartpole_scene):
    sc, me, no = cartpole_scene
    one = oracle.render_hard(sc, me, no, precision="f32", nthreads=1)["pixels"]
    many = oracle.render_hard(sc, me, no, precision="f32", nthreads=7)["pixels"]
    assert np.array_equal(one, many)


def test_fp32_baseline_known_answers(oracle):
    mesh = K.screen_mesh(K.SQUARE, K.SQUARE_TRIS)
    sc = K.scene(strength=1.0, ambient=K.FACE_AMBIENT, ldir=(0.0, 0.0, 2.0), lcol=(1.0, 1.0, 1.0))
    got = oracle.render_hard(sc, [mesh], [K.node(0, color=K.FACE_COLOR)], want_winner=True, want_depth=True,
                             precision="f32")
    cov = got["winner"][0] >= 0
    assert np.array_equal(cov, K.square_expected())
    for c in range(3):
        assert np.all(got["pixels"][0][c][cov] == K.FACE_EXPECT[c])
    assert np.all(got["depth"][0][cov] == 0.625)


@pytest.mark.parametrize("workload", ["many_cubes", "uneven"])
def test_fp32_baseline_matches_fp64_on_other_workloads(oracle, workload):
    from pybatchrender_gb300 import workloads
    if workload == "many_cubes":
        r = workloads.many_cubes(num_scenes=8, res=64, instances=16, device="cpu")
    else:
        r = workloads.uneven(num_scenes=8, res=48, max_instances=24, device="cpu")
    sc, me, no = r.export_scene()
    ref = oracle.render_hard(sc, me, no, want_winner=True, want_ambiguous=True)
    got = oracle.render_hard(sc, me, no, want_winner=True, precision="f32", nthreads=3)
    ok = ~ref["ambiguous"]
    assert np.array_equal(got["winner"][ok], ref["winner"][ok])
    diff = np.abs(got["pixels"].astype(np.int16) - ref["pixels"].astype(np.int16)).max(axis=1)
    assert diff[ok].max(initial=0) <= 1
    assert (ref["winner"] >= 0).sum() > 100
