"""Code written against the reference package's module paths runs unchanged
after ``install_as_pybatchrender()`` (CPU)."""
import importlib
import sys
import textwrap

import pytest

import pybatchrender_gb300 as ours
from pybatchrender_gb300.compat import install_as_pybatchrender


@pytest.fixture
def alias():
    saved = {k: v for k, v in sys.modules.items() if k == "pybatchrender" or k.startswith("pybatchrender.")}
    install_as_pybatchrender(force=True)
    yield
    for k in [k for k in sys.modules if k == "pybatchrender" or k.startswith("pybatchrender.")]:
        del sys.modules[k]
    sys.modules.update(saved)


def test_reference_import_paths(alias):
    import pybatchrender as pbr
    from pybatchrender.config import PBRConfig
    from pybatchrender.env import PBREnv
    from pybatchrender.envs.cartpole.renderer import CartPoleRenderer
    from pybatchrender.renderer.frame_grabber import GPUFrameGrabber
    from pybatchrender.renderer.renderer import PBRRenderer
    assert pbr is ours and PBRRenderer is ours.PBRRenderer and PBRConfig is ours.PBRConfig and PBREnv is ours.PBREnv
    assert CartPoleRenderer.__module__ == "pybatchrender_gb300.envs.cartpole.renderer"
    assert GPUFrameGrabber is None
    assert "CartPole-v0" in pbr.envs.list_envs()


def test_user_env_written_for_the_reference(alias, tmp_path, monkeypatch):
    pkg = tmp_path / "myenv"
    pkg.mkdir()
    (pkg / "__init__.py").write_text(textwrap.dedent("""
        import torch
        from pybatchrender.config import PBRConfig
        from pybatchrender.renderer.renderer import PBRRenderer

        class BoxRenderer(PBRRenderer):
            def __init__(self, cfg=None):
                super().__init__(cfg)
                self.box = self.add_node("models/box", instances_per_scene=2)
                self.add_camera()
                self.add_light()
                self.setup_environment()

            def _step(self, state_batch=None):
                if state_batch is not None:
                    self.box.set_positions(state_batch)
    """))
    monkeypatch.syspath_prepend(str(tmp_path))
    mod = importlib.import_module("myenv")
    r = mod.BoxRenderer(ours.PBRConfig(num_scenes=3, device="cpu"))
    assert isinstance(r, ours.PBRRenderer) and r.box.buf_instances == 6


def test_refuses_to_replace_another_package():
    saved = sys.modules.get("pybatchrender")
    sys.modules["pybatchrender"] = type(sys)("pybatchrender")
    try:
        with pytest.raises(ValueError):
            install_as_pybatchrender()
    finally:
        if saved is None:
            del sys.modules["pybatchrender"]
        else:
            sys.modules["pybatchrender"] = saved
