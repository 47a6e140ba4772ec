"""Run code written against the reference package's module paths unchanged.

``install_as_pybatchrender()`` registers this package under the reference's
module names, so that ``import pybatchrender as pbr``,
``from pybatchrender.renderer.renderer import PBRRenderer``,
``from pybatchrender.env import PBREnv`` or an environment package that does
``from pybatchrender.config import PBRConfig`` resolve to this renderer.
``pybatchrender.renderer.frame_grabber`` becomes a module whose grabbers are
None: there is no readback here, pixels are written straight into the output
tensor.
"""
from __future__ import annotations

import importlib
import sys
import types

_MODULES = {
    "pybatchrender": "pybatchrender_gb300",
    "pybatchrender.config": "pybatchrender_gb300.config",
    "pybatchrender.env": "pybatchrender_gb300.env",
    "pybatchrender.envs": "pybatchrender_gb300.envs",
    "pybatchrender.envs.cartpole": "pybatchrender_gb300.envs.cartpole",
    "pybatchrender.envs.cartpole.config": "pybatchrender_gb300.envs.cartpole.config",
    "pybatchrender.envs.cartpole.env": "pybatchrender_gb300.envs.cartpole.env",
    "pybatchrender.envs.cartpole.renderer": "pybatchrender_gb300.envs.cartpole.renderer",
    "pybatchrender.envs.steering": "pybatchrender_gb300.envs.steering",
    "pybatchrender.envs.steering.config": "pybatchrender_gb300.envs.steering.config",
    "pybatchrender.envs.steering.env": "pybatchrender_gb300.envs.steering.env",
    "pybatchrender.envs.steering.renderer": "pybatchrender_gb300.envs.steering.renderer",
    "pybatchrender.envs._template": "pybatchrender_gb300.envs._template",
    "pybatchrender.envs._template.config": "pybatchrender_gb300.envs._template.config",
    "pybatchrender.envs._template.env": "pybatchrender_gb300.envs._template.env",
    "pybatchrender.envs._template.renderer": "pybatchrender_gb300.envs._template.renderer",
    "pybatchrender.renderer": "pybatchrender_gb300.renderer",
    "pybatchrender.renderer.renderer": "pybatchrender_gb300.renderer.renderer",
    "pybatchrender.renderer.node": "pybatchrender_gb300.renderer.node",
    "pybatchrender.renderer.camera": "pybatchrender_gb300.renderer.camera",
    "pybatchrender.renderer.light": "pybatchrender_gb300.renderer.light",
    "pybatchrender.renderer.shader_context": "pybatchrender_gb300.renderer.shader_context",
}


def install_as_pybatchrender(force: bool = False) -> None:
    """Register the aliases in ``sys.modules``.  Refuses (ValueError) when a
    module named ``pybatchrender`` that is not this package is already
    imported, unless ``force``."""
    existing = sys.modules.get("pybatchrender")
    if existing is not None and getattr(existing, "__name__", "") != "pybatchrender_gb300" and not force:
        raise ValueError("another 'pybatchrender' package is already imported; pass force=True to replace it")
    for alias, real in _MODULES.items():
        sys.modules[alias] = importlib.import_module(real)
    grabber = types.ModuleType("pybatchrender.renderer.frame_grabber")
    grabber.GPUFrameGrabber = None
    grabber.CPUFrameGrabber = None
    grabber.GPU_AVAILABLE = sys.modules["pybatchrender_gb300"].GPU_AVAILABLE
    sys.modules["pybatchrender.renderer.frame_grabber"] = grabber
