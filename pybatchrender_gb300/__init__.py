"""pybatchrender_gb300: a GB300 (sm_103a) batch renderer with PyBatchRender's API.

``import pybatchrender_gb300 as pbr`` gives the names the reference package
exports (``pybatchrender/__init__.py``): ``PBRConfig``, ``PBRRenderer``,
``PBRNode``, ``PBRCam``, ``PBRLight``, ``PBRShaderContext``, ``PBREnv`` and the
``envs`` registry.  There are no frame grabbers: pixels are written straight
into the output tensor, so ``GPUFrameGrabber`` / ``CPUFrameGrabber`` /
``FrameGrabber`` are None and ``GPU_AVAILABLE`` reports whether a CUDA device
is present.
"""
__version__ = "0.1.0"

from .config import PBRConfig  # noqa: F401
from .renderer import PBRCam, PBRLight, PBRNode, PBRRenderer, PBRShaderContext  # noqa: F401
from ._capi import PBRError, RendererUnavailable  # noqa: F401
from .env import GraphedEnvStep, PBREnv  # noqa: F401
from . import envs  # noqa: F401
from .compat import install_as_pybatchrender  # noqa: F401

GPUFrameGrabber = None
CPUFrameGrabber = None
FrameGrabber = None
try:
    import torch as _torch
    GPU_AVAILABLE = bool(_torch.cuda.is_available())
except Exception:  # pragma: no cover
    GPU_AVAILABLE = False

__all__ = [
    "PBRConfig", "PBREnv", "GraphedEnvStep", "PBRRenderer", "PBRNode", "PBRCam", "PBRLight", "PBRShaderContext",
    "GPUFrameGrabber", "CPUFrameGrabber", "FrameGrabber", "envs", "__version__", "PBRError",
    "RendererUnavailable", "install_as_pybatchrender",
]
