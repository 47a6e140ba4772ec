"""Renderer API: PBRRenderer, PBRNode, PBRCam, PBRLight, PBRShaderContext."""
from .camera import PBRCam
from .light import PBRLight
from .meshes import Mesh, cylinder, icosphere, resolve_model, unit_cube
from .node import PBRNode
from .renderer import PBRRenderer
from .shader_context import PBRShaderContext

__all__ = ["PBRRenderer", "PBRNode", "PBRCam", "PBRLight", "PBRShaderContext", "Mesh", "unit_cube", "cylinder",
           "icosphere", "resolve_model"]
