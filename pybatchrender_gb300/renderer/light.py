"""Global lighting (``renderer/light.py``): ambient + one directional light
with a strength in [0,1], the uniforms of ``shaders/basic.frag:13-18``.
The direction points *towards* the light (``ndl = dot(n, normalize(dir))``)."""
from __future__ import annotations

from typing import Literal

from .shader_context import PBRShaderContext


class PBRLight(PBRShaderContext):
    def __init__(self, showbase,
                 ambient: tuple[float, float, float] = (0.2, 0.2, 0.25),
                 dir_dir: tuple[float, float, float] = (0.4, -0.6, -0.7),
                 dir_col: tuple[float, float, float] = (1.0, 1.0, 1.0),
                 strength: float = 1.0,
                 backend: Literal["loop", "instanced"] = "instanced") -> None:
        super().__init__(showbase, backend=backend)
        self.set_strength(strength)
        self.set_directional(dir_dir, dir_col)
        self.set_ambient(ambient)
        self._register_self()

    def set_strength(self, strength: float) -> None:
        self.strength = float(strength)
        self._changed()

    def set_directional(self, dir_dir, dir_col) -> None:
        self.dir_dir = tuple(float(x) for x in dir_dir)
        self.dir_col = tuple(float(x) for x in dir_col)
        if len(self.dir_dir) != 3 or len(self.dir_col) != 3:
            raise ValueError("dir_dir and dir_col must have 3 components")
        self._changed()

    def set_ambient(self, amb_col) -> None:
        self.ambient = tuple(float(x) for x in amb_col)
        if len(self.ambient) != 3:
            raise ValueError("ambient must have 3 components")
        self._changed()

    def attach(self, node) -> None:
        return None

    def _changed(self) -> None:
        if all(hasattr(self, a) for a in ("strength", "dir_dir", "dir_col", "ambient")):
            notify = getattr(self.base, "_light_changed", None)
            if notify is not None:
                notify(self)

    def _register_self(self) -> None:
        self.base._pbr_light = self
        self._changed()
