"""Renderer configuration (the reference's ``PBRConfig``, ``config.py:17-199``).

Field names, defaults, ``process_resolution`` (atlas tiling and its error
conventions), ``process_device`` and ``from_config`` follow the reference so
existing configs and env subclasses keep working.  The Panda3D-only fields
(``panda3d_backend``, ``extra_prc_file_data``, ``cuda_gl_interop``, ...) are
accepted and ignored.  New fields at the end select the GB300 renderer's
raster method/mode and launch tuning.
"""
from __future__ import annotations

import logging
import math
import os
from dataclasses import asdict, dataclass
from typing import TypeVar

import torch

T = TypeVar("T", bound="PBRConfig")

SOFT_SIGMA_DEFAULT = 0.5 / (2.0 * math.log(9.0))  # 10%-90% edge transition of 0.5 px


@dataclass
class PBRConfig:
    offscreen: bool = True

    num_scenes: int | None = None
    tiles: tuple[int, int] | int | None = None
    tile_resolution: tuple[int, int] | None = None
    window_resolution: tuple[int, int] | None = None

    num_channels: int = 3
    batch_inner_dim: int | None = None

    clip_camera: tuple[float, float] = (3.0, 500.0)
    min_objects: int = 50
    max_objects: int = 100
    device: str | None = None
    panda3d_backend: str | None = 'arm'
    log_level: int = logging.DEBUG
    extra_prc_file_data: str = (
        'audio-library-name null\n'
        'textures-power-2 none\n'
        'sync-video 0\n'
    )

    render_mode: str = 'rgb_array'
    dt: float = 1 / 60
    warmup_steps: int = 5

    report_fps: bool = True
    report_fps_interval: float = 1.0

    manual_camera_control: bool = False
    cuda_gl_interop: bool = True

    interactive: bool = False

    # TorchRL env-related
    direct_obs_dim: int | None = None
    action_n: int | None = None
    action_type: str = 'discrete'
    max_steps: int = 500
    auto_reset: bool = True

    num_workers: int = 1

    # ---- GB300 renderer (no reference counterpart) ----
    raster_method: str = 'batched'   # 'batched' (one fused launch) | 'plain' (per-node launches, host-built matrices)
    raster_mode: str = 'hard'        # 'hard' (uint8 pixels) | 'soft' (float32, differentiable)
    raster_kernel: str = 'auto'      # 'auto' | 'warp' (scene per warp, small scenes) | 'tile' (CTA per region)
                                     # | 'binned' (soft mode: global per-block candidate masks, large scenes)
    raster_threads: int = 256        # threads per CTA: 128 | 256 | 512 (warp kernel: 128 | 224 | 448)
    bin_size: int = 16               # binner tile size in pixels: 8 | 16 | 32
    tri_cap: int = 0                 # triangles per shared-memory chunk (0 = automatic)
    cluster_cull: bool = True        # tile kernel: skip groups of 32 triangles that cannot be drawn (meshes of 128+)
    tile_pretest: str = 'auto'       # tile kernel: coverage-and-depth pre-test of small triangles: 'auto' | 'on' | 'off'
    persistent: bool = False         # persistent work-stealing schedule
    autotune: bool = False           # time the launch configurations at setup_environment()
    cuda_graph: bool = False         # capture _step + render into a CUDA graph on the first step
    return_depth: bool = False       # step() also returns float32 [N,H,W] window depth
    reuse_output: bool = False       # return the same output buffer every step (no allocation)
    soft_sigma: float = SOFT_SIGMA_DEFAULT
    soft_gamma: float = 1e-3

    def process_resolution(self) -> None:
        """Tiles / tile / window resolution bookkeeping (``config.py:61-126``)."""
        if self.tiles is None and self.num_scenes is not None:
            self.tiles = self.num_scenes

        if isinstance(self.tiles, int):
            cols = math.ceil(math.sqrt(self.tiles))
            rows = math.ceil(self.tiles / cols)
            self.tiles = (cols, rows)

        num_nones = sum(1 for x in [self.tiles, self.tile_resolution, self.window_resolution] if x is None)

        if num_nones == 0:
            if (
                self.window_resolution[0] != self.tiles[0] * self.tile_resolution[0]
                or self.window_resolution[1] != self.tiles[1] * self.tile_resolution[1]
            ):
                raise ValueError(
                    "window_resolution must equal tiles * tile_resolution. "
                    f"Got window_resolution={self.window_resolution}, tiles={self.tiles}, "
                    f"tile_resolution={self.tile_resolution}."
                )
        elif num_nones > 1:
            default_tiles = (1, 1)
            default_tile_resolution = (64, 64)
            if self.tiles is not None:
                self.tile_resolution = default_tile_resolution
                self.window_resolution = (64 * self.tiles[0], 64 * self.tiles[1])
            elif self.tile_resolution is not None:
                self.tiles = default_tiles
                self.window_resolution = (self.tile_resolution[0], self.tile_resolution[1])
            elif self.window_resolution is not None:
                self.tiles = default_tiles
                self.tile_resolution = (self.window_resolution[0], self.window_resolution[1])
            else:
                self.tiles = default_tiles
                self.tile_resolution = default_tile_resolution
                self.window_resolution = (default_tile_resolution[0] * default_tiles[0],
                                          default_tile_resolution[1] * default_tiles[1])
        else:
            if self.tiles is None:
                self.tiles = (
                    self.window_resolution[0] // self.tile_resolution[0],
                    self.window_resolution[1] // self.tile_resolution[1],
                )
            elif self.tile_resolution is None:
                self.tile_resolution = (
                    self.window_resolution[0] // self.tiles[0],
                    self.window_resolution[1] // self.tiles[1],
                )
            elif self.window_resolution is None:
                self.window_resolution = (
                    self.tiles[0] * self.tile_resolution[0],
                    self.tiles[1] * self.tile_resolution[1],
                )

        if self.num_scenes is None:
            self.num_scenes = self.tiles[0] * self.tiles[1]
        elif self.num_scenes > self.tiles[0] * self.tiles[1]:
            raise ValueError(f'{self.num_scenes=} can\'t fit into {self.tiles=}')

        if self.batch_inner_dim is None:
            self.batch_inner_dim = self.tiles[0] * self.tiles[1]
        elif self.batch_inner_dim != self.tiles[0] * self.tiles[1]:
            raise ValueError("batch_inner_dim must equal tiles[0] * tiles[1]")

    def process_device(self) -> None:
        """Device selection and validation (``config.py:128-145``)."""
        if self.device is not None and self.device not in ['cpu', 'cuda', 'mps']:
            raise ValueError(f"Invalid device: {self.device}")
        if self.device is None:
            self.device = 'cuda' if torch.cuda.is_available() else 'cpu'
        if self.device == 'cuda' and not torch.cuda.is_available():
            raise RuntimeError("device is set to CUDA but CUDA is not available")
        elif self.device == 'mps' and not torch.backends.mps.is_available():
            raise RuntimeError("device is set to MPS but MPS is not available")

    def process_renderer(self) -> None:
        if self.raster_method not in ('batched', 'plain'):
            raise ValueError(f"raster_method must be 'batched' or 'plain', got {self.raster_method!r}")
        if self.raster_mode not in ('hard', 'soft'):
            raise ValueError(f"raster_mode must be 'hard' or 'soft', got {self.raster_mode!r}")
        if self.tile_pretest not in ('auto', 'on', 'off'):
            raise ValueError(f"tile_pretest must be 'auto', 'on' or 'off', got {self.tile_pretest!r}")
        if self.raster_kernel not in ('auto', 'warp', 'tile', 'binned'):
            raise ValueError("raster_kernel must be 'auto', 'warp', 'tile' or 'binned'")
        if self.raster_threads not in (128, 256, 512) and not (self.raster_kernel == 'warp'
                                                               and self.raster_threads in (224, 448)):
            raise ValueError("raster_threads must be 128, 256 or 512 (224 or 448 with raster_kernel='warp')")
        if self.bin_size not in (8, 16, 32):
            raise ValueError("bin_size must be 8, 16 or 32")
        if not 1 <= int(self.num_channels) <= 4:
            raise ValueError("num_channels must be between 1 and 4")

    def __post_init__(self) -> None:
        if isinstance(self.tiles, list):
            self.tiles = tuple(self.tiles)
        if isinstance(self.tile_resolution, list):
            self.tile_resolution = tuple(self.tile_resolution)
        if isinstance(self.window_resolution, list):
            self.window_resolution = tuple(self.window_resolution)
        self.process_resolution()
        self.process_device()
        self.process_renderer()

    @classmethod
    def from_config(cls: type[T], cfg: T | dict | None = None, **overrides) -> T:
        """Build a config from an instance or dict plus keyword overrides
        (``config.py:152-174``); an instance keeps its subclass."""
        if isinstance(cfg, cls):
            cfg_dict = asdict(cfg)
            cls = cfg.__class__
        elif isinstance(cfg, PBRConfig):
            cfg_dict = asdict(cfg)
            cls = cfg.__class__
        elif isinstance(cfg, dict):
            cfg_dict = dict(cfg)
        else:
            cfg_dict = {}
        if overrides:
            cfg_dict.update(overrides)
        return cls(**cfg_dict)

    def build_prc(self) -> str:
        """Panda3D PRC text the reference feeds to ``loadPrcFileData``
        (``config.py:176-191``).  Nothing here consumes it; kept so code that
        inspects it keeps working."""
        if self.window_resolution is None:
            self.process_resolution()
        prc = [f"window-type {'offscreen' if self.offscreen else 'onscreen'}\n",
               f"win-size {self.window_resolution[0]} {self.window_resolution[1]}\n"]
        if self.panda3d_backend == 'arm':
            prc.append('gl-version 3 2\n')
        else:
            os.environ.setdefault("PYOPENGL_PLATFORM", "egl")
            prc.append('threading-model Cull/Draw\n')
        prc.append(self.extra_prc_file_data)
        return ''.join(prc)

    def __repr__(self):
        repr_string = "PBRConfig(\n"
        for key, value in asdict(self).items():
            repr_string += f"    {key}: {value!r}\n"
        repr_string += ")"
        return repr_string
