"""Template environment configuration (``envs/_template/config.py``)."""
from dataclasses import dataclass

from ...config import PBRConfig


@dataclass
class MyEnvConfig(PBRConfig):
    """Environment parameters on top of every ``PBRConfig`` field."""

    # TorchRL env defaults
    direct_obs_dim: int | None = 2      # observation: (x, x_dot)
    action_n: int | None = 2            # discrete: push left / push right
    action_type: str = "discrete"
    max_steps: int = 200
    auto_reset: bool = True

    # rendering defaults
    num_channels: int = 3
    tile_resolution: tuple[int, int] | None = (64, 64)
    offscreen: bool = True
    report_fps: bool = False

    # dynamics
    push: float = 0.5                   # velocity change per step
    dt: float = 0.05
    limit: float = 3.0
    init_x_range: tuple[float, float] = (-0.5, 0.5)

    seed: int = 0
    render: bool = True

    # parallel env controls
    worker_index: int = 0
    num_workers: int = 1
