"""Steering configuration (``envs/steering/config.py:10-111``): the
reference's fields and defaults.  Two model defaults differ because the
reference's files are not part of this package: the obstacle sphere is the
built-in ``"models/smiley"`` stand-in (an untextured icosphere; Panda3D's
bundled smiley is a textured sphere) and the lane rails are the procedural
``"models/cylinder"`` (the reference loads ``models/cylinder/scene.gltf``,
which ``add_node`` can still load from a file path)."""
from dataclasses import dataclass, field

from ...config import PBRConfig


@dataclass
class SteeringConfig(PBRConfig):
    # TorchRL env defaults
    direct_obs_dim: int = 6  # player x, player y, speed, grace active, next obstacle x, next obstacle y
    action_n: int = 1
    action_type: str = "continuous"
    action_low: float = -327.68
    action_high: float = 327.68
    max_steps: int = 10000
    auto_reset: bool = True

    # Rendering defaults
    num_channels: int = 3
    tile_resolution: tuple[int, int] = (64, 64)
    offscreen: bool = True
    report_fps: bool = False

    # Camera
    fov_y_deg: float = 40.0
    z_near: float = 0.5
    z_far: float = 1000.0
    camera_eye_offset: tuple[float, float, float] = (0.0, -16.3, 4.0)
    camera_forward_vector: tuple[float, float, float] = (0.0, 1.0, 0.0)

    # Lighting
    ambient_light: tuple[float, float, float] = (0.2, 0.2, 0.2)
    directional_light_dir: tuple[float, float, float] = (0.22, 0.44, 0.88)
    directional_light_color: tuple[float, float, float] = (0.8, 0.8, 0.8)

    # Colours
    red_obstacle_color: tuple[float, float, float, float] = (1.0, 0.0, 0.0, 1.0)
    gold_obstacle_color: tuple[float, float, float, float] = (1.0, 0.5, 0.0, 1.0)
    player_color: tuple[float, float, float, float] = (0.0, 0.0, 1.0, 1.0)
    edge_color: tuple[float, float, float, float] = (0.2, 0.2, 0.2, 1.0)
    background_color: tuple[float, float, float, float] = (0.0, 0.0, 0.0, 1.0)
    crash_player_color: tuple[float, float, float, float] = (0.4, 0.4, 0.4, 1.0)

    # Models
    player_model: str = "models/box"
    obstacle_sphere_model: str = "models/smiley"
    obstacle_cone_model: str = "models/cone.egg"
    border_model: str = "models/cylinder/scene.gltf"

    # Scene layout
    lane_width: float = 25.0
    obstacle_dimensions: tuple[float, float, float] = (2.0, 2.0, 2.0)
    player_dimensions: tuple[float, float, float] = (2.0, 2.0, 2.0)
    rail_dimensions: tuple[float, float, float] = (0.2, 1012.0, 0.2)
    rail_offset: tuple[float, float, float] = (0.0, -12.0, 0.5)
    track_length: float = 1000.0

    player_pivot_relative_point: tuple[float, float, float] = (0.5, 0.5, 0.5)
    obstacle_pivot_relative_point: tuple[float, float, float] = (0.5, 0.5, 0.5)
    rail_pivot_relative_point: tuple[float, float, float] = (0.5, 0.5, 0.0)
    player_model_hpr: tuple[float, float, float] = (0.0, 0.0, 0.0)
    obstacle_model_hpr: tuple[float, float, float] = (0.0, 0.0, 0.0)
    border_model_hpr: tuple[float, float, float] = (0.0, 0.0, 0.0)

    # Obstacle generation
    obstacle_seed: int | None = None
    prob_gold: float = 0.2
    prob_cone: float = 0.5
    distance_to_first_obstacle: float = 6
    number_of_obstacles: int = 100
    obstacle_y_spacing: float = 12.0
    obstacle_x_position: list[int] = field(default_factory=lambda: list(range(-11, 12, 2)))

    # Physics
    speed_initial: float = 96.0
    minimal_speed: float = 18.0
    speed_increment: float = 0.072
    speed_decrement: float = 6.12
    grace_period: float = 100.0 / 60.0
    steering_speed: float = 20.0

    # RL
    tau: float = 1.0 / 60.0
    wheel_sensitivity: float = 800.0
    collision_penalty: float = -1.0
    terminate_on_collision: bool = False
    terminate_on_track_end: bool = True

    # Saving / debug
    seed: int = 0
    render: bool = True
    save_every_steps: int = -1
    save_examples_num: int = 16
    save_out_dir: str | None = None

    # Parallel env controls
    worker_index: int = 0
    num_workers: int = 1
