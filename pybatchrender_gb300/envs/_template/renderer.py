"""Template environment renderer (``envs/_template/renderer.py``): one box
per scene whose x follows state column 0, a camera and a light."""
import torch

from ...config import PBRConfig
from ...renderer.renderer import PBRRenderer


class MyEnvRenderer(PBRRenderer):
    def __init__(self, cfg: PBRConfig | dict | None = None):
        super().__init__(cfg)
        n = int(self.cfg.num_scenes)
        # scene nodes: shared_across_scenes=True for geometry that is the same in every scene
        self.box = self.add_node("models/box", model_pivot_relative_point=(0.5, 0.5, 0.5),
                                 model_scale=(0.6, 0.6, 0.6), instances_per_scene=1, shared_across_scenes=False)
        self.box.set_colors(torch.tensor([0.3, 0.7, 1.0, 1.0]).repeat(n, 1))
        self.add_camera(fov_y_deg=45.0)
        self._pbr_cam.set_positions_and_lookat(torch.tensor([0.0, -9.0, 2.0]), torch.tensor([0.0, 0.0, 0.0]))
        self.add_light()
        # optional: read box x from state column 0 inside the raster launch (no copy kernel per step)
        self.bind_state(self.box, "x", 0)
        # required: the last call of __init__
        self.setup_environment()

    def _step(self, state_batch: torch.Tensor | None = None):
        """Write the state into the node buffers (used when the state cannot
        be bound, e.g. on the CPU): state [B, obs_dim], column 0 = x."""
        if state_batch is None:
            return
        s = torch.as_tensor(state_batch, dtype=torch.float32).to(self.state_device)
        self.box.pos[: s.shape[0], 0].copy_(s[:, 0])
