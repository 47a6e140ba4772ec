"""``PBREnv``: TorchRL environment base over a ``PBRRenderer`` (``pybatchrender/env.py``).

When TorchRL and tensordict are installed ``PBREnv`` subclasses
``torchrl.envs.EnvBase`` and uses its specs, exactly like the reference
(``env.py:18-95,360-440``).  Without them (neither package is part of this
project's environments) a small stand-in with the same ``reset`` / ``step``
contract is used: tensordicts become :class:`TensorDictLite`, a dict keyed by
strings or nested tuples with a ``batch_size``.
"""
from __future__ import annotations

from abc import abstractmethod

import torch

from .config import PBRConfig

try:  # pragma: no cover - depends on the environment
    from tensordict import TensorDict as _TensorDict
    from torchrl.data.tensor_specs import Categorical, Composite, Unbounded
    from torchrl.envs import EnvBase as _EnvBase
    from torchrl.envs import ParallelEnv as _ParallelEnv
    HAVE_TORCHRL = True
except Exception:
    HAVE_TORCHRL = False
    _TensorDict = None
    _ParallelEnv = None


class TensorDictLite(dict):
    """Minimal tensordict stand-in: string or nested-tuple keys, ``batch_size``."""

    def __init__(self, fields=None, batch_size=None):
        super().__init__()
        self.batch_size = torch.Size(batch_size or [])
        for k, v in (fields or {}).items():
            self[k] = v

    def __getitem__(self, key):
        if isinstance(key, tuple):
            cur = self
            for k in key:
                cur = dict.__getitem__(cur, k)
            return cur
        return dict.__getitem__(self, key)

    def __setitem__(self, key, value):
        if isinstance(key, tuple):
            cur = self
            for k in key[:-1]:
                if k not in cur:
                    dict.__setitem__(cur, k, TensorDictLite(batch_size=self.batch_size))
                cur = dict.__getitem__(cur, k)
            dict.__setitem__(cur, key[-1], value)
        else:
            dict.__setitem__(self, key, value)

    def get(self, key, default=None):
        try:
            return self[key]
        except KeyError:
            return default

    def keys(self, include_nested: bool = False):
        return list(dict.keys(self))

    def clone(self) -> "TensorDictLite":
        out = TensorDictLite(batch_size=self.batch_size)
        for k, v in dict.items(self):
            dict.__setitem__(out, k, v.clone() if hasattr(v, "clone") else v)
        return out


def TensorDict(fields, batch_size=None):  # noqa: N802 - mirrors the tensordict constructor
    if HAVE_TORCHRL:
        return _TensorDict(fields, batch_size=batch_size)
    return TensorDictLite(fields, batch_size=batch_size)


class _SpecLite:
    def __init__(self, shape, dtype, device, n=None, low=None, high=None):
        self.shape, self.dtype, self.device, self.n = torch.Size(shape), dtype, device, n
        self.low, self.high = low, high

    def rand(self):
        if self.n is not None:
            return torch.randint(0, self.n, self.shape, dtype=self.dtype, device=self.device)
        if self.low is not None:
            return torch.empty(self.shape, dtype=self.dtype, device=self.device).uniform_(self.low, self.high)
        return torch.randn(self.shape, dtype=self.dtype, device=self.device)

    def zero(self):
        return torch.zeros(self.shape, dtype=self.dtype, device=self.device)


class _EnvBaseLite:
    """The slice of ``torchrl.envs.EnvBase`` the PBR envs use."""

    def __init__(self, device="cpu", batch_size=torch.Size([]), **kwargs):
        self.device = torch.device(device)
        self.batch_size = torch.Size(batch_size)

    def reset(self, tensordict=None):
        return self._reset(tensordict)

    def step(self, tensordict):
        nxt = self._step(tensordict)
        tensordict["next"] = nxt
        return tensordict

    def rand_action(self, tensordict=None):
        td = tensordict if tensordict is not None else TensorDict({}, batch_size=self.batch_size)
        td["action"] = self.action_spec.rand()
        return td

    def set_seed(self, seed: int, static_seed: bool = False):
        self._set_seed(seed)
        return seed


_Base = _EnvBase if HAVE_TORCHRL else _EnvBaseLite


class PBREnv(_Base):
    """Environment base: owns a renderer and renders pixels per step."""

    def __init__(self, renderer, cfg: PBRConfig | None = None, device: str | torch.device = "cpu",
                 batch_size: torch.Size = torch.Size([128]), **kwargs) -> None:
        super().__init__(device=torch.device(device), batch_size=batch_size, **kwargs)
        self._renderer = renderer
        self.cfg = cfg if cfg is not None else renderer.cfg

    def set_default_specs(self, *, direct_obs_dim: int | None = None, actions: int | None = None,
                          with_pixels: bool = False, pixels_only: bool = False,
                          discrete_actions: bool = True, action_low: float | None = None,
                          action_high: float | None = None) -> None:
        """Observation / action / reward / done specs (``env.py:33-82``);
        continuous actions are bounded when ``action_low`` / ``action_high``
        are given (``envs/steering/env.py:142-156``)."""
        assert with_pixels or not pixels_only, "Cannot set both with_pixels and pixels_only to True."
        bs = self.batch_size if self.batch_size != torch.Size([]) else torch.Size([1])
        C = int(self.cfg.num_channels)
        W, H = int(self.cfg.tile_resolution[0]), int(self.cfg.tile_resolution[1])
        if not pixels_only and direct_obs_dim is None:
            raise ValueError("direct_obs_dim must be provided when pixels_only=False.")
        if actions is None:
            raise ValueError("actions must be provided.")
        if HAVE_TORCHRL:  # pragma: no cover
            fields = {}
            if with_pixels:
                fields["pixels"] = Unbounded(shape=bs + torch.Size([C, H, W]), dtype=torch.uint8, device=self.device)
            if not pixels_only:
                fields["observation"] = Unbounded(shape=bs + torch.Size([int(direct_obs_dim)]), dtype=torch.float32,
                                                  device=self.device)
            self.observation_spec = Composite(**fields, shape=bs)
            if discrete_actions:
                self.action_spec = Categorical(n=int(actions), shape=bs, dtype=torch.long, device=self.device)
            elif action_low is not None:
                from torchrl.data.tensor_specs import Bounded
                self.action_spec = Bounded(low=float(action_low), high=float(action_high),
                                           shape=bs + torch.Size([int(actions)]), dtype=torch.float32,
                                           device=self.device)
            else:
                self.action_spec = Unbounded(shape=bs + torch.Size([int(actions)]), dtype=torch.float32,
                                             device=self.device)
            self.reward_spec = Unbounded(shape=bs + torch.Size([1]), dtype=torch.float32, device=self.device)
            self.done_spec = Unbounded(shape=bs + torch.Size([1]), dtype=torch.bool, device=self.device)
            return
        self.observation_spec = {}
        if with_pixels:
            self.observation_spec["pixels"] = _SpecLite(bs + torch.Size([C, H, W]), torch.uint8, self.device)
        if not pixels_only:
            self.observation_spec["observation"] = _SpecLite(bs + torch.Size([int(direct_obs_dim)]), torch.float32,
                                                             self.device)
        if discrete_actions:
            self.action_spec = _SpecLite(bs, torch.long, self.device, n=int(actions))
        else:
            self.action_spec = _SpecLite(bs + torch.Size([int(actions)]), torch.float32, self.device,
                                         low=None if action_low is None else float(action_low),
                                         high=None if action_high is None else float(action_high))
        self.reward_spec = _SpecLite(bs + torch.Size([1]), torch.float32, self.device)
        self.done_spec = _SpecLite(bs + torch.Size([1]), torch.bool, self.device)

    @abstractmethod
    def _step(self, tensordict):
        pass

    @abstractmethod
    def _reset(self, tensordict=None):
        pass

    def render_pixels(self, obs: torch.Tensor | None = None) -> torch.Tensor:
        """Render ``obs`` through the renderer (``env.py:92-95``)."""
        if self._renderer is None:
            raise RuntimeError("Renderer is not initialized. Construct env with a renderer and pass it to PBREnv.")
        return self._renderer.step(obs)

    # ------------------------------------------------------------ snapshots
    def _is_secondary_worker(self) -> bool:
        return int(getattr(self.cfg, "num_workers", 1) or 1) > 1 and int(getattr(self.cfg, "worker_index", 0) or 0) != 0

    @staticmethod
    def _snapshot_path(out_dir: str | None, prefix: str, ext: str):
        import random
        import time
        from pathlib import Path
        out = Path(out_dir) if out_dir is not None else Path(".")
        out.mkdir(parents=True, exist_ok=True)
        name = f"{prefix}_{time.strftime('%Y%m%d_%H%M%S')}_{random.randint(0, 999999):06d}.{ext}"
        return (out / name).resolve()

    def _make_grid_frame(self, pixels: torch.Tensor, indices: list[int] | None = None, num: int = 16,
                         scale: int = 1):
        """Grid image of the batch (``env.py:186-241``)."""
        from .imagefile import make_grid
        return make_grid(pixels, indices, num, scale)

    def save_batch_examples(self, *, pixels: torch.Tensor | None = None, obs: torch.Tensor | None = None,
                            indices: list[int] | None = None, num: int = 16, scale: int = 1,
                            out_dir: str | None = "./outputs", filename_prefix: str = "batch_example",
                            return_bytes: bool = False):
        """Save one PNG grid of batch elements (``env.py:97-184``); returns the
        path, or ``(path, png_bytes)`` when ``return_bytes``.  Worker processes
        other than worker 0 return None."""
        from .imagefile import encode_png
        if self._is_secondary_worker():
            return None
        if pixels is None:
            pixels = self.render_pixels(obs)
        if pixels is None:
            raise RuntimeError("No pixels available to save.")
        data = encode_png(self._make_grid_frame(pixels, indices, num, scale))
        path = self._snapshot_path(out_dir, filename_prefix, "png")
        path.write_bytes(data)
        return (str(path), data) if return_bytes else str(path)

    def save_batch_gif(self, *, num_steps: int = 100, frame_interval: int = 2, indices: list[int] | None = None,
                       num: int = 16, scale: int = 2, duration_ms: int = 100, out_dir: str | None = "./outputs",
                       filename_prefix: str = "batch_animation", return_bytes: bool = False):
        """Reset, run ``num_steps`` random-action steps and save an animated GIF
        of the batch grid, one frame every ``frame_interval`` steps
        (``env.py:243-358``)."""
        from .imagefile import encode_gif
        if self._is_secondary_worker():
            return None
        frames = []
        td = self._reset()
        pixels = td.get("pixels", None)
        if pixels is None:
            pixels = self.render_pixels(td.get("observation", None))
        if pixels is not None:
            frames.append(self._make_grid_frame(pixels, indices, num, scale))
        for step in range(1, int(num_steps) + 1):
            td["action"] = self.action_spec.rand()
            td = self.step(td)
            td = td["next"]
            if step % int(frame_interval) == 0:
                pixels = td.get("pixels", None)
                if pixels is None:
                    pixels = self.render_pixels(td.get("observation", None))
                if pixels is not None:
                    frames.append(self._make_grid_frame(pixels, indices, num, scale))
        if not frames:
            raise RuntimeError("No frames captured. Ensure rendering is enabled.")
        data = encode_gif(frames, duration_ms=duration_ms, loop=0)
        path = self._snapshot_path(out_dir, filename_prefix, "gif")
        path.write_bytes(data)
        return (str(path), data) if return_bytes else str(path)

    @classmethod
    def make_parallel_env(cls, *, config: PBRConfig, renderer_cls, num_workers: int,
                          mp_start_method: str = "spawn", shared_memory: bool = True, devices=None):
        """``num_workers`` spawned replicas, each with its own renderer
        (``env.py:360-416``): TorchRL's ``ParallelEnv`` when TorchRL is
        installed, else :class:`~pybatchrender_gb300.parallel_env.ParallelEnvLite`
        with the same ``reset`` / ``step`` contract and batch
        ``[num_workers, num_scenes]``.  ``devices`` (no reference counterpart):
        one device per worker, e.g. ``["cuda:0", "cuda:1"]``, to spread the
        replicas over GPUs; by default every worker uses ``config.device``."""
        num_workers = int(num_workers)
        if devices is not None and len(devices) != num_workers:
            raise ValueError("devices needs one entry per worker")
        kwargs = []
        for i in range(num_workers):
            cfg = config if devices is None else PBRConfig.from_config(config, device=str(devices[i]))
            kwargs.append({"env_cls": cls, "renderer_cls": renderer_cls, "config": cfg, "worker_index": i,
                           "num_workers": num_workers})
        if not HAVE_TORCHRL:
            from .parallel_env import ParallelEnvLite
            return ParallelEnvLite(num_workers, create_env_fn=cls._make_env_worker, create_env_kwargs=kwargs,
                                   mp_start_method=mp_start_method, shared_memory=shared_memory)
        import multiprocessing as mp  # pragma: no cover
        try:
            mp.set_start_method(mp_start_method, force=True)
        except RuntimeError:
            pass
        return _ParallelEnv(num_workers, create_env_fn=cls._make_env_worker, shared_memory=shared_memory,
                            mp_start_method=mp_start_method, create_env_kwargs=kwargs)

    @staticmethod
    def _make_env_worker(env_cls, renderer_cls, config: PBRConfig, worker_index: int, num_workers: int):
        """Spawn-safe worker factory (``env.py:418-440``): seed offset by the
        worker index."""
        cfg = PBRConfig.from_config(config, worker_index=worker_index, num_workers=num_workers)
        cfg.worker_index = worker_index
        try:
            if getattr(cfg, "seed", None) is not None:
                cfg.seed = int(cfg.seed) + int(worker_index)
        except Exception:
            pass
        renderer = renderer_cls(cfg)
        return env_cls(renderer=renderer, cfg=cfg)


class GraphedEnvStep:
    """``env._step`` replayed as one CUDA graph: the env's device-side
    dynamics, termination, reward, auto-reset and the render launch it makes
    (for CartPole a single state-bound raster launch) are captured on the
    first call and replayed afterwards, so a step costs one graph launch
    instead of a few dozen kernel launches from Python.

    ``step(tensordict)`` takes ``observation``, ``action`` and optionally
    ``step_count`` and returns the next tensordict of ``_step``.  Its tensors
    are the graph's static outputs: they are overwritten by the next call, so
    copy what must outlive it.  The graph is captured again when the input
    shapes or dtypes change.  Random numbers (auto-reset states) come from
    the CUDA generator through PyTorch's graph-safe RNG."""

    def __init__(self, env: PBREnv, warmup: int = 2):
        self.env = env
        self.warmup = int(warmup)
        self._graph = None
        self._sig = None
        self._static_in: dict = {}
        self._static_out = None

    def _inputs(self, tensordict) -> dict:
        obs = tensordict["observation"]
        ins = {"observation": obs, "action": tensordict["action"]}
        sc = tensordict.get("step_count", None)
        ins["step_count"] = sc if sc is not None else torch.zeros(obs.shape[:-1], dtype=torch.long, device=obs.device)
        return {k: v.to(self.env.device) for k, v in ins.items()}

    def _capture(self, ins: dict) -> None:
        self._static_in = {k: v.detach().clone() for k, v in ins.items()}
        td = TensorDict(dict(self._static_in), batch_size=self.env.batch_size)
        side = torch.cuda.Stream(self.env.device)
        side.wait_stream(torch.cuda.current_stream(self.env.device))
        with torch.cuda.stream(side):
            for _ in range(self.warmup):
                self.env._step(td)
        torch.cuda.current_stream(self.env.device).wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._static_out = self.env._step(td)
        self._graph = g

    def step(self, tensordict):
        ins = self._inputs(tensordict)
        sig = tuple((k, tuple(v.shape), v.dtype) for k, v in sorted(ins.items()))
        if self._graph is None or sig != self._sig:
            self._capture(ins)
            self._sig = sig
        else:
            for k, v in ins.items():
                self._static_in[k].copy_(v, non_blocking=True)
        self._graph.replay()
        return self._static_out

    __call__ = step
