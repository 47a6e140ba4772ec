"""Environment registry (``pybatchrender/envs/__init__.py``).

Gym-style factory: ``register``, ``unregister``, ``list_envs``,
``is_registered``, ``get_env_classes``, ``make``, ``make_parallel``.  Built-ins:
``CartPole-v0``.  Third-party packages register through the entry-point group
``pybatchrender.envs`` (the reference's group, ``pyproject.toml:73-79``) or
``pybatchrender_gb300.envs``.  Unlike the reference there is no one-renderer-
per-process limit: renderers are independent CUDA contexts.
"""
from __future__ import annotations

import warnings
from typing import Dict, Tuple, Type

_ENV_REGISTRY: Dict[str, Tuple[type, type, type]] = {}

ENTRY_POINT_GROUPS = ("pybatchrender.envs", "pybatchrender_gb300.envs")


def register(name: str, env_cls: Type, renderer_cls: Type, config_cls: Type) -> None:
    if name in _ENV_REGISTRY:
        warnings.warn(f"Environment '{name}' is already registered. Overwriting.")
    _ENV_REGISTRY[name] = (env_cls, renderer_cls, config_cls)


def unregister(name: str) -> None:
    _ENV_REGISTRY.pop(name, None)


def list_envs() -> list[str]:
    return sorted(_ENV_REGISTRY.keys())


def is_registered(name: str) -> bool:
    return name in _ENV_REGISTRY


def get_env_classes(name: str) -> Tuple[type, type, type]:
    if name not in _ENV_REGISTRY:
        raise ValueError(f"Unknown environment: '{name}'. Available: {list_envs()}")
    return _ENV_REGISTRY[name]


def make(name: str, **config_overrides):
    """``config_cls(**overrides)`` -> ``renderer_cls(cfg)`` -> ``env_cls(renderer, cfg)``."""
    if name not in _ENV_REGISTRY:
        raise ValueError(f"Unknown environment: '{name}'. Available: {list_envs()}")
    env_cls, renderer_cls, config_cls = _ENV_REGISTRY[name]
    cfg = config_cls(**config_overrides)
    renderer = renderer_cls(cfg)
    return env_cls(renderer=renderer, cfg=cfg)


def make_parallel(name: str, num_workers: int, shared_memory: bool = True, devices=None, **config_overrides):
    """``num_workers`` spawned replicas of env ``name``, each with its own
    renderer, as one env of batch ``[num_workers, num_scenes]``
    (``envs/__init__.py:127-164``): TorchRL's ``ParallelEnv`` when TorchRL is
    installed, else the process-replica stand-in of ``parallel_env``.
    ``devices``: optional device per worker (see ``PBREnv.make_parallel_env``)."""
    if name not in _ENV_REGISTRY:
        raise ValueError(f"Unknown environment: '{name}'. Available: {list_envs()}")
    env_cls, renderer_cls, config_cls = _ENV_REGISTRY[name]
    cfg = config_cls(**config_overrides)
    return env_cls.make_parallel_env(config=cfg, renderer_cls=renderer_cls, num_workers=num_workers,
                                     mp_start_method="spawn", shared_memory=shared_memory, devices=devices)


def _register_builtins() -> None:
    from .cartpole import CartPoleConfig, CartPoleEnv, CartPoleRenderer
    register("CartPole-v0", CartPoleEnv, CartPoleRenderer, CartPoleConfig)
    from .steering import SteeringConfig, SteeringEnv, SteeringRenderer
    register("Steering-v0", SteeringEnv, SteeringRenderer, SteeringConfig)


def _register_from_entry_points() -> None:
    try:
        from importlib.metadata import entry_points
    except ImportError:  # pragma: no cover
        return
    for group in ENTRY_POINT_GROUPS:
        try:
            eps = entry_points(group=group)
        except TypeError:  # pragma: no cover
            eps = entry_points().get(group, [])
        for ep in eps:
            try:
                fn = ep.load()
                if callable(fn):
                    fn()
            except Exception as e:  # pragma: no cover
                warnings.warn(f"Failed to load environment entry point '{ep.name}': {e}")


_register_builtins()
_register_from_entry_points()

__all__ = ["register", "unregister", "list_envs", "is_registered", "get_env_classes", "make", "make_parallel"]
