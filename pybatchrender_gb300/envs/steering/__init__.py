"""Steering-v0: config, renderer and environment (``envs/steering``)."""
from .config import SteeringConfig
from .env import SteeringEnv
from .renderer import SteeringRenderer

__all__ = ["SteeringConfig", "SteeringEnv", "SteeringRenderer"]
