"""CartPole-v0: config, renderer and environment."""
from .config import CartPoleConfig
from .env import CartPoleEnv
from .renderer import CartPoleRenderer

__all__ = ["CartPoleConfig", "CartPoleEnv", "CartPoleRenderer"]
