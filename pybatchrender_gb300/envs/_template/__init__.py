"""Template environment: a working starting point for a new environment
(``envs/_template/`` in the reference).

Copy this directory, rename the classes (``MyEnv`` -> ``PendulumEnv`` ...),
replace the toy dynamics, and register the result::

    from pybatchrender_gb300.envs import register
    register("Pendulum-v0", PendulumEnv, PendulumRenderer, PendulumConfig)

The toy task: a box slides along x; actions push it left or right; an
episode ends when it leaves [-limit, limit] or after ``max_steps``.
"""
from .config import MyEnvConfig
from .env import MyEnv
from .renderer import MyEnvRenderer

__all__ = ["MyEnvConfig", "MyEnvRenderer", "MyEnv"]
