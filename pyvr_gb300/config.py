"""Render quality settings for the CUDA ray marcher.

Mirrors pyvr's ``RenderConfig`` (pyvr/config.py:11-368): same fields, same
validation, same five presets.  Only ``step_size``, ``max_steps`` and
``reference_step_size`` reach the marcher, exactly as in the reference
renderer (pyvr/moderngl_renderer/renderer.py:303-309); the early-termination
fields are carried for API compatibility but the march always stops at an
accumulated alpha of 0.99 (pyvr/shaders/volume.frag.glsl:87).
"""

from __future__ import annotations

import warnings
from dataclasses import dataclass, replace


@dataclass
class RenderConfig:
    step_size: float = 0.01
    max_steps: int = 500
    early_ray_termination: bool = True
    opacity_threshold: float = 0.95
    reference_step_size: float = 0.01

    def __post_init__(self):
        self.validate()

    def validate(self) -> None:
        """Field checks of pyvr/config.py:64-94 (errors and warnings alike)."""
        if self.step_size <= 0:
            raise ValueError("step_size must be positive")
        if self.step_size > 1.0:
            warnings.warn(f"step_size {self.step_size} is very large and may produce poor quality",
                          UserWarning)
        if self.max_steps < 1:
            raise ValueError("max_steps must be at least 1")
        if self.max_steps > 10000:
            warnings.warn(f"max_steps {self.max_steps} is very large and may be slow", UserWarning)
        if not (0.0 <= self.opacity_threshold <= 1.0):
            raise ValueError("opacity_threshold must be between 0.0 and 1.0")

    # Presets: pyvr/config.py:96-227.  (step, max_steps, ert, threshold)
    @classmethod
    def preview(cls) -> "RenderConfig":
        return cls(0.05, 50, True, 0.80)

    @classmethod
    def fast(cls) -> "RenderConfig":
        return cls(0.02, 100, True, 0.90)

    @classmethod
    def balanced(cls) -> "RenderConfig":
        return cls(0.01, 500, True, 0.95)

    @classmethod
    def high_quality(cls) -> "RenderConfig":
        return cls(0.005, 1000, True, 0.98)

    @classmethod
    def ultra_quality(cls) -> "RenderConfig":
        return cls(0.001, 2000, False, 1.0)

    @classmethod
    def custom(cls, step_size: float, max_steps: int, early_ray_termination: bool = True,
               opacity_threshold: float = 0.95) -> "RenderConfig":
        # Like pyvr/config.py:229-261, reference_step_size is not a parameter
        # here and keeps its default.
        return cls(step_size=step_size, max_steps=max_steps,
                   early_ray_termination=early_ray_termination,
                   opacity_threshold=opacity_threshold)

    def copy(self) -> "RenderConfig":
        return replace(self)

    def with_step_size(self, step_size: float) -> "RenderConfig":
        cfg = self.copy()
        cfg.step_size = step_size
        cfg.validate()
        return cfg

    def with_max_steps(self, max_steps: int) -> "RenderConfig":
        cfg = self.copy()
        cfg.max_steps = max_steps
        cfg.validate()
        return cfg

    def estimate_samples_per_ray(self) -> int:
        """Unit-cube diagonal / step, capped at max_steps (pyvr/config.py:319-336)."""
        return min(int(1.732 / self.step_size), self.max_steps)

    def estimate_render_time_relative(self) -> float:
        return self.estimate_samples_per_ray() / RenderConfig.balanced().estimate_samples_per_ray()

    def __repr__(self) -> str:
        return (f"RenderConfig(step_size={self.step_size}, max_steps={self.max_steps}, "
                f"early_termination={self.early_ray_termination}, "
                f"~{self.estimate_samples_per_ray()} samples/ray)")


class RenderConfigError(Exception):
    pass
