"""Light source description, mirroring pyvr's ``Light`` (pyvr/lighting/light.py:14-425).

The marcher only consumes four values of it (pyvr/moderngl_renderer/renderer.py:311-316):
``ambient_intensity``, ``diffuse_intensity``, ``position`` and ``target``; the
shading direction is ``normalize(target - position)`` (pyvr/shaders/volume.frag.glsl:107).
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np


def _vec3(values) -> np.ndarray:
    return np.array(values, dtype=np.float32)


class LightError(Exception):
    pass


@dataclass
class Light:
    position: np.ndarray = field(default_factory=lambda: _vec3([1.0, 1.0, 1.0]))
    target: np.ndarray = field(default_factory=lambda: _vec3([0.0, 0.0, 0.0]))
    ambient_intensity: float = 0.2
    diffuse_intensity: float = 0.8
    _is_linked: bool = field(default=False, init=False, repr=False)
    _camera_offsets: Optional[dict] = field(default=None, init=False, repr=False)

    def __post_init__(self):
        self.validate()

    def validate(self) -> None:
        for name in ("position", "target"):
            vec = getattr(self, name)
            if not isinstance(vec, np.ndarray) or vec.shape != (3,):
                raise ValueError(f"{name} must be a 3D numpy array")
        if not (0.0 <= self.ambient_intensity <= 1.0):
            raise ValueError("ambient_intensity must be between 0.0 and 1.0")
        if not (0.0 <= self.diffuse_intensity <= 1.0):
            raise ValueError("diffuse_intensity must be between 0.0 and 1.0")

    @classmethod
    def directional(cls, direction, ambient: float = 0.2, diffuse: float = 0.8,
                    distance: float = 10.0) -> "Light":
        """Light placed ``distance`` back along the unit direction, aimed at the
        origin (pyvr/lighting/light.py:68-110)."""
        d = np.array(direction, dtype=np.float32)
        d = d / np.linalg.norm(d)
        return cls(position=-d * distance, target=_vec3([0.0, 0.0, 0.0]),
                   ambient_intensity=ambient, diffuse_intensity=diffuse)

    @classmethod
    def point_light(cls, position, target=None, ambient: float = 0.2,
                    diffuse: float = 0.8) -> "Light":
        tgt = _vec3([0.0, 0.0, 0.0]) if target is None else np.array(target, dtype=np.float32)
        return cls(position=np.array(position, dtype=np.float32), target=tgt,
                   ambient_intensity=ambient, diffuse_intensity=diffuse)

    @classmethod
    def default(cls) -> "Light":
        return cls()

    @classmethod
    def ambient_only(cls, intensity: float = 0.5) -> "Light":
        return cls(position=_vec3([0.0, 0.0, 0.0]), target=_vec3([0.0, 0.0, 0.0]),
                   ambient_intensity=intensity, diffuse_intensity=0.0)

    @classmethod
    def camera_linked(cls, azimuth_offset: float = 0.0, elevation_offset: float = 0.0,
                      distance_offset: float = 0.0, ambient: float = 0.2,
                      diffuse: float = 0.8) -> "Light":
        light = cls(ambient_intensity=ambient, diffuse_intensity=diffuse)
        return light.link_to_camera(azimuth_offset, elevation_offset, distance_offset)

    def get_direction(self) -> np.ndarray:
        d = self.target - self.position
        n = np.linalg.norm(d)
        if n < 1e-9:
            return _vec3([0.0, 0.0, -1.0])
        return d / n

    def copy(self) -> "Light":
        out = Light(position=self.position.copy(), target=self.target.copy(),
                    ambient_intensity=self.ambient_intensity,
                    diffuse_intensity=self.diffuse_intensity)
        out._is_linked = self._is_linked
        out._camera_offsets = None if self._camera_offsets is None else dict(self._camera_offsets)
        return out

    # -- headlight mode (pyvr/lighting/light.py:274-401) ----------------------
    @property
    def is_linked(self) -> bool:
        return self._is_linked

    def link_to_camera(self, azimuth_offset: float = 0.0, elevation_offset: float = 0.0,
                       distance_offset: float = 0.0) -> "Light":
        self._is_linked = True
        self._camera_offsets = {"azimuth": azimuth_offset, "elevation": elevation_offset,
                                "distance": distance_offset}
        return self

    def unlink_from_camera(self) -> "Light":
        self._is_linked = False
        self._camera_offsets = None
        return self

    def update_from_camera(self, camera) -> None:
        """Headlight: the light sits at the camera and points at its target."""
        if not self._is_linked or self._camera_offsets is None:
            raise ValueError("Light is not linked to camera. Call link_to_camera() first.")
        if not hasattr(camera, "get_camera_vectors"):
            raise ValueError("camera must be a Camera instance")
        pos, _ = camera.get_camera_vectors()
        self.position = np.array(pos).copy()
        self.target = np.array(camera.target).copy()

    def get_offsets(self) -> Optional[dict]:
        return dict(self._camera_offsets) if self._camera_offsets else None

    def __repr__(self) -> str:
        return (f"Light(position={self.position}, target={self.target}, "
                f"ambient={self.ambient_intensity:.2f}, diffuse={self.diffuse_intensity:.2f})")
