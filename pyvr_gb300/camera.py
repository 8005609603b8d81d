"""Orbit camera: spherical parameters -> position/up -> GL view/projection.

Mirrors pyvr's ``Camera`` (pyvr/camera/camera.py:16-380) and
``get_camera_pos`` (pyvr/camera/control.py:238-374).  The position is built
from three axis-angle rotations (azimuth about ``init_up``, elevation about
``init_up x view_dir``, roll about ``view_dir``), composed azimuth*elevation*roll
and applied to the distance-scaled initial offset.  The reference composes
them as quaternions through scipy; here each one is a Rodrigues matrix in
float64, which agrees to ~1e-16.

The two matrices keep the reference's memory layout because the renderer
sends their raw bytes as GL uniforms (pyvr/moderngl_renderer/manager.py:192):
the row-major numpy view matrix is read by GL as the column-major lookAt
matrix, and the projection matrix is read transposed.
"""

from __future__ import annotations

import json
from dataclasses import dataclass, field
from pathlib import Path
from typing import Any, Dict, Optional, Tuple, Union

import numpy as np


class CameraError(Exception):
    pass


def validate_camera_angles(azimuth: float, elevation: float, roll: float) -> None:
    for name, value in (("azimuth", azimuth), ("elevation", elevation), ("roll", roll)):
        if not isinstance(value, (int, float)):
            raise CameraError(f"{name} must be numeric, got {type(value)}")
        if not np.isfinite(value):
            raise CameraError(f"{name} must be finite, got {value}")


def _axis_angle_matrix(rotvec: np.ndarray) -> np.ndarray:
    """3x3 rotation by |rotvec| radians about rotvec (right-handed), float64."""
    v = np.asarray(rotvec, dtype=np.float64)
    theta = float(np.sqrt(v @ v))
    if theta == 0.0:
        return np.eye(3)
    k = v / theta
    kx = np.array([[0.0, -k[2], k[1]], [k[2], 0.0, -k[0]], [-k[1], k[0], 0.0]])
    return np.eye(3) + np.sin(theta) * kx + (1.0 - np.cos(theta)) * (kx @ kx)


def get_camera_pos(target: np.ndarray, azimuth: float, elevation: float, roll: float,
                   distance: float, init_pos: Optional[np.ndarray] = None,
                   init_up: Optional[np.ndarray] = None) -> Tuple[np.ndarray, np.ndarray]:
    """Camera position and up vector (float64), pyvr/camera/control.py:238-351."""
    validate_camera_angles(azimuth, elevation, roll)
    if not isinstance(target, np.ndarray) or target.shape != (3,):
        raise ValueError("target must be a 3D numpy array")
    if not isinstance(distance, (int, float)) or distance <= 0:
        raise ValueError("distance must be positive")
    if init_pos is None:
        init_pos = np.array([0, 0, distance], dtype=np.float32)
    if init_up is None:
        init_up = np.array([0, 1, 0], dtype=np.float32)
    for name, vec in (("init_pos", init_pos), ("init_up", init_up)):
        if not isinstance(vec, np.ndarray) or vec.shape != (3,):
            raise ValueError(f"{name} must be a 3D numpy array")

    # The reference works in float32 up to the rotations.
    tgt = target.astype(np.float32)
    up0 = init_up.astype(np.float32)
    offset = init_pos.astype(np.float32) - tgt
    n = np.linalg.norm(offset)
    if n == 0:
        raise ValueError("init_pos must not be the zero vector (relative to target)")
    offset = offset / n * distance

    view_dir = -offset / np.linalg.norm(offset)
    elev_axis = np.cross(up0, view_dir)
    elev_len = np.linalg.norm(elev_axis)
    if elev_len < 1e-6:  # init_up parallel to the view direction
        alt = np.array([1, 0, 0]) if abs(up0[0]) < 0.9 else np.array([0, 0, 1])
        elev_axis = np.cross(up0, alt)
        elev_len = np.linalg.norm(elev_axis)
    elev_axis = elev_axis / elev_len

    rot = (_axis_angle_matrix(azimuth * up0)
           @ _axis_angle_matrix(elevation * elev_axis)
           @ _axis_angle_matrix(roll * view_dir))
    position = rot @ offset.astype(np.float64) + tgt
    up = rot @ up0.astype(np.float64)
    return position, up


def get_camera_pos_from_params(params: "Camera") -> Tuple[np.ndarray, np.ndarray]:
    return get_camera_pos(params.target, params.azimuth, params.elevation, params.roll,
                          params.distance, params.init_pos, params.init_up)


def _vec3(values) -> np.ndarray:
    return np.array(values, dtype=np.float32)


@dataclass
class Camera:
    """Orbit camera with the field set and validation of pyvr/camera/camera.py:37-113."""

    target: np.ndarray = field(default_factory=lambda: _vec3([0.0, 0.0, 0.0]))
    azimuth: float = 0.0
    elevation: float = 0.0
    roll: float = 0.0
    distance: float = 3.0
    init_pos: np.ndarray = field(default_factory=lambda: _vec3([1.0, 0.0, 0.0]))
    init_up: np.ndarray = field(default_factory=lambda: _vec3([0.0, 0.0, 1.0]))
    fov: float = np.pi / 4
    near_plane: float = 0.1
    far_plane: float = 100.0

    def __post_init__(self):
        self.validate()

    def validate(self) -> None:
        if not isinstance(self.target, np.ndarray) or self.target.shape != (3,):
            raise ValueError("target must be a 3D numpy array")
        for name in ("azimuth", "elevation", "roll"):
            if not isinstance(getattr(self, name), (int, float)):
                raise ValueError(f"{name} must be numeric")
        if not isinstance(self.distance, (int, float)) or self.distance <= 0:
            raise ValueError("distance must be positive")
        for name in ("init_pos", "init_up"):
            vec = getattr(self, name)
            if not isinstance(vec, np.ndarray) or vec.shape != (3,):
                raise ValueError(f"{name} must be a 3D numpy array")
        if np.linalg.norm(self.init_pos - self.target) < 1e-9:
            raise ValueError("init_pos must not be at the same location as target")
        if np.linalg.norm(self.init_up) < 1e-9:
            raise ValueError("init_up must not be the zero vector")
        if self.fov <= 0 or self.fov >= np.pi:
            raise ValueError("fov must be between 0 and π radians")
        if self.near_plane <= 0:
            raise ValueError("near_plane must be positive")
        if self.far_plane <= self.near_plane:
            raise ValueError("far_plane must be greater than near_plane")

    # -- constructors (pyvr/camera/camera.py:115-194) -------------------------
    @classmethod
    def from_spherical(cls, target: np.ndarray, azimuth: float, elevation: float, roll: float,
                       distance: float, **kwargs) -> "Camera":
        return cls(target=target, azimuth=azimuth, elevation=elevation, roll=roll,
                   distance=distance, **kwargs)

    @classmethod
    def _preset(cls, target, distance, azimuth, elevation) -> "Camera":
        if target is None:
            target = _vec3([0.0, 0.0, 0.0])
        return cls(target=target, azimuth=azimuth, elevation=elevation, roll=0.0,
                   distance=distance)

    @classmethod
    def front_view(cls, target: Optional[np.ndarray] = None, distance: float = 3.0) -> "Camera":
        return cls._preset(target, distance, 0.0, 0.0)

    @classmethod
    def side_view(cls, target: Optional[np.ndarray] = None, distance: float = 3.0) -> "Camera":
        return cls._preset(target, distance, np.pi / 2, 0.0)

    @classmethod
    def top_view(cls, target: Optional[np.ndarray] = None, distance: float = 3.0) -> "Camera":
        return cls._preset(target, distance, 0.0, np.pi / 2)

    @classmethod
    def isometric_view(cls, target: Optional[np.ndarray] = None,
                       distance: float = 3.0) -> "Camera":
        return cls._preset(target, distance, np.pi / 4, np.pi / 6)

    # -- serialisation (pyvr/camera/camera.py:196-267) ------------------------
    def to_dict(self) -> Dict[str, Any]:
        return {"target": self.target.tolist(), "azimuth": float(self.azimuth),
                "elevation": float(self.elevation), "roll": float(self.roll),
                "distance": float(self.distance), "init_pos": self.init_pos.tolist(),
                "init_up": self.init_up.tolist(), "fov": float(self.fov),
                "near_plane": float(self.near_plane), "far_plane": float(self.far_plane)}

    @classmethod
    def from_dict(cls, data: Dict[str, Any]) -> "Camera":
        return cls(target=_vec3(data["target"]), azimuth=data["azimuth"],
                   elevation=data["elevation"], roll=data["roll"], distance=data["distance"],
                   init_pos=_vec3(data["init_pos"]), init_up=_vec3(data["init_up"]),
                   fov=data.get("fov", np.pi / 4), near_plane=data.get("near_plane", 0.1),
                   far_plane=data.get("far_plane", 100.0))

    def save_to_file(self, filepath: Union[str, Path]) -> None:
        with open(filepath, "w") as f:
            json.dump(self.to_dict(), f, indent=2)

    @classmethod
    def load_from_file(cls, filepath: Union[str, Path]) -> "Camera":
        with open(filepath) as f:
            return cls.from_dict(json.load(f))

    def copy(self) -> "Camera":
        return Camera.from_dict(self.to_dict())

    # -- matrices -------------------------------------------------------------
    def get_camera_vectors(self) -> Tuple[np.ndarray, np.ndarray]:
        return get_camera_pos_from_params(self)

    def get_view_matrix(self) -> np.ndarray:
        """lookAt with the basis in the first three COLUMNS of a row-major array
        (pyvr/camera/camera.py:292-334); GL reads its bytes column-major."""
        position, up = self.get_camera_vectors()
        return self._view_from(position, up)

    def _view_from(self, position: np.ndarray, up: np.ndarray) -> np.ndarray:
        """get_view_matrix from already computed camera vectors."""
        fwd = self.target - position
        fwd = fwd / np.linalg.norm(fwd)
        right = np.cross(fwd, up)
        right = right / np.linalg.norm(right)
        up_c = np.cross(right, fwd)
        m = np.zeros((4, 4), dtype=np.float64)
        m[:3, 0], m[:3, 1], m[:3, 2] = right, up_c, -fwd
        m[3, :3] = (-np.dot(right, position), -np.dot(up_c, position), np.dot(fwd, position))
        m[3, 3] = 1.0
        return m.astype(np.float32)

    def get_projection_matrix(self, aspect_ratio: float) -> np.ndarray:
        """Perspective matrix in the reference's row-major layout
        (pyvr/camera/camera.py:336-369)."""
        f = 1.0 / np.tan(self.fov / 2.0)
        n, fa = self.near_plane, self.far_plane
        m = np.zeros((4, 4), dtype=np.float64)
        m[0, 0] = f / aspect_ratio
        m[1, 1] = f
        m[2, 2] = (fa + n) / (n - fa)
        m[2, 3] = (2 * fa * n) / (n - fa)
        m[3, 2] = -1.0
        return m.astype(np.float32)

    def __repr__(self) -> str:
        return (f"Camera(target={self.target}, azimuth={self.azimuth:.3f} rad, "
                f"elevation={self.elevation:.3f} rad, roll={self.roll:.3f} rad, "
                f"distance={self.distance:.2f})")
