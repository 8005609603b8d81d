"""Volume container and the gradient normal producer.

``Volume`` mirrors pyvr/volume/data.py:15-174 (data (D,H,W), optional
normals (D,H,W,3), world-space bounds).  ``compute_normal_volume`` restates
pyvr/datasets/synthetic.py:109-122: central differences inside, one-sided
differences on the faces (numpy.gradient, unit spacing), divided by
``|g| + 1e-8`` and stored as float32 with the components in array-axis order.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional, Tuple

import numpy as np


def _gradient_axis(v: np.ndarray, axis: int) -> np.ndarray:
    """np.gradient along one axis with unit spacing and first-order edges."""
    v = np.moveaxis(v, axis, 0)
    out = np.empty(v.shape, dtype=np.result_type(v.dtype, np.float64)
                   if v.dtype.kind in "iub" else v.dtype)
    n = v.shape[0]
    if n < 2:
        raise ValueError("Shape of array too small to calculate a numerical gradient, "
                         "at least (edge_order + 1) elements are required.")
    if v.dtype.kind in "iub":
        v = v.astype(np.float64)
    out[1:-1] = (v[2:] - v[:-2]) / 2.0
    out[0] = v[1] - v[0]
    out[-1] = v[-1] - v[-2]
    return np.moveaxis(out, 0, axis)


def compute_normal_volume(volume: np.ndarray) -> np.ndarray:
    """Unit gradient per voxel, shape (D, H, W, 3), float32."""
    volume = np.asarray(volume)
    g = np.stack([_gradient_axis(volume, a) for a in range(3)], axis=-1)
    # float16 input stays float16 (as in numpy.gradient): there 1e-8 rounds to
    # 0 and a zero gradient gives NaN, exactly as the reference produces it.
    with np.errstate(divide="ignore", invalid="ignore"):
        norm = np.sqrt(np.sum(g * g, axis=-1, keepdims=True)) + 1e-8
        return (g / norm).astype(np.float32)


class VolumeError(Exception):
    pass


def _vec3(values) -> np.ndarray:
    return np.array(values, dtype=np.float32)


@dataclass
class Volume:
    data: np.ndarray
    normals: Optional[np.ndarray] = None
    min_bounds: np.ndarray = field(default_factory=lambda: _vec3([-0.5, -0.5, -0.5]))
    max_bounds: np.ndarray = field(default_factory=lambda: _vec3([0.5, 0.5, 0.5]))
    name: Optional[str] = None

    def __post_init__(self):
        self.validate()

    def validate(self) -> None:
        if not isinstance(self.data, np.ndarray):
            raise ValueError("Volume data must be a numpy array")
        if self.data.ndim != 3:
            raise ValueError(f"Volume data must be 3D, got shape {self.data.shape}")
        if self.normals is not None:
            if not isinstance(self.normals, np.ndarray):
                raise ValueError("Normal volume must be a numpy array")
            want = self.data.shape + (3,)
            if self.normals.shape != want:
                raise ValueError(f"Normal volume must have shape {want}, "
                                 f"got {self.normals.shape}")
        for name in ("min_bounds", "max_bounds"):
            b = getattr(self, name)
            if not isinstance(b, np.ndarray) or b.shape != (3,):
                raise ValueError(f"{name} must be a 3D numpy array")
        if np.any(self.max_bounds <= self.min_bounds):
            raise ValueError("max_bounds must be greater than min_bounds")

    @property
    def shape(self) -> Tuple[int, int, int]:
        return self.data.shape

    @property
    def dimensions(self) -> np.ndarray:
        return self.max_bounds - self.min_bounds

    @property
    def center(self) -> np.ndarray:
        return (self.min_bounds + self.max_bounds) / 2.0

    @property
    def has_normals(self) -> bool:
        return self.normals is not None

    @property
    def voxel_spacing(self) -> np.ndarray:
        return self.dimensions / np.array(self.shape, dtype=np.float32)

    def compute_normals(self, method: str = "gradient") -> None:
        if method != "gradient":
            raise ValueError(f"Unsupported method: {method}")
        self.normals = compute_normal_volume(self.data)

    def normalize(self, method: str = "minmax") -> "Volume":
        d = self.data
        if method == "minmax":
            lo, hi = d.min(), d.max()
            out = np.zeros_like(d) if hi - lo < 1e-9 else (d - lo) / (hi - lo)
        elif method == "zscore":
            mu, sd = d.mean(), d.std()
            out = np.zeros_like(d) if sd < 1e-9 else (d - mu) / sd
        else:
            raise ValueError(f"Unsupported method: {method}")
        return Volume(data=out.astype(np.float32),
                      normals=None if self.normals is None else self.normals.copy(),
                      min_bounds=self.min_bounds.copy(), max_bounds=self.max_bounds.copy(),
                      name=f"{self.name}_normalized" if self.name else None)

    def copy(self) -> "Volume":
        return Volume(data=self.data.copy(),
                      normals=None if self.normals is None else self.normals.copy(),
                      min_bounds=self.min_bounds.copy(), max_bounds=self.max_bounds.copy(),
                      name=self.name)

    def __repr__(self) -> str:
        nm = f"'{self.name}'" if self.name else "unnamed"
        nrm = "with normals" if self.has_normals else "no normals"
        return (f"Volume({nm}, shape={self.shape}, "
                f"bounds=[{self.min_bounds}, {self.max_bounds}], {nrm})")
