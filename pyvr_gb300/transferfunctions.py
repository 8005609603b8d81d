"""Piecewise-linear colour and opacity transfer functions and the RGBA LUT.

Mirrors pyvr/transferfunctions (base.py:15-161, color.py:18-248,
opacity.py:18-214): control points sorted by scalar, validated to [0, 1],
sampled into a lookup table with ``np.interp`` on ``linspace(0, 1, size)``.
``rgba_lut`` builds the combined (size, 4) float32 table exactly as
pyvr/moderngl_renderer/manager.py:162-175 does before uploading it.
"""

from __future__ import annotations

from typing import List, Optional, Sequence, Tuple

import numpy as np


class TransferFunctionError(Exception):
    pass


class InvalidControlPointError(TransferFunctionError):
    pass


def _check_points(points: Sequence, width: int) -> None:
    """Shape/type checks of pyvr/transferfunctions/base.py:111-161."""
    if not points:
        raise InvalidControlPointError("Control points cannot be empty")
    for i, p in enumerate(points):
        if not isinstance(p, (tuple, list)) or len(p) != 2:
            raise InvalidControlPointError(f"Control point {i} must be a (scalar, value) tuple, got {p}")
        s, v = p
        if not isinstance(s, (int, float)):
            raise InvalidControlPointError(f"Control point {i} scalar must be numeric, got {type(s)}")
        if width == 1:
            if not isinstance(v, (int, float)):
                raise InvalidControlPointError(f"Control point {i} value must be numeric, got {type(v)}")
        else:
            if not isinstance(v, (tuple, list, np.ndarray)) or len(v) != width:
                raise InvalidControlPointError(
                    f"Control point {i} value must be a {width}-element sequence, got {v}")
            for j, c in enumerate(v):
                if not isinstance(c, (int, float)):
                    raise InvalidControlPointError(
                        f"Control point {i} value component {j} must be numeric, got {type(c)}")
        if not (0.0 <= s <= 1.0):
            raise ValueError(f"Control point scalar {s} outside valid range [0.0, 1.0]")


class BaseTransferFunction:
    _width = 1

    def __init__(self, control_points: Optional[List[Tuple]] = None, lut_size: int = 256):
        if control_points is None:
            control_points = self._default_points()
        self.control_points = sorted(control_points, key=lambda p: p[0])
        self.lut_size = lut_size
        _check_points(self.control_points, self._width)
        self._check_values()

    def _default_points(self):
        raise NotImplementedError

    def _check_values(self):
        raise NotImplementedError

    def to_lut(self, size: Optional[int] = None) -> np.ndarray:
        raise NotImplementedError

    def __call__(self, size: Optional[int] = None) -> np.ndarray:
        return self.to_lut(size)

    def _samples(self, size: Optional[int]) -> np.ndarray:
        return np.linspace(0, 1, size or self.lut_size)


class OpacityTransferFunction(BaseTransferFunction):
    """Scalar -> opacity, pyvr/transferfunctions/opacity.py."""

    _width = 1

    def _default_points(self):
        return [(0.0, 0.0), (1.0, 1.0)]

    def _check_values(self):
        for i, (_, a) in enumerate(self.control_points):
            if not (0.0 <= a <= 1.0):
                raise InvalidControlPointError(
                    f"Control point {i} opacity {a} outside valid range [0.0, 1.0]")

    @classmethod
    def linear(cls, low: float = 0.0, high: float = 1.0, lut_size: int = 256):
        return cls([(0.0, low), (1.0, high)], lut_size=lut_size)

    @classmethod
    def one_step(cls, step: float = 0.5, low: float = 0.0, high: float = 1.0,
                 lut_size: int = 256):
        eps = 1e-12
        return cls([(0.0, low), (step, low), (step + eps, high), (1.0, high)], lut_size=lut_size)

    @classmethod
    def peaks(cls, peaks: List[float], opacity: float = 1.0, eps: float = 0.02,
              lut_size: int = 256, base: float = 0.0):
        """Triangular peaks over a base level (pyvr/transferfunctions/opacity.py:93-151)."""
        if not peaks:
            raise ValueError("At least one peak position must be specified")
        for p in peaks:
            if not (0.0 <= p <= 1.0):
                raise ValueError(f"Peak position {p} must be between 0 and 1")
        pts = [(0.0, base)]
        for p in sorted(peaks):
            lo, hi = max(0.0, p - eps), min(1.0, p + eps)
            if lo > pts[-1][0]:
                pts.append((lo, base))
            pts.append((p, opacity))
            if hi > p:
                pts.append((hi, base))
        if pts[-1][0] < 1.0:
            pts.append((1.0, base))
        return cls(pts, lut_size=lut_size)

    def to_lut(self, size: Optional[int] = None) -> np.ndarray:
        xs, ys = zip(*self.control_points)
        return np.interp(self._samples(size), xs, ys).astype(np.float32)

    def apply_to_array(self, scalars: np.ndarray) -> np.ndarray:
        xs, ys = zip(*self.control_points)
        return np.interp(scalars.ravel(), xs, ys).reshape(scalars.shape).astype(np.float32)

    def __repr__(self) -> str:
        return f"OpacityTransferFunction(control_points={self.control_points}, lut_size={self.lut_size})"


class ColorTransferFunction(BaseTransferFunction):
    """Scalar -> RGB, pyvr/transferfunctions/color.py."""

    _width = 3

    def _default_points(self):
        return [(0.0, (0.0, 0.0, 0.0)), (1.0, (1.0, 1.0, 1.0))]

    def _check_values(self):
        for i, (_, rgb) in enumerate(self.control_points):
            for j, c in enumerate(rgb):
                if not (0.0 <= c <= 1.0):
                    raise InvalidControlPointError(
                        f"Control point {i} RGB component {j} value {c} outside valid range [0.0, 1.0]")

    @classmethod
    def grayscale(cls, lut_size: int = 256):
        return cls([(0.0, (0.0, 0.0, 0.0)), (1.0, (1.0, 1.0, 1.0))], lut_size=lut_size)

    @classmethod
    def single_color(cls, color, lut_size: int = 256):
        return cls([(0.0, color), (1.0, color)], lut_size=lut_size)

    @classmethod
    def two_color_ramp(cls, color1, color2, lut_size: int = 256):
        return cls([(0.0, color1), (1.0, color2)], lut_size=lut_size)

    @classmethod
    def from_colormap(cls, colormap_name: str, value_range=(0.0, 1.0), lut_size: int = 256):
        """Sample a matplotlib colormap into control points (needs matplotlib)."""
        try:
            import matplotlib
            cmap = matplotlib.colormaps.get_cmap(colormap_name)
        except ImportError:
            raise ImportError("matplotlib is required for from_colormap method")
        except Exception as e:  # unknown name
            raise ValueError(f"Unknown colormap name '{colormap_name}': {e}")
        x = np.linspace(0, 1, lut_size)
        rgb = cmap(x)[:, :3]
        lo, hi = value_range
        xm = lo + x * (hi - lo)
        return cls([(float(a), tuple(map(float, c))) for a, c in zip(xm, rgb)], lut_size=lut_size)

    def to_lut(self, size: Optional[int] = None) -> np.ndarray:
        x = self._samples(size)
        xs, cs = zip(*self.control_points)
        cs = np.array(cs)
        lut = np.empty((x.size, 3), dtype=np.float32)
        for c in range(3):
            lut[:, c] = np.interp(x, xs, cs[:, c])
        return lut

    def apply_to_array(self, scalars: np.ndarray) -> np.ndarray:
        xs, cs = zip(*self.control_points)
        cs = np.array(cs)
        flat = scalars.ravel()
        out = np.empty((flat.size, 3), dtype=np.float32)
        for c in range(3):
            out[:, c] = np.interp(flat, xs, cs[:, c])
        return out.reshape(scalars.shape + (3,))

    def get_color_at(self, scalar: float):
        xs, cs = zip(*self.control_points)
        cs = np.array(cs)
        return tuple(float(np.float32(np.interp(scalar, xs, cs[:, c]))) for c in range(3))

    def __repr__(self) -> str:
        return (f"ColorTransferFunction({len(self.control_points)} control points, "
                f"lut_size={self.lut_size})")


def rgba_lut(color_tf, opacity_tf, size: Optional[int] = None) -> np.ndarray:
    """Combined (size, 4) float32 RGBA table: size defaults to the larger of
    the two functions' ``lut_size`` (pyvr/moderngl_renderer/manager.py:162-175)."""
    if size is None:
        size = max(color_tf.lut_size, opacity_tf.lut_size)
    out = np.empty((size, 4), dtype=np.float32)
    out[:, :3] = color_tf.to_lut(size)
    out[:, 3] = opacity_tf.to_lut(size)
    return out
