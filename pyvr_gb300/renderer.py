"""CUDA drop-in for pyvr's ``ModernGLVolumeRenderer`` / ``VolumeRenderer``.

Same constructor, methods, return values and exceptions as
pyvr/moderngl_renderer/renderer.py:19-320; the GL manager underneath is
replaced by the C ABI of ``libpyvr_gb300.so`` (include/pyvr_gb300.h).
Scene objects may be this package's (``pyvr_gb300.camera.Camera`` ...) or
pyvr's own: anything with the reference's class name and attributes is
accepted.
"""

from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _native
from ._native import check
from .camera import Camera
from .config import RenderConfig
from .lighting import Light


def _is_kind(obj, cls, name: str) -> bool:
    """isinstance(obj, cls), or obj is pyvr's class of the same name."""
    if isinstance(obj, cls):
        return True
    return any(c.__name__ == name for c in type(obj).__mro__)


def volume_storage(data: np.ndarray):
    """(contiguous array, dtype code) for upload.  uint8 / float16 / float32
    keep their storage; anything else is converted to float32 like
    pyvr/moderngl_renderer/manager.py:91-92."""
    if data.ndim != 3:
        raise ValueError("Volume data must be 3D")
    if data.dtype == np.uint8:
        code = _native.PVR_U8
    elif data.dtype == np.float16:
        code = _native.PVR_F16
    else:
        data = data.astype(np.float32, copy=False)
        code = _native.PVR_F32
    return np.ascontiguousarray(data), code


def rgba_lut(color_tf, opacity_tf, size: Optional[int] = None) -> np.ndarray:
    """(size, 4) float32 RGBA table as manager.py:162-175 builds it."""
    if size is None:
        size = max(color_tf.lut_size, opacity_tf.lut_size)
    lut = np.empty((size, 4), dtype=np.float32)
    lut[:, :3] = color_tf.to_lut(size)
    lut[:, 3] = opacity_tf.to_lut(size)
    return lut


def camera_uniforms(camera, width: int, height: int):
    """(view, proj, position) float32 arrays as renderer.py:160-172 sends them
    (this package's Camera computes its camera vectors once for both)."""
    if isinstance(camera, Camera):
        pos, up = camera.get_camera_vectors()
        view = camera._view_from(pos, up)
    else:
        view = camera.get_view_matrix()
        pos, _ = camera.get_camera_vectors()
    view = np.ascontiguousarray(view, dtype=np.float32)
    proj = np.ascontiguousarray(camera.get_projection_matrix(width / height), dtype=np.float32)
    return view, proj, np.asarray(pos, dtype=np.float32)


class CudaVolumeRenderer:
    """GB300 volume renderer with the API of ModernGLVolumeRenderer."""

    def __init__(self, width=512, height=512, config=None, light=None):
        self.width = width
        self.height = height
        self.volume = None
        self.camera = None
        if config is None:
            self.config = RenderConfig.balanced()
        else:
            if not _is_kind(config, RenderConfig, "RenderConfig"):
                raise TypeError(f"Expected RenderConfig instance, got {type(config)}")
            self.config = config
        if light is None:
            self.light = Light.default()
        else:
            if not _is_kind(light, Light, "Light"):
                raise TypeError(f"Expected Light instance, got {type(light)}")
            self.light = light
        self._lib = _native.load()
        handle = ctypes.c_void_p()
        check(self._lib.pvr_create(int(width), int(height), ctypes.byref(handle)))
        self._h = handle
        self._value_scale = 1.0
        self._update_render_config()
        self._update_light()

    # -- lifetime (ModernGLManager.cleanup, manager.py:238-256) ---------------
    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.pvr_destroy(h)
            self._h = None

    cleanup = close

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _handle(self):
        if self._h is None:
            raise RuntimeError("renderer has been closed")
        return self._h

    # -- scene state -----------------------------------------------------------
    def load_volume(self, volume, value_scale: Optional[float] = None) -> None:
        """renderer.py:107-146.  ``value_scale`` (extension) multiplies the
        sampled stored value; the default 1.0 samples uint8 voxels as 0..255
        exactly like the reference, 1/255 reads them as UNORM."""
        from .volume import Volume
        if not _is_kind(volume, Volume, "Volume"):
            raise TypeError(
                f"Expected Volume instance, got {type(volume)}. "
                "Create a Volume instance: from pyvr.volume import Volume; "
                "volume = Volume(data=your_array)")
        data, code = volume_storage(np.asarray(volume.data))
        scale = 1.0 if value_scale is None else float(value_scale)
        bmin = np.asarray(volume.min_bounds, dtype=np.float32)
        bmax = np.asarray(volume.max_bounds, dtype=np.float32)
        d, h, w = data.shape
        check(self._lib.pvr_load_volume(self._handle(), data.ctypes.data, code, d, h, w, scale,
                                        _native.fptr(bmin), _native.fptr(bmax)))
        self.volume = volume
        self._value_scale = scale
        if getattr(volume, "normals", None) is not None:
            nrm = np.asarray(volume.normals)
            if nrm.shape[-1] != 3:
                raise ValueError("Normal volume must have 3 channels (last dimension).")
            if nrm.shape[:3] != data.shape:
                raise ValueError(f"Normal volume must have shape {data.shape + (3,)}, got {nrm.shape}")
            nrm = np.ascontiguousarray(nrm, dtype=np.float32)
            check(self._lib.pvr_load_normals(self._handle(), nrm.ctypes.data))

    def set_camera(self, camera) -> None:
        if not _is_kind(camera, Camera, "Camera"):
            raise TypeError(f"Expected Camera instance, got {type(camera)}")
        self.camera = camera
        view, proj, pos = camera_uniforms(camera, self.width, self.height)
        check(self._lib.pvr_set_camera(self._handle(), _native.fptr(view), _native.fptr(proj),
                                       _native.fptr(pos)))

    def set_light(self, light) -> None:
        if not _is_kind(light, Light, "Light"):
            raise TypeError(f"Expected Light instance, got {type(light)}")
        self.light = light
        self._update_light()

    def set_transfer_functions(self, color_transfer_function, opacity_transfer_function,
                               size: Optional[int] = None) -> None:
        lut = rgba_lut(color_transfer_function, opacity_transfer_function, size)
        check(self._lib.pvr_set_lut(self._handle(), lut.ctypes.data, int(lut.shape[0])))

    def set_config(self, config) -> None:
        if not _is_kind(config, RenderConfig, "RenderConfig"):
            raise TypeError(f"Expected RenderConfig instance, got {type(config)}")
        self.config = config
        self._update_render_config()

    def get_config(self):
        return self.config

    def get_light(self):
        return self.light

    def get_volume(self):
        return self.volume

    def get_camera(self):
        return self.camera

    # -- rendering ---------------------------------------------------------------
    def render_array(self) -> np.ndarray:
        """(height, width, 4) uint8 RGBA, row 0 = bottom (no bytes copy)."""
        out = np.empty((self.height, self.width, 4), dtype=np.uint8)
        check(self._lib.pvr_render(self._handle(), out.ctypes.data, None))
        return out

    def render(self) -> bytes:
        """renderer.py:209-219: W*H*4 RGBA8 bytes, bottom row first (copied
        once, from the handle's page-locked image)."""
        p = ctypes.c_void_p()
        check(self._lib.pvr_render_pinned(self._handle(), ctypes.byref(p)))
        return ctypes.string_at(p.value, self.width * self.height * 4)

    def render_float(self):
        """(rgba8, float32 (H, W, 4) pre-blend fragment colour)."""
        out8 = np.empty((self.height, self.width, 4), dtype=np.uint8)
        outf = np.empty((self.height, self.width, 4), dtype=np.float32)
        check(self._lib.pvr_render(self._handle(), out8.ctypes.data, outf.ctypes.data))
        return out8, outf

    def render_to_pil(self, data=None):
        from PIL import Image
        if data is None:
            data = self.render()
        image = Image.frombytes("RGBA", (self.width, self.height), data)
        return image.transpose(Image.FLIP_TOP_BOTTOM)

    def compute_normals(self) -> None:
        """Volume.compute_normals on the GPU for the loaded volume (the
        normals numpy's compute_normal_volume would give, bit for bit)."""
        check(self._lib.pvr_compute_normals(self._handle()))

    def set_tuning(self, tile_w: int = 16, tile_h: int = 16, steps_per_iter: int = 1,
                   blocks_per_sm: int = 0) -> None:
        """Launch shape of the march (any valid shape gives the same image)."""
        t = _native.PvrTuning(tile_w, tile_h, steps_per_iter, blocks_per_sm)
        check(self._lib.pvr_set_tuning(self._handle(), ctypes.byref(t)))

    def last_sample_count(self) -> int:
        n = ctypes.c_longlong(0)
        check(self._lib.pvr_last_sample_count(self._handle(), ctypes.byref(n)))
        return int(n.value)

    def last_sample_counts(self):
        """(in-box samples, shaded samples) of the most recent render."""
        a, b = ctypes.c_longlong(0), ctypes.c_longlong(0)
        check(self._lib.pvr_last_sample_counts(self._handle(), ctypes.byref(a), ctypes.byref(b)))
        return int(a.value), int(b.value)

    def device_bytes(self) -> int:
        n = ctypes.c_longlong(0)
        check(self._lib.pvr_device_bytes(self._handle(), ctypes.byref(n)))
        return int(n.value)

    # -- uniform updates (renderer.py:303-316) -------------------------------------
    def _update_render_config(self):
        c = self.config
        check(self._lib.pvr_set_config(self._handle(), float(c.step_size), int(c.max_steps),
                                       float(c.reference_step_size)))

    def _update_light(self):
        lt = self.light
        pos = np.asarray(lt.position, dtype=np.float32)
        tgt = np.asarray(lt.target, dtype=np.float32)
        check(self._lib.pvr_set_light(self._handle(), _native.fptr(pos), _native.fptr(tgt),
                                      float(lt.ambient_intensity), float(lt.diffuse_intensity)))


VolumeRenderer = CudaVolumeRenderer
ModernGLVolumeRenderer = CudaVolumeRenderer
