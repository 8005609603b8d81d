"""Differentiable rendering: gradients of an image loss with respect to the
RGBA transfer-function LUT and the voxel values, from a hand-written CUDA
backward (``pvr_diff_backward``) behind ``torch.autograd.Function``.

The forward is the renderer's march (pyvr/shaders/volume.frag.glsl:70-122)
over an FP32 volume in its (D, H, W) layout, for several views of one scene
at once; its float image is the renderer's float image bit for bit.  The
backward marches each ray a second time in reverse and rebuilds the
transmittance from the final alpha (T_i = T_{i+1} / (1 - alpha_i)), so no
per-sample state is stored: only the loop length of each pixel.  Normals (a
given normal volume, or none) are constants of the scene.

    scene = DiffScene(cameras, light, config, width, height)
    image = render_views(volume, lut, scene)      # (views, H, W, 4)
    loss = ((image - target) ** 2).mean()
    loss.backward()                               # volume.grad, lut.grad
"""

from __future__ import annotations

import ctypes
from typing import Sequence

import numpy as np

from . import _native
from ._native import check
from .renderer import camera_uniforms


def _lib():
    return _native.load()


class DiffScene:
    """Views, light, march settings and volume bounds of a differentiable
    render; cameras are pyvr-style ``Camera`` objects (matrices as the
    renderer computes them, pyvr/moderngl_renderer/renderer.py:160-172)."""

    def __init__(self, cameras: Sequence, light, config, width: int, height: int,
                 min_bounds=(-1.0, -1.0, -1.0), max_bounds=(1.0, 1.0, 1.0), value_scale: float = 1.0):
        self.width, self.height = int(width), int(height)
        self.n_views = len(cameras)
        if self.n_views < 1:
            raise ValueError("at least one camera is needed")
        self._views = (_native.PvrDiffView * self.n_views)()
        for v, cam in zip(self._views, cameras):
            view, proj, pos = camera_uniforms(cam, self.width, self.height)
            v.view[:] = view.ravel().tolist()
            v.proj[:] = proj.ravel().tolist()
            v.camera_pos[:] = pos.tolist()
        self.light = light
        self.config = config
        self.min_bounds = np.asarray(min_bounds, np.float32)
        self.max_bounds = np.asarray(max_bounds, np.float32)
        self.value_scale = float(value_scale)

    def c_scene(self, volume, lut, normals=None) -> _native.PvrDiffScene:
        s = _native.PvrDiffScene()
        s.volume = volume.data_ptr()
        s.normals = normals.data_ptr() if normals is not None else None
        s.d, s.h, s.w = (int(x) for x in volume.shape)
        s.value_scale = self.value_scale
        s.lut = lut.data_ptr()
        s.lut_size = int(lut.shape[0])
        s.min_bounds[:] = self.min_bounds.tolist()
        s.max_bounds[:] = self.max_bounds.tolist()
        lp = np.asarray(self.light.position, np.float32)
        lt = np.asarray(self.light.target, np.float32)
        s.light_pos[:] = lp.tolist()
        s.light_target[:] = lt.tolist()
        s.ambient = float(self.light.ambient_intensity)
        s.diffuse = float(self.light.diffuse_intensity)
        s.step_size = float(self.config.step_size)
        s.reference_step_size = float(self.config.reference_step_size)
        s.max_steps = int(self.config.max_steps)
        s.width, s.height = self.width, self.height
        s.n_views = self.n_views
        s.views = ctypes.cast(self._views, ctypes.c_void_p)
        return s


def _check_inputs(volume, lut, normals):
    import torch
    if volume.dtype != torch.float32 or volume.dim() != 3 or not volume.is_cuda:
        raise TypeError("volume must be a CUDA float32 tensor of shape (D, H, W)")
    if lut.dtype != torch.float32 or lut.dim() != 2 or lut.shape[1] != 4 or not lut.is_cuda:
        raise TypeError("lut must be a CUDA float32 tensor of shape (size, 4)")
    if normals is not None and (normals.dtype != torch.float32 or not normals.is_cuda or
                                tuple(normals.shape) != tuple(volume.shape) + (3,)):
        raise TypeError("normals must be a CUDA float32 tensor of shape (D, H, W, 3)")
    devices = {volume.device, lut.device} | ({normals.device} if normals is not None else set())
    if len(devices) != 1:
        raise ValueError("volume, lut and normals must be on one device")


def _march_function():
    import torch

    class _March(torch.autograd.Function):
        @staticmethod
        def forward(ctx, volume, lut, normals, scene):
            _check_inputs(volume, lut, normals)
            volume = volume.contiguous()
            lut = lut.contiguous()
            normals = normals.contiguous() if normals is not None else None
            v, h, w = scene.n_views, scene.height, scene.width
            image = torch.empty((v, h, w, 4), dtype=torch.float32, device=volume.device)
            steps = torch.empty((v, h, w), dtype=torch.int32, device=volume.device)
            c = scene.c_scene(volume, lut, normals)
            stream = torch.cuda.current_stream(volume.device).cuda_stream
            check(_lib().pvr_diff_forward(ctypes.byref(c), image.data_ptr(), steps.data_ptr(), stream))
            ctx.scene = scene
            ctx.save_for_backward(volume, lut, normals, image, steps)
            ctx.mark_non_differentiable(steps)
            return image, steps

        @staticmethod
        def backward(ctx, gimage, _gsteps):
            volume, lut, normals, image, steps = ctx.saved_tensors
            need_vol, need_lut = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
            gvol = torch.zeros_like(volume) if need_vol else None
            glut = torch.zeros_like(lut) if need_lut else None
            if need_vol or need_lut:
                gimage = gimage.contiguous()
                c = ctx.scene.c_scene(volume, lut, normals)
                stream = torch.cuda.current_stream(volume.device).cuda_stream
                check(_lib().pvr_diff_backward(ctypes.byref(c), image.data_ptr(), steps.data_ptr(),
                                               gimage.data_ptr(), glut.data_ptr() if glut is not None else None,
                                               gvol.data_ptr() if gvol is not None else None, stream))
            return gvol, glut, None, None

    return _March


_MARCH = None


def render_views(volume, lut, scene: DiffScene, normals=None, return_steps: bool = False):
    """Float RGBA images (views, H, W, 4) of ``volume`` (CUDA float32 (D, H, W))
    under ``lut`` (CUDA float32 (size, 4)), differentiable in both.  With
    return_steps, also the per-pixel loop lengths."""
    global _MARCH
    if _MARCH is None:
        _MARCH = _march_function()
    if normals is not None and normals.requires_grad:
        raise ValueError("normals are constants of the scene; detach them")
    image, steps = _MARCH.apply(volume, lut, normals, scene)
    return (image, steps) if return_steps else image
