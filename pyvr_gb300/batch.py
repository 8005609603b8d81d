"""Batched rendering: many renders of different volumes, LUTs, cameras and
sizes in one persistent kernel launch (captured as a CUDA graph).

``DeviceVolume`` and ``DeviceLUT`` are the device resources of the C ABI
(``pvr_volume`` / ``pvr_lut``); ``BatchRenderer`` queues lists of
``RenderJob`` on a ``pvr_batch`` launcher.  Output buffers are torch CUDA
tensors (plumbing only: the kernels are the library's).
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _native
from ._native import check
from .renderer import camera_uniforms, rgba_lut, volume_storage


def _lib():
    return _native.load()


class DeviceVolume:
    """A volume resident on the GPU in the march layout.

    normals: "given" (use ``volume.normals``), "device" (compute with
    numpy.gradient semantics on the GPU), "none", or "auto" (given if the
    volume has normals, else none).
    """

    def __init__(self, volume, value_scale: float = 1.0, normals: str = "auto",
                 brick_log2: int = 0):
        data, code = volume_storage(np.asarray(volume.data))
        mode = normals
        if mode == "auto":
            mode = "given" if getattr(volume, "normals", None) is not None else "none"
        nrm_ptr = None
        self._keep = None
        if mode == "given":
            nrm = np.ascontiguousarray(volume.normals, dtype=np.float32)
            if nrm.shape != data.shape + (3,):
                raise ValueError(f"Normal volume must have shape {data.shape + (3,)}, got {nrm.shape}")
            nrm_ptr = nrm.ctypes.data
            self._keep = nrm
        codes = {"none": _native.PVR_NORMALS_NONE, "given": _native.PVR_NORMALS_GIVEN,
                 "device": _native.PVR_NORMALS_DEVICE}
        if mode not in codes:
            raise ValueError(f"unknown normals mode {normals!r}")
        bmin = np.asarray(volume.min_bounds, dtype=np.float32)
        bmax = np.asarray(volume.max_bounds, dtype=np.float32)
        h = ctypes.c_void_p()
        d0, d1, d2 = data.shape
        check(_lib().pvr_volume_create(data.ctypes.data, code, d0, d1, d2, float(value_scale),
                                       _native.fptr(bmin), _native.fptr(bmax), nrm_ptr, codes[mode],
                                       int(brick_log2), ctypes.byref(h)))
        self._keep = None
        self.handle = h
        self.shape = data.shape
        self.dtype = data.dtype
        self.normals_mode = mode
        self.brick_log2 = brick_log2 or 3

    def device_bytes(self) -> int:
        n = ctypes.c_longlong(0)
        check(_lib().pvr_volume_device_bytes(self.handle, ctypes.byref(n)))
        return int(n.value)

    def read_normals(self) -> np.ndarray:
        out = np.empty(self.shape + (3,), dtype=np.float32)
        check(_lib().pvr_volume_read_normals(self.handle, out.ctypes.data))
        return out

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            _lib().pvr_volume_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceLUT:
    """An RGBA LUT on the GPU (the table of set_transfer_functions)."""

    def __init__(self, color_tf=None, opacity_tf=None, size: Optional[int] = None,
                 rgba: Optional[np.ndarray] = None):
        lut = rgba if rgba is not None else rgba_lut(color_tf, opacity_tf, size)
        lut = np.ascontiguousarray(lut, dtype=np.float32)
        h = ctypes.c_void_p()
        check(_lib().pvr_lut_create(lut.ctypes.data, int(lut.shape[0]), ctypes.byref(h)))
        self.handle = h
        self.size = int(lut.shape[0])

    def update(self, rgba: np.ndarray) -> None:
        """Replace the table; no batch reading this LUT may be in flight."""
        lut = np.ascontiguousarray(rgba, dtype=np.float32)
        check(_lib().pvr_lut_update(self.handle, lut.ctypes.data, int(lut.shape[0])))
        self.size = int(lut.shape[0])

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            _lib().pvr_lut_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class RenderJob:
    """One render: resources, camera/light/config objects (pyvr's or ours),
    output size, and device outputs (torch uint8 (H*W*4,) / float32
    (H*W*4,) tensors or raw device pointers; either may be None)."""

    volume: DeviceVolume
    lut: DeviceLUT
    camera: object
    light: object
    config: object
    width: int
    height: int
    out_rgba8: object = None
    out_rgba32f: object = None
    counters: object = None  # torch int64 (2,) zeroed: [in-box, shaded] samples


def _ptr(x) -> Optional[int]:
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return int(x.data_ptr())


def make_job_struct(job: RenderJob, out: Optional[_native.PvrJob] = None) -> _native.PvrJob:
    j = out if out is not None else _native.PvrJob()
    view, proj, pos = camera_uniforms(job.camera, job.width, job.height)
    j.volume = job.volume.handle.value
    j.lut = job.lut.handle.value
    j.width, j.height = int(job.width), int(job.height)
    j.view[:] = view.ravel().tolist()
    j.proj[:] = proj.ravel().tolist()
    j.camera_pos[:] = pos.tolist()
    lp = np.asarray(job.light.position, np.float32)
    lt = np.asarray(job.light.target, np.float32)
    j.light_pos[:] = lp.tolist()
    j.light_target[:] = lt.tolist()
    j.ambient = float(job.light.ambient_intensity)
    j.diffuse = float(job.light.diffuse_intensity)
    j.step_size = float(job.config.step_size)
    j.reference_step_size = float(job.config.reference_step_size)
    j.max_steps = int(job.config.max_steps)
    j.d_rgba8 = _ptr(job.out_rgba8)
    j.d_rgba32f = _ptr(job.out_rgba32f)
    j.d_counters = _ptr(job.counters)
    return j


@dataclass
class Tuning:
    tile_w: int = 16
    tile_h: int = 16
    steps_per_iter: int = 1
    blocks_per_sm: int = 0
    brick_log2: int = 3

    def c(self) -> _native.PvrTuning:
        return _native.PvrTuning(self.tile_w, self.tile_h, self.steps_per_iter, self.blocks_per_sm)


class BatchRenderer:
    """Queues batches of RenderJob on one persistent-kernel launcher."""

    def __init__(self, capacity: int = 64, slots: int = 3, tuning: Optional[Tuning] = None):
        h = ctypes.c_void_p()
        check(_lib().pvr_batch_create(int(capacity), int(slots), ctypes.byref(h)))
        self.handle = h
        self.capacity = capacity
        self._arr = (_native.PvrJob * capacity)()
        if tuning is not None:
            self.set_tuning(tuning)

    def set_tuning(self, tuning: Tuning) -> None:
        t = tuning.c()
        check(_lib().pvr_batch_set_tuning(self.handle, ctypes.byref(t)))
        self.tuning = tuning

    def render(self, jobs: Sequence[RenderJob], stream=None) -> None:
        """Queue the jobs (asynchronous).  ``stream``: a torch.cuda.Stream,
        a raw handle, or None for the launcher's own stream."""
        if len(jobs) > self.capacity:
            raise ValueError(f"batch of {len(jobs)} exceeds capacity {self.capacity}")
        for i, job in enumerate(jobs):
            make_job_struct(job, self._arr[i])
        s = getattr(stream, "cuda_stream", stream)
        check(_lib().pvr_batch_render(self.handle, ctypes.cast(self._arr, ctypes.c_void_p),
                                      len(jobs), s))

    def render_structs(self, structs, n: int, stream=None) -> None:
        """Queue n prepared PvrJob structs (an array of at least n)."""
        s = getattr(stream, "cuda_stream", stream)
        check(_lib().pvr_batch_render(self.handle, ctypes.cast(structs, ctypes.c_void_p), int(n), s))

    def synchronize(self) -> None:
        check(_lib().pvr_batch_synchronize(self.handle))

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            _lib().pvr_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
