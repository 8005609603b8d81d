"""Batched rendering: many renders of different volumes, LUTs, cameras and
sizes in one persistent kernel launch (captured as a CUDA graph).

``DeviceVolume`` and ``DeviceLUT`` are the device resources of the C ABI
(``pvr_volume`` / ``pvr_lut``); ``BatchRenderer`` queues lists of
``RenderJob`` on a ``pvr_batch`` launcher.  Output buffers are torch CUDA
tensors (plumbing only: the kernels are the library's).
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _native
from ._native import check
from .renderer import rgba_lut, volume_storage


def _lib():
    return _native.load()


class _PageLocked:
    """One pvr_host_alloc block; freed when the last array viewing it goes."""

    def __init__(self, nbytes: int):
        p = ctypes.c_void_p()
        check(_lib().pvr_host_alloc(int(nbytes), ctypes.byref(p)))
        self.ptr, self.nbytes = p.value, int(nbytes)

    def __del__(self):
        if getattr(self, "ptr", None):
            try:
                _lib().pvr_host_free(ctypes.c_void_p(self.ptr))
            except Exception:
                pass
            self.ptr = None


def page_locked_empty(shape, dtype) -> np.ndarray:
    """A numpy array in page-locked host memory (``pvr_host_alloc``):
    volumes uploaded from it (``DeviceVolume``, the render server's loads)
    move at the link's full speed.  The memory is freed with the array."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape)) * dtype.itemsize
    owner = _PageLocked(max(n, 1))
    buf = (ctypes.c_uint8 * max(n, 1)).from_address(owner.ptr)
    buf._owner = owner  # the array's base (buf) keeps the block alive
    return np.frombuffer(buf, dtype=np.uint8, count=n).view(dtype).reshape(shape)


class PageLockedArena:
    """One pvr_host_alloc block handing out numpy arrays (``array``), each at
    a 4 KiB boundary: many volumes in one page-locked allocation instead of
    one each.  The block is freed when the arena and every array from it
    are gone."""

    ALIGN = 4096

    def __init__(self, nbytes: int):
        self._owner = _PageLocked(max(int(nbytes), 1))
        self._off = 0

    @classmethod
    def size_for(cls, arrays) -> int:
        """Bytes an arena needs to hold copies of ``arrays``."""
        return sum((int(a.nbytes) + cls.ALIGN - 1) // cls.ALIGN * cls.ALIGN for a in arrays)

    def array(self, shape, dtype) -> np.ndarray:
        dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * dtype.itemsize
        if self._off + n > self._owner.nbytes:
            raise MemoryError(f"page-locked arena of {self._owner.nbytes} bytes is full")
        buf = (ctypes.c_uint8 * max(n, 1)).from_address(self._owner.ptr + self._off)
        buf._owner = self._owner
        self._off += (n + self.ALIGN - 1) // self.ALIGN * self.ALIGN
        return np.frombuffer(buf, dtype=np.uint8, count=n).view(dtype).reshape(shape)

    def copy(self, a: np.ndarray) -> np.ndarray:
        out = self.array(a.shape, a.dtype)
        out[...] = a
        return out


def page_locked_copy(a: np.ndarray) -> np.ndarray:
    """``a`` copied into page-locked host memory (C order)."""
    out = page_locked_empty(a.shape, a.dtype)
    out[...] = a
    return out


class DeviceVolume:
    """A volume resident on the GPU in the march layout.

    normals: "given" (use ``volume.normals``), "device" (compute with
    numpy.gradient semantics on the GPU), "none", or "auto" (given if the
    volume has normals, else none).  half_records: store the records as
    halves if every value and normal is a half exactly (``compact``).
    """

    def __init__(self, volume, value_scale: float = 1.0, normals: str = "auto",
                 brick_log2: int = 0, half_records: bool = False, wait: bool = True):
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
        # wait=False: the upload and layout are only queued (the renders of
        # the volume wait for them on the device); the host arrays stay
        # referenced until ready() has seen the layout complete
        create = _lib().pvr_volume_create if wait else _lib().pvr_volume_create_async
        check(create(data.ctypes.data, code, d0, d1, d2, float(value_scale), _native.fptr(bmin),
                     _native.fptr(bmax), nrm_ptr, codes[mode], int(brick_log2), ctypes.byref(h)))
        self._keep = None if wait else (data, self._keep)
        self.handle = h
        self.shape = data.shape
        self.dtype = data.dtype
        self.normals_mode = mode
        self.brick_log2 = brick_log2 or 3
        if half_records:
            self.compact()

    def ready(self) -> bool:
        """True once the layout has completed (always after wait=True)."""
        r = ctypes.c_int(0)
        check(_lib().pvr_volume_ready(self.handle, ctypes.byref(r)))
        if r.value:
            self._keep = None
        return bool(r.value)

    def compact(self) -> bool:
        """Records as halves if every one of their floats is a half exactly
        (the images stay the same); True if they are halves afterwards.  Waits
        for all work queued on the volume's device first; no render of the
        volume may be queued while it runs."""
        c = ctypes.c_int(0)
        check(_lib().pvr_volume_compact(self.handle, ctypes.byref(c)))
        return bool(c.value)

    def device_bytes(self) -> int:
        n = ctypes.c_longlong(0)
        check(_lib().pvr_volume_device_bytes(self.handle, ctypes.byref(n)))
        return int(n.value)

    def record_bytes(self) -> int:
        """16 (float records) or 8 (half records: every value and normal of
        the volume is a half exactly)."""
        n = ctypes.c_int(0)
        check(_lib().pvr_volume_record_bytes(self.handle, ctypes.byref(n)))
        return int(n.value)

    def records_exact(self) -> bool:
        """True if the records hold the values and normals exactly (False:
        half records with the normals rounded to half)."""
        e = ctypes.c_int(0)
        check(_lib().pvr_volume_records_exact(self.handle, ctypes.byref(e)))
        return bool(e.value)

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


_RECORD_MODES = {"float": 0, "half_exact": 1, "half_normals": 2}


def set_compact_records(mode) -> None:
    """Record form of volumes laid out from now on: "float" (or False; 16-byte
    float records), "half_exact" (or True; 8-byte half records where every
    value and normal component is a half exactly: identical images) or
    "half_normals" (half records for volumes whose values are halves exactly
    -- uint8 and float16 -- with the normal components rounded to half)."""
    if isinstance(mode, bool):
        mode = "half_exact" if mode else "float"
    if mode not in _RECORD_MODES:
        raise ValueError(f"record mode must be one of {sorted(_RECORD_MODES)}, got {mode!r}")
    check(_lib().pvr_set_compact_records(_RECORD_MODES[mode]))


def get_compact_records() -> str:
    m = ctypes.c_int(0)
    check(_lib().pvr_get_compact_records(ctypes.byref(m)))
    return {v: k for k, v in _RECORD_MODES.items()}[m.value]


_ARITHMETIC = {"fast": 0, "exact": 1}


def set_arithmetic(mode: str) -> None:
    """Arithmetic of renders queued from now on, on every entry point:
    "fast" (the default: FMA-contracted shading with hardware exp and
    1/sqrt, within 1 LSB per RGBA8 channel of "exact") or "exact" (every
    operation rounded as the CPU oracle rounds it: bit-identical images)."""
    if mode not in _ARITHMETIC:
        raise ValueError(f"arithmetic must be 'fast' or 'exact', got {mode!r}")
    check(_lib().pvr_set_arithmetic(_ARITHMETIC[mode]))


def get_arithmetic() -> str:
    m = ctypes.c_int(0)
    check(_lib().pvr_get_arithmetic(ctypes.byref(m)))
    return {v: k for k, v in _ARITHMETIC.items()}[m.value]


class arithmetic:
    """Context manager: ``with arithmetic("exact"): ...`` renders with the
    given arithmetic and restores the previous one on exit."""

    def __init__(self, mode: str):
        self.mode = mode

    def __enter__(self):
        self.prev = get_arithmetic()
        set_arithmetic(self.mode)
        return self

    def __exit__(self, *exc):
        set_arithmetic(self.prev)
        return False


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

    @classmethod
    def on_device(cls, color_tf, opacity_tf, size: Optional[int] = None, stream=None) -> "DeviceLUT":
        """A LUT built on the GPU from the transfer functions' control points."""
        n = int(size or max(color_tf.lut_size, opacity_tf.lut_size))
        lut = cls(rgba=np.zeros((n, 4), np.float32))
        lut.build(color_tf, opacity_tf, n, stream)
        return lut

    def build(self, color_tf, opacity_tf, size: Optional[int] = None, stream=None) -> None:
        """Rebuild the table on the GPU from control points (``pvr_lut_build``,
        queued on ``stream``): the same float32 entries as ``rgba_lut`` computes
        on the host.  No batch reading this LUT may be in flight."""
        n = int(size or max(color_tf.lut_size, opacity_tf.lut_size))
        cx = np.ascontiguousarray([float(p[0]) for p in color_tf.control_points], np.float64)
        crgb = np.ascontiguousarray([[float(c) for c in p[1]] for p in color_tf.control_points], np.float64)
        ox = np.ascontiguousarray([float(p[0]) for p in opacity_tf.control_points], np.float64)
        oa = np.ascontiguousarray([float(p[1]) for p in opacity_tf.control_points], np.float64)
        s = getattr(stream, "cuda_stream", stream)
        check(_lib().pvr_lut_build(self.handle, cx.ctypes.data, crgb.ctypes.data, len(cx), ox.ctypes.data,
                                   oa.ctypes.data, len(ox), n, s))
        self.size = n

    def read(self) -> np.ndarray:
        """The table as (size, 4) float32 (waits for the device)."""
        out = np.empty((self.size, 4), np.float32)
        check(_lib().pvr_lut_read(self.handle, out.ctypes.data))
        return out

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


def _ptr(x, n: int = 0, dtype: str = "", what: str = "buffer") -> Optional[int]:
    """Device address of an output: None, a raw device pointer (int, taken
    as it is), or a CUDA tensor of at least n elements of dtype."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if not getattr(x, "is_cuda", False):
        raise TypeError(f"{what} must be a CUDA tensor or a device pointer")
    if dtype and str(x.dtype) != f"torch.{dtype}":
        raise TypeError(f"{what} must be {dtype}, got {x.dtype}")
    if x.numel() < n or not x.is_contiguous():
        raise ValueError(f"{what} must be contiguous with at least {n} elements")
    return int(x.data_ptr())


_F3 = ctypes.c_float * 3


def _f3(v) -> "ctypes.Array":
    return _F3(float(v[0]), float(v[1]), float(v[2]))


def fill_camera(camera, width: int, height: int, view, proj, pos) -> None:
    """Orbit camera -> float32 view / projection / position, computed natively
    in double precision (``pvr_camera_spherical``) into the ctypes arrays
    ``view`` (16), ``proj`` (16) and ``pos`` (3).  Same construction as
    ``Camera.get_view_matrix`` / ``get_projection_matrix`` /
    ``get_camera_vectors`` (pyvr/camera/camera.py:292-369,
    pyvr/camera/control.py:238-351), agreeing with them to float32 rounding,
    at a few microseconds instead of a few hundred.  A camera whose up vector
    ends parallel to the view direction has a basis made of rounding noise;
    that case takes the ``Camera`` methods' matrices."""
    rc = _lib().pvr_camera_spherical(
        _f3(camera.target), float(camera.azimuth), float(camera.elevation), float(camera.roll),
        float(camera.distance), _f3(camera.init_pos), _f3(camera.init_up), float(camera.fov),
        float(camera.near_plane), float(camera.far_plane), float(width) / float(height),
        view, proj, pos)
    if rc == _native.PVR_ERR_VALUE and b"parallel" in _lib().pvr_last_error():
        from .renderer import camera_uniforms
        v, p, c = camera_uniforms(camera, width, height)
        for dst, src in ((view, v), (proj, p), (pos, c)):
            for i, x in enumerate(src.ravel().tolist()):
                dst[i] = x
        return
    check(rc)


def job_camera_uniforms(camera, width: int, height: int):
    """(view, proj, position) float32 numpy arrays as the batch path computes
    them (``fill_camera``)."""
    view = np.zeros((4, 4), np.float32)
    proj = np.zeros((4, 4), np.float32)
    pos = np.zeros(3, np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    fill_camera(camera, width, height, view.ctypes.data_as(fp), proj.ctypes.data_as(fp),
                pos.ctypes.data_as(fp))
    return view, proj, pos


def fill_job(j: _native.PvrJob, volume: int, lut: int, camera, light, config, width: int,
             height: int, d_rgba8: Optional[int] = None, d_rgba32f: Optional[int] = None,
             d_counters: Optional[int] = None) -> None:
    """Fill a ``pvr_job`` in place from raw handles / device addresses (ints)
    and camera / light / config objects (pyvr's or this package's)."""
    fill_camera(camera, width, height, j.view, j.proj, j.camera_pos)
    j.volume = volume
    j.lut = lut
    j.width = width
    j.height = height
    lp, lt = light.position, light.target
    j.light_pos[0], j.light_pos[1], j.light_pos[2] = float(lp[0]), float(lp[1]), float(lp[2])
    j.light_target[0], j.light_target[1], j.light_target[2] = float(lt[0]), float(lt[1]), float(lt[2])
    j.ambient = float(light.ambient_intensity)
    j.diffuse = float(light.diffuse_intensity)
    j.step_size = float(config.step_size)
    j.reference_step_size = float(config.reference_step_size)
    j.max_steps = int(config.max_steps)
    j.d_rgba8 = d_rgba8
    j.d_rgba32f = d_rgba32f
    j.d_counters = d_counters


def make_job_struct(job: RenderJob, out: Optional[_native.PvrJob] = None) -> _native.PvrJob:
    """A ``pvr_job`` for ``job``.  The camera goes through ``fill_camera``
    (native double-precision setup), so an oracle scene for a batch render is
    built from ``job_camera_uniforms``."""
    j = out if out is not None else _native.PvrJob()
    n = int(job.width) * int(job.height) * 4
    fill_job(j, job.volume.handle.value, job.lut.handle.value, job.camera, job.light, job.config,
             int(job.width), int(job.height), _ptr(job.out_rgba8, n, "uint8", "out_rgba8"),
             _ptr(job.out_rgba32f, n, "float32", "out_rgba32f"), _ptr(job.counters, 2, "int64", "counters"))
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


def render_static(structs, n: int, tuning: Optional["Tuning"] = None, stream=None) -> None:
    """Queue n prepared PvrJob structs through ``pvr_batch_render_static``:
    the batch march with no launcher and no memory allocation (scratch in a
    static device array; at most 6144 jobs per call; calls that may overlap on
    the GPU must be ordered, e.g. on one stream)."""
    t = tuning.c() if tuning is not None else None
    s = getattr(stream, "cuda_stream", stream)
    check(_lib().pvr_batch_render_static(ctypes.cast(structs, ctypes.c_void_p), int(n),
                                         ctypes.addressof(t) if t is not None else None, s))
