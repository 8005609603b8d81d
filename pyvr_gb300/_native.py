"""Build and load ``libpyvr_gb300.so``, the CUDA (sm_103a) library behind the C ABI
declared in ``include/pyvr_gb300.h``.

The library is compiled in-tree with nvcc (one object per ``csrc/*.cu``, built
in parallel, then linked).  There is no CPU fallback: if the library cannot
be built or loaded, every renderer call raises.
"""

from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB_PATH = os.path.join(PKG, "libpyvr_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: no implicit multiply-add contraction; the kernels write
# fmaf() where a fused operation is meant (see csrc/pvr_device.cuh).
# -ffp-contract=off: the host-side derivations (matrix inverses, light
# direction) must not be fused into FMAs either -- aarch64 compilers fuse by
# default, x86-64 ones do not, and the results must not depend on the host.
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fno-fast-math", "-Xcompiler", "-ffp-contract=off", f"-I{INCLUDE}"]

# status codes of include/pyvr_gb300.h
PVR_OK, PVR_ERR_VALUE, PVR_ERR_TYPE, PVR_ERR_STATE, PVR_ERR_CUDA, PVR_ERR_NOMEM, PVR_ERR_TIMEOUT = range(7)
PVR_U8, PVR_F16, PVR_F32 = 0, 1, 2


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the pyvr_gb300 CUDA library cannot be built")
    return exe


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    files = _sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC)
                          if f.endswith((".cuh", ".h"))]
    files.append(os.path.join(INCLUDE, "pyvr_gb300.h"))
    return files


def needs_build() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(f) > t for f in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every csrc/*.cu for sm_103a and link the shared library."""
    if not force and not needs_build():
        return LIB_PATH
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        cmd = [exe, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = [exe, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None

# exported symbol -> (restype, argtypes)
_VP, _I, _F, _LL = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_longlong
_FP = ctypes.POINTER(ctypes.c_float)
SIGNATURES = {
    "pvr_abi_version": (_I, []),
    "pvr_last_error": (ctypes.c_char_p, []),
    "pvr_create": (_I, [_I, _I, ctypes.POINTER(_VP)]),
    "pvr_destroy": (_I, [_VP]),
    "pvr_load_volume": (_I, [_VP, _VP, _I, _I, _I, _I, _F, _FP, _FP]),
    "pvr_load_normals": (_I, [_VP, _VP]),
    "pvr_set_lut": (_I, [_VP, _VP, _I]),
    "pvr_set_camera": (_I, [_VP, _FP, _FP, _FP]),
    "pvr_set_light": (_I, [_VP, _FP, _FP, _F, _F]),
    "pvr_set_config": (_I, [_VP, _F, _I, _F]),
    "pvr_render": (_I, [_VP, _VP, _VP]),
    "pvr_volume_record_bytes": (_I, [_VP, ctypes.POINTER(_I)]),
    "pvr_set_compact_records": (_I, [_I]),
    "pvr_get_compact_records": (_I, [ctypes.POINTER(_I)]),
    "pvr_volume_records_exact": (_I, [_VP, ctypes.POINTER(_I)]),
    "pvr_set_arithmetic": (_I, [_I]),
    "pvr_reserve_volume_memory": (_I, [_LL]),
    "pvr_host_alloc": (_I, [_LL, ctypes.POINTER(_VP)]),
    "pvr_volume_create_async": (_I, [_VP, _I, _I, _I, _I, _F, _FP, _FP, _VP, _I, _I, ctypes.POINTER(_VP)]),
    "pvr_volume_ready": (_I, [_VP, ctypes.POINTER(_I)]),
    "pvr_host_free": (_I, [_VP]),
    "pvr_get_arithmetic": (_I, [ctypes.POINTER(_I)]),
    "pvr_volume_compact": (_I, [_VP, ctypes.POINTER(_I)]),
    "pvr_render_pinned": (_I, [_VP, ctypes.POINTER(_VP)]),
    "pvr_render_device": (_I, [_VP, _VP, _VP, _VP]),
    "pvr_last_sample_count": (_I, [_VP, ctypes.POINTER(_LL)]),
    "pvr_last_sample_counts": (_I, [_VP, ctypes.POINTER(_LL), ctypes.POINTER(_LL)]),
    "pvr_device_bytes": (_I, [_VP, ctypes.POINTER(_LL)]),
    "pvr_frame_constants": (_I, [_FP, _FP, _FP, _FP, _FP, _FP, _F, _F, _FP]),
    "pvr_compute_normals": (_I, [_VP]),
    "pvr_set_tuning": (_I, [_VP, _VP]),
    "pvr_volume_create": (_I, [_VP, _I, _I, _I, _I, _F, _FP, _FP, _VP, _I, _I, ctypes.POINTER(_VP)]),
    "pvr_volume_destroy": (_I, [_VP]),
    "pvr_volume_release": (_I, [_VP, _VP]),
    "pvr_volume_device_bytes": (_I, [_VP, ctypes.POINTER(_LL)]),
    "pvr_volume_read_normals": (_I, [_VP, _VP]),
    "pvr_lut_create": (_I, [_VP, _I, ctypes.POINTER(_VP)]),
    "pvr_lut_update": (_I, [_VP, _VP, _I]),
    "pvr_lut_destroy": (_I, [_VP]),
    "pvr_batch_create": (_I, [_I, _I, ctypes.POINTER(_VP)]),
    "pvr_batch_destroy": (_I, [_VP]),
    "pvr_batch_set_tuning": (_I, [_VP, _VP]),
    "pvr_batch_get_tuning": (_I, [_VP, _VP]),
    "pvr_batch_render": (_I, [_VP, _VP, _I, _VP]),
    "pvr_batch_synchronize": (_I, [_VP]),
    "pvr_batch_render_static": (_I, [_VP, _I, _VP, _VP]),
    "pvr_server_create": (_I, [_VP, ctypes.POINTER(_VP)]),
    "pvr_server_submit": (_I, [_VP, _VP]),
    "pvr_server_poll": (_I, [_VP, _VP, _I, _I, ctypes.POINTER(_I)]),
    "pvr_server_pause": (_I, [_VP, _I]),
    "pvr_server_get_stats": (_I, [_VP, _VP]),
    "pvr_server_reset_stats": (_I, [_VP]),
    "pvr_server_last_error": (ctypes.c_char_p, [_VP]),
    "pvr_server_destroy": (_I, [_VP]),
    "pvr_lut_build": (_I, [_VP, _VP, _VP, _I, _VP, _VP, _I, _I, _VP]),
    "pvr_lut_read": (_I, [_VP, _VP]),
    "pvr_diff_forward": (_I, [_VP, _VP, _VP, _VP]),
    "pvr_diff_backward": (_I, [_VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "pvr_camera_spherical": (_I, [_FP, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                  _FP, _FP, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_double, _FP, _FP, _FP]),
}

PVR_NORMALS_NONE, PVR_NORMALS_GIVEN, PVR_NORMALS_DEVICE = 0, 1, 2


class PvrTuning(ctypes.Structure):
    """pvr_tuning of include/pyvr_gb300.h."""
    _fields_ = [("tile_w", _I), ("tile_h", _I), ("steps_per_iter", _I), ("blocks_per_sm", _I)]


_D = ctypes.c_double
PVR_CAMERA_MATRICES, PVR_CAMERA_ORBIT = 0, 1


class PvrRequest(ctypes.Structure):
    """pvr_request of include/pyvr_gb300.h."""
    _fields_ = [("volume", _VP), ("lut", _VP), ("camera_mode", _I),
                ("view", _F * 16), ("proj", _F * 16), ("camera_pos", _F * 3),
                ("target", _F * 3), ("azimuth", _D), ("elevation", _D), ("roll", _D), ("distance", _D),
                ("init_pos", _F * 3), ("init_up", _F * 3), ("fov", _D), ("near_plane", _D), ("far_plane", _D),
                ("light_pos", _F * 3), ("light_target", _F * 3), ("ambient", _F), ("diffuse", _F),
                ("step_size", _F), ("reference_step_size", _F), ("max_steps", _I),
                ("width", _I), ("height", _I), ("out_rgba8", _VP), ("out_pinned", _I),
                ("wait_event", _VP), ("tag", ctypes.c_ulonglong)]


class PvrCompletion(ctypes.Structure):
    """pvr_completion of include/pyvr_gb300.h."""
    _fields_ = [("tag", ctypes.c_ulonglong), ("status", _I), ("t_submit_ns", _LL), ("t_launch_ns", _LL),
                ("t_done_ns", _LL)]


class PvrServerConfig(ctypes.Structure):
    """pvr_server_config of include/pyvr_gb300.h."""
    _fields_ = [("max_batch", _I), ("slots", _I), ("per_frame", _I), ("instrument", _I), ("linger_us", _I),
                ("tuning", PvrTuning), ("batch_pixels", _LL)]


class PvrServerStats(ctypes.Structure):
    """pvr_server_stats of include/pyvr_gb300.h."""
    _fields_ = [("submitted", _LL), ("batches", _LL), ("jobs", _LL), ("max_jobs", _I), ("kernel_ms", _D),
                ("inbox_samples", _LL), ("shaded_samples", _LL), ("algorithmic_bytes", _D), ("queued", _LL),
                ("instrumented_batches", _LL), ("instrumented_jobs", _LL)]


class PvrDiffView(ctypes.Structure):
    """pvr_diff_view of include/pyvr_gb300.h."""
    _fields_ = [("view", _F * 16), ("proj", _F * 16), ("camera_pos", _F * 3)]


class PvrDiffScene(ctypes.Structure):
    """pvr_diff_scene of include/pyvr_gb300.h."""
    _fields_ = [("volume", _VP), ("normals", _VP), ("d", _I), ("h", _I), ("w", _I),
                ("value_scale", _F), ("lut", _VP), ("lut_size", _I),
                ("min_bounds", _F * 3), ("max_bounds", _F * 3),
                ("light_pos", _F * 3), ("light_target", _F * 3), ("ambient", _F), ("diffuse", _F),
                ("step_size", _F), ("reference_step_size", _F), ("max_steps", _I),
                ("width", _I), ("height", _I), ("n_views", _I), ("views", _VP)]


class PvrJob(ctypes.Structure):
    """pvr_job of include/pyvr_gb300.h."""
    _fields_ = [("volume", _VP), ("lut", _VP), ("width", _I), ("height", _I),
                ("view", _F * 16), ("proj", _F * 16), ("camera_pos", _F * 3),
                ("light_pos", _F * 3), ("light_target", _F * 3), ("ambient", _F), ("diffuse", _F),
                ("step_size", _F), ("reference_step_size", _F), ("max_steps", _I),
                ("d_rgba8", _VP), ("d_rgba32f", _VP), ("d_counters", _VP)]


def load(path: str = LIB_PATH, build_if_missing: bool = True):
    """Load (building first if needed) and type the exported functions."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing and (not os.path.exists(path) or (path == LIB_PATH and needs_build())):
        build()
    if not os.path.exists(path):
        raise RuntimeError(f"pyvr_gb300 CUDA library missing at {path}")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class PvrError(RuntimeError):
    pass


_EXC = {PVR_ERR_VALUE: ValueError, PVR_ERR_TYPE: TypeError, PVR_ERR_STATE: RuntimeError,
        PVR_ERR_CUDA: RuntimeError, PVR_ERR_NOMEM: MemoryError, PVR_ERR_TIMEOUT: TimeoutError}


def check(rc: int) -> None:
    """Raise the Python exception the reference would raise for this status."""
    if rc == PVR_OK:
        return
    msg = _lib.pvr_last_error().decode(errors="replace") if _lib is not None else f"status {rc}"
    raise _EXC.get(rc, PvrError)(msg)


def fptr(arr):
    return arr.ctypes.data_as(_FP)
