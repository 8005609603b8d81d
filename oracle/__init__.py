"""CPU oracle for the pyvr ray-marching path -- TEST INFRASTRUCTURE ONLY.

Loaded by tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline, never by the ``pyvr_gb300`` package.  ``march_ref.c`` is the
float32 restatement of pyvr/shaders/volume.frag.glsl and the GL fixed
function around it (the RGBA8 parity oracle and the timed CPU baseline);
``march_fp64.py`` is the float64 NumPy marcher used for float-image error
statistics.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libpvr_oracle.so")

DTYPES = {np.dtype(np.uint8): 0, np.dtype(np.float16): 1, np.dtype(np.float32): 2}


class OracleScene(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int),
                ("view", ctypes.c_float * 16), ("proj", ctypes.c_float * 16),
                ("cam_pos", ctypes.c_float * 3),
                ("volume", ctypes.c_void_p), ("dtype", ctypes.c_int),
                ("dims", ctypes.c_int * 3), ("value_scale", ctypes.c_float),
                ("normals", ctypes.c_void_p),
                ("bmin", ctypes.c_float * 3), ("bmax", ctypes.c_float * 3),
                ("lut", ctypes.c_void_p), ("lut_size", ctypes.c_int),
                ("step_size", ctypes.c_float), ("reference_step_size", ctypes.c_float),
                ("max_steps", ctypes.c_int),
                ("light_pos", ctypes.c_float * 3), ("light_target", ctypes.c_float * 3),
                ("ambient", ctypes.c_float), ("diffuse", ctypes.c_float)]


def build(force: bool = False) -> str:
    """Compile march_ref.c with gcc (OpenMP, no FP contraction)."""
    src = os.path.join(HERE, "march_ref.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
                           "-fno-fast-math", "-fopenmp", src, "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.oracle_render_rows.argtypes = [ctypes.POINTER(OracleScene), ctypes.c_int,
                                            ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong),
                                            ctypes.c_int]
        _lib.oracle_expf_array.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong]
        _lib.oracle_max_threads.restype = ctypes.c_int
        _lib.oracle_frame_constants.argtypes = [ctypes.POINTER(OracleScene), ctypes.c_void_p]
    return _lib


def _f3(v):
    return (ctypes.c_float * 3)(*[float(x) for x in np.asarray(v, dtype=np.float32)])


def make_scene(scene: dict):
    """Build the C struct; returns (struct, keepalive list)."""
    vol = np.ascontiguousarray(scene["volume"])
    if vol.dtype not in DTYPES:
        vol = vol.astype(np.float32)
    keep = [vol]
    s = OracleScene()
    s.width, s.height = int(scene["width"]), int(scene["height"])
    s.view = (ctypes.c_float * 16)(*np.asarray(scene["view"], np.float32).ravel())
    s.proj = (ctypes.c_float * 16)(*np.asarray(scene["proj"], np.float32).ravel())
    s.cam_pos = _f3(scene["cam_pos"])
    s.volume = vol.ctypes.data
    s.dtype = DTYPES[vol.dtype]
    s.dims = (ctypes.c_int * 3)(*vol.shape)
    s.value_scale = float(scene.get("value_scale", 1.0))
    nrm = scene.get("normals")
    if nrm is not None:
        nrm = np.ascontiguousarray(nrm, dtype=np.float32)
        keep.append(nrm)
        s.normals = nrm.ctypes.data
    s.bmin, s.bmax = _f3(scene["bmin"]), _f3(scene["bmax"])
    lut = np.ascontiguousarray(scene["lut"], dtype=np.float32)
    keep.append(lut)
    s.lut, s.lut_size = lut.ctypes.data, lut.shape[0]
    s.step_size = float(scene["step_size"])
    s.reference_step_size = float(scene["reference_step_size"])
    s.max_steps = int(scene["max_steps"])
    s.light_pos, s.light_target = _f3(scene["light_pos"]), _f3(scene["light_target"])
    s.ambient, s.diffuse = float(scene["ambient"]), float(scene["diffuse"])
    return s, keep


def render(scene: dict, rows=None, want_float: bool = True, nthreads: int = 0,
           want_counts: bool = False):
    """(rgba8 (H,W,4) uint8, float image (H,W,4) or None, in-box sample count);
    with ``want_counts`` the count is an (H, W) int32 array per pixel."""
    s, keep = make_scene(scene)
    H, W = s.height, s.width
    out8 = np.zeros((H, W, 4), dtype=np.uint8)
    outf = np.zeros((H, W, 4), dtype=np.float32) if want_float else None
    counts = np.zeros((H, W), dtype=np.int32) if want_counts else None
    n = ctypes.c_longlong(0)
    r0, r1 = rows if rows is not None else (0, 0)
    rc = lib().oracle_render_rows(ctypes.byref(s), r0, r1, out8.ctypes.data,
                                  None if outf is None else outf.ctypes.data,
                                  None if counts is None else counts.ctypes.data,
                                  ctypes.byref(n), int(nthreads))
    if rc != 0:
        raise ValueError("oracle: singular view or projection matrix")
    return out8, outf, (counts if want_counts else int(n.value))


def frame_constants(scene: dict) -> np.ndarray:
    """The 27 derived per-frame floats (see pvr_frame_constants)."""
    s, keep = make_scene(scene)
    out = np.zeros(27, dtype=np.float32)
    if lib().oracle_frame_constants(ctypes.byref(s), out.ctypes.data) != 0:
        raise ValueError("oracle: singular view or projection matrix")
    return out


def expf(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty_like(x)
    lib().oracle_expf_array(x.ctypes.data, y.ctypes.data, x.size)
    return y


def max_threads() -> int:
    return int(lib().oracle_max_threads())
