"""The C-ABI library builds, loads and exports every symbol include/*.h declares.

No compute call is made here (no GPU needed): only entry points whose
argument checks fail before touching CUDA are called.
"""

import ctypes
import glob
import os
import re

import pytest

from pyvr_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(pvr_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "pvr_render" in names and "pvr_create" in names and len(names) >= 10


def test_library_exports_every_declared_symbol(native_lib):
    missing = [n for n in declared_functions() if not hasattr(native_lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    assert set(declared_functions()) <= set(_native.SIGNATURES)


def test_abi_version(native_lib):
    assert native_lib.pvr_abi_version() == 1


def test_null_handle_errors(native_lib):
    lib = native_lib
    assert lib.pvr_destroy(None) == _native.PVR_OK
    lut = (ctypes.c_float * 4)(0, 0, 0, 0)
    assert lib.pvr_set_lut(None, lut, 1) == _native.PVR_ERR_VALUE
    assert b"null renderer" in lib.pvr_last_error()
    with pytest.raises(ValueError, match="null renderer"):
        _native.check(lib.pvr_set_config(None, 0.01, 10, 0.01))
    out = ctypes.c_void_p()
    assert lib.pvr_create(0, 5, ctypes.byref(out)) == _native.PVR_ERR_VALUE
    assert not out.value


def test_argument_checks_before_any_device_work(native_lib):
    """Entry points added beside the renderer reject bad arguments up front
    (no device is touched, so these run anywhere)."""
    lib = native_lib
    V, E = _native.PVR_OK, _native.PVR_ERR_VALUE
    out = ctypes.c_void_p()
    cfg = _native.PvrServerConfig(0, 3, 0, 0, 0, _native.PvrTuning(0, 0, 0, 0))
    assert lib.pvr_server_create(ctypes.byref(cfg), ctypes.byref(out)) == E and not out.value
    cfg = _native.PvrServerConfig(8, 99, 0, 0, 0, _native.PvrTuning(0, 0, 0, 0))
    assert lib.pvr_server_create(ctypes.byref(cfg), ctypes.byref(out)) == E
    assert lib.pvr_server_create(None, ctypes.byref(out)) == E
    req = _native.PvrRequest()
    assert lib.pvr_server_submit(None, ctypes.byref(req)) == E
    n = ctypes.c_int(0)
    assert lib.pvr_server_poll(None, None, 1, 0, ctypes.byref(n)) == E
    assert lib.pvr_server_destroy(None) == V
    assert lib.pvr_lut_build(None, None, None, 1, None, None, 1, 256, None) == E
    assert lib.pvr_diff_forward(None, None, None, None) == E
    scene = _native.PvrDiffScene()
    assert lib.pvr_diff_forward(ctypes.byref(scene), None, None, None) == E  # no volume / LUT / views
    assert lib.pvr_batch_render_static(None, 1, None, None) == E
    assert lib.pvr_batch_render_static(None, -1, None, None) == E
    assert lib.pvr_batch_render(None, None, 0, None) == E
    cfg = _native.PvrServerConfig(8, 3, 0, 0, 0, _native.PvrTuning(0, 0, 0, 0), -1)
    assert lib.pvr_server_create(ctypes.byref(cfg), ctypes.byref(out)) == E  # negative pixel budget
    assert b"batch_pixels" in lib.pvr_last_error()
    img = ctypes.c_void_p(1)
    assert lib.pvr_render_pinned(None, ctypes.byref(img)) == E and not img.value
    nbytes = ctypes.c_int(0)
    assert lib.pvr_volume_record_bytes(None, ctypes.byref(nbytes)) == E


def test_compact_records_switch(native_lib):
    assert native_lib.pvr_set_compact_records(1) == _native.PVR_OK
    assert native_lib.pvr_set_compact_records(0) == _native.PVR_OK  # back to the default


def test_error_code_mapping():
    for code, exc in [(_native.PVR_ERR_VALUE, ValueError), (_native.PVR_ERR_TYPE, TypeError),
                      (_native.PVR_ERR_STATE, RuntimeError), (_native.PVR_ERR_NOMEM, MemoryError),
                      (_native.PVR_ERR_TIMEOUT, TimeoutError)]:
        with pytest.raises(exc):
            _native.check(code)


def test_frame_constants_match_oracle_bit_for_bit(native_lib):
    """The host-side derivations (double inverses, light direction, box
    reciprocal, step ratio) agree with the oracle's to the bit."""
    import numpy as np

    import oracle
    from pyvr_gb300 import Camera, Light, RenderConfig
    from pyvr_gb300 import workloads as W
    from pyvr_gb300.renderer import camera_uniforms

    rng = np.random.default_rng(3)
    lights = [Light.directional([1, -1, 0]), Light.default(), Light.ambient_only(0.3),
              Light.point_light(np.array([0.3, -2.0, 5.0]))]
    for i in range(40):
        cam = Camera.from_spherical(rng.uniform(-0.5, 0.5, 3).astype(np.float32),
                                    float(rng.uniform(-6, 6)), float(rng.uniform(-1.5, 1.5)),
                                    float(rng.uniform(-1, 1)), float(rng.uniform(0.5, 6)),
                                    fov=float(rng.uniform(0.2, 2.5)))
        w, h = int(rng.integers(1, 2000)), int(rng.integers(1, 2000))
        view, proj, pos = camera_uniforms(cam, w, h)
        light = lights[i % len(lights)]
        bmin = rng.uniform(-2, 0, 3).astype(np.float32)
        bmax = bmin + rng.uniform(0.1, 3, 3).astype(np.float32)
        cfg = RenderConfig(step_size=float(rng.uniform(0.001, 0.05)), max_steps=10,
                           reference_step_size=float(rng.uniform(0.002, 0.03)))
        lp = np.asarray(light.position, np.float32)
        lt = np.asarray(light.target, np.float32)
        got = np.zeros(27, np.float32)
        f = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        assert native_lib.pvr_frame_constants(f(view), f(proj), f(lp), f(lt), f(bmin), f(bmax),
                                              cfg.step_size, cfg.reference_step_size,
                                              got.ctypes.data_as(ctypes.POINTER(ctypes.c_float))) == 0
        scene = dict(width=w, height=h, view=view, proj=proj, cam_pos=pos,
                     volume=np.zeros((2, 2, 2), np.float32), bmin=bmin, bmax=bmax,
                     lut=np.zeros((1, 4), np.float32), step_size=cfg.step_size,
                     reference_step_size=cfg.reference_step_size, max_steps=10,
                     light_pos=lp, light_target=lt, ambient=0.2, diffuse=0.8)
        want = oracle.frame_constants(scene)
        # equal values (a structurally zero inverse entry may be +0 or -0)
        np.testing.assert_array_equal(got, want)


def test_job_outputs_must_be_device_buffers():
    torch = pytest.importorskip("torch")
    from pyvr_gb300.batch import _ptr
    assert _ptr(None) is None and _ptr(123456) == 123456  # raw device pointers pass as they are
    with pytest.raises(TypeError, match="CUDA"):
        _ptr(torch.zeros(64, dtype=torch.uint8), 64, "uint8", "out_rgba8")
