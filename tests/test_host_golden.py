"""Host-side value objects against golden vectors produced by pyvr itself
(tests/golden/make_golden.py imports the reference and records them)."""

import os

import numpy as np
import pytest

from pyvr_gb300 import (Camera, ColorTransferFunction, Light, OpacityTransferFunction,
                        RenderConfig, Volume, compute_normal_volume)
from pyvr_gb300.renderer import rgba_lut

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_host.npz"))


def _camera(p):
    return Camera.from_spherical(
        target=np.array(p[0:3], dtype=np.float32), azimuth=float(p[3]), elevation=float(p[4]),
        roll=float(p[5]), distance=float(p[6]), fov=float(p[7]),
        init_pos=np.array(p[9:12], dtype=np.float32), init_up=np.array(p[12:15], dtype=np.float32))


@pytest.mark.parametrize("i", range(len(G["camera_params"])))
def test_camera_matches_reference(i):
    p = G["camera_params"][i]
    cam = _camera(p)
    pos, up = cam.get_camera_vectors()
    np.testing.assert_allclose(pos, G["camera_pos"][i], rtol=0, atol=1e-12)
    np.testing.assert_allclose(up, G["camera_up"][i], rtol=0, atol=1e-12)
    # float32 matrices: equal up to the last bit of entries that are ~0
    np.testing.assert_allclose(cam.get_view_matrix(), G["camera_view"][i], rtol=2e-7, atol=1e-12)
    np.testing.assert_array_equal(cam.get_projection_matrix(float(p[8])), G["camera_proj"][i])


@pytest.mark.parametrize("i", range(len(G["camera_params"])))
def test_batch_camera_setup_matches_reference(i, native_lib):
    # the batch path's native camera setup takes the reference's float32
    # steps in float32: its float32 matrices equal the reference's as the
    # Camera methods' do (up to the last bit of entries that are ~0)
    from pyvr_gb300.batch import job_camera_uniforms
    p = G["camera_params"][i]
    view, proj, pos = job_camera_uniforms(_camera(p), float(p[8]), 1.0)
    np.testing.assert_allclose(pos, G["camera_pos"][i].astype(np.float32), rtol=0, atol=0)
    np.testing.assert_allclose(view, G["camera_view"][i], rtol=2e-7, atol=1e-12)
    np.testing.assert_allclose(proj, G["camera_proj"][i], rtol=2e-7, atol=0)


def test_batch_camera_setup_equals_camera_methods(native_lib):
    # 4000 orbit cameras: the native setup and Camera.get_view_matrix /
    # get_projection_matrix / get_camera_vectors give the same float32 arrays,
    # every entry bit for bit except the ones that are rounding noise of 0
    from pyvr_gb300.batch import job_camera_uniforms
    from pyvr_gb300.renderer import camera_uniforms
    rng = np.random.default_rng(11)
    for k in range(4000):
        cam = Camera.from_spherical(np.zeros(3, np.float32), float(rng.uniform(-4, 4)),
                                    float(rng.uniform(-1.5, 1.5)), float(rng.uniform(-0.5, 0.5)) if k % 2 else 0.0,
                                    float(rng.uniform(2.0, 5.0)))
        w, h = [(512, 512), (1024, 768), (37, 91)][k % 3]
        for a, b in zip(job_camera_uniforms(cam, w, h), camera_uniforms(cam, w, h)):
            differ = a != b
            assert np.all(np.abs(a[differ]) < 1e-12) and np.all(np.abs(b[differ]) < 1e-12), (k, a, b)


def test_batch_camera_setup_rejects_bad_cameras(native_lib):
    import ctypes
    f3 = ctypes.c_float * 3
    f16 = ctypes.c_float * 16
    args = lambda **kw: [f3(0, 0, 0), 0.0, 0.0, 0.0, kw.get("dist", 3.0), f3(*kw.get("pos", (1, 0, 0))),
                         f3(0, 0, 1), kw.get("fov", 0.785), 0.1, kw.get("far", 100.0), 1.0,
                         f16(), f16(), f3()]
    assert native_lib.pvr_camera_spherical(*args()) == 0
    for bad in (dict(dist=0.0), dict(dist=-1.0), dict(pos=(0, 0, 0)), dict(fov=0.0), dict(fov=3.2),
                dict(far=0.05)):
        assert native_lib.pvr_camera_spherical(*args(**bad)) == 1, bad  # PVR_ERR_VALUE
    # up parallel to the view direction: no basis to give
    bad = args(pos=(0, 0, 2))
    bad[6] = f3(0, 0, 1)
    assert native_lib.pvr_camera_spherical(*bad) == 1
    assert b"parallel" in native_lib.pvr_last_error()


def test_camera_default_position():
    # reference tests/test_camera/test_control.py:22-32: default init -> [0,0,3]-like pins
    cam = Camera.from_spherical(np.zeros(3, np.float32), np.pi / 4, np.pi / 6, 0.0, 3.0)
    pos, _ = cam.get_camera_vectors()
    np.testing.assert_allclose(pos, [1.8371173, 1.8371173, 1.5], atol=1e-6)


def test_lights_match_reference():
    lights = [Light.directional([1, -1, 0], ambient=0.2, diffuse=0.8), Light.default(),
              Light.point_light(np.array([2.0, 3.0, -1.0]), ambient=0.1, diffuse=0.7),
              Light.ambient_only(0.4),
              Light.directional(np.array([0.0, 0.0, -2.0]), 0.3, 0.6, distance=5.0)]
    got = np.array([[*l.position, *l.target, l.ambient_intensity, l.diffuse_intensity]
                    for l in lights])
    np.testing.assert_array_equal(got, G["light_uniforms"])


def test_config_presets_match_reference():
    got = np.array([[c.step_size, c.max_steps, float(c.early_ray_termination),
                     c.opacity_threshold, c.reference_step_size, c.estimate_samples_per_ray()]
                    for c in (RenderConfig.preview(), RenderConfig.fast(),
                              RenderConfig.balanced(), RenderConfig.high_quality(),
                              RenderConfig.ultra_quality())])
    np.testing.assert_array_equal(got, G["config_presets"])


def test_luts_match_reference():
    otfs = [OpacityTransferFunction.linear(0.0, 0.1),
            OpacityTransferFunction.one_step(0.4, 0.05, 0.9),
            OpacityTransferFunction.peaks([0.3, 0.7], opacity=0.9, eps=0.05, base=0.1),
            OpacityTransferFunction([(0.0, 0.0), (0.3, 0.1), (0.8, 0.9), (1.0, 0.5)], lut_size=100)]
    ctfs = [ColorTransferFunction.grayscale(),
            ColorTransferFunction([(0.0, (0.0, 0.0, 0.0)), (0.5, (1.0, 0.0, 0.0)),
                                   (1.0, (1.0, 1.0, 1.0))]),
            ColorTransferFunction.two_color_ramp((0.1, 0.2, 0.3), (0.9, 0.5, 0.0), lut_size=64)]
    for i, o in enumerate(otfs):
        np.testing.assert_array_equal(o.to_lut(), G[f"otf_lut_{i}"])
        np.testing.assert_array_equal(o.to_lut(37), G[f"otf_lut_{i}_37"])
    for i, c in enumerate(ctfs):
        np.testing.assert_array_equal(c.to_lut(), G[f"ctf_lut_{i}"])
        np.testing.assert_array_equal(c.to_lut(37), G[f"ctf_lut_{i}_37"])
    # combined table: size = max of the two lut_size values (manager.py:163-166)
    lut = rgba_lut(ctfs[2], otfs[3])
    assert lut.shape == (100, 4) and lut.dtype == np.float32


@pytest.mark.parametrize("name", ["rand_f32", "rand_u8", "flat"])
def test_normals_match_reference(name):
    out = compute_normal_volume(G[f"normals_in_{name}"])
    assert out.dtype == np.float32
    np.testing.assert_array_equal(out, G[f"normals_out_{name}"])


def test_opacity_lut_endpoints():
    # reference tests/test_transferfunctions/test_opacity.py:31-44
    lut = OpacityTransferFunction.linear(0.2, 0.8).to_lut(256)
    assert lut[0] == pytest.approx(0.2) and lut[-1] == pytest.approx(0.8)


def test_value_object_validation():
    with pytest.raises(ValueError):
        RenderConfig(step_size=0.0)
    with pytest.raises(ValueError):
        RenderConfig(max_steps=0)
    with pytest.raises(ValueError):
        Volume(data=np.zeros((2, 2), np.float32))
    with pytest.raises(ValueError):
        Volume(data=np.zeros((2, 2, 2), np.float32), normals=np.zeros((2, 2, 2, 2), np.float32))
    with pytest.raises(ValueError):
        Light(ambient_intensity=1.5)
    with pytest.raises(ValueError):
        Camera(distance=-1.0)
    from pyvr_gb300 import InvalidControlPointError
    with pytest.raises(InvalidControlPointError):
        OpacityTransferFunction([(0.0, 1.5)])
