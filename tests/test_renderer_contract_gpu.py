"""The renderer's API contract, as pyvr's own renderer tests state it
(tests/test_moderngl_renderer/test_volume_renderer.py: defaults, setters and
getters, type errors with the reference's messages, call shapes), run on the
CUDA backend instead of a mocked GL context."""

import numpy as np
import pytest

from pyvr_gb300 import (Camera, Light, OpacityTransferFunction, RenderConfig, Volume, VolumeRenderer,
                        compute_normal_volume)
from pyvr_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _volume(n=12, normals=True, seed=0):
    data = W.value_noise((n, n, n), seed=seed).astype(np.float32)
    return Volume(data=data, normals=compute_normal_volume(data) if normals else None)


def test_defaults_and_custom_construction():
    with VolumeRenderer() as r:
        assert (r.width, r.height) == (512, 512)
        assert r.config.step_size == 0.01 and r.config.max_steps == 500  # balanced preset
        assert isinstance(r.light, Light) and isinstance(r.get_light(), Light)
    cfg = RenderConfig(step_size=0.005, max_steps=500)
    with VolumeRenderer(width=1024, height=768, config=cfg, light=Light.ambient_only(0.5)) as r:
        assert (r.width, r.height) == (1024, 768)
        assert r.get_config() is cfg and r.light.ambient_intensity == 0.5


@pytest.mark.parametrize("bad", [object(), np.zeros((4, 4, 4)), "volume"])
def test_type_errors_carry_the_reference_messages(bad):
    with pytest.raises(TypeError, match="Expected RenderConfig instance"):
        VolumeRenderer(config=bad)
    with pytest.raises(TypeError, match="Expected Light instance"):
        VolumeRenderer(light=bad)
    with VolumeRenderer(32, 32) as r:
        with pytest.raises(TypeError, match="Expected Volume instance"):
            r.load_volume(bad)
        with pytest.raises(TypeError, match="Expected Camera instance"):
            r.set_camera(bad)
        with pytest.raises(TypeError, match="Expected Light instance"):
            r.set_light(bad)
        with pytest.raises(TypeError, match="Expected RenderConfig instance"):
            r.set_config(bad)


def test_setters_and_getters():
    vol, cam = _volume(), Camera.front_view(distance=3.0)
    with VolumeRenderer(32, 24) as r:
        assert r.get_volume() is None and r.get_camera() is None
        r.load_volume(vol)
        r.set_camera(cam)
        light = Light.point_light(position=[2.0, 2.0, 2.0]) if hasattr(Light, "point_light") else Light.default()
        r.set_light(light)
        r.set_config(RenderConfig.ultra_quality())
        assert r.get_volume() is vol and r.get_camera() is cam and r.get_light() is light
        assert r.config.step_size == 0.001 and r.config.max_steps == 2000


def test_tiny_volume_minimal_setup_and_repeat_frames():
    with VolumeRenderer(40, 30) as r:
        r.set_camera(Camera.front_view(distance=3.0))
        frame = r.render()  # camera only, no volume: a transparent frame of the right size
        assert isinstance(frame, bytes) and len(frame) == 40 * 30 * 4 and not any(frame)
        r.load_volume(Volume(data=np.random.default_rng(1).random((1, 1, 1)).astype(np.float32)))
        r.set_transfer_functions(W.standin_colormap(0), OpacityTransferFunction.linear(0.0, 0.8))
        a, b = r.render(), r.render()
        assert a == b and len(a) == 40 * 30 * 4


def test_render_before_camera_or_lut_is_a_reasonable_error():
    with VolumeRenderer(16, 16) as r:
        r.load_volume(_volume())
        with pytest.raises((ValueError, RuntimeError, AttributeError)):
            r.render()
        r.set_camera(Camera.isometric_view())
        with pytest.raises((ValueError, RuntimeError, AttributeError)):
            r.render()


def test_volume_replacement_and_custom_bounds():
    cam = Camera.isometric_view(distance=3.0)
    with VolumeRenderer(48, 48) as r:
        r.set_camera(cam)
        r.set_transfer_functions(W.standin_colormap(1), OpacityTransferFunction.linear(0.0, 0.5))
        r.load_volume(_volume(seed=1))
        first = r.render()
        small = _volume(seed=1)
        small.min_bounds = np.full(3, -0.25, np.float32)
        small.max_bounds = np.full(3, 0.25, np.float32)
        r.load_volume(small)
        second = r.render()
        assert first != second  # the box is smaller on screen
        alpha = np.frombuffer(second, np.uint8).reshape(48, 48, 4)[..., 3]
        assert alpha[:8].sum() == 0 and alpha[-8:].sum() == 0 and alpha.sum() > 0


def test_light_and_config_changes_take_effect():
    with VolumeRenderer(32, 32) as r:
        r.load_volume(_volume(seed=2))
        r.set_camera(Camera.front_view(distance=3.0))
        r.set_transfer_functions(W.standin_colormap(2), OpacityTransferFunction.linear(0.0, 0.5))
        frames = []
        for light in (Light.default(), Light.ambient_only(0.2), Light.directional([1, -1, 0], 0.1, 0.9)):
            r.set_light(light)
            frames.append(r.render())
        for cfg in (RenderConfig.fast(), RenderConfig.high_quality()):
            r.set_config(cfg)
            frames.append(r.render())
        assert len(set(frames)) == len(frames)


def test_normals_shape_is_checked():
    vol = _volume(normals=False)
    vol.normals = np.zeros((12, 12, 12, 2), np.float32)
    with VolumeRenderer(16, 16) as r:
        with pytest.raises(ValueError):
            r.load_volume(vol)


def test_render_bytes_come_from_the_pinned_image():
    with VolumeRenderer(40, 24) as r:
        r.load_volume(_volume(seed=3))
        r.set_camera(Camera.isometric_view(distance=3.0))
        r.set_transfer_functions(W.standin_colormap(3), OpacityTransferFunction.linear(0.0, 0.5))
        a = r.render()
        assert isinstance(a, bytes) and a == r.render_array().tobytes()
        r.set_camera(Camera.front_view(distance=3.0))
        b = r.render()
        assert b != a and b == r.render_array().tobytes()
        r.set_camera(Camera.isometric_view(distance=3.0))
        assert r.render_array().tobytes() == a  # the first result was a copy, not a view
