"""The CPU oracle itself: known-answer cases, the FP64 marcher, the exp restatement.

The reference has no image-level golden data (its renderer tests mock GL),
so these cases pin the oracle's shader restatement analytically.
"""

import numpy as np
import pytest

import oracle
from oracle import march_fp64
from pyvr_gb300 import Camera, Light, RenderConfig
from pyvr_gb300 import workloads as W
from pyvr_gb300.renderer import camera_uniforms, rgba_lut


def scene(data, lut, cam=None, width=8, height=8, light=None, config=None, normals=None,
          bmin=(-0.5, -0.5, -0.5), bmax=(0.5, 0.5, 0.5), value_scale=1.0):
    cam = cam or Camera.front_view(distance=3.0)
    light = light or Light.default()
    config = config or RenderConfig.balanced()
    view, proj, pos = camera_uniforms(cam, width, height)
    return dict(width=width, height=height, view=view, proj=proj, cam_pos=pos, volume=data,
                normals=normals, value_scale=value_scale, bmin=np.array(bmin, np.float32),
                bmax=np.array(bmax, np.float32), lut=lut, step_size=config.step_size,
                reference_step_size=config.reference_step_size, max_steps=config.max_steps,
                light_pos=light.position, light_target=light.target,
                ambient=light.ambient_intensity, diffuse=light.diffuse_intensity)


def const_lut(rgb, a, n=4):
    lut = np.empty((n, 4), np.float32)
    lut[:, :3] = rgb
    lut[:, 3] = a
    return lut


def test_expf_accuracy():
    x = np.linspace(-87.0, 88.0, 400001, dtype=np.float32)
    x = np.concatenate([x, np.linspace(-1, 0, 100001, dtype=np.float32)])
    y = oracle.expf(x).astype(np.float64)
    ref = np.exp(x.astype(np.float64))
    ulp = np.spacing(ref.astype(np.float32)).astype(np.float64)
    err = np.abs(y - ref) / ulp
    assert err.max() <= 2.0, err.max()
    assert oracle.expf(np.array([0.0], np.float32))[0] == 1.0
    assert oracle.expf(np.array([-100.0], np.float32))[0] == 0.0


def test_miss_is_transparent():
    # camera looking away from the box
    cam = Camera.from_spherical(np.array([0.0, 0.0, 10.0], np.float32), 0.0, 0.0, 0.0, 3.0)
    s = scene(np.ones((4, 4, 4), np.float32), const_lut((1, 1, 1), 1.0), cam=cam)
    o8, of, n = oracle.render(s)
    assert n == 0 and not o8.any() and not of.any()


def test_ert_cutoff_counts_five_samples():
    # alpha_tf = 1 at step == reference: alpha = 1 - e^-1 per sample, so the
    # accumulated alpha first reaches 0.99 after 5 samples (frag:87).
    s = scene(np.ones((4, 4, 4), np.float32), const_lut((1, 1, 1), 1.0), width=1, height=1)
    o8, of, n = oracle.render(s)
    assert n == 5
    a = 1 - np.exp(-1.0)
    assert of[0, 0, 3] == pytest.approx(1 - (1 - a) ** 5, abs=1e-6)


def test_constant_volume_closed_form():
    # constant density, constant LUT, no normals -> n = normalize(d,0,0) = +x,
    # light along -x...: k = ambient + diffuse*max(L.x, 0)
    lut = const_lut((0.5, 0.25, 1.0), 0.02)
    light = Light.directional([1.0, 0.0, 0.0], ambient=0.3, diffuse=0.6)
    s = scene(np.full((5, 6, 7), 0.4, np.float32), lut, width=1, height=1, light=light)
    o8, of, n = oracle.render(s)
    a = 1 - np.exp(-0.02)
    acc_a = 1 - (1 - a) ** n
    k = 0.3 + 0.6 * 1.0
    assert n > 50
    np.testing.assert_allclose(of[0, 0], [0.5 * k * acc_a, 0.25 * k * acc_a, 1.0 * k * acc_a, acc_a],
                               rtol=2e-5)


def test_zero_normals_shade_ambient_only():
    lut = const_lut((1.0, 1.0, 1.0), 0.05)
    data = np.full((4, 4, 4), 0.5, np.float32)
    nz = np.zeros((4, 4, 4, 3), np.float32)
    light = Light.directional([0.0, 0.0, -1.0], ambient=0.25, diffuse=0.75)
    s = scene(data, lut, width=1, height=1, normals=nz, light=light)
    _, of, n = oracle.render(s)
    acc_a = of[0, 0, 3]
    np.testing.assert_allclose(of[0, 0, :3], 0.25 * acc_a, rtol=1e-5)


def test_single_voxel_volume():
    lut = np.array([[0, 0, 0, 0], [1, 0, 0, 0.01]], np.float32)
    s = scene(np.full((1, 1, 1), 0.75, np.float32), lut, width=1, height=1)
    _, of, n = oracle.render(s)
    # density 0.75 -> LUT coordinate 0.75*2-0.5 = 1.0 -> entry 1 exactly
    a = 1 - np.exp(-0.01)
    assert n in (100, 101)  # unit box crossed along its axis at step 0.01
    assert of[0, 0, 3] == pytest.approx(1 - (1 - a) ** n, rel=1e-5)
    assert of[0, 0, 1] == 0.0 and of[0, 0, 2] == 0.0


def test_uint8_raw_saturates_lut():
    # uint8 voxels sample as 0..255 (manager.py:91-92, no /255): any voxel >= 1
    # reads the last LUT entry
    lut = np.zeros((256, 4), np.float32)
    lut[-1] = (1.0, 1.0, 1.0, 0.05)
    s_u8 = scene(np.full((4, 4, 4), 3, np.uint8), lut, width=2, height=2)
    s_f = scene(np.full((4, 4, 4), 1.0, np.float32), lut, width=2, height=2)
    np.testing.assert_array_equal(oracle.render(s_u8)[1], oracle.render(s_f)[1])
    # with the UNORM scale the same bytes read as 3/255
    s_un = scene(np.full((4, 4, 4), 3, np.uint8), lut, width=2, height=2, value_scale=1 / 255)
    assert not oracle.render(s_un)[1].any()


def test_noncubic_buffer_reinterpretation():
    # texture size (D,H,W) reads flat[z + D*(y + H*x)]: a volume whose
    # C-order (D,H,W) buffer is reinterpreted as (W,H,D) indexed [x,y,z]
    rng = np.random.default_rng(5)
    data = rng.random((6, 5, 9), dtype=np.float32)
    lut = np.stack([np.linspace(0, 1, 16)] * 4, 1).astype(np.float32) * 0.2
    cam = Camera.from_spherical(np.zeros(3, np.float32), 0.7, 0.4, 0.0, 2.5)
    s = scene(data, lut, cam=cam, width=24, height=24)
    o8, of, cnt = oracle.render(s, want_counts=True)
    f64, c64 = march_fp64.render_fp64(s)
    # a grazing ray may gain, lose or shift one boundary sample in float32
    err = np.abs(of - f64).max(axis=-1)
    assert (cnt == c64).mean() > 0.95
    assert (err < 1e-4).mean() > 0.95 and np.median(err) < 1e-6


def test_oracle_against_fp64_config_small():
    c = W.config_small()
    c["width"] = c["height"] = 96
    lut = rgba_lut(c["ctf"], c["otf"])
    s = W.frame_inputs(c["volume"], c["camera"], c["light"], c["config"], lut, 96, 96)
    o8, of, cnt = oracle.render(s, want_counts=True)
    f64, s64 = march_fp64.render_fp64(s)
    assert abs(int(cnt.sum()) - int(s64.sum())) <= 10
    same = cnt == s64
    assert np.abs(of - f64)[same].max() < 1e-4
    d = np.abs(march_fp64.blend_rgba8(f64).astype(int) - o8.astype(int))
    assert d.max() <= 1 and (d > 0).mean() < 1e-3
    assert (o8[..., 3] > 0).sum() > 1000


def test_row_subset_matches_full_render():
    c = W.config_small()
    lut = rgba_lut(c["ctf"], c["otf"])
    s = W.frame_inputs(c["volume"], c["camera"], c["light"], c["config"], lut, 64, 64)
    full, _, _ = oracle.render(s, want_float=False)
    part, _, _ = oracle.render(s, rows=(20, 30), want_float=False)
    np.testing.assert_array_equal(full[20:30], part[20:30])
    assert not part[:20].any()


def test_serving_workload_snapshot_restarts_the_same_stream():
    wl = W.ServingWorkload(n_volumes=4, n_extra=2, min_dim=16, max_dim=24,
                           generator=lambda n, s: W.value_noise((n, n, n), s))
    snap = wl.snapshot()
    first = [(kw["volume_id"], kw["tag"], kw["camera"].azimuth, tuple(kw["opacity_tf"].control_points))
             for _, kw in wl.requests(2000.0, 0.3, 9)]
    wl.requests(2000.0, 0.3, 10)  # the state moves on
    wl.restore(snap)
    again = [(kw["volume_id"], kw["tag"], kw["camera"].azimuth, tuple(kw["opacity_tf"].control_points))
             for _, kw in wl.requests(2000.0, 0.3, 9)]
    assert first == again and any(t == "load" for _, t, _, _ in first)
