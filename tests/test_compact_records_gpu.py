"""Half (8-byte) texel records: a volume gets them exactly when every stored
value and normal is a half (float16 volumes with normals computed in half
precision, uint8 or float16 values without normals), and renders the same
bytes and floats from them as from float records, in batches and alone."""

import numpy as np
import pytest

from pyvr_gb300 import Volume, compute_normal_volume
from pyvr_gb300 import workloads as W
from pyvr_gb300.batch import DeviceVolume, set_compact_records

from test_batch_gpu import _mixed_scenes, _run_batch

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture
def half_records():
    set_compact_records(True)
    yield
    set_compact_records(False)


def _both(scenes, **kw):
    set_compact_records(True)
    try:
        half = _run_batch(scenes, **kw)
    finally:
        set_compact_records(False)
    full = _run_batch(scenes, **kw)
    return half, full


def test_record_form_follows_exactness(half_records):
    base = W.value_noise((12, 14, 16), seed=21)
    cases = {
        ("f16", "device"): 8, ("f16", "none"): 8, ("u8", "none"): 8, ("u8", "device"): 16,
        ("f32", "device"): 16, ("f32", "none"): 16,
    }
    for (dtype, normals), want in cases.items():
        data = W.to_storage(base, dtype)
        dv = DeviceVolume(Volume(data=data), normals=normals)
        assert dv.record_bytes() == want, (dtype, normals)
        if normals == "device":  # the normals read back are the same floats either way
            got = dv.read_normals()
            ref = compute_normal_volume(data)
            assert np.array_equal(np.isnan(got), np.isnan(ref))
            assert np.array_equal(got[~np.isnan(got)], ref[~np.isnan(ref)])
    # float16 values with float32 normals that are not halves: float records
    data = W.to_storage(base, "f16")
    nrm = compute_normal_volume(base.astype(np.float32))
    assert DeviceVolume(Volume(data=data, normals=nrm), normals="given").record_bytes() == 16


def test_float_records_by_default():
    data = W.to_storage(W.value_noise((10, 10, 10), seed=2), "f16")
    assert DeviceVolume(Volume(data=data), normals="device").record_bytes() == 16


def test_per_volume_half_records():
    """DeviceVolume(half_records=True) compacts that volume alone, when exact."""
    from pyvr_gb300 import Camera, Light, OpacityTransferFunction, RenderConfig
    from pyvr_gb300.batch import BatchRenderer, DeviceLUT, RenderJob
    base = W.value_noise((20, 18, 22), seed=5)
    f16 = Volume(data=W.to_storage(base, "f16"), min_bounds=np.full(3, -1.0, np.float32),
                 max_bounds=np.full(3, 1.0, np.float32))
    half = DeviceVolume(f16, normals="device", half_records=True)
    full = DeviceVolume(f16, normals="device")
    assert half.record_bytes() == 8 and full.record_bytes() == 16
    u8 = DeviceVolume(Volume(data=W.to_storage(base, "u8")), normals="device")
    assert u8.compact() is False and u8.record_bytes() == 16
    lut = DeviceLUT(W.standin_colormap(4), OpacityTransferFunction.linear(0.0, 0.4))
    cam = Camera.from_spherical(np.zeros(3, np.float32), 0.4, 0.3, 0.0, 3.0)
    outs = []
    br = BatchRenderer(capacity=2, slots=2)
    for dv in (half, full):
        o8 = torch.zeros(64 * 48 * 4, dtype=torch.uint8, device="cuda")
        of = torch.zeros(64 * 48 * 4, dtype=torch.float32, device="cuda")
        br.render([RenderJob(dv, lut, cam, Light.default(), RenderConfig.balanced(), 64, 48, o8, of)])
        br.synchronize()
        outs.append((o8.cpu().numpy(), of.cpu().numpy()))
    br.close()
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    assert outs[0][0].reshape(-1, 4)[:, 3].max() > 0


@pytest.mark.parametrize("n_jobs", [1, 9])
def test_half_records_render_the_same_images(n_jobs):
    scenes = _mixed_scenes(n_jobs if n_jobs > 1 else 3, seed=31)
    if n_jobs == 1:  # one job per launch: the single-job kernel of each variant
        pairs = [_both([s]) for s in scenes]
        half = [h[0] for h, _ in pairs]
        full = [f[0] for _, f in pairs]
    else:
        half, full = _both(scenes)
    for (a8, af, ac), (b8, bf, bc) in zip(half, full):
        assert np.array_equal(a8, b8)
        assert np.array_equal(af, bf)
        assert np.array_equal(ac, bc)
