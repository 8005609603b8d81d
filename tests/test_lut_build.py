"""Device LUT build from control points (pvr_lut_build) against the host
table (rgba_lut, numpy.interp), entry for entry, and in rendered images."""

import numpy as np
import pytest

from pyvr_gb300 import ColorTransferFunction as CTF
from pyvr_gb300 import OpacityTransferFunction as OTF
from pyvr_gb300 import workloads as W
from pyvr_gb300.renderer import rgba_lut

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _cases():
    rng = np.random.default_rng(11)
    out = [(W.standin_colormap(k), W.random_opacity(rng, int(rng.integers(4, 13)), 0.3), None)
           for k in range(6)]
    out += [
        (CTF.grayscale(), OTF.linear(0.0, 0.1), None),
        (W.standin_colormap(1), OTF.one_step(0.3), 1000),
        (W.standin_colormap(2), OTF.peaks([0.2, 0.7]), 4096),
        (CTF([(0.3, (1.0, 0.5, 0.0))]), OTF([(0.5, 0.4)]), 7),           # single points
        (W.standin_colormap(3), OTF([(0.0, 0.0), (0.5, 0.2), (0.5, 0.8), (1.0, 1.0)]), 9),  # duplicate x
        (CTF([(0.2, (0, 0, 1)), (0.6, (1, 1, 0))]), OTF([(0.1, 0.0), (0.9, 0.5)]), 256),   # partial range
        (W.standin_colormap(4), W.random_opacity(rng, 8, 0.3), 1),
        (W.standin_colormap(5), W.random_opacity(rng, 8, 0.3), 2),
        (W.standin_colormap(6), W.random_opacity(rng, 8, 0.3), 65536),
    ]
    return out


def test_device_table_equals_host_table():
    from pyvr_gb300.batch import DeviceLUT
    for ctf, otf, size in _cases():
        want = rgba_lut(ctf, otf, size)
        lut = DeviceLUT.on_device(ctf, otf, size)
        got = lut.read()
        assert got.shape == want.shape
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (size, np.abs(got - want).max())
        lut.close()


def test_rebuild_in_place_and_renders_identically():
    from pyvr_gb300 import Camera, Light, RenderConfig, Volume
    from pyvr_gb300.batch import BatchRenderer, DeviceLUT, DeviceVolume, RenderJob
    data = W.value_noise((24, 20, 28), seed=8).astype(np.float32)
    vol = Volume(data=data, min_bounds=np.full(3, -1.0, np.float32), max_bounds=np.full(3, 1.0, np.float32))
    dv = DeviceVolume(vol, normals="device")
    cam = Camera.from_spherical(np.zeros(3, np.float32), 0.4, 0.3, 0.0, 3.0)
    rng = np.random.default_rng(3)
    ctf, otf = W.standin_colormap(7), OTF.peaks([0.3, 0.6], opacity=0.5)
    host = DeviceLUT(ctf, otf)
    dev = DeviceLUT.on_device(W.standin_colormap(1), W.random_opacity(rng, 5, 0.3))
    dev.build(ctf, otf)  # rebuilt in place
    outs = [torch.zeros(64 * 64 * 4, dtype=torch.uint8, device="cuda") for _ in range(2)]
    br = BatchRenderer(capacity=2, slots=1)
    br.render([RenderJob(dv, lut, cam, Light.default(), RenderConfig.balanced(), 64, 64, out_rgba8=o)
               for lut, o in zip((host, dev), outs)])
    br.synchronize()
    a, b = outs[0].cpu().numpy(), outs[1].cpu().numpy()
    assert a.any() and np.array_equal(a, b)
    br.close()


def test_bad_control_points_rejected():
    from pyvr_gb300.batch import DeviceLUT
    lut = DeviceLUT(rgba=np.zeros((4, 4), np.float32))

    class Pts:
        def __init__(self, pts, n=256):
            self.control_points, self.lut_size = pts, n

    with pytest.raises(ValueError, match="sorted"):
        lut.build(Pts([(0.5, (0, 0, 0)), (0.1, (1, 1, 1))]), Pts([(0.0, 0.0)]))
    with pytest.raises(ValueError, match="control points"):
        lut.build(Pts([(i / 300, (0, 0, 0)) for i in range(300)]), Pts([(0.0, 0.0)]))
    with pytest.raises(ValueError, match="size"):
        lut.build(Pts([(0.0, (0, 0, 0))], 1 << 17), Pts([(0.0, 0.0)], 4))
