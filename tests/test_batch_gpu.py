"""GPU tests of the batch path (persistent kernel + CUDA graph), device
normals, brick sizes and launch tunings -- all against the CPU oracle or
numpy, bit for bit."""

import numpy as np
import pytest

import oracle
from pyvr_gb300 import (Camera, Light, OpacityTransferFunction, RenderConfig, Volume,
                        VolumeRenderer, compute_normal_volume)
from pyvr_gb300 import workloads as W
from pyvr_gb300.batch import BatchRenderer, DeviceLUT, DeviceVolume, RenderJob, Tuning
from pyvr_gb300.renderer import rgba_lut

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def nan_equal(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


@pytest.mark.parametrize("dims,brick_log2", [((13, 17, 22), 3), ((33, 33, 33), 3), ((16, 16, 16), 4),
                                              ((2, 2, 2), 2), ((21, 21, 21), 2), ((40, 40, 40), 4)])
@pytest.mark.parametrize("dtype", ["u8", "f16", "f32"])
def test_device_normals_match_numpy(dtype, dims, brick_log2):
    # cubic volumes take the normals from the neighbours staged in shared
    # memory, non-cubic ones from global memory; both must equal numpy
    base = W.value_noise(dims, seed=3)
    data = W.to_storage(base, dtype)
    if min(dims) > 6:
        data[2:5, 3:6, :] = data[3, 4, 0]  # flat patches: zero gradients (NaN for float16)
    vol = Volume(data=data)
    dv = DeviceVolume(vol, normals="device", brick_log2=brick_log2)
    got = dv.read_normals()
    want = compute_normal_volume(data)
    assert nan_equal(got, want), np.nanmax(np.abs(got - want))
    if dtype == "f16" and min(dims) > 6:
        assert np.isnan(want).any()  # the reference's own float16 behaviour


@pytest.mark.parametrize("dtype", ["u8", "f16", "f32"])
def test_half_normal_records(dtype):
    # "half_normals": uint8 / float16 volumes get 8-byte records holding the
    # values exactly and the normals rounded to half; float32 keeps floats
    from pyvr_gb300.batch import set_compact_records
    data = W.to_storage(W.value_noise((24, 24, 24), seed=5), dtype)
    set_compact_records("half_normals")
    try:
        dv = DeviceVolume(Volume(data=data), normals="device", brick_log2=3)
    finally:
        set_compact_records("float")
    want = compute_normal_volume(data)
    if dtype == "f32":
        assert dv.record_bytes() == 16 and dv.records_exact()
        assert nan_equal(dv.read_normals(), want)
    else:
        assert dv.record_bytes() == 8
        assert dv.records_exact() == (dtype == "f16")
        assert nan_equal(dv.read_normals(), want.astype(np.float16).astype(np.float32))


def test_page_locked_volume_data():
    # volumes uploaded from pvr_host_alloc memory lay out like any other
    from pyvr_gb300.batch import page_locked_copy, page_locked_empty
    data = W.to_storage(W.value_noise((20, 22, 24), seed=6), "u8")
    pl = page_locked_copy(data)
    assert pl.dtype == data.dtype and pl.shape == data.shape and np.array_equal(pl, data)
    a = DeviceVolume(Volume(data=data), normals="device", brick_log2=3)
    b = DeviceVolume(Volume(data=pl), normals="device", brick_log2=3)
    assert nan_equal(a.read_normals(), b.read_normals())
    e = page_locked_empty((3, 4, 5), np.float16)
    assert e.shape == (3, 4, 5) and e.dtype == np.float16
    del pl, e  # freed with the arrays
    from pyvr_gb300.batch import PageLockedArena
    arrays = [data, data.astype(np.float16)]
    arena = PageLockedArena(PageLockedArena.size_for(arrays))
    got = [arena.copy(a) for a in arrays]
    assert all(np.array_equal(g, a) and g.dtype == a.dtype for g, a in zip(got, arrays))
    assert got[1].ctypes.data % PageLockedArena.ALIGN == 0
    with pytest.raises(MemoryError):
        arena.array((1,), np.uint8)
    c = DeviceVolume(Volume(data=got[0]), normals="device", brick_log2=3)
    assert nan_equal(a.read_normals(), c.read_normals())


@pytest.mark.parametrize("dtype", ["u8", "f32"])
def test_queued_layout_renders_like_a_finished_one(dtype):
    # pvr_volume_create_async: the batch launch waits on the device for the
    # layout; images, normals and record form equal the synchronous volume's
    data = W.to_storage(W.value_noise((48, 40, 44), seed=8), dtype)
    vol = Volume(data=data)
    a = DeviceVolume(vol, normals="device", brick_log2=3)
    b = DeviceVolume(vol, normals="device", brick_log2=3, wait=False)
    rng = np.random.default_rng(3)
    lut = DeviceLUT(W.standin_colormap(3), W.random_opacity(rng, 8, 0.3))
    cam = Camera.from_spherical(np.zeros(3, np.float32), 0.7, 0.4, 0.0, 3.0)
    outs = []
    br = BatchRenderer(capacity=4, slots=2)
    for dv in (b, a):  # the queued volume first, straight after its creation
        o8, of, _ = _job_outputs(64, 48)
        br.render([RenderJob(dv, lut, cam, Light.directional([1, -1, 0], 0.2, 0.8), RenderConfig.balanced(),
                             64, 48, o8, of)])
        outs.append((o8, of))
    torch.cuda.synchronize()
    assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][1], outs[1][1])
    assert b.ready() and b.record_bytes() == a.record_bytes()
    assert nan_equal(a.read_normals(), b.read_normals())
    br.close()


def test_queued_layout_released_before_it_completes():
    # a volume released right after its creation is freed behind its layout
    from pyvr_gb300 import _native
    data = W.to_storage(W.value_noise((96, 96, 96), seed=9), "f16")
    dv = DeviceVolume(Volume(data=data), normals="device", brick_log2=4, wait=False)
    s = torch.cuda.Stream()
    _native.check(_native.load().pvr_volume_release(dv.handle, s.cuda_stream))
    dv.handle = None
    s.synchronize()
    torch.cuda.synchronize()


def test_given_normals_roundtrip():
    data = W.value_noise((9, 10, 11), seed=4)
    vol = Volume(data=data, normals=compute_normal_volume(data))
    for b in (2, 3, 4):
        dv = DeviceVolume(vol, normals="given", brick_log2=b)
        assert nan_equal(dv.read_normals(), vol.normals)


def _job_outputs(w, h):
    return (torch.zeros(w * h * 4, dtype=torch.uint8, device="cuda"),
            torch.zeros(w * h * 4, dtype=torch.float32, device="cuda"),
            torch.zeros(2, dtype=torch.int64, device="cuda"))


def _mixed_scenes(n, seed=0, brick_log2=3):
    rng = np.random.default_rng(seed)
    scenes = []
    for i in range(n):
        dims = tuple(int(x) for x in np.exp(rng.uniform(np.log(6), np.log(40), 3)))
        dtype = ["u8", "f16", "f32"][i % 3]
        data = W.to_storage(W.value_noise(dims, seed=100 + i), dtype)
        vs = 1 / 255 if dtype == "u8" else 1.0
        vol = Volume(data=data, normals=compute_normal_volume(data) if i % 4 else None,
                     min_bounds=np.full(3, -1.0, np.float32), max_bounds=np.full(3, 1.0, np.float32))
        otf = W.random_opacity(rng, int(rng.integers(4, 13)), 0.3)
        ctf = W.standin_colormap(int(rng.integers(0, 12)))
        r = float(rng.uniform(2.5, 4.0))
        cam = Camera.from_spherical(np.zeros(3, np.float32), float(rng.uniform(-np.pi, np.pi)),
                                    float(rng.uniform(-1.2, 1.2)), 0.0, r)
        w, h = [(48, 48), (64, 40), (24, 56), (33, 17)][i % 4]
        cfg = [RenderConfig.balanced(), RenderConfig.fast(), RenderConfig.high_quality()][i % 3]
        light = [Light.directional([1, -1, 0]), Light.default(), Light.ambient_only(0.6)][i % 3]
        scenes.append(dict(vol=vol, vs=vs, otf=otf, ctf=ctf, cam=cam, w=w, h=h, cfg=cfg, light=light))
    return scenes


def _run_batch(scenes, tuning=None, brick_log2=3, repeat=1):
    dev = [(DeviceVolume(s["vol"], value_scale=s["vs"], brick_log2=brick_log2),
            DeviceLUT(s["ctf"], s["otf"])) for s in scenes]
    br = BatchRenderer(capacity=len(scenes), slots=2, tuning=tuning)
    outs = [_job_outputs(s["w"], s["h"]) for s in scenes]
    jobs = [RenderJob(dv, dl, s["cam"], s["light"], s["cfg"], s["w"], s["h"], o8, of, cnt)
            for s, (dv, dl), (o8, of, cnt) in zip(scenes, dev, outs)]
    for _ in range(repeat):
        for _, _, cnt in outs:
            cnt.zero_()
        br.render(jobs)
        br.synchronize()
    res = [(o8.cpu().numpy().reshape(s["h"], s["w"], 4), of.cpu().numpy().reshape(s["h"], s["w"], 4),
            cnt.cpu().numpy()) for s, (o8, of, cnt) in zip(scenes, outs)]
    br.close()
    return res


def _oracle(s):
    lut = rgba_lut(s["ctf"], s["otf"])
    return oracle.render(W.frame_inputs(s["vol"], s["cam"], s["light"], s["cfg"], lut, s["w"], s["h"],
                                        s["vs"], batch_camera=True))


def test_batch_of_mixed_jobs_matches_oracle():
    scenes = _mixed_scenes(12)
    res = _run_batch(scenes, repeat=2)
    for s, (g8, gf, cnt) in zip(scenes, res):
        o8, of, on = _oracle(s)
        assert np.array_equal(g8, o8)
        assert np.array_equal(gf, of)
        assert int(cnt[0]) == on


@pytest.mark.parametrize("brick_log2", [2, 4])
def test_brick_sizes_give_identical_images(brick_log2):
    scenes = _mixed_scenes(6, seed=5)
    base = _run_batch(scenes, brick_log2=3)
    other = _run_batch(scenes, brick_log2=brick_log2)
    for (a8, af, ac), (b8, bf, bc) in zip(base, other):
        assert np.array_equal(a8, b8) and np.array_equal(af, bf) and np.array_equal(ac, bc)


@pytest.mark.parametrize("tuning", [Tuning(32, 8, 1, 0), Tuning(8, 32, 4, 0), Tuning(64, 4, 4, 2),
                                    Tuning(16, 16, 4, 1)])
def test_tunings_give_identical_images(tuning):
    scenes = _mixed_scenes(6, seed=9)
    base = _run_batch(scenes)
    other = _run_batch(scenes, tuning=tuning)
    for (a8, af, ac), (b8, bf, bc) in zip(base, other):
        assert np.array_equal(a8, b8) and np.array_equal(af, bf) and np.array_equal(ac, bc)


def test_graph_replay_with_new_contents():
    """Consecutive batches through the same slots (graphs replayed with new
    descriptors) give each job the image it gets alone."""
    scenes = _mixed_scenes(8, seed=13)
    dev = [(DeviceVolume(s["vol"], value_scale=s["vs"]), DeviceLUT(s["ctf"], s["otf"])) for s in scenes]
    br = BatchRenderer(capacity=8, slots=2)
    outs = [_job_outputs(s["w"], s["h"]) for s in scenes]
    jobs = [RenderJob(dv, dl, s["cam"], s["light"], s["cfg"], s["w"], s["h"], o8, of, cnt)
            for s, (dv, dl), (o8, of, cnt) in zip(scenes, dev, outs)]
    groups = [jobs[0:3], jobs[3:8], jobs[1:2], jobs[2:7]]
    for g in groups:
        br.render(g)
    br.synchronize()
    for s, (o8, of, cnt) in zip(scenes, outs):
        want8, wantf, _ = _oracle(s)
        assert np.array_equal(o8.cpu().numpy().reshape(s["h"], s["w"], 4), want8)


def test_renderer_device_normals_match_host_normals():
    data = W.value_noise((30, 26, 34), seed=17)
    host = Volume(data=data, normals=compute_normal_volume(data))
    bare = Volume(data=data)
    cam = Camera.from_spherical(np.zeros(3, np.float32), 0.6, 0.3, 0.0, 3.0)
    ctf, otf = W.standin_colormap(2), OpacityTransferFunction.linear(0.0, 0.2)
    outs = []
    for vol, device in ((host, False), (bare, True)):
        with VolumeRenderer(64, 64) as r:
            r.load_volume(vol)
            if device:
                r.compute_normals()
            r.set_camera(cam)
            r.set_transfer_functions(ctf, otf)
            outs.append(r.render_float())
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
