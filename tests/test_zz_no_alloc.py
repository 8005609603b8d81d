"""pvr_batch_render_static (the batch march that allocates nothing, scratch in
a static device array) against pvr_batch_render on the same jobs: identical
bytes, samples and counters, on two calls in a row; calls of different sizes
queued back to back on one stream; and a warmed call that leaves the device's
free memory, the default memory pool and torch's allocator untouched.  Kept
in its own file, collected last, so that it also runs after every other GPU
test."""

import ctypes
import gc
import os

import numpy as np
import pytest

from pyvr_gb300 import Camera, Light, RenderConfig, Volume, compute_normal_volume
from pyvr_gb300 import _native
from pyvr_gb300 import workloads as W
from pyvr_gb300.batch import (BatchRenderer, DeviceLUT, DeviceVolume, RenderJob, Tuning,
                              make_job_struct, render_static)

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _scenes(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        dims = tuple(int(x) for x in np.exp(rng.uniform(np.log(5), np.log(30), 3)))
        dtype = ["u8", "f16", "f32"][i % 3]
        data = W.to_storage(W.value_noise(dims, seed=500 + i), dtype)
        vol = Volume(data=data, normals=compute_normal_volume(data) if i % 2 else None,
                     min_bounds=np.full(3, -1.0, np.float32), max_bounds=np.full(3, 1.0, np.float32))
        cam = Camera.from_spherical(np.zeros(3, np.float32), float(rng.uniform(-np.pi, np.pi)),
                                    float(rng.uniform(-1.2, 1.2)), 0.0, float(rng.uniform(2.5, 4.0)))
        w, h = [(40, 40), (48, 24), (17, 33)][i % 3]
        out.append(dict(vol=vol, vs=1 / 255 if dtype == "u8" else 1.0, cam=cam, w=w, h=h,
                        otf=W.random_opacity(rng, int(rng.integers(4, 10)), 0.3),
                        ctf=W.standin_colormap(int(rng.integers(0, 12))),
                        cfg=[RenderConfig.balanced(), RenderConfig.fast()][i % 2],
                        light=[Light.directional([1, -1, 0]), Light.default()][i % 2]))
    return out


class _Setup:
    """Device resources of the scenes (made up front: the static entry point
    itself allocates nothing) and one set of outputs per render call."""

    def __init__(self, scenes, calls):
        self.scenes = scenes
        self.res = [(DeviceVolume(s["vol"], value_scale=s["vs"]), DeviceLUT(s["ctf"], s["otf"]))
                    for s in scenes]
        self.outs = [[(torch.zeros(s["w"] * s["h"] * 4, dtype=torch.uint8, device="cuda"),
                       torch.zeros(s["w"] * s["h"] * 4, dtype=torch.float32, device="cuda"),
                       torch.zeros(2, dtype=torch.int64, device="cuda")) for s in scenes]
                     for _ in range(calls)]

    def structs(self, call):
        arr = (_native.PvrJob * len(self.scenes))()
        for k, (s, (dv, dl), (o8, of, cnt)) in enumerate(zip(self.scenes, self.res, self.outs[call])):
            make_job_struct(RenderJob(dv, dl, s["cam"], s["light"], s["cfg"], s["w"], s["h"], o8, of, cnt),
                            arr[k])
        return arr

    def results(self, call):
        return [(o8.cpu().numpy(), of.cpu().numpy(), cnt.cpu().numpy()) for o8, of, cnt in self.outs[call]]


def _compare(scenes, tuning=None):
    setup = _Setup(scenes, calls=3)
    stream = torch.cuda.Stream()
    # call 0: the launcher entry point (pvr_batch_render)
    br = BatchRenderer(capacity=len(scenes), slots=1, tuning=tuning)
    br.render_structs(setup.structs(0), len(scenes), stream=stream)
    stream.synchronize()
    br.close()
    # calls 1 and 2: the static entry point, back to back on one stream
    s1, s2 = setup.structs(1), setup.structs(2)
    render_static(s1, len(scenes), tuning=tuning, stream=stream)
    render_static(s2, len(scenes), tuning=tuning, stream=stream)
    stream.synchronize()
    want = setup.results(0)
    assert sum(int(c[0]) for _, _, c in want) > 0  # the renders really sample the volumes
    for call in (1, 2):
        got = setup.results(call)
        for k, ((g8, gf, gc), (w8, wf, wc)) in enumerate(zip(got, want)):
            assert np.array_equal(g8, w8), (call, k)
            assert np.array_equal(gf.view(np.uint32), wf.view(np.uint32)), (call, k)
            assert np.array_equal(gc, wc), (call, k)


def test_static_batch_equals_launcher():
    _compare(_scenes(7, seed=1))


def test_static_batch_equals_launcher_with_tuning():
    _compare(_scenes(5, seed=2), tuning=Tuning(tile_w=32, tile_h=8, steps_per_iter=4, blocks_per_sm=2))


def test_static_batch_over_several_launches():
    # 200 jobs: three launches (96 + 96 + 8), one static tile counter each
    _compare(_scenes(200, seed=3))


def test_static_batch_rejects_bad_calls():
    lib = _native.load()
    setup = _Setup(_scenes(1, seed=4), calls=1)
    one = setup.structs(0)
    assert lib.pvr_batch_render_static(None, 0, None, None) == _native.PVR_OK
    big = (_native.PvrJob * 6145)()
    ctypes.memmove(big, one, ctypes.sizeof(one))
    with pytest.raises(ValueError, match="at most 6144"):
        render_static(big, 6145)
    with pytest.raises(ValueError, match="tuning"):
        render_static(one, 1, tuning=Tuning(tile_w=16, tile_h=8))
    bad = (_native.PvrJob * 1)()
    ctypes.memmove(bad, one, ctypes.sizeof(one))
    bad[0].lut = None
    with pytest.raises(ValueError, match="without volume or LUT"):
        render_static(bad, 1)
    torch.cuda.synchronize()


def test_static_batch_calls_of_different_sizes_back_to_back():
    # a 200-job call (3 launches) and a 7-job call queued on one stream with
    # no synchronisation between them: the second call's clear of the static
    # counters runs behind every launch of the first
    big, small = _scenes(200, seed=5), _scenes(7, seed=6)
    sb, ss = _Setup(big, calls=2), _Setup(small, calls=2)
    stream = torch.cuda.Stream()
    br = BatchRenderer(capacity=200, slots=1)
    br.render_structs(sb.structs(0), 200, stream=stream)
    br.render_structs(ss.structs(0), 7, stream=stream)
    stream.synchronize()
    br.close()
    render_static(sb.structs(1), 200, stream=stream)
    render_static(ss.structs(1), 7, stream=stream)
    stream.synchronize()
    for setup in (sb, ss):
        want, got = setup.results(0), setup.results(1)
        for k, ((g8, gf, gc), (w8, wf, wc)) in enumerate(zip(got, want)):
            assert np.array_equal(g8, w8), k
            assert np.array_equal(gf.view(np.uint32), wf.view(np.uint32)), k
            assert np.array_equal(gc, wc), k


def _cudart():
    """The CUDA runtime library torch loaded in this process (ctypes), or None."""
    try:
        with open("/proc/self/maps") as f:
            paths = {line.split()[-1] for line in f if "libcudart.so" in line}
    except OSError:
        return None
    for p in sorted(paths):
        if os.path.exists(p):
            try:
                return ctypes.CDLL(p)
            except OSError:
                continue
    return None


def _pool_used_bytes(rt, device):
    """Bytes in use from the device's default stream-ordered memory pool."""
    pool = ctypes.c_void_p()
    if rt.cudaDeviceGetDefaultMemPool(ctypes.byref(pool), device) != 0:
        return None
    used = ctypes.c_uint64()
    if rt.cudaMemPoolGetAttribute(pool, 7, ctypes.byref(used)) != 0:  # cudaMemPoolAttrUsedMemCurrent
        return None
    return int(used.value)


def test_static_batch_allocates_nothing():
    setup = _Setup(_scenes(9, seed=7), calls=1)
    structs = setup.structs(0)
    stream = torch.cuda.Stream()
    render_static(structs, 9, stream=stream)  # warm: module loaded, address looked up
    stream.synchronize()
    dev = torch.cuda.current_device()
    rt = _cudart()
    # objects of earlier tests freed meanwhile would change the free memory
    gc.collect()
    gc.disable()
    try:
        _measure_calls(structs, stream, dev, rt)
    finally:
        gc.enable()


def _measure_calls(structs, stream, dev, rt):
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    pool0 = _pool_used_bytes(rt, dev) if rt is not None else None
    stats0 = torch.cuda.memory_stats()
    for _ in range(3):
        render_static(structs, 9, stream=stream)
    stream.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, "device memory changed across the calls"
    if pool0 is not None:
        assert _pool_used_bytes(rt, dev) == pool0, "the default memory pool grew"
    stats1 = torch.cuda.memory_stats()
    for k in ("allocation.all.allocated", "segment.all.allocated"):
        assert stats1.get(k, 0) == stats0.get(k, 0), k
