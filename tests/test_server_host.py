"""Host logic of the serving layer, on CPU with stand-ins for the device
objects: the volume cache (byte budget, LRU, pinning), the LUT cache
(content keys, reservation, eviction, pinning), the sustained-rate search and
the latency statistics, and the bench's clock-sample parsing."""

import os

import numpy as np
import pytest

from pyvr_gb300 import OpacityTransferFunction, Volume
from pyvr_gb300 import server as S
from pyvr_gb300 import workloads as W


class FakeDeviceVolume:
    made = []

    def __init__(self, volume, value_scale=1.0, normals="auto", brick_log2=0, half_records=False, wait=True):
        self.waited = wait
        self.shape = volume.data.shape
        d, h, w = volume.data.shape
        lb = brick_log2 or 3  # the cache's own estimate of records + voxels
        self.bytes = (16 * ((w >> lb) + 1) * ((h >> lb) + 1) * ((d >> lb) + 1) * ((1 << lb) + 1) ** 3
                      + int(volume.data.nbytes))
        self.closed = False
        FakeDeviceVolume.made.append(self)

    def device_bytes(self):
        return self.bytes

    def ready(self):
        return True

    def close(self):
        self.closed = True


class FakeDeviceLUT:
    made = 0

    def __init__(self, color_tf=None, opacity_tf=None, size=None, rgba=None):
        FakeDeviceLUT.made += 1
        self.size = int(rgba.shape[0]) if rgba is not None else 256
        self.table = None
        self.closed = False

    def update(self, rgba):
        self.table = np.array(rgba)
        self.size = int(rgba.shape[0])

    def close(self):
        self.closed = True


@pytest.fixture
def fake_device(monkeypatch):
    FakeDeviceVolume.made = []
    FakeDeviceLUT.made = 0
    monkeypatch.setattr(S, "DeviceVolume", FakeDeviceVolume)
    monkeypatch.setattr(S, "DeviceLUT", FakeDeviceLUT)


def _vol(n):
    return Volume(data=np.zeros((n, n, n), np.uint8))


def test_volume_cache_budget_lru_and_pins(fake_device):
    one = FakeDeviceVolume(_vol(16), brick_log2=3).device_bytes()
    FakeDeviceVolume.made = []
    cache = S.VolumeCache(budget_bytes=int(one * 2.2), brick_log2=3)  # room for two
    released = []
    cache.insert(1, _vol(16), 1.0, released.append)
    cache.insert(2, _vol(16), 1.0, released.append)
    assert cache.loads == 2 and cache.uploaded_bytes == 2 * 16 ** 3
    # a resident volume is not loaded again and becomes the most recent
    assert cache.insert(1, _vol(16), 1.0, released.append) is cache.get(1)
    assert cache.loads == 2
    # 1 is pinned by an in-flight request: loading 3 evicts 2, the least recent unpinned
    cache.acquire(1)
    cache.insert(3, _vol(16), 1.0, released.append)
    assert cache.get(2) is None and cache.get(1) is not None and cache.get(3) is not None
    assert len(released) == 1 and cache.evictions >= 1
    # everything pinned: go over budget rather than stall, and count it
    cache.acquire(3)
    assert cache.over_budget == 0
    cache.insert(4, _vol(16), 1.0, released.append)
    assert cache.get(1) is not None and cache.get(3) is not None and cache.get(4) is not None
    assert cache.over_budget == 1 and cache.used > cache.budget
    cache.release(1)
    cache.release(3)
    vols = [cache.get(i) for i in (1, 3, 4)]
    cache.clear()
    assert all(v.closed for v in vols) and cache.used == 0


def test_volume_cache_evict_except_keeps_pinned_and_kept(fake_device):
    cache = S.VolumeCache(budget_bytes=1 << 30, brick_log2=3)
    for vid in range(4):
        cache.insert(vid, _vol(8), 1.0, lambda dv: None)
    cache.acquire(2)  # in flight: stays
    out = cache.evict_except({0})
    assert len(out) == 2 and sorted(cache._vols) == [0, 2]
    assert cache.evictions == 0 and cache.used == sum(cache._bytes.values())


def test_volume_cache_queues_layouts_when_asked(fake_device):
    # the native server's cache hands new volumes on with their layout queued
    # (DeviceVolume(wait=False)); the default cache waits for it
    S.VolumeCache(budget_bytes=1 << 30, brick_log2=3).insert(1, _vol(8), 1.0, lambda dv: None)
    S.VolumeCache(budget_bytes=1 << 30, brick_log2=3, queue_layouts=True).insert(2, _vol(8), 1.0, lambda dv: None)
    assert [v.waited for v in FakeDeviceVolume.made] == [True, False]


def test_volume_cache_evicts_and_retries_when_allocation_fails(fake_device, monkeypatch):
    """A layout that runs out of device memory (the budget assumed more room
    than there is) evicts the least recently used unpinned volume and is
    retried; with nothing left to evict the MemoryError reaches the caller."""
    one = FakeDeviceVolume(_vol(16), brick_log2=3).device_bytes()
    FakeDeviceVolume.made = []
    failures = {"left": 2}

    class Flaky(FakeDeviceVolume):
        def __init__(self, *a, **kw):
            if failures["left"] > 0:
                failures["left"] -= 1
                raise MemoryError("out of device memory (injected)")
            super().__init__(*a, **kw)

    monkeypatch.setattr(S, "DeviceVolume", FakeDeviceVolume)
    waits = []
    cache = S.VolumeCache(budget_bytes=one * 10, brick_log2=3, release_wait=lambda: waits.append(1))
    released = []
    for vid in (1, 2, 3):
        cache.insert(vid, _vol(16), 1.0, released.append)
    cache.acquire(3)  # pinned: never a victim
    monkeypatch.setattr(S, "DeviceVolume", Flaky)
    cache.insert(4, _vol(16), 1.0, released.append)
    # two failed attempts: volumes 1 then 2 (least recent first) were evicted
    assert cache.alloc_retries == 2 and len(waits) == 2
    assert cache.get(1) is None and cache.get(2) is None
    assert cache.get(3) is not None and cache.get(4) is not None
    assert cache.evictions == 2 and len(released) == 2
    # nothing evictable left (3 and 4 pinned): the failure propagates
    cache.acquire(4)
    failures["left"] = 5
    with pytest.raises(MemoryError):
        cache.insert(5, _vol(16), 1.0, released.append)
    assert cache.get(5) is None and cache.alloc_retries == 2


def test_volume_cache_estimate_follows_record_form(monkeypatch):
    import pyvr_gb300.batch as B
    cache = S.VolumeCache(budget_bytes=1 << 40, brick_log2=4)
    vol8 = Volume(data=np.zeros((32, 32, 32), np.uint8))
    vol32 = Volume(data=np.zeros((32, 32, 32), np.float32))
    records = 3 ** 3 * 17 ** 3
    monkeypatch.setattr(B, "get_compact_records", lambda: "half_normals")
    assert cache.estimate_bytes(vol8) == 8 * records + 32 ** 3
    assert cache.estimate_bytes(vol32) == 16 * records + 4 * 32 ** 3
    monkeypatch.setattr(B, "get_compact_records", lambda: "float")
    assert cache.estimate_bytes(vol8) == 16 * records + 32 ** 3


def test_deadlines_expire_in_order():
    d = S.Deadlines()
    for tag, when in ((1, 5.0), (2, 1.0), (3, 3.0)):
        d.add(tag, when)
    assert d.expired(0.5) == [] and len(d) == 3
    assert d.expired(3.0) == [2, 3]
    assert d.expired(10.0) == [1] and len(d) == 0


def _tfs(seed):
    rng = np.random.default_rng(seed)
    return W.standin_colormap(seed % 12), W.random_opacity(rng, 5, 0.3)


def test_tf_key_is_content_based():
    c, o = _tfs(3)
    c2, o2 = _tfs(3)
    assert S.tf_key(c, o) == S.tf_key(c2, o2)
    assert S.tf_key(c, o) != S.tf_key(*_tfs(4))
    # lists and tuples of the same points give the same key
    pts = [(0.0, 0.0), (0.5, 0.25), (1.0, 1.0)]
    a = OpacityTransferFunction(list(pts))
    b = OpacityTransferFunction([tuple(p) for p in pts])
    assert S.tf_key(c, a) == S.tf_key(c, b)
    hash(S.tf_key(c, a))


def test_lut_cache_reserve_hits_eviction_and_pins(fake_device):
    cache = S.LutCache(capacity=3, device_build=False)
    cache.reserve(256, 3)
    assert FakeDeviceLUT.made == 3
    keys = []
    for s in range(3):
        k, lut = cache.acquire(*_tfs(s))
        keys.append(k)
        assert lut.table is not None and lut.table.shape == (256, 4)
    assert FakeDeviceLUT.made == 3 and cache.misses == 3  # built into the reserved tables
    k, _ = cache.acquire(*_tfs(0))
    assert k == keys[0] and cache.hits == 1
    for k in keys + [keys[0]]:
        cache.release(k)
    # a fourth table evicts the least recently used unpinned one and reuses its memory
    cache.acquire(*_tfs(7))
    assert FakeDeviceLUT.made == 3 and len(cache._luts) == 3 and keys[1] not in cache._luts
    # every resident table pinned by a queued request: the cache grows rather than stall
    cache.acquire(*_tfs(0))
    cache.acquire(*_tfs(2))
    cache.acquire(*_tfs(8))
    assert len(cache._luts) == 4 and FakeDeviceLUT.made == 4
    cache.clear()
    assert len(cache._luts) == 0


def test_latency_stats():
    reqs = []
    for i in range(100):
        r = S.RenderRequest("render", 0, None, None, None, None, None, 1, 1)
        r.arrival = float(i)
        r.done_at = float(i) + (i + 1) / 1000.0  # 1 .. 100 ms
        reqs.append(r)
    st = S.latency_stats(reqs)
    assert st["n"] == 100 and st["max_ms"] == pytest.approx(100.0)
    assert st["p50_ms"] == pytest.approx(50.5) and 99.0 <= st["p99_ms"] <= 100.0
    assert S.latency_stats([]) == {"n": 0}


def test_sustained_rate_search(monkeypatch):
    """A service that keeps up to 5,000 req/s: doubling probes pass up to 3,200,
    fail at 6,400 (each failure repeated once), then bisection closes in."""
    capacity = 5000.0

    class Workload:
        def requests(self, rate, duration, seed):
            return [(0.0, {"rate": rate})]

    def fake_drive(impl, stream):
        rate = stream[0][1]["rate"]
        r = S.RenderRequest("render", 0, None, None, None, None, None, 1, 1)
        r.arrival, r.done_at = 0.0, (0.005 if rate <= capacity else 0.5)
        return [r] * int(rate), 1.0

    monkeypatch.setattr(S, "drive", fake_drive)
    resets = []
    best, probes = S.sustained_rate(None, Workload(), [400.0 * 2 ** k for k in range(6)], 1.0, 7,
                                    refine=4, reset=lambda: resets.append(1))
    assert 4600.0 <= best <= capacity
    failed = [p for p in probes if not p["ok"]]
    assert {p["repeat"] for p in failed if p["offered"] == 6400.0} == {0, 1}
    assert len(resets) == len(probes)


def test_clock_sampler_parses_samples(tmp_path):
    import bench

    class Done:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    cs = bench.ClockSampler(gpu_index=0)
    for lines in (["0, 2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active",
                   "1, 1000, 2070, 100.0, 0x0, Active, Not Active, Not Active, Not Active"],
                  ["0, 2060, 2070, 1200.0, 0x4, Not Active, Not Active, Not Active, Active",
                   "garbage"]):
        cs.path = str(tmp_path / f"clk{len(cs.sm)}.csv")
        with open(cs.path, "w") as f:
            f.write("\n".join(lines) + "\n")
        cs.fh = open(os.devnull, "w")
        cs.proc = Done()
        cs.pause()
    out = cs.stop()
    # only GPU 0's rows count; sw_power_cap was active once
    assert out["samples"] == 2 and out["sm_max_mhz"] == 2070.0
    assert out["sm_mhz"] == pytest.approx(2065.0) and out["reasons"] == ["sw_power_cap"]
