"""Serving: every result of the continuously batched server equals the same
request rendered alone (and the CPU oracle), with and without evictions."""

import numpy as np
import pytest

import oracle
from pyvr_gb300 import workloads as W
from pyvr_gb300.renderer import rgba_lut
from pyvr_gb300.server import PyRenderServer, RenderRequest, SerialRenderer, latency_stats

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _workload():
    return W.ServingWorkload(n_volumes=5, n_extra=3, min_dim=16, max_dim=40, res=48, capture_res=64,
                             generator=lambda n, s: W.value_noise((n, n, n), s))


def _run(budget, n_req=160):
    wl = _workload()
    stream = wl.requests(rate=4000.0, duration=1.0, seed=3)[:n_req]
    server = PyRenderServer(budget_bytes=budget, max_batch=16, slots=3)
    serial = SerialRenderer()
    for slot in range(wl.n_catalog):
        vol, vs = wl.volumes[slot]
        server.cache.insert(slot, vol, vs, server._release_after_inflight)
        serial.cache.insert(slot, vol, vs, serial._free_now)
    reqs = [RenderRequest(**kw) for _, kw in stream]
    futs = [server.submit(r) for r in reqs]
    got = [f.result(timeout=120) for f in futs]
    want = []
    for _, kw in stream:
        want.append(serial.handle(RenderRequest(**kw)))
    stats = dict(batches=server.batches, sizes=list(server.batch_sizes),
                 evictions=server.cache.evictions, loads=server.cache.loads, lat=latency_stats(reqs))
    server.close()
    serial.close()
    return wl, stream, got, want, stats


def test_server_results_equal_results_alone():
    wl, stream, got, want, stats = _run(budget=40 << 30)
    assert len(got) == len(want) == len(stream)
    for g, w in zip(got, want):
        assert g == w
    assert max(stats["sizes"]) > 1, stats["sizes"]  # requests were really batched
    tags = {kw["tag"] for _, kw in stream}
    assert {"orbit", "tf_edit", "capture", "load"} <= tags
    # a few results against the CPU oracle
    for (_, kw), g in list(zip(stream, got))[:6]:
        vol, vs = wl.volumes[kw["volume_id"]]
        from pyvr_gb300 import compute_normal_volume, Volume
        v = Volume(data=vol.data, normals=compute_normal_volume(vol.data), min_bounds=vol.min_bounds,
                   max_bounds=vol.max_bounds)
        lut = rgba_lut(kw["color_tf"], kw["opacity_tf"])
        o8, _, _ = oracle.render(W.frame_inputs(v, kw["camera"], kw["light"], kw["config"], lut,
                                                kw["width"], kw["height"], vs, batch_camera=True),
                                 want_float=False)
        assert g == o8.tobytes()


def test_server_with_evictions():
    # room for about two of the small volumes: loads and re-loads evict others
    wl, stream, got, want, stats = _run(budget=3 << 20, n_req=120)
    for g, w in zip(got, want):
        assert g == w
    assert stats["evictions"] > 0


def _run_native(budget, n_req=160, per_frame=False, max_batch=16, slots=3, batch_pixels=0,
                half_records=False):
    """Results of the native server (batched or per-frame) and of the serial
    Python renderer for the same stream."""
    from pyvr_gb300.server import NativeRenderServer
    wl = _workload()
    stream = wl.requests(rate=4000.0, duration=1.0, seed=3)[:n_req]
    server = NativeRenderServer(budget_bytes=budget, max_batch=max_batch, slots=slots, per_frame=per_frame,
                                instrument=1, batch_pixels=batch_pixels, half_records=half_records)
    serial = SerialRenderer()
    for slot in range(wl.n_catalog):
        vol, vs = wl.volumes[slot]
        server.cache.insert(slot, vol, vs, server._free_volume)
        serial.cache.insert(slot, vol, vs, serial._free_now)
    reqs = [RenderRequest(**kw) for _, kw in stream]
    # the first half is held and released at once (full batches), the second
    # half is served as it arrives
    server.pause(True)
    futs = [server.submit(r) for r in reqs[:n_req // 2]]
    server.pause(False)
    futs += [server.submit(r) for r in reqs[n_req // 2:]]
    got = [f.result(timeout=120) for f in futs]
    want = [serial.handle(RenderRequest(**kw)) for _, kw in stream]
    stats = server.stats()
    stats.update(evictions=server.cache.evictions, lat=latency_stats(reqs))
    server.close()
    serial.close()
    return wl, stream, got, want, stats


@pytest.mark.parametrize("per_frame", [False, True])
def test_native_server_results_equal_results_alone(per_frame):
    wl, stream, got, want, stats = _run_native(budget=40 << 30, per_frame=per_frame)
    for (_, kw), g, w in zip(stream, got, want):
        assert g.dtype == np.uint8 and g.size == kw["width"] * kw["height"] * 4
        assert g.tobytes() == w
    assert stats["jobs"] == len(stream) and stats["shaded_samples"] > 0
    if per_frame:
        assert stats["max_jobs"] == 1 and stats["batches"] == len(stream)
    else:
        assert stats["max_jobs"] == 16  # held requests formed full batches
    assert stats["lat"]["n"] == len(stream)


def test_native_server_concurrent_launches_complete_out_of_order():
    """max_batch=1 over several slots: every request is its own launch, the
    launches overlap on the device, results equal the results alone, and a
    short render launched after a long one is handed back when it is done."""
    from pyvr_gb300 import RenderConfig
    from pyvr_gb300.server import NativeRenderServer
    wl, stream, got, want, stats = _run_native(budget=40 << 30, max_batch=1, slots=8)
    for g, w in zip(got, want):
        assert g.tobytes() == w
    assert stats["max_jobs"] == 1 and stats["batches"] == len(stream)
    server = NativeRenderServer(budget_bytes=1 << 30, max_batch=1, slots=8)
    vol, vs = wl.volumes[0]
    server.cache.insert(0, vol, vs, server._free_volume)
    base = dict(stream[0][1], volume_id=0, kind="render")
    long = RenderRequest(**dict(base, width=1024, height=1024, config=RenderConfig.ultra_quality()))
    short = [RenderRequest(**dict(base, width=32, height=32)) for _ in range(6)]
    server.pause(True)
    futs = [server.submit(r) for r in [long] + short]
    server.pause(False)
    for f in futs:
        f.result(timeout=60)
    server.close()
    assert all(s.launched_at >= long.launched_at for s in short)
    assert any(s.done_at < long.done_at for s in short), [(s.launched_at, s.done_at) for s in short]


def test_native_server_half_records_same_results():
    # float16 volumes (device normals) held as half records: the same bytes as
    # the float records of the per-request renderer
    wl, stream, got, want, stats = _run_native(budget=40 << 30, max_batch=8, half_records=True)
    for g, w in zip(got, want):
        assert g.tobytes() == w


def test_native_server_pixel_budget_per_launch():
    # 48^2 renders pair up within 2 x 48^2 pixels; a 64^2 capture goes alone
    wl, stream, got, want, stats = _run_native(budget=40 << 30, max_batch=16, batch_pixels=2 * 48 * 48)
    for g, w in zip(got, want):
        assert g.tobytes() == w
    assert stats["max_jobs"] == 2 and stats["jobs"] == len(stream)


def test_native_server_with_evictions_and_bad_requests():
    wl, stream, got, want, stats = _run_native(budget=3 << 20, n_req=120)
    for g, w in zip(got, want):
        assert g.tobytes() == w
    assert stats["evictions"] > 0
    from pyvr_gb300.server import NativeRenderServer
    server = NativeRenderServer(budget_bytes=1 << 30)
    vol, vs = wl.volumes[0]
    server.cache.insert(0, vol, vs, server._free_volume)
    kw = dict(stream[0][1], volume_id=0, width=0, kind="render")
    with pytest.raises(ValueError, match="size"):
        server.submit(RenderRequest(**kw)).result(timeout=30)
    kw = dict(stream[0][1], volume_id=99, kind="render", volume=None)
    with pytest.raises(KeyError):
        server.submit(RenderRequest(**kw)).result(timeout=30)
    server.close()


def test_native_server_request_deadline():
    """A request whose image is not back within its timeout fails with
    TimeoutError (launches held by pause()); its launch still completes and
    the server keeps serving: a later request returns the same image as a
    request without a deadline."""
    from pyvr_gb300.server import NativeRenderServer
    wl = _workload()
    stream = wl.requests(rate=4000.0, duration=0.2, seed=5)
    server = NativeRenderServer(budget_bytes=1 << 30, max_batch=4, slots=2)
    vol, vs = wl.volumes[0]
    server.cache.insert(0, vol, vs, server._free_volume)
    base = dict(stream[0][1], volume_id=0, kind="render")
    server.pause(True)
    late = RenderRequest(**dict(base, timeout_s=0.05))
    fut = server.submit(late)
    with pytest.raises(TimeoutError):
        fut.result(timeout=10)
    server.pause(False)
    a = server.submit(RenderRequest(**base)).result(timeout=30)
    b = server.submit(RenderRequest(**dict(base, timeout_s=10.0))).result(timeout=30)
    assert a.tobytes() == b.tobytes() and server.timeouts == 1
    server.close()
