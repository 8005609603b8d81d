"""Serving: a request loop over HBM-resident volumes with continuous batching.

The reference renders one frame per call on one GL context
(pyvr/moderngl_renderer/renderer.py:209-219) from an interactive loop
(pyvr/interface/matplotlib_interface.py:168-247: orbit re-renders, TF edits,
high-quality captures).  ``RenderServer`` serves that access pattern for many
clients at once:

* volumes stay resident in HBM as march records (``DeviceVolume``); a byte
  budget is enforced with LRU eviction, and an evicted volume's memory is
  freed in stream order behind the last batch that read it;
* new volumes are uploaded and laid out (normals computed on the GPU) by a
  loader thread on its own stream while renders continue;
* a scheduler thread forms batches from whatever requests are pending and
  launches them as soon as one of ``slots`` launch slots is free: requests
  that arrive while others are on the GPU are admitted into the next batch,
  and up to ``slots`` batches overlap on the device (each on its own stream,
  its read-back overlapping the next batch's march);
* each result is copied to pinned host memory and handed back as RGBA8 bytes
  (bottom row first, as ``render()`` returns them).

``SerialRenderer`` is the per-frame baseline: the same resident volumes, one
request at a time, each rendered and read back before the next starts.
"""

from __future__ import annotations

import collections
import queue
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import _native
from .batch import BatchRenderer, DeviceLUT, DeviceVolume, RenderJob, Tuning, make_job_struct
from .renderer import rgba_lut


@dataclass
class RenderRequest:
    """One client request.  kind: 'render' (orbit re-render / TF edit /
    capture: a render of a resident volume) or 'load' (a new volume, then a
    render of it).  ``volume`` is the pyvr-style Volume to upload for 'load'."""

    kind: str
    volume_id: int
    camera: object
    light: object
    config: object
    color_tf: object
    opacity_tf: object
    width: int
    height: int
    value_scale: float = 1.0
    volume: object = None
    arrival: float = 0.0
    tag: str = ""
    future: Future = field(default_factory=Future)
    done_at: float = 0.0


class VolumeCache:
    """HBM-resident volumes with a byte budget and LRU eviction."""

    def __init__(self, budget_bytes: int, brick_log2: int = 3):
        self.budget = int(budget_bytes)
        self.brick_log2 = brick_log2
        self._vols: "collections.OrderedDict[int, DeviceVolume]" = collections.OrderedDict()
        self._bytes: Dict[int, int] = {}
        self._users: Dict[int, int] = collections.defaultdict(int)  # in-flight batches
        self._lock = threading.Lock()
        self.evictions = 0
        self.loads = 0

    @property
    def used(self) -> int:
        return sum(self._bytes.values())

    def get(self, vid: int) -> Optional[DeviceVolume]:
        with self._lock:
            dv = self._vols.get(vid)
            if dv is not None:
                self._vols.move_to_end(vid)
            return dv

    def acquire(self, vid: int) -> Optional[DeviceVolume]:
        """The resident volume, pinned against eviction (None if not resident)."""
        with self._lock:
            dv = self._vols.get(vid)
            if dv is not None:
                self._vols.move_to_end(vid)
                self._users[vid] += 1
            return dv

    def release(self, vid: int) -> None:
        with self._lock:
            self._users[vid] -= 1

    def _evict_for(self, need: int, release_after) -> None:
        while self.used + need > self.budget:
            victim = next((k for k in self._vols if self._users.get(k, 0) == 0), None)
            if victim is None:
                break  # everything is in use: go over budget rather than stall
            dv = self._vols.pop(victim)
            self._bytes.pop(victim)
            release_after(dv)
            self.evictions += 1

    def insert(self, vid: int, volume, value_scale: float, release_after) -> DeviceVolume:
        """Upload + lay out (device normals) a volume and make it resident
        (a volume that is already resident is kept as it is)."""
        with self._lock:
            if vid in self._vols:
                self._vols.move_to_end(vid)
                return self._vols[vid]
        d, h, w = volume.data.shape
        est = int(16 * ((w >> self.brick_log2) + 1) * ((h >> self.brick_log2) + 1) *
                  ((d >> self.brick_log2) + 1) * ((1 << self.brick_log2) + 1) ** 3
                  + volume.data.nbytes)
        with self._lock:
            self._evict_for(est, release_after)
        normals = "given" if getattr(volume, "normals", None) is not None else "device"
        dv = DeviceVolume(volume, value_scale=value_scale, normals=normals,
                          brick_log2=self.brick_log2)
        with self._lock:
            if vid in self._vols:  # loaded meanwhile by another request
                release_after(dv)
                return self._vols[vid]
            self._vols[vid] = dv
            self._bytes[vid] = dv.device_bytes()
            self.loads += 1
        return dv


class _Pool:
    """Free lists of reusable objects keyed by a shape key."""

    def __init__(self, factory):
        self._factory = factory
        self._free = collections.defaultdict(list)

    def get(self, key):
        lst = self._free[key]
        return lst.pop() if lst else self._factory(key)

    def put(self, key, obj):
        self._free[key].append(obj)


class RenderServer:
    """Continuous-batching render server (see module docstring)."""

    def __init__(self, budget_bytes: int = 40 << 30, max_batch: int = 64, slots: int = 3,
                 tuning: Optional[Tuning] = None, brick_log2: int = 3):
        import torch
        self.torch = torch
        self.cache = VolumeCache(budget_bytes, brick_log2)
        self.max_batch = max_batch
        self.launcher = BatchRenderer(capacity=max_batch, slots=slots, tuning=tuning)
        self.streams = [torch.cuda.Stream() for _ in range(slots)]
        self._slot_busy = [None] * slots  # in-flight batch per slot
        self._pending: "collections.deque[RenderRequest]" = collections.deque()
        self._incoming: "queue.Queue[RenderRequest]" = queue.Queue()
        self._loads: "queue.Queue[RenderRequest]" = queue.Queue()
        self._wake = threading.Event()
        self._stop = False
        self._out_pool = _Pool(lambda wh: (torch.empty(wh[0] * wh[1] * 4, dtype=torch.uint8, device="cuda"),
                                           torch.empty(wh[0] * wh[1] * 4, dtype=torch.uint8).pin_memory()))
        self._lut_pool = _Pool(lambda n: DeviceLUT(rgba=np.zeros((n, 4), np.float32)))
        self._structs = (_native.PvrJob * max_batch)()
        self._release_stream = torch.cuda.Stream()
        self.batches = 0
        self.batch_sizes: List[int] = []
        self._threads = [threading.Thread(target=self._schedule, daemon=True, name="pvr-sched"),
                         threading.Thread(target=self._load_loop, daemon=True, name="pvr-loader")]
        for t in self._threads:
            t.start()

    # -- client API -------------------------------------------------------------
    def submit(self, req: RenderRequest) -> Future:
        if not req.arrival:
            req.arrival = time.perf_counter()
        if req.kind == "load":
            self._loads.put(req)
        else:
            self._incoming.put(req)
            self._wake.set()
        return req.future

    def close(self) -> None:
        self._stop = True
        self._wake.set()
        self._loads.put(None)
        for t in self._threads:
            t.join(timeout=30)
        self.torch.cuda.synchronize()
        self.launcher.close()

    # -- volume loading ---------------------------------------------------------------
    def _release_after_inflight(self, dv: DeviceVolume) -> None:
        """Free an evicted volume in stream order behind every batch queued so
        far (no batch formed later can use it: it is no longer resident)."""
        for s in self.streams:
            self._release_stream.wait_stream(s)
        _native.check(_native.load().pvr_volume_release(dv.handle, self._release_stream.cuda_stream))
        dv.handle = None

    def _load_loop(self) -> None:
        while True:
            req = self._loads.get()
            if req is None or self._stop:
                return
            try:
                self.cache.insert(req.volume_id, req.volume, req.value_scale,
                                  self._release_after_inflight)
            except Exception as e:  # surface the failure to the client
                req.future.set_exception(e)
                continue
            req.kind = "render"
            self._incoming.put(req)
            self._wake.set()

    # -- scheduling -------------------------------------------------------------------
    def _drain_incoming(self) -> None:
        while True:
            try:
                self._pending.append(self._incoming.get_nowait())
            except queue.Empty:
                return

    def _complete(self, slot: int) -> None:
        ev, reqs, bufs, luts, vids = self._slot_busy[slot]
        ev.synchronize()
        now = time.perf_counter()
        for req, (wh, (dev, host)) in zip(reqs, bufs):
            data = host.numpy().tobytes()
            req.done_at = now
            req.future.set_result(data)
            self._out_pool.put(wh, (dev, host))
        for lut in luts:
            self._lut_pool.put(lut.size, lut)
        for vid in vids:
            self.cache.release(vid)
        self._slot_busy[slot] = None

    def _abandon(self, slot: int) -> None:
        busy = self._slot_busy[slot]
        self._slot_busy[slot] = None
        if busy is None:
            return
        _, _, bufs, luts, vids = busy
        for wh, pair in bufs:
            self._out_pool.put(wh, pair)
        for lut in luts:
            self._lut_pool.put(lut.size, lut)
        for vid in vids:
            self.cache.release(vid)

    def _launch(self, slot: int, reqs: List[RenderRequest]) -> None:
        torch = self.torch
        stream = self.streams[slot]
        bufs, luts, vids, ready = [], [], [], []
        for req in reqs:
            dv = self.cache.acquire(req.volume_id)
            if dv is None:  # evicted meanwhile: reload it, then render
                if req.volume is None:
                    req.future.set_exception(KeyError(f"volume {req.volume_id} is not resident"))
                else:
                    req.kind = "load"
                    self._loads.put(req)
                continue
            ready.append((req, dv))
        if not ready:
            return
        reqs = [r for r, _ in ready]
        vids = [r.volume_id for r in reqs]
        # resources belong to the slot from here on: released by _complete
        # or, on failure, by _abandon
        self._slot_busy[slot] = (None, reqs, bufs, luts, vids)
        for i, (req, dv) in enumerate(ready):
            table = rgba_lut(req.color_tf, req.opacity_tf)
            lut = self._lut_pool.get(table.shape[0])
            lut.update(table)
            luts.append(lut)
            wh = (req.width, req.height)
            dev, host = self._out_pool.get(wh)
            bufs.append((wh, (dev, host)))
            job = RenderJob(dv, lut, req.camera, req.light, req.config, req.width, req.height,
                            out_rgba8=dev)
            make_job_struct(job, self._structs[i])
        self.launcher.render_structs(self._structs, len(reqs), stream=stream)
        ev = torch.cuda.Event()
        with torch.cuda.stream(stream):
            for _, (dev, host) in bufs:
                host.copy_(dev, non_blocking=True)
            ev.record(stream)
        self._slot_busy[slot] = (ev, reqs, bufs, luts, vids)
        self.batches += 1
        self.batch_sizes.append(len(reqs))

    def _schedule(self) -> None:
        torch = self.torch
        torch.cuda.set_device(torch.cuda.current_device())
        while not self._stop or any(self._slot_busy) or self._pending:
            self._drain_incoming()
            # retire finished batches
            for s, busy in enumerate(self._slot_busy):
                if busy is not None and busy[0].query():
                    self._complete(s)
            free = [s for s, b in enumerate(self._slot_busy) if b is None]
            if free and self._pending:
                batch = []
                while self._pending and len(batch) < self.max_batch:
                    batch.append(self._pending.popleft())
                try:
                    self._launch(free[0], batch)
                except Exception as e:  # fail this batch's renders, keep serving
                    busy = self._slot_busy[free[0]]
                    for req in (busy[1] if busy else []):
                        if not req.future.done():
                            req.future.set_exception(e)
                    torch.cuda.synchronize()
                    self._abandon(free[0])
                continue
            if self._stop and not self._pending and not any(self._slot_busy):
                return
            if not self._pending and not any(self._slot_busy):
                self._wake.wait(timeout=0.005)
                self._wake.clear()
            elif not free:
                # all slots busy: wait for the oldest batch to finish
                busy = [b for b in self._slot_busy if b is not None]
                busy[0][0].synchronize()
            else:
                time.sleep(0.0002)


class SerialRenderer:
    """Per-frame baseline: the same resident volumes (shared cache policy),
    one request at a time, each rendered and read back before the next."""

    def __init__(self, budget_bytes: int = 40 << 30, tuning: Optional[Tuning] = None,
                 brick_log2: int = 3):
        import torch
        self.torch = torch
        self.cache = VolumeCache(budget_bytes, brick_log2)
        self.launcher = BatchRenderer(capacity=1, slots=1, tuning=tuning)
        self.stream = torch.cuda.Stream()
        self._bufs = {}
        self._lut = DeviceLUT(rgba=np.zeros((256, 4), np.float32))
        self._struct = (_native.PvrJob * 1)()

    def _free_now(self, dv: DeviceVolume) -> None:
        self.torch.cuda.synchronize()
        dv.close()

    def handle(self, req: RenderRequest) -> bytes:
        torch = self.torch
        if req.kind == "load":
            self.cache.insert(req.volume_id, req.volume, req.value_scale, self._free_now)
        dv = self.cache.get(req.volume_id)
        table = rgba_lut(req.color_tf, req.opacity_tf)
        self._lut.update(table)
        wh = (req.width, req.height)
        if wh not in self._bufs:
            self._bufs[wh] = (torch.empty(wh[0] * wh[1] * 4, dtype=torch.uint8, device="cuda"),
                              torch.empty(wh[0] * wh[1] * 4, dtype=torch.uint8).pin_memory())
        dev, host = self._bufs[wh]
        make_job_struct(RenderJob(dv, self._lut, req.camera, req.light, req.config, req.width,
                                  req.height, out_rgba8=dev), self._struct[0])
        self.launcher.render_structs(self._struct, 1, stream=self.stream)
        with torch.cuda.stream(self.stream):
            host.copy_(dev, non_blocking=True)
        self.stream.synchronize()
        return host.numpy().tobytes()

    def close(self) -> None:
        self.torch.cuda.synchronize()
        self.launcher.close()


def latency_stats(reqs: List[RenderRequest]) -> dict:
    lat = np.array([(r.done_at - r.arrival) * 1000.0 for r in reqs if r.done_at])
    if lat.size == 0:
        return {"n": 0}
    return {"n": int(lat.size), "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat.max()),
            "mean_ms": float(lat.mean())}
