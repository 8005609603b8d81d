"""Serving: a request loop over HBM-resident volumes with continuous batching.

The reference renders one frame per call on one GL context
(pyvr/moderngl_renderer/renderer.py:209-219) from an interactive loop
(pyvr/interface/matplotlib_interface.py:168-247: orbit re-renders, TF edits,
high-quality captures).  ``RenderServer`` (= ``NativeRenderServer``, on the
native serving runtime) and ``PyRenderServer`` (the same design with a
Python scheduler) serve that access pattern for many clients at once:

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
* transfer-function tables stay resident too, keyed by their content (an
  orbit re-render reuses its session's table: no upload);
* a batch writes its images into one device arena of its slot and comes back
  in one copy to pinned host memory; each result is handed back as RGBA8
  bytes (bottom row first, as ``render()`` returns them).

``SerialRenderer`` is the per-frame baseline: the same resident volumes, one
request at a time, each rendered and read back before the next starts.
"""

from __future__ import annotations

import collections
import ctypes
import gc
import heapq
import queue
import threading
import time
import weakref
from concurrent.futures import Future
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import _native
from .batch import BatchRenderer, DeviceLUT, DeviceVolume, Tuning, fill_job
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
    # > 0: the request fails with TimeoutError if its image is not back this
    # many seconds after its arrival (native server)
    timeout_s: float = 0.0
    arrival: float = 0.0
    tag: str = ""
    future: Future = field(default_factory=Future)
    done_at: float = 0.0
    launched_at: float = 0.0


class VolumeCache:
    """HBM-resident volumes with a byte budget and LRU eviction.

    Failure handling: when every resident volume is pinned by in-flight
    requests, a new volume is admitted over budget rather than stalling the
    request stream (counted in ``over_budget``); when a layout fails for lack
    of device memory (``MemoryError``), unpinned volumes are evicted, least
    recently used first, and the layout is retried (counted in
    ``alloc_retries``) until it succeeds or nothing is left to evict."""

    def __init__(self, budget_bytes: int, brick_log2: int = 3, half_records: bool = False,
                 release_wait=None, queue_layouts: bool = False):
        self.budget = int(budget_bytes)
        self.brick_log2 = brick_log2
        self.half_records = half_records
        # queue_layouts: insert() returns once a new volume's upload and
        # layout are queued (DeviceVolume(wait=False)); its renders wait for
        # them on the device
        self.queue_layouts = queue_layouts
        # release_wait(): wait until the memory of volumes released so far is
        # free again (before retrying a failed layout)
        self.release_wait = release_wait
        self._vols: "collections.OrderedDict[int, DeviceVolume]" = collections.OrderedDict()
        self._bytes: Dict[int, int] = {}
        self._users: Dict[int, int] = collections.defaultdict(int)  # in-flight batches
        self._lock = threading.Lock()
        self.evictions = 0
        self.loads = 0
        self.uploaded_bytes = 0  # host bytes of the volumes uploaded so far
        self.over_budget = 0     # admissions past the budget (every resident volume pinned)
        self.alloc_retries = 0   # layouts retried after evicting on a failed allocation

    def estimate_bytes(self, volume) -> int:
        """Device bytes a layout of ``volume`` needs at its peak: the records
        (8-byte halves for uint8 / float16 volumes when the library lays them
        out that way, else 16-byte floats) plus the uploaded voxels."""
        d, h, w = volume.data.shape
        rec = 16
        if np.asarray(volume.data).dtype in (np.uint8, np.float16):
            from .batch import get_compact_records
            try:
                rec = 8 if get_compact_records() == "half_normals" else 16
            except Exception:
                rec = 16
        lb = self.brick_log2
        return int(rec * ((w >> lb) + 1) * ((h >> lb) + 1) * ((d >> lb) + 1) * ((1 << lb) + 1) ** 3
                   + volume.data.nbytes)

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

    def clear(self) -> None:
        """Free every resident volume (nothing may be in flight)."""
        with self._lock:
            vols = list(self._vols.values())
            self._vols.clear()
            self._bytes.clear()
            self._users.clear()
        for dv in vols:
            dv.close()

    def evict_except(self, keep) -> list:
        """Take every volume whose id is not in ``keep`` and that no request
        in flight uses out of the cache (without counting them as
        evictions); the caller releases their memory."""
        with self._lock:
            out = []
            for vid in [k for k in self._vols if k not in keep and self._users.get(k, 0) == 0]:
                out.append(self._vols.pop(vid))
                self._bytes.pop(vid)
            return out

    def _evict_one(self):
        """Take the least recently used unpinned volume out of the cache (the
        caller releases its memory, outside the lock); None if none."""
        victim = next((k for k in self._vols if self._users.get(k, 0) == 0), None)
        if victim is None:
            return None
        dv = self._vols.pop(victim)
        self._bytes.pop(victim)
        self.evictions += 1
        return dv

    def _evict_for(self, need: int) -> list:
        out = []
        while self.used + need > self.budget:
            dv = self._evict_one()
            if dv is None:
                self.over_budget += 1  # everything is in use: go over budget rather than stall
                break
            out.append(dv)
        return out

    def insert(self, vid: int, volume, value_scale: float, release_after) -> DeviceVolume:
        """Upload + lay out (device normals) a volume and make it resident
        (a volume that is already resident is kept as it is).  Evicted
        volumes are handed to ``release_after`` outside the cache's lock, so
        that no device call holds up the requests that look volumes up."""
        with self._lock:
            if vid in self._vols:
                self._vols.move_to_end(vid)
                return self._vols[vid]
        est = self.estimate_bytes(volume)
        with self._lock:
            evicted = self._evict_for(est)
        for dv in evicted:
            release_after(dv)
        normals = "given" if getattr(volume, "normals", None) is not None else "device"
        while True:
            try:
                dv = DeviceVolume(volume, value_scale=value_scale, normals=normals,
                                  brick_log2=self.brick_log2, half_records=self.half_records,
                                  wait=not self.queue_layouts)
                break
            except MemoryError:
                # the device is fuller than the budget assumed (other memory
                # users, fragmentation): make room and try again
                with self._lock:
                    victim = self._evict_one()
                if victim is None:
                    raise
                release_after(victim)
                self.alloc_retries += 1
                if self.release_wait is not None:
                    self.release_wait()
        with self._lock:
            other = self._vols.get(vid)
            if other is None:
                self._vols[vid] = dv
                self._bytes[vid] = dv.device_bytes()
                self.loads += 1
                self.uploaded_bytes += int(volume.data.nbytes)
        if other is not None:  # loaded meanwhile by another request
            release_after(dv)
            return other
        return dv


class Deadlines:
    """Request deadlines by tag: ``expired(now)`` pops the tags whose
    deadline has passed, earliest first."""

    def __init__(self):
        self._heap: List[tuple] = []
        self._lock = threading.Lock()

    def add(self, tag, when: float) -> None:
        with self._lock:
            heapq.heappush(self._heap, (when, tag))

    def expired(self, now: float) -> list:
        out = []
        with self._lock:
            while self._heap and self._heap[0][0] <= now:
                out.append(heapq.heappop(self._heap)[1])
        return out

    def __len__(self) -> int:
        return len(self._heap)


def tf_key(color_tf, opacity_tf) -> tuple:
    """Content key of a transfer-function pair: equal keys give equal tables
    (``rgba_lut`` depends on the control points and LUT sizes alone).  Control
    points held as tuples of numbers are keyed as they are; anything else
    (lists, arrays) is normalised to tuples of floats first."""
    key = (tuple(color_tf.control_points), tuple(opacity_tf.control_points),
           color_tf.lut_size, opacity_tf.lut_size)
    try:
        hash(key)
        return key
    except TypeError:
        return (tuple((float(x), tuple(float(c) for c in rgb)) for x, rgb in color_tf.control_points),
                tuple((float(x), float(a)) for x, a in opacity_tf.control_points),
                int(color_tf.lut_size), int(opacity_tf.lut_size))


class LutCache:
    """Device LUTs keyed by transfer-function content (``tf_key``), LRU with a
    fixed number of entries.  A LUT in use by a queued batch is pinned
    (``acquire`` / ``release``) and never rewritten; an evicted LUT's memory
    is reused for the next new table.  New tables are built on the GPU from
    the control points (``DeviceLUT.build``) on the stream of the batch that
    first needs them; ``lut.ready`` = (event, stream) lets batches on other
    streams wait for the build.  Used from one thread."""

    def __init__(self, capacity: int = 1024, device_build: bool = True):
        self.capacity = capacity
        self.device_build = device_build
        self._luts: "collections.OrderedDict[tuple, DeviceLUT]" = collections.OrderedDict()
        self._users: Dict[tuple, int] = collections.defaultdict(int)
        self._free = _Pool(lambda n: DeviceLUT(rgba=np.zeros((n, 4), np.float32)))
        self.hits = 0
        self.misses = 0

    def acquire(self, color_tf, opacity_tf, stream=None, sync: bool = False):
        """(key, DeviceLUT) of the pair, built if new; pinned until release(key).
        sync: wait for a new table's build before returning."""
        key = tf_key(color_tf, opacity_tf)
        lut = self._luts.get(key)
        if lut is None:
            self._evict()
            n = max(int(color_tf.lut_size), int(opacity_tf.lut_size))
            lut = self._free.get(n)
            if self.device_build and stream is not None:
                import torch
                lut.build(color_tf, opacity_tf, n, stream)
                if sync:
                    stream.synchronize()
                    lut.ready = None
                else:
                    ev = getattr(lut, "_event", None)
                    if ev is None:
                        ev = lut._event = torch.cuda.Event()
                    ev.record(stream)
                    lut.ready = (ev, stream)
            else:
                lut.update(rgba_lut(color_tf, opacity_tf))
                lut.ready = None
            self._luts[key] = lut
            self.misses += 1
        else:
            self._luts.move_to_end(key)
            self.hits += 1
        self._users[key] += 1
        return key, lut

    def release(self, key) -> None:
        self._users[key] -= 1

    def reserve(self, size: int, count: int) -> None:
        """Allocate ``count`` tables of ``size`` entries up front, so that new
        transfer functions are built into memory that already exists."""
        for _ in range(count):
            self._free.put(size, DeviceLUT(rgba=np.zeros((size, 4), np.float32)))

    def clear(self) -> None:
        """Free every table (nothing may be in flight)."""
        luts = list(self._luts.values()) + self._free.drain()
        self._luts.clear()
        self._users.clear()
        for lut in luts:
            lut.close()

    def _evict(self) -> None:
        while len(self._luts) >= self.capacity:
            victim = next((k for k in self._luts if self._users.get(k, 0) == 0), None)
            if victim is None:
                return  # all in use: grow rather than stall
            lut = self._luts.pop(victim)
            self._users.pop(victim, None)
            self._free.put(lut.size, lut)


class _Arena:
    """A slot's output images: one device buffer and one pinned host buffer,
    grown (never shrunk) to the largest batch seen."""

    def __init__(self, torch):
        self.torch = torch
        self.nbytes = 0
        self.dev = None
        self.host = None
        self.view = None

    def reserve(self, nbytes: int) -> None:
        if nbytes <= self.nbytes:
            return
        n = 1 << max(20, (nbytes - 1).bit_length())
        self.dev = self.torch.empty(n, dtype=self.torch.uint8, device="cuda")
        self.host = self.torch.empty(n, dtype=self.torch.uint8).pin_memory()
        self.view = self.host.numpy()
        self.nbytes = n


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

    def drain(self) -> list:
        """Every free object, removed from the pool."""
        out = [o for lst in self._free.values() for o in lst]
        self._free.clear()
        return out


class PyRenderServer:
    """Continuous-batching render server with its scheduler in Python (see
    the module docstring); ``RenderServer`` is the native one."""

    def __init__(self, budget_bytes: int = 40 << 30, max_batch: int = 64, slots: int = 3,
                 tuning: Optional[Tuning] = None, brick_log2: int = 3, loaders: int = 2,
                 instrument: bool = False):
        import torch
        self.torch = torch
        # instrument: CUDA events around every batch kernel and per-job sample
        # counters (kernel_ms, samples, shaded) for roofline accounting
        self.instrument = instrument
        self.kernel_records: List[tuple] = []
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
        self.luts = LutCache()
        self._arenas = [_Arena(torch) for _ in range(slots)]
        self._structs = (_native.PvrJob * max_batch)()
        self._release_stream = torch.cuda.Stream()
        self.batches = 0
        self.batch_sizes: List[int] = []
        self._counters = torch.zeros((slots, max_batch, 2), dtype=torch.int64, device="cuda")
        self._threads = [threading.Thread(target=self._schedule, daemon=True, name="pvr-sched")]
        self._threads += [threading.Thread(target=self._load_loop, daemon=True, name=f"pvr-loader{i}")
                          for i in range(loaders)]
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
        for _ in self._threads:
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
        self.torch.cuda.set_device(self.torch.cuda.current_device())
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
        ev, reqs, offs, luts, vids = self._slot_busy[slot][:5]
        ev.synchronize()
        now = time.perf_counter()
        if self.instrument:
            k0, k1 = self._slot_busy[slot][5]
            per_job = self._counters[slot, :len(reqs)].tolist()
            self.kernel_records.append((k0.elapsed_time(k1), sum(c[0] for c in per_job),
                                        sum(c[1] for c in per_job),
                                        [(r.width, r.height, r.value_scale, c[1])
                                         for r, c in zip(reqs, per_job)]))
        view = self._arenas[slot].view
        for req, off in zip(reqs, offs):
            data = view[off:off + req.width * req.height * 4].tobytes()
            req.done_at = now
            req.future.set_result(data)
        for key in luts:
            self.luts.release(key)
        for vid in vids:
            self.cache.release(vid)
        self._slot_busy[slot] = None

    def _abandon(self, slot: int) -> None:
        busy = self._slot_busy[slot]
        self._slot_busy[slot] = None
        if busy is None:
            return
        _, _, _, luts, vids = busy[:5]
        for key in luts:
            self.luts.release(key)
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
        offs = []
        # resources belong to the slot from here on: released by _complete
        # or, on failure, by _abandon
        self._slot_busy[slot] = (None, reqs, offs, luts, vids)
        total = 0
        for req in reqs:  # images packed at 256-byte aligned offsets
            offs.append(total)
            total += (req.width * req.height * 4 + 255) & ~255
        arena = self._arenas[slot]
        arena.reserve(total)
        base = arena.dev.data_ptr()
        cbase = self._counters[slot].data_ptr() if self.instrument else None
        waited = set()
        for i, (req, dv) in enumerate(ready):
            key, lut = self.luts.acquire(req.color_tf, req.opacity_tf, stream)
            luts.append(key)
            rd = getattr(lut, "ready", None)
            if rd is not None and rd[1] is not stream and id(lut) not in waited:
                stream.wait_event(rd[0])  # built on another slot's stream
                waited.add(id(lut))
            fill_job(self._structs[i], dv.handle.value, lut.handle.value, req.camera, req.light,
                     req.config, int(req.width), int(req.height), base + offs[i], None,
                     cbase + 16 * i if cbase is not None else None)
        kev = None
        if self.instrument:
            kev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            with torch.cuda.stream(stream):
                self._counters[slot].zero_()
                kev[0].record(stream)
        self.launcher.render_structs(self._structs, len(reqs), stream=stream)
        ev = torch.cuda.Event()
        with torch.cuda.stream(stream):
            if kev:
                kev[1].record(stream)
            arena.host[:total].copy_(arena.dev[:total], non_blocking=True)
            ev.record(stream)
        self._slot_busy[slot] = (ev, reqs, offs, luts, vids, kev)
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
        self.luts = LutCache()
        self._struct = (_native.PvrJob * 1)()

    def _free_now(self, dv: DeviceVolume) -> None:
        self.torch.cuda.synchronize()
        dv.close()

    def handle(self, req: RenderRequest) -> bytes:
        torch = self.torch
        dv = None if req.kind == "load" else self.cache.get(req.volume_id)
        if dv is None:  # a new volume, or one evicted earlier: load it first
            if req.volume is None:
                raise KeyError(f"volume {req.volume_id} is not resident")
            dv = self.cache.insert(req.volume_id, req.volume, req.value_scale, self._free_now)
        key, lut = self.luts.acquire(req.color_tf, req.opacity_tf, self.stream)
        self.luts.release(key)  # nothing is queued after this request returns
        wh = (req.width, req.height)
        if wh not in self._bufs:
            self._bufs[wh] = (torch.empty(wh[0] * wh[1] * 4, dtype=torch.uint8, device="cuda"),
                              torch.empty(wh[0] * wh[1] * 4, dtype=torch.uint8).pin_memory())
        dev, host = self._bufs[wh]
        fill_job(self._struct[0], dv.handle.value, lut.handle.value, req.camera, req.light,
                 req.config, int(req.width), int(req.height), dev.data_ptr())
        self.launcher.render_structs(self._struct, 1, stream=self.stream)
        with torch.cuda.stream(self.stream):
            host.copy_(dev, non_blocking=True)
        self.stream.synchronize()
        return host.numpy().tobytes()

    def close(self) -> None:
        self.torch.cuda.synchronize()
        self.launcher.close()


class _PinnedPool:
    """Page-locked result buffers carved from one pinned block and recycled:
    a result array hands its slab back when it is garbage-collected.
    Bounded: once the block is used up, results go to ordinary memory."""

    def __init__(self, torch, cap_bytes: int = 1 << 30):
        self._block = torch.empty(cap_bytes, dtype=torch.uint8).pin_memory()
        self._np = self._block.numpy()
        self._base = self._block.data_ptr()
        self._top = 0
        self._cap = cap_bytes
        self._free = collections.defaultdict(list)  # slab size -> offsets
        self._lock = threading.Lock()

    def get(self, n: int) -> Optional[int]:
        """Offset of a free slab of n bytes (256-byte aligned), or None."""
        with self._lock:
            lst = self._free[n]
            if lst:
                return lst.pop()
            size = (n + 255) & ~255
            if self._top + size > self._cap:
                return None
            off = self._top
            self._top += size
            return off

    def put(self, n: int, off: int) -> None:
        with self._lock:
            self._free[n].append(off)

    def address(self, off: int) -> int:
        return self._base + off

    def wrap(self, n: int, off: int) -> np.ndarray:
        """The slab as a numpy array that hands the slab back when it dies."""
        arr = self._np[off:off + n]
        weakref.finalize(arr, self.put, n, off)
        return arr


class NativeRenderServer:
    """Continuous-batching render server on the native runtime
    (``pvr_server_*``): batch formation, launches, read-back and completion
    run on C++ threads; Python resolves residency (volumes, LUTs) at submit
    and hands results back.

    A result is the request's RGBA8 image as a flat uint8 array (H*W*4,
    bottom row first: the bytes ``render()`` returns).  per_frame=True is
    the per-frame baseline on the same runtime (one request per launch, each
    read back before the next starts).  instrument=N times every N-th batch
    kernel and counts its samples (``stats()``).

    Batching: up to ``slots`` launches are in flight, each on its own stream,
    so requests that arrive while others are on the GPU start as soon as a
    slot frees up and overlap with them on the device; a slot hands its
    results back as soon as its own work is done.  A launch takes queued
    requests up to ``max_batch`` and, with ``batch_pixels`` > 0, while their
    pixel counts sum to at most ``batch_pixels``: small renders are fused
    into one persistent launch, while renders of that size or larger run as
    launches of their own (the single-render kernel) side by side.  The
    defaults (8 slots, 512^2 pixels per launch) measured best on a mixed
    512^2 / 1024^2 stream.  ``lut_reserve`` tables of 256 entries are
    allocated at start, so that new transfer functions are built into
    existing memory.  half_records: resident volumes whose values and normals
    are all halves exactly (float16 volumes with device normals) keep their
    records as halves: half the memory, the same images.  ``loaders``
    threads upload and lay out new volumes (one measured best: concurrent
    uploads of large volumes slow each other down).  close() frees the
    resident volumes and tables."""

    def __init__(self, budget_bytes: int = 40 << 30, max_batch: int = 64, slots: int = 8,
                 tuning: Optional[Tuning] = None, brick_log2: int = 3, loaders: int = 1,
                 instrument: int = 0, per_frame: bool = False, linger_us: int = 0,
                 batch_pixels: int = 512 * 512, lut_reserve: int = 1024, half_records: bool = False):
        import torch
        self.torch = torch
        self._release_stream = torch.cuda.Stream()
        self.cache = VolumeCache(budget_bytes, brick_log2, half_records,
                                 release_wait=self._release_stream.synchronize, queue_layouts=True)
        # the volume memory pool holds the budget (and room for a layout in
        # progress) from the start: loads and evictions then reuse pool
        # memory instead of mapping new memory while renders run
        _native.check(_native.load().pvr_reserve_volume_memory(int(budget_bytes * 1.1)))
        self.luts = LutCache()
        self.luts.reserve(256, lut_reserve)
        self.per_frame = per_frame
        self._deadlines = Deadlines()
        self.timeouts = 0
        self._lut_stream = torch.cuda.Stream()
        self._lock = threading.Lock()  # LUT cache and in-flight table
        self._pool = _PinnedPool(torch)
        self._lib = _native.load()
        cfg = _native.PvrServerConfig(int(max_batch), int(slots), int(per_frame), int(instrument),
                                      int(linger_us),
                                      tuning.c() if tuning is not None else _native.PvrTuning(0, 0, 0, 0),
                                      int(batch_pixels))
        h = ctypes.c_void_p()
        _native.check(self._lib.pvr_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._inflight: Dict[int, tuple] = {}
        self._next_tag = 1
        self._loads: "queue.Queue[RenderRequest]" = queue.Queue()
        self._stop = False
        self._threads = [threading.Thread(target=self._poll_loop, daemon=True, name="pvr-poll")]
        self._threads += [threading.Thread(target=self._load_loop, daemon=True, name=f"pvr-load{i}")
                          for i in range(loaders)]
        for t in self._threads:
            t.start()

    # -- client API -------------------------------------------------------------
    def submit(self, req: RenderRequest) -> Future:
        """Queue a request; its future gets the image (or the exception).  In
        the per-frame baseline a new-volume load runs here, in the caller's
        thread, before the request's render is queued: a serial renderer
        serves the load before anything that arrives after it."""
        if not req.arrival:
            req.arrival = time.perf_counter()
        if req.kind == "load":
            if self.per_frame:
                self._load_then_render(req)
            else:
                self._loads.put(req)
        else:
            self._submit_render(req)
        return req.future

    def pause(self, paused: bool = True) -> None:
        """Hold launches (submissions queue up) or resume them."""
        _native.check(self._lib.pvr_server_pause(self._h, int(paused)))

    def stats(self) -> dict:
        st = _native.PvrServerStats()
        _native.check(self._lib.pvr_server_get_stats(self._h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def reset_stats(self) -> None:
        _native.check(self._lib.pvr_server_reset_stats(self._h))

    def close(self) -> None:
        if self._h is None:
            return
        deadline = time.time() + 120
        while self._inflight and time.time() < deadline:
            time.sleep(0.001)
        self._stop = True
        for _ in self._threads:
            self._loads.put(None)
        for t in self._threads:  # the poller exits once nothing is in flight
            t.join(timeout=30)
        h, self._h = self._h, None
        self._lib.pvr_server_destroy(h)
        self.torch.cuda.synchronize()
        self.cache.clear()
        with self._lock:
            self.luts.clear()

    # -- internals -----------------------------------------------------------------
    def _free_volume(self, dv: DeviceVolume) -> None:
        """An evicted volume: no request uses it any more (every batch that read
        it has completed), so it is freed in the order of a private stream
        (behind its layout, if that is still queued).  Its host arrays are
        let go only once the upload has read them."""
        while not dv.ready():
            time.sleep(0.0002)
        _native.check(self._lib.pvr_volume_release(dv.handle, self._release_stream.cuda_stream))
        dv.handle = None

    def _load_then_render(self, req: RenderRequest) -> None:
        if req.timeout_s > 0 and time.perf_counter() > req.arrival + req.timeout_s:
            self.timeouts += 1
            req.future.set_exception(TimeoutError(f"request timed out after {req.timeout_s} s before its load"))
            return
        try:
            self.cache.insert(req.volume_id, req.volume, req.value_scale, self._free_volume)
        except Exception as e:
            req.future.set_exception(e)
            return
        req.kind = "render"
        self._submit_render(req)

    def _load_loop(self) -> None:
        self.torch.cuda.set_device(self.torch.cuda.current_device())
        while True:
            req = self._loads.get()
            if req is None or self._stop:
                return
            self._load_then_render(req)

    def _submit_render(self, req: RenderRequest) -> None:
        dv = self.cache.acquire(req.volume_id)
        if dv is None:  # not resident (evicted meanwhile): load it, then render
            if req.volume is None:
                req.future.set_exception(KeyError(f"volume {req.volume_id} is not resident"))
            else:
                req.kind = "load"
                self._loads.put(req)
            return
        key = tag = out = None
        try:
            with self._lock:
                key, lut = self.luts.acquire(req.color_tf, req.opacity_tf, self._lut_stream)
                tag = self._next_tag
                self._next_tag += 1
            nbytes = req.width * req.height * 4
            slab = self._pool.get(nbytes) if nbytes > 0 else None
            out = (nbytes, slab) if slab is not None else np.empty(nbytes, np.uint8)
            r = _native.PvrRequest()
            r.camera_mode = _native.PVR_CAMERA_ORBIT
            r.volume = dv.handle.value
            r.lut = lut.handle.value
            rd = getattr(lut, "ready", None)
            r.wait_event = rd[0].cuda_event if rd is not None else None
            cam = req.camera
            t, ip, iu = cam.target, cam.init_pos, cam.init_up
            r.target[0], r.target[1], r.target[2] = float(t[0]), float(t[1]), float(t[2])
            r.init_pos[0], r.init_pos[1], r.init_pos[2] = float(ip[0]), float(ip[1]), float(ip[2])
            r.init_up[0], r.init_up[1], r.init_up[2] = float(iu[0]), float(iu[1]), float(iu[2])
            r.azimuth, r.elevation, r.roll = float(cam.azimuth), float(cam.elevation), float(cam.roll)
            r.distance, r.fov = float(cam.distance), float(cam.fov)
            r.near_plane, r.far_plane = float(cam.near_plane), float(cam.far_plane)
            lp, lt, light = req.light.position, req.light.target, req.light
            r.light_pos[0], r.light_pos[1], r.light_pos[2] = float(lp[0]), float(lp[1]), float(lp[2])
            r.light_target[0], r.light_target[1], r.light_target[2] = float(lt[0]), float(lt[1]), float(lt[2])
            r.ambient, r.diffuse = float(light.ambient_intensity), float(light.diffuse_intensity)
            cfg = req.config
            r.step_size, r.reference_step_size = float(cfg.step_size), float(cfg.reference_step_size)
            r.max_steps = int(cfg.max_steps)
            r.width, r.height = int(req.width), int(req.height)
            r.out_rgba8 = self._pool.address(slab) if slab is not None else out.ctypes.data
            r.out_pinned = int(slab is not None)
            r.tag = tag
            self._inflight[tag] = (req, req.volume_id, key, out)
            if req.timeout_s > 0:
                self._deadlines.add(tag, req.arrival + req.timeout_s)
            rc = self._lib.pvr_server_submit(self._h, ctypes.byref(r))
            if rc == _native.PVR_ERR_VALUE and b"parallel" in self._lib.pvr_last_error():
                # degenerate orbit camera: the Camera methods' matrices
                from .renderer import camera_uniforms
                v, p, c = camera_uniforms(cam, req.width, req.height)
                r.camera_mode = _native.PVR_CAMERA_MATRICES
                r.view[:] = v.ravel().tolist()
                r.proj[:] = p.ravel().tolist()
                r.camera_pos[:] = c.tolist()
                rc = self._lib.pvr_server_submit(self._h, ctypes.byref(r))
            _native.check(rc)
        except Exception as e:
            self._inflight.pop(tag, None)
            if isinstance(out, tuple):
                self._pool.put(*out)
            self.cache.release(req.volume_id)
            if key is not None:
                with self._lock:
                    self.luts.release(key)
            req.future.set_exception(e)

    def _poll_loop(self) -> None:
        comps = (_native.PvrCompletion * 256)()
        n = ctypes.c_int(0)
        h = self._h
        while True:
            if self._lib.pvr_server_poll(h, comps, 256, 20, ctypes.byref(n)) != 0:
                return
            for c in comps[:n.value]:
                req, vid, key, out = self._inflight.pop(c.tag)
                self.cache.release(vid)
                with self._lock:
                    self.luts.release(key)
                req.done_at = c.t_done_ns / 1e9
                req.launched_at = c.t_launch_ns / 1e9
                if req.future.done():  # failed by its deadline: the image is dropped
                    if not isinstance(out, np.ndarray):
                        self._pool.put(*out)
                    continue
                if not isinstance(out, np.ndarray):
                    if c.status == 0:
                        out = self._pool.wrap(*out)
                    else:
                        self._pool.put(*out)
                if c.status == 0:
                    req.future.set_result(out)
                else:
                    req.future.set_exception(RuntimeError(
                        f"render failed (status {c.status}): "
                        f"{self._lib.pvr_server_last_error(self._h).decode(errors='replace')}"))
            if len(self._deadlines):
                # requests past their deadline fail now; their launches still
                # finish (their memory stays in use until then)
                for tag in self._deadlines.expired(time.perf_counter()):
                    entry = self._inflight.get(tag)
                    if entry is not None and not entry[0].future.done():
                        self.timeouts += 1
                        entry[0].future.set_exception(
                            TimeoutError(f"request timed out after {entry[0].timeout_s} s"))
            if self._stop and not self._inflight:
                return


def latency_stats(reqs: List[RenderRequest]) -> dict:
    lat = np.array([(r.done_at - r.arrival) * 1000.0 for r in reqs if r.done_at])
    if lat.size == 0:
        return {"n": 0}
    return {"n": int(lat.size), "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat.max()),
            "mean_ms": float(lat.mean())}


def latency_by_tag(reqs: List[RenderRequest]) -> dict:
    """latency_stats of the requests of each tag."""
    tags: Dict[str, list] = {}
    for r in reqs:
        tags.setdefault(r.tag, []).append(r)
    return {k: latency_stats(v) for k, v in sorted(tags.items())}


def bounded(reqs: List[RenderRequest], tags=None) -> List[RenderRequest]:
    """The requests a latency bound applies to: those whose tag is in `tags`
    (all requests if tags is None)."""
    return list(reqs) if tags is None else [r for r in reqs if r.tag in tags]


def _wait_until(t: float) -> None:
    while True:
        dt = t - time.perf_counter()
        if dt <= 0:
            return
        time.sleep(dt - 0.0003 if dt > 0.0006 else 0.00005)


_CONSUMED: Future = Future()
_CONSUMED.set_result(None)


def _consume(req: RenderRequest):
    """Done-callback of a load-generating client: the image is taken and
    dropped at once (its buffer can be reused), the timings stay."""
    def cb(f):
        if f.exception() is None:
            req.future = _CONSUMED
    return cb


def drive(impl, stream, timeout: float = 300.0):
    """Replay a request stream [(arrival offset s, RenderRequest kwargs)] in
    real time against a server or a SerialRenderer (open loop: a client
    thread submits at the arrival times whatever the service does, and drops
    each image as soon as it arrives).  Returns (requests, seconds from the
    first arrival to the last completion)."""
    reqs = [RenderRequest(**kw) for _, kw in stream]
    if not reqs:
        return reqs, 0.0
    # the request objects (and everything else alive now) are moved out of the
    # cyclic collector's reach, and the collector is off for the replay (as
    # in a latency-bound service): no collection pause holds up a submission
    gc.collect()
    gc.freeze()
    enabled = gc.isenabled()
    gc.disable()
    try:
        return _replay(impl, stream, reqs, timeout)
    finally:
        if enabled:
            gc.enable()
        gc.unfreeze()


def _replay(impl, stream, reqs, timeout):
    if not isinstance(impl, SerialRenderer):
        t0 = time.perf_counter()
        for (off, _), req in zip(stream, reqs):
            _wait_until(t0 + off)
            # the scheduled arrival: a submission that runs late (the client
            # thread held up) counts against the request's latency
            req.arrival = t0 + off
            impl.submit(req).add_done_callback(_consume(req))
        for req in reqs:
            req.future.result(timeout=timeout)
        return reqs, max(r.done_at for r in reqs) - t0
    # serial: one worker thread serves a FIFO in order
    q: "queue.Queue" = queue.Queue()

    def worker():
        while True:
            req = q.get()
            if req is None:
                return
            try:
                req.future.set_result(impl.handle(req))
            except Exception as e:
                req.future.set_exception(e)
            req.done_at = time.perf_counter()

    th = threading.Thread(target=worker, daemon=True)
    th.start()
    t0 = time.perf_counter()
    for (off, _), req in zip(stream, reqs):
        _wait_until(t0 + off)
        req.arrival = t0 + off
        q.put(req)
    q.put(None)
    for req in reqs:
        req.future.result(timeout=timeout)
    th.join()
    return reqs, max(r.done_at for r in reqs) - t0


def sustained_rate(impl, workload, rates, probe_s: float, seed: int, p99_ms: float = 20.0,
                   refine: int = 0, reset=None, bound_tags=None):
    """Highest offered rate that `impl` serves with p99 latency <= p99_ms and
    completions keeping up with arrivals: probes `rates` (ascending) up to the
    first failure, then bisects `refine` times between the last passing and
    the first failing rate.  A failing probe is repeated once (another stream
    at the same rate), so that one transient stall does not end the sweep.
    reset(): called before every probe (e.g. to restart a workload whose
    state evolves from the same point).  bound_tags: the request tags the p99
    bound applies to (all requests if None).  Returns (rate or None, [probe
    results])."""
    probes = []

    def probe(rate, k):
        for attempt in range(2):
            if reset is not None:
                reset()
            stream = workload.requests(rate, probe_s, seed + k + 1000 * attempt)
            reqs, elapsed = drive(impl, stream)
            st = latency_stats(reqs)
            st.update(offered=rate, completed_per_s=len(reqs) / elapsed if elapsed else 0.0, repeat=attempt)
            st["bound_p99_ms"] = latency_stats(bounded(reqs, bound_tags)).get("p99_ms", 1e9)
            st["ok"] = bool(st["bound_p99_ms"] <= p99_ms and st["completed_per_s"] >= 0.9 * rate)
            probes.append(st)
            if st["ok"]:
                return True
        return False

    best, fail = None, None
    for rate in rates:
        if not probe(rate, len(probes)):
            fail = rate
            break
        best = rate
    if best is not None and fail is not None:
        lo, hi = best, fail
        for _ in range(refine):
            mid = 0.5 * (lo + hi)
            if probe(mid, len(probes)):
                lo = mid
            else:
                hi = mid
        best = lo
    return best, probes


# the serving API: the native runtime
RenderServer = NativeRenderServer
