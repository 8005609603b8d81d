"""Autotuner of the persistent batch march: tile shape, brick size, steps per
loop iteration and resident blocks per SM, picked by timing the real batch.

A candidate is a ``Tuning``.  Its brick size fixes the volumes' march layout
(bricks of 4^3, 8^3 or 16^3 texels), so the batch's volumes are laid out once
per brick size; its tile shape (pixels per 256-thread block), unroll of the
march loop and blocks per SM are launch settings.  Every candidate renders
the same jobs, so every candidate yields the same images; it is timed with
CUDA events over a few launches after one warm-up, and the median decides.
The winner is cached in a JSON file keyed by the GPU and a signature of the
workload, so later runs skip the search.

No reference counterpart: the reference renders one frame per GL draw.
"""

from __future__ import annotations

import dataclasses
import hashlib
import itertools
import json
import os
import statistics
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .batch import BatchRenderer, DeviceLUT, DeviceVolume, RenderJob, Tuning

TILES = ((16, 16), (32, 8), (8, 32))
BRICKS = (2, 3, 4)
STEPS = (1, 4)
BLOCKS = (0, 3, 4, 5)  # 0: as many as fit


def default_cache_path() -> str:
    return os.environ.get("PVR_TUNING_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "pyvr_gb300", "tuning.json"))


def candidates(tiles=TILES, bricks=BRICKS, steps=STEPS, blocks=BLOCKS) -> List[Tuning]:
    return [Tuning(tile_w=tw, tile_h=th, steps_per_iter=s, blocks_per_sm=b, brick_log2=br)
            for br, (tw, th), s, b in itertools.product(bricks, tiles, steps, blocks)]


def workload_signature(scenes: Sequence[dict]) -> str:
    """Stable digest of what the timing depends on: volume extents and
    storage, image sizes, march settings and the opacity functions."""
    h = hashlib.sha1()
    for s in scenes:
        v = s["volume"]
        h.update(repr((tuple(v.data.shape), str(v.data.dtype), s["width"], s["height"],
                       float(s["config"].step_size), int(s["config"].max_steps),
                       tuple(map(tuple, s["otf"].control_points)))).encode())
    return h.hexdigest()[:16]


def device_key() -> str:
    import torch
    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    return f"{p.name}|sm{p.multi_processor_count}"


class _Bench:
    """The scenes' device resources per brick size, their outputs, and timed
    batch launches."""

    def __init__(self, scenes: Sequence[dict]):
        import torch
        self.torch = torch
        self.scenes = scenes
        self.luts = [DeviceLUT(s["ctf"], s["otf"]) for s in scenes]
        self.outs = [torch.empty(s["width"] * s["height"] * 4, dtype=torch.uint8, device="cuda")
                     for s in scenes]
        self.stream = torch.cuda.Stream()
        self._vols: Dict[int, List[DeviceVolume]] = {}

    def volumes(self, brick_log2: int) -> List[DeviceVolume]:
        if brick_log2 not in self._vols:
            self._vols.clear()  # one layout at a time: bounded device memory
            self._vols[brick_log2] = [
                DeviceVolume(s["volume"], value_scale=s["value_scale"], normals=s.get("normals", "device"),
                             brick_log2=brick_log2) for s in self.scenes]
        return self._vols[brick_log2]

    def jobs(self, brick_log2: int) -> List[RenderJob]:
        vols = self.volumes(brick_log2)
        return [RenderJob(v, l, s["camera"], s["light"], s["config"], s["width"], s["height"], out_rgba8=o)
                for v, l, s, o in zip(vols, self.luts, self.scenes, self.outs)]

    def time(self, tuning: Tuning, repeats: int) -> float:
        torch = self.torch
        jobs = self.jobs(tuning.brick_log2)
        br = BatchRenderer(capacity=len(jobs), slots=1, tuning=tuning)
        try:
            br.render(jobs, stream=self.stream)  # warm-up (graph build)
            ms = []
            for _ in range(repeats):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(self.stream)
                br.render(jobs, stream=self.stream)
                b.record(self.stream)
                b.synchronize()
                ms.append(a.elapsed_time(b))
            return statistics.median(ms)
        finally:
            br.synchronize()
            br.close()

    def images(self) -> List[np.ndarray]:
        self.torch.cuda.synchronize()
        return [o.cpu().numpy() for o in self.outs]


def autotune(scenes: Sequence[dict], repeats: int = 5, cands: Optional[Sequence[Tuning]] = None,
             cache_path: Optional[str] = None, use_cache: bool = True
             ) -> Tuple[Tuning, List[Tuple[Tuning, float]]]:
    """Best ``Tuning`` for a batch of scenes (dicts with volume, value_scale,
    camera, light, ctf, otf, config, width, height) and the timings of all
    candidates (empty when the result came from the cache)."""
    cache_path = cache_path or default_cache_path()
    key = f"{device_key()}|{workload_signature(scenes)}"
    if use_cache and os.path.exists(cache_path):
        try:
            with open(cache_path) as f:
                hit = json.load(f).get(key)
            if hit:
                return Tuning(**hit), []
        except (OSError, ValueError, TypeError):
            pass
    bench = _Bench(scenes)
    cands = list(cands or candidates())
    cands.sort(key=lambda t: t.brick_log2)  # one layout at a time
    results = [(t, bench.time(t, repeats)) for t in cands]
    best = min(results, key=lambda r: r[1])[0]
    try:
        os.makedirs(os.path.dirname(cache_path), exist_ok=True)
        data = {}
        if os.path.exists(cache_path):
            with open(cache_path) as f:
                data = json.load(f)
        data[key] = dataclasses.asdict(best)
        tmp = cache_path + f".tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1)
        os.replace(tmp, cache_path)
    except (OSError, ValueError):
        pass  # the cache is an optimisation only
    return best, results
