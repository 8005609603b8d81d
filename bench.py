#!/usr/bin/env python
"""Benchmark of the pyvr ray-marching path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Headline ("renders/s & p50/p99 ms: batched server vs per-frame CUDA"): the
serving workload.  A catalog of 32 HBM-resident volumes (cubic, extents
log-uniform in 128..512, uint8 or float16 value noise, normals computed on
the GPU) sits under a 40 GB budget with LRU eviction, and a seeded Poisson
request stream mixes 70% orbit re-renders (512^2, balanced), 20% TF edits
(512^2), 5% high-quality 1024^2 captures and 5% new-volume loads.  Both
arms run on the native serving runtime over the same resident volumes: the
continuously batching server, and the per-frame renderer (one request per
launch, each read back before the next starts).  For each, an untimed sweep
of offered rates (doubling from 400 req/s, then bisection) finds the highest
rate served with p99 latency <= 20 ms over the 512^2 frames (orbit re-renders,
TF edits, and new-volume loads with their render; the 1024^2 captures are
reported beside them); then K timed one-second steps run at that rate,
backing off by 15% (at most 7 times) until the timed run meets the bound.  value = requests completed per second by the server, arrival ->
RGBA8 image in host memory (the whole path is end to end); the per-frame
rate, the ratio and p50/p99 of both (also at the nominal 400 req/s) are
reported beside it.  The roofline is the batch march kernel's
(event-timed launches in the timed steps; bytes = 8 voxel texels in the
stored type + 8 float32x3 normal texels per shaded in-box sample).

Nested sections: "plain" (the per-frame renderer on 256^3 value noise in
u8/f16/f32, 16 orbit cameras, 1024^2, high_quality; one step = 48 frames),
"batching_c3" (64 uneven renders per persistent launch with the autotuner's
settings) and "differentiation" (TF recovery with the hand-written backward).

--impl reference: the CPU restatement of the reference shader (the oracle,
all host cores) rendering whole frames of the same request mix.
"""

import argparse
import ctypes
import dataclasses
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_SAMPLE = {"u8": 8 * 1 + 8 * 12, "f16": 8 * 2 + 8 * 12, "f32": 8 * 4 + 8 * 12}
DTYPES = ("u8", "f16", "f32")
RES = 1024
N_VOL = 256
NOMINAL_RATE = 400.0
# Per shaded sample of the single-render march kernel (fast arithmetic,
# half-normal records for uint8/float16), from ncu (smsp__inst_executed.sum
# and dram__bytes_read/write.sum over the captured launches, divided by their
# shaded-sample counters): the serving requests of a 6-volume catalog
# (272^3-397^3) and of a 512^3 catalog, the upper end of the serving range
# (profiles/march_single_kernel_serving_mix.md), and the plain 256^3 1024^2
# high_quality frames (profiles/march_single_kernel_256cube_1024px.md)
SERVING_WARP_INSTR_PER_SAMPLE = 7.51
SERVING_DRAM_BYTES_PER_SAMPLE = 8.31
SERVING_512_WARP_INSTR_PER_SAMPLE = 7.82
SERVING_512_DRAM_BYTES_PER_SAMPLE = 23.4
PLAIN_WARP_INSTR_PER_SAMPLE = 6.68
PLAIN_DRAM_BYTES_PER_SAMPLE = 0.80
# ... and of the persistent batch kernel on the 64 uneven renders
# (profiles/march_batch_kernel_batching64.md)
BATCH_WARP_INSTR_PER_SAMPLE = 7.20
BATCH_DRAM_BYTES_PER_SAMPLE = 1.20
P99_MS = 20.0
# the requests whose latency the p99 bound applies to: the 512^2 frames
# (orbit re-renders, TF edits, and the renders of newly loaded volumes, the
# load included); the 1024^2 captures are reported beside them
FRAME_TAGS = ("orbit", "tf_edit", "load")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="oracle seconds of the CPU baseline")
    ap.add_argument("--probe-s", type=float, default=0.0,
                    help="seconds per rate probe (0: as long as the timed run, --steps seconds)")
    ap.add_argument("--refine", type=int, default=4, help="bisection probes after the doubling sweep")
    ap.add_argument("--slots", type=int, default=8, help="server: launches in flight (streams)")
    ap.add_argument("--max-batch", type=int, default=64, help="server: requests per launch")
    ap.add_argument("--batch-pixels", type=int, default=512 * 512,
                    help="server: pixels per launch (renders this large run as launches of their own, "
                         "side by side on the slots' streams)")
    ap.add_argument("--linger-us", type=int, default=0, help="server: hold a partial batch this long")
    ap.add_argument("--serving-brick-log2", type=int, default=4, help="brick size of the resident volumes")
    ap.add_argument("--serving-volumes", type=int, default=32)
    ap.add_argument("--serving-max-dim", type=int, default=512)
    ap.add_argument("--serving-extra", type=int, default=224,
                    help="volumes outside the catalog: the pool new-volume loads draw from (its records "
                         "exceed the byte budget, so loads upload volumes that are not resident)")
    ap.add_argument("--records", default="half_normals", choices=["float", "half_exact", "half_normals"],
                    help="record form of the volumes laid out by the benchmark")
    ap.add_argument("--arithmetic", default="fast", choices=["fast", "exact"],
                    help="arithmetic of the march")
    # smaller cases for profiling captures
    ap.add_argument("--only", choices=["all", "plain", "serving", "diff", "batching", "loaders", "requests"],
                    default="all")
    ap.add_argument("--serving-min-dim", type=int, default=128)
    ap.add_argument("--loaders", type=int, default=1, help="server: loader threads for new volumes")
    ap.add_argument("--switch-interval-us", type=float, default=0.0,
                    help="serving: Python thread switch interval during the replays (0: unchanged)")
    ap.add_argument("--requests", type=int, default=24, help="requests section: renders of the stream")
    ap.add_argument("--loaders-volume", type=int, default=256, help="loaders section: volume extent")
    ap.add_argument("--diff-steps", type=int, default=200, help="Adam steps of the differentiation section")
    ap.add_argument("--no-tune", action="store_true", help="batching section: default tuning, no search")
    ap.add_argument("--storages", default=",".join(DTYPES))
    ap.add_argument("--plain-volume", type=int, default=N_VOL, help="plain section: volume extent")
    ap.add_argument("--plain-res", type=int, default=RES, help="plain section: image size")
    ap.add_argument("--plain-config", default="high_quality", choices=["high_quality", "balanced"],
                    help="plain section: RenderConfig preset")
    ap.add_argument("--cameras", type=int, default=16)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region (one or
    more start/pause intervals, summarised by stop)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, gpu_index):
        self.gpu_index = gpu_index
        self.proc = None
        self.available = True
        self.sm, self.smax, self.reasons = [], None, set()

    def start(self):
        self.path = tempfile.mktemp(prefix="pvr_clocks_", suffix=".csv")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            self.available = False

    def pause(self):
        if self.proc is None:
            return
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.proc = None
        self.fh.close()
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9 or not parts[0].isdigit() or int(parts[0]) != self.gpu_index:
                    continue
                try:
                    self.sm.append(float(parts[1]))
                    self.smax = float(parts[2])
                except ValueError:
                    continue
                for n, v in zip(self.NAMES, parts[5:9]):
                    if v.lower().startswith("active"):
                        self.reasons.add(n)
        os.unlink(self.path)

    def stop(self):
        self.pause()
        if not self.available:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        return {"sm_mhz": statistics.median(self.sm) if self.sm else None, "sm_max_mhz": self.smax,
                "reasons": sorted(self.reasons), "samples": len(self.sm)}


def gpu_index(local_rank):
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    ids = [v for v in vis.split(",") if v.strip()]
    if ids and all(v.strip().isdigit() for v in ids) and local_rank < len(ids):
        return int(ids[local_rank])
    return local_rank


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (a checker here, timed; never the product path)
# ---------------------------------------------------------------------------

class ReferenceServer:
    """The reference's own host path serving the request mix, request by
    request (no GPU, nothing of the pyvr_gb300 library): a new volume is
    converted to float32 and gets its normals from ``compute_normal_volume``
    (numpy, pyvr/datasets/synthetic.py:109-122) as the reference's
    load_volume path does (pyvr/moderngl_renderer/renderer.py:107-146,
    manager.py:88-97); the transfer functions become an RGBA table on the
    host (manager.py:162-175); the camera matrices come from the ``Camera``
    methods (pyvr/camera/camera.py:292-369); the frame is marched by the CPU
    restatement of the shader (the oracle) on all host cores.  Volumes stay
    resident (voxels + normals) under a host byte budget with LRU eviction."""

    def __init__(self, budget_bytes=40 << 30):
        import oracle
        oracle.build()
        self.oracle = oracle
        self.budget = budget_bytes
        self.resident = {}  # volume id -> (Volume, bytes), in LRU order

    def _load(self, vid, vol):
        from pyvr_gb300 import Volume, compute_normal_volume
        self.resident.pop(vid, None)
        data = vol.data.astype(np.float32)  # the reference uploads float32 textures
        v = Volume(data=data, normals=compute_normal_volume(vol.data), min_bounds=vol.min_bounds,
                   max_bounds=vol.max_bounds)
        nbytes = data.nbytes + v.normals.nbytes
        while self.resident and sum(b for _, b in self.resident.values()) + nbytes > self.budget:
            self.resident.pop(next(iter(self.resident)))
        self.resident[vid] = (v, nbytes)
        return v

    def make_resident(self, vid, vol):
        """Untimed: the catalog volumes the stream starts with."""
        if vid not in self.resident:
            self._load(vid, vol)

    def handle(self, kw):
        """One request; returns (in-box samples, seconds of host work)."""
        from pyvr_gb300 import workloads as W
        from pyvr_gb300.renderer import rgba_lut
        t = time.perf_counter()
        vid = kw["volume_id"]
        if kw["kind"] == "load" or vid not in self.resident:
            v = self._load(vid, kw["volume"])
        else:
            v = self.resident.pop(vid)[0]
            self.resident[vid] = (v, v.data.nbytes + v.normals.nbytes)
        lut = rgba_lut(kw["color_tf"], kw["opacity_tf"])
        s = W.frame_inputs(v, kw["camera"], kw["light"], kw["config"], lut, kw["width"], kw["height"],
                           kw["value_scale"])
        _, _, n = self.oracle.render(s, want_float=False)
        return n, time.perf_counter() - t


def reference_serving_steps(wl, steps, seconds_per_step, seed, server=None):
    """Request after request of the serving stream through ReferenceServer,
    each step until `seconds_per_step` of host work; the catalog volumes a
    request finds resident are made resident untimed.  Returns (per-step
    [(requests, seconds, samples, loads)], threads)."""
    server = server or ReferenceServer()
    out = []

    def requests():
        k = 0
        while True:  # 10-second chunks of the stream
            for item in wl.requests(NOMINAL_RATE, 10.0, seed + 7919 * k):
                yield item
            k += 1

    stream = requests()
    for _ in range(steps):
        nreq = ns = loads = 0
        el = 0.0
        while el < seconds_per_step:
            _, kw = next(stream)
            if kw["kind"] != "load":
                server.make_resident(kw["volume_id"], kw["volume"])
            n, dt = server.handle(kw)
            nreq += 1
            ns += n
            el += dt
            loads += kw["kind"] == "load"
        out.append((nreq, el, ns, loads))
    return out, server.oracle.max_threads()


# ---------------------------------------------------------------------------
# Serving (headline)
# ---------------------------------------------------------------------------

def pin_host_volumes(workload):
    """The host copies of the volumes (the data a client hands in) in
    page-locked memory from pvr_host_alloc, all in one allocation.
    (Registering the numpy arrays with cudaHostRegister instead made uploads
    of 100-250 MB volumes take 10-70 ms at times on Grace-Blackwell, against
    about 1-2 ms from this memory.)"""
    from pyvr_gb300.batch import PageLockedArena
    vols = [vol for vol, _ in workload.volumes]
    arena = PageLockedArena(PageLockedArena.size_for([v.data for v in vols]))
    for vol in vols:
        vol.data = arena.copy(vol.data)


def serving_section(args, torch):
    """The batched server and the per-frame baseline, both on the native
    serving runtime (pvr_server_*), each measured alone: its own runtime and
    its own resident copies of the same volumes, closed before the other arm
    starts, over the same request streams."""
    from pyvr_gb300 import workloads as W
    from pyvr_gb300.replicas import all_ok, barrier
    from pyvr_gb300.server import NativeRenderServer, bounded, drive, latency_by_tag, latency_stats, sustained_rate
    t_setup = time.perf_counter()
    wl = W.ServingWorkload(n_volumes=args.serving_volumes, n_extra=args.serving_extra,
                           min_dim=args.serving_min_dim, max_dim=args.serving_max_dim, seed=0)
    wl.volumes.materialize()  # the clients' data exists before the stream starts
    pin_host_volumes(wl)
    start = wl.snapshot()
    setup_s = time.perf_counter() - t_setup
    from pyvr_gb300.server import VolumeCache
    est = VolumeCache(0, args.serving_brick_log2)
    pool = {"volumes": len(wl.volumes), "catalog": wl.n_catalog,
            "host_bytes": int(sum(v.data.nbytes for v, _ in wl.volumes)),
            "device_bytes_estimate": int(sum(est.estimate_bytes(v) - v.data.nbytes for v, _ in wl.volumes)),
            "budget_bytes": 40 << 30}
    clocks = ClockSampler(gpu_index(dist_env()[2]))
    if args.switch_interval_us:
        sys.setswitchinterval(args.switch_interval_us * 1e-6)

    def timed_run(impl, rate, seed, reset):
        """K one-second steps at `rate`; a run whose p99 exceeds the bound is
        repeated at 0.85x the rate (at most 7 times), so that the reported
        rate is one served within the bound."""
        attempts = []
        for _ in range(8):
            torch.cuda.synchronize()
            barrier()
            reset()
            impl.reset_stats()
            c = impl.cache
            m0, up0, ld0, ev0, ob0, ar0 = (impl.luts.misses, c.uploaded_bytes, c.loads, c.evictions,
                                           c.over_budget, c.alloc_retries)
            clocks.start()
            reqs, el = drive(impl, wl.requests(rate, float(args.steps), seed))
            torch.cuda.synchronize()
            clocks.pause()
            barrier()
            lat = latency_stats(reqs)
            frames = latency_stats(bounded(reqs, FRAME_TAGS))
            load_lat = latency_stats([r for r in reqs if r.tag == "load"])
            attempts.append({"offered": rate, "completed_per_s": len(reqs) / el, "p99_ms": lat.get("p99_ms"),
                             "frames_512_p99_ms": frames.get("p99_ms"), "by_tag": latency_by_tag(reqs),
                             "lut_builds": impl.luts.misses - m0,
                             "uploaded_bytes": c.uploaded_bytes - up0, "volume_loads": c.loads - ld0,
                             "evictions": c.evictions - ev0, "over_budget": c.over_budget - ob0,
                             "alloc_retries": c.alloc_retries - ar0,
                             "load_requests": sum(r.tag == "load" for r in reqs),
                             "load_p50_ms": load_lat.get("p50_ms"), "load_p99_ms": load_lat.get("p99_ms"),
                             "resident_bytes": c.used,
                             "device_free_bytes": int(torch.cuda.mem_get_info()[0])})
            # the ranks repeat together, so that their barriers stay paired
            if all_ok(frames.get("p99_ms", 1e9) <= P99_MS, device="cuda"):
                break
            rate *= 0.85
        return reqs, el, impl.stats(), attempts

    def measure(impl, warm_seed):
        """Warm-up, the latency at the nominal rate, the untimed rate sweep and
        the timed steps of one implementation."""
        def make_catalog_resident():
            # untimed: the steady state of a running service with a full
            # cache -- the catalog's volumes (the ones being served), then the
            # volumes that left the catalog most recently, up to the budget;
            # anything else (e.g. admitted over the budget while requests in
            # flight pinned every volume) is let go first
            cache = impl.cache
            for dv in cache.evict_except(set(wl.catalog)):
                impl._free_volume(dv)
            for slot in range(wl.n_catalog):
                vid = wl.catalog[slot]
                vol, vs = wl.volumes[vid]
                cache.insert(vid, vol, vs, impl._free_volume)
            for vid in reversed(wl.outside):
                vol, vs = wl.volumes[vid]
                if cache.used + cache.estimate_bytes(vol) > cache.budget:
                    break
                cache.insert(vid, vol, vs, impl._free_volume)
            torch.cuda.synchronize()

        wl.restore(start)
        make_catalog_resident()
        # warm-up: W untimed one-second segments at the nominal rate (the same
        # streams for both implementations)
        for w in range(args.warmup):
            drive(impl, wl.requests(NOMINAL_RATE, 1.0, warm_seed + w))
        # the workload's state (catalog churn, orbits, TF edits) evolves with
        # every stream: each measurement below restarts from this point, so
        # that all of them see the same mix
        snap = wl.snapshot()

        def reset():
            # the same workload state (catalog, sessions) for every run, with
            # the catalog resident as it was at the snapshot
            wl.restore(snap)
            make_catalog_resident()

        reset()
        reqs, el = drive(impl, wl.requests(NOMINAL_RATE, 3.0, 200))
        nominal = latency_stats(reqs)
        nominal["completed_per_s"] = len(reqs) / el
        # untimed sweep: highest rate with p99 <= 20 ms (a failing probe is
        # repeated once)
        rates = [NOMINAL_RATE * (2 ** k) for k in range(8)]
        # probes as long as the timed run: a loader that falls behind shows
        # its queue only after a few seconds
        probe_s = args.probe_s or float(args.steps)
        rate, probes = sustained_rate(impl, wl, rates, probe_s, 300, refine=args.refine, reset=reset,
                                      bound_tags=FRAME_TAGS)
        reqs, el, st, attempts = timed_run(impl, rate or NOMINAL_RATE, 500, reset)
        return dict(nominal=nominal, probes=probes, reqs=reqs, el=el, stats=st, attempts=attempts,
                    loads=impl.cache.loads, evictions=impl.cache.evictions, lut_hits=impl.luts.hits,
                    lut_misses=impl.luts.misses)

    # kernel events and sample counters on every 8th launch (the roofline);
    # the clocks are sampled during the timed steps of both
    server = NativeRenderServer(budget_bytes=40 << 30, max_batch=args.max_batch, slots=args.slots, instrument=8,
                                batch_pixels=args.batch_pixels,
                                linger_us=args.linger_us, brick_log2=args.serving_brick_log2,
                                loaders=args.loaders)
    srv = measure(server, 100)
    server.close()
    del server
    torch.cuda.synchronize()
    serial = NativeRenderServer(budget_bytes=40 << 30, per_frame=True, brick_log2=args.serving_brick_log2)
    ser = measure(serial, 100)
    serial.close()
    del serial
    clk = clocks.stop()
    srv_reqs, srv_el, st, srv_attempts = srv["reqs"], srv["el"], srv["stats"], srv["attempts"]
    ser_reqs, ser_el, ser_attempts = ser["reqs"], ser["el"], ser["attempts"]
    nom = {"server": srv["nominal"], "serial": ser["nominal"]}
    probes_server, probes_serial = srv["probes"], ser["probes"]
    # our kernels in the timed region: the server's marches (one launch per
    # batch), the per-frame marches, LUT builds of new transfer functions and
    # the layout of every uploaded volume
    launches = (st["batches"] + ser["stats"]["batches"] + srv_attempts[-1]["lut_builds"]
                + ser_attempts[-1]["lut_builds"] + srv_attempts[-1]["volume_loads"]
                + ser_attempts[-1]["volume_loads"])
    r_server, r_serial = srv_attempts[-1]["offered"], ser_attempts[-1]["offered"]
    # roofline of the server's march over the timed steps: algorithmic bytes
    # of the shaded samples (measured on every 8th launch, scaled to all
    # launches) over the timed wall time.  Launches overlap on the device,
    # so their own event times add up to more than the time the GPU spent;
    # the wall time includes idle gaps, so this is a lower bound.
    peak, peak_kind = measured_peaks()
    k_ms = st["kernel_ms"]
    inst = max(1, st["instrumented_batches"])
    alg_per_launch = st["algorithmic_bytes"] / inst
    achieved = alg_per_launch * st["batches"] / srv_el / 1e9
    d2h = sum(r.width * r.height * 4 for r in srv_reqs)
    # uploads: volumes not yet resident (tables of new transfer functions are
    # built on the device from their control points, passed as kernel
    # parameters)
    h2d = srv_attempts[-1]["uploaded_bytes"]
    out = dict(value=len(srv_reqs) / srv_el, serial_value=len(ser_reqs) / ser_el,
               counts=(len(srv_reqs), srv_el, len(ser_reqs), ser_el),
               lut_builds=srv_attempts[-1]["lut_builds"], launches=launches,
               server=latency_stats(srv_reqs), serial=latency_stats(ser_reqs), nominal=nom,
               server_frames=latency_stats(bounded(srv_reqs, FRAME_TAGS)),
               serial_frames=latency_stats(bounded(ser_reqs, FRAME_TAGS)),
               by_tag={"server": latency_by_tag(srv_reqs), "serial": latency_by_tag(ser_reqs)},
               rate_server=r_server, rate_serial=r_serial, probes_server=probes_server,
               probes_serial=probes_serial, attempts={"server": srv_attempts, "serial": ser_attempts},
               batches=st["batches"],
               mean_batch=st["jobs"] / max(1, st["batches"]), max_batch=st["max_jobs"],
               kernel_ms=k_ms, inbox_samples=st["inbox_samples"], shaded_samples=st["shaded_samples"],
               mean_inbox_per_request=st["inbox_samples"] / max(1, st["instrumented_jobs"]),
               summed_launch_time_over_wall=k_ms * st["batches"] / inst / 1000.0 / srv_el,
               roofline=march_roofline(st["shaded_samples"] / inst * st["batches"], srv_el, clk,
                                       SERVING_WARP_INSTR_PER_SAMPLE, SERVING_DRAM_BYTES_PER_SAMPLE,
                                       alg_per_launch * st["batches"], torch,
                                       kernel=("march_single_kernel" if st["max_jobs"] <= 1
                                               else "march_batch_kernel + march_single_kernel"),
                                       launches=st["batches"], launches_instrumented=st["instrumented_batches"],
                                       note="samples of all timed launches (counted on every 8th launch, "
                                            "scaled) over the timed wall time, idle gaps included: a lower "
                                            "bound; launches overlap on the device",
                                       per_sample_512cube={"warp_instr": SERVING_512_WARP_INSTR_PER_SAMPLE,
                                                           "dram_bytes": SERVING_512_DRAM_BYTES_PER_SAMPLE,
                                                           "note": "the same kernel on 512^3 uint8 volumes "
                                                                   "(upper end of the catalog): bound by L1 "
                                                                   "traffic (84 %) and gather latency"},
                                       profile="profiles/march_single_kernel_serving_mix.md"),
               clocks=clk, h2d=h2d / args.steps, d2h=d2h / args.steps, setup_s=setup_s, pool=pool,
               loads=srv["loads"], evictions=srv["evictions"],
               lut_hits=srv["lut_hits"], lut_misses=srv["lut_misses"], workload=wl)
    return out


def march_roofline(samples, seconds, clocks, warp_instr_per_sample, dram_bytes_per_sample, alg_bytes, torch,
                   **extra):
    """Roofline of the march kernels.  They are bound by instruction issue
    (the working sets of cached volumes sit in L1/L2) or by memory latency
    (large volumes), not by HBM bandwidth.  bound "issue": warp instructions
    per shaded sample (ncu, smsp__inst_executed.sum over the kernel's sample
    counters) x shaded samples per second, against 4 issue slots per SM per
    cycle at the median SM clock sampled during the timed region.  Beside it:
    the DRAM bytes the kernel moves (ncu dram__bytes per sample x samples/s)
    as a fraction of the measured HBM bandwidth, and the algorithmic bytes
    (8 voxel + 8 float32x3 normal texels per sample, cache hits included)."""
    peak_hbm, peak_kind = measured_peaks()
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    sms = props.multi_processor_count
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz") or 2070.0
    peak_issue = sms * 4 * mhz * 1e6 / 1e9  # G warp instructions / s
    rate = samples / seconds if seconds > 0 else 0.0
    issue = warp_instr_per_sample * rate / 1e9
    dram = dram_bytes_per_sample * rate / 1e9
    out = {"bound": "issue", "achieved": issue, "peak": peak_issue, "unit": "G warp-instr/s",
           "frac": issue / peak_issue if peak_issue else None,
           "traffic": dram_bytes_per_sample * samples / max(1, extra.get("launches") or 1),
           "traffic_note": "DRAM bytes per launch: ncu bytes per shaded sample x samples per launch",
           "samples_per_s": rate, "warp_instr_per_sample": warp_instr_per_sample,
           "issue_peak_note": f"{sms} SMs x 4 schedulers x {mhz:.0f} MHz (median sampled SM clock)",
           "dram": {"achieved": dram, "peak": peak_hbm, "unit": "GB/s", "frac": dram / peak_hbm,
                    "bytes_per_sample": dram_bytes_per_sample, "peak_kind": peak_kind},
           "algorithmic": {"achieved": alg_bytes / seconds / 1e9 if seconds > 0 else 0.0, "unit": "GB/s",
                           "frac_of_hbm": (alg_bytes / seconds / 1e9 / peak_hbm) if seconds > 0 else 0.0,
                           "note": "8 voxel + 8 float32x3 normal texels per sample, L1/L2 hits included"}}
    out.update(extra)
    return out


# ---------------------------------------------------------------------------
# Batching (nested section)
# ---------------------------------------------------------------------------

def batching_section(args, torch):
    """64 uneven renders (volumes 32..384 per axis, u8/f16/f32, 128^2..1024^2,
    random cameras and TFs) in one persistent launch replayed as a CUDA graph,
    with the autotuner's tile shape / brick size / steps per iteration /
    blocks per SM; beside it the default tuning and the same 64 renders as 64
    single-render launches."""
    from pyvr_gb300 import workloads as W
    from pyvr_gb300.autotune import _Bench, autotune
    from pyvr_gb300.batch import BatchRenderer, Tuning
    scenes = W.config_batching(64, noise=W.value_noise_device)
    t_tune = time.perf_counter()
    if args.no_tune:
        best, results = Tuning(), []
    else:
        best, results = autotune(scenes, repeats=3, use_cache=False)
    tune_s = time.perf_counter() - t_tune
    bench = _Bench(scenes)
    counters = torch.zeros((len(scenes), 2), dtype=torch.int64, device="cuda")

    def timed(tuning, per_frame=False, count=False):
        jobs = bench.jobs(tuning.brick_log2)
        if count:
            for i, j in enumerate(jobs):
                j.counters = counters[i]
        br = BatchRenderer(capacity=len(jobs), slots=2, tuning=tuning)
        st = bench.stream

        def launch():
            if per_frame:
                for j in jobs:
                    br.render([j], stream=st)
            else:
                br.render(jobs, stream=st)

        for _ in range(args.warmup):
            launch()
        if count:
            st.synchronize()  # the warm-up launches also add to the counters
            with torch.cuda.stream(st):
                counters.zero_()
            launch()
            st.synchronize()
            for j in jobs:  # count one batch only
                j.counters = None
        st.synchronize()
        ev = []
        for _ in range(args.steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            launch()
            b.record(st)
            ev.append((a, b))
        st.synchronize()
        br.close()
        return statistics.mean(a.elapsed_time(b) for a, b in ev)

    ms_best = timed(best, count=True)
    per = counters.cpu().numpy()
    default = Tuning()
    ms_default = timed(default)
    ms_frames = timed(best, per_frame=True)
    dtypes = [s["dtype"] for s in scenes]
    shaded_bytes = sum(int(c[1]) * BYTES_PER_SAMPLE[dt] for c, dt in zip(per, dtypes))
    return {"renders_per_s": len(scenes) / (ms_best / 1000.0), "ms_per_batch": ms_best,
            "default_tuning_ms_per_batch": ms_default, "per_frame_launches_ms": ms_frames,
            "tuning": dataclasses.asdict(best), "tuning_search_s": tune_s, "candidates": len(results),
            "candidate_ms": sorted(round(ms, 3) for _, ms in results)[:5],
            "samples_inbox": int(per[:, 0].sum()), "samples_shaded": int(per[:, 1].sum()),
            "roofline": march_roofline(int(per[:, 1].sum()), ms_best / 1000.0, None, BATCH_WARP_INSTR_PER_SAMPLE,
                                       BATCH_DRAM_BYTES_PER_SAMPLE, shaded_bytes, torch,
                                       kernel="march_batch_kernel", launches=1,
                                       note="one batch (a persistent launch per kernel variant) over its "
                                            "CUDA-event time",
                                       profile="profiles/march_batch_kernel_batching64.md"),
            "config": {"renders": len(scenes), "volumes": "32..384 per axis log-uniform, u8/f16/f32 value noise",
                       "resolutions": "128^2..1024^2", "render_config": "balanced", "steps": args.steps}}


# ---------------------------------------------------------------------------
# Differentiation (nested section)
# ---------------------------------------------------------------------------

def diff_section(args, torch):
    """Transfer-function recovery: 128^3 FP32 value noise (seed 3), 8 views at
    512^2 rendered as float RGBA, MSE against targets rendered from another
    seeded TF, Adam on the 256-entry LUT; each step = forward + loss +
    hand-written backward + Adam update, timed with CUDA events."""
    import numpy as np
    from pyvr_gb300 import Camera, Light, RenderConfig, compute_normal_volume
    from pyvr_gb300 import workloads as W
    from pyvr_gb300.diff import DiffScene, render_views
    from pyvr_gb300.renderer import rgba_lut
    n, res, views = 128, 512, 8
    data = W.value_noise((n, n, n), seed=3).astype(np.float32)
    nrm = torch.tensor(compute_normal_volume(data), device="cuda")
    vol = torch.tensor(data, device="cuda")
    rng = np.random.default_rng(3)
    ctf = W.standin_colormap(3)
    lut0 = torch.tensor(rgba_lut(ctf, W.random_opacity(rng, 8, 0.3)), device="cuda")
    lut_t = torch.tensor(rgba_lut(ctf, W.random_opacity(rng, 8, 0.3)), device="cuda")
    cams = [Camera.from_spherical(np.zeros(3, np.float32), 2 * np.pi * k / views, np.pi / 6, 0.0, 3.0)
            for k in range(views)]
    scene = DiffScene(cams, Light.directional([1, -1, 0], 0.2, 0.8), RenderConfig.balanced(), res, res)
    with torch.no_grad():
        target, steps_t = render_views(vol, lut_t, scene, nrm, return_steps=True)

    def run(n_steps, with_volume):
        lut = lut0.clone().requires_grad_(True)
        v = vol.clone().requires_grad_(with_volume)
        opt = torch.optim.Adam([lut], lr=0.01)
        ev = []
        losses = []
        for _ in range(n_steps):
            e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            e[0].record()
            opt.zero_grad(set_to_none=True)
            img = render_views(v, lut, scene, nrm)
            e[1].record()
            loss = ((img - target) ** 2).mean()
            loss.backward()
            e[2].record()
            opt.step()
            with torch.no_grad():
                lut.clamp_(0.0, 1.0)
            e[3].record()
            ev.append(e)
            losses.append(loss.detach())
        torch.cuda.synchronize()
        step = [a.elapsed_time(d) for a, _, _, d in ev]
        fwd = [a.elapsed_time(b) for a, b, _, _ in ev]
        bwd = [b.elapsed_time(c) for _, b, c, _ in ev]
        return step, fwd, bwd, [float(x) for x in losses]

    run(args.warmup, False)
    step, fwd, bwd, losses = run(args.diff_steps, False)
    vstep, vfwd, vbwd, _ = run(max(args.warmup, 10), True)
    return {"ms_per_step": statistics.mean(step), "ms_per_step_median": statistics.median(step),
            "forward_ms": statistics.mean(fwd), "backward_ms": statistics.mean(bwd), "steps": args.diff_steps,
            "loss_first": losses[0], "loss_last": losses[-1],
            "with_volume_gradient": {"ms_per_step": statistics.mean(vstep), "forward_ms": statistics.mean(vfwd),
                                     "backward_ms": statistics.mean(vbwd)},
            "mean_loop_iterations_per_ray": float(steps_t.float().mean()),
            "config": {"volume": "128^3 FP32 value noise seed 3 (normals constant)", "views": views,
                       "resolution": f"{res}x{res}", "lut": 256, "render_config": "balanced",
                       "loss": "MSE over float RGBA", "optimizer": "Adam lr 0.01 on the LUT, clamped to [0,1]"}}


# ---------------------------------------------------------------------------
# Plain per-frame renderer (nested section)
# ---------------------------------------------------------------------------

def make_scenes(storages=DTYPES, n=N_VOL, res=RES):
    from pyvr_gb300 import workloads as W
    noise = W.config_scale_volume(n)
    return {dt: W.config_scale(dt, n=n, res=res, noise=noise) for dt in storages}


def loaders_section(args, torch):
    """The paths either side of the march, each against the host path the
    reference takes: volume layout with device normals against numpy normals
    plus their upload, LUT builds on the device against numpy tables plus
    upload, the FP64 orbit-camera setup against numpy, and .vti reading."""
    import numpy as np
    from pyvr_gb300 import Volume, compute_normal_volume
    from pyvr_gb300.batch import DeviceLUT, DeviceVolume
    from pyvr_gb300 import workloads as W
    from pyvr_gb300.batch import fill_camera
    from pyvr_gb300.renderer import camera_uniforms, rgba_lut
    from pyvr_gb300.vti import load_vtk_volume, write_vti
    from pyvr_gb300.camera import Camera
    out = {}

    def wall(fn, reps=1):
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            r = fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t) / reps, r

    # (1) volume layout with normals computed on the device
    n = args.loaders_volume
    base = W.value_noise_device(n, 0)
    loads = {}
    for dt in ("u8", "f16"):
        data = W.to_storage(base, dt)
        vol = Volume(data=data)
        DeviceVolume(vol, normals="device", brick_log2=4).close()  # warm-up
        ts = []
        for _ in range(args.steps):
            t, dv = wall(lambda: DeviceVolume(vol, normals="device", brick_log2=4))
            rec_bytes = dv.device_bytes()
            dv.close()
            ts.append(t)
        entry = {"device_ms": 1000 * statistics.median(ts), "voxels": int(data.size),
                 "device_bytes": rec_bytes, "gvoxels_per_s": data.size / statistics.median(ts) / 1e9}
        if not args.skip_cpu:
            t_np, nrm = wall(lambda: compute_normal_volume(data))
            t_up, dv = wall(lambda: DeviceVolume(Volume(data=data, normals=nrm), normals="given",
                                                  brick_log2=4))
            dv.close()
            entry.update({"host_normals_ms": 1000 * t_np, "host_normals_upload_ms": 1000 * t_up,
                          "speedup": (t_np + t_up) / statistics.median(ts)})
        loads[dt] = entry
    out["volume_load"] = {"volume": f"{n}^3 value noise seed 0, 16^3 bricks", "per_storage": loads,
                          "note": "wall time of DeviceVolume(...) to a ready layout, pageable upload "
                                  "included; host path = numpy normals (reference semantics) + upload"}

    # (2) LUTs built on the device from control points
    rng = np.random.default_rng(1)
    tfs = [(W.standin_colormap(i % 12), W.random_opacity(rng, int(rng.integers(4, 13)), 0.3))
           for i in range(200)]
    stream = torch.cuda.Stream()
    lut = DeviceLUT.on_device(*tfs[0], 256)
    for ctf, otf in tfs[:10]:
        lut.build(ctf, otf, 256, stream)
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t = time.perf_counter()
    e0.record(stream)
    for ctf, otf in tfs:
        lut.build(ctf, otf, 256, stream)
    e1.record(stream)
    stream.synchronize()
    t_dev = (time.perf_counter() - t) / len(tfs)
    t_host, _ = wall(lambda: [lut.update(rgba_lut(c, o, 256)) for c, o in tfs])
    lut.close()
    out["lut_build"] = {"entries": 256, "tables": len(tfs), "device_us_per_table": 1e6 * t_dev,
                        "device_stream_us_per_table": 1000 * e0.elapsed_time(e1) / len(tfs),
                        "host_us_per_table": 1e6 * t_host / len(tfs),
                        "note": "device: pvr_lut_build queued per table (host call included); "
                                "host: numpy to_lut (reference) + pvr_lut_update upload"}

    # (3) orbit camera setup in FP64 (native) against numpy
    cams = [Camera.from_spherical(np.zeros(3, np.float32), float(a), float(e), 0.0, float(d))
            for a, e, d in zip(rng.uniform(-np.pi, np.pi, 2000), rng.uniform(-1.4, 1.4, 2000),
                               rng.uniform(2.5, 4.0, 2000))]
    view, proj, pos = (ctypes.c_float * 16)(), (ctypes.c_float * 16)(), (ctypes.c_float * 3)()
    t = time.perf_counter()
    for c in cams:
        fill_camera(c, 512, 512, view, proj, pos)
    t_nat = (time.perf_counter() - t) / len(cams)
    t = time.perf_counter()
    for c in cams:
        camera_uniforms(c, 512, 512)
    t_np = (time.perf_counter() - t) / len(cams)
    out["camera_setup"] = {"cameras": len(cams), "native_us": 1e6 * t_nat, "numpy_us": 1e6 * t_np}

    # (4) .vti reading: the reference's loader (host normals) against reading
    # plus device normals
    vn = min(n, 256)
    raw = W.value_noise_device(vn, 2)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "noise.vti")
        write_vti(path, raw.astype(np.float32), spacing=(1.0, 1.0, 1.0), compress=True)
        size = os.path.getsize(path)
        t_ref, _ = wall(lambda: load_vtk_volume(path))
        t_read, vol = wall(lambda: load_vtk_volume(path, compute_normals=False))
        t_dev, dv = wall(lambda: DeviceVolume(vol, normals="device", brick_log2=4))
        dv.close()
    out["vti_load"] = {"volume": f"{vn}^3 float32, zlib blocks", "file_bytes": size,
                       "reference_loader_ms": 1000 * t_ref, "read_ms": 1000 * t_read,
                       "device_layout_ms": 1000 * t_dev,
                       "speedup": t_ref / (t_read + t_dev)}
    return out


def requests_section(args, torch):
    """The render requests of the serving stream one after the other, each a
    single-render launch on one stream with sample counters: per launch, the
    request's kind, volume, resolution, in-box and shaded samples and its
    CUDA-event time.  Launch k of the march kernel here is request k, which
    is what a profiler capture of these launches is matched against."""
    from pyvr_gb300 import workloads as W
    from pyvr_gb300.batch import BatchRenderer, DeviceLUT, DeviceVolume, RenderJob
    wl = W.ServingWorkload(n_volumes=args.serving_volumes, n_extra=args.serving_extra,
                           min_dim=args.serving_min_dim, max_dim=args.serving_max_dim, seed=0)
    kws = [kw for _, kw in wl.requests(NOMINAL_RATE, 5.0, 31) if kw["kind"] == "render"][:args.requests]
    vols, luts = {}, {}
    for kw in kws:
        if kw["volume_id"] not in vols:
            vols[kw["volume_id"]] = DeviceVolume(kw["volume"], value_scale=kw["value_scale"], normals="device",
                                                 brick_log2=args.serving_brick_log2)
    br = BatchRenderer(capacity=1, slots=2)
    stream = torch.cuda.Stream()
    out = []
    for kw in kws:
        lut = DeviceLUT(kw["color_tf"], kw["opacity_tf"])
        o8 = torch.empty(kw["width"] * kw["height"] * 4, dtype=torch.uint8, device="cuda")
        cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        br.render([RenderJob(vols[kw["volume_id"]], lut, kw["camera"], kw["light"], kw["config"], kw["width"],
                             kw["height"], o8, None, cnt)], stream=stream)
        b.record(stream)
        stream.synchronize()
        v = kw["volume"].data
        out.append({"tag": kw["tag"], "volume": list(v.shape), "storage": str(v.dtype), "res": kw["width"],
                    "inbox": int(cnt[0]), "shaded": int(cnt[1]), "ms": a.elapsed_time(b)})
        luts[len(out)] = lut
    br.close()
    return {"launches": out, "shaded": sum(r["shaded"] for r in out),
            "config": {"catalog": f"{args.serving_volumes} volumes {args.serving_min_dim}..{args.serving_max_dim}",
                       "records": args.records, "arithmetic": args.arithmetic}}


def c1_section(args, torch):
    """The small plain case (64^3 float32 double sphere, 256^2, balanced):
    device-timed frames, frames through render(), and the oracle on all host
    cores."""
    from pyvr_gb300 import VolumeRenderer, _native
    from pyvr_gb300 import workloads as W
    from pyvr_gb300.renderer import rgba_lut
    c = W.config_small()
    w, h = c["width"], c["height"]
    lib = _native.load()
    stream = torch.cuda.Stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)
    out = torch.empty(w * h * 4, dtype=torch.uint8, device="cuda")
    frames = 200
    with VolumeRenderer(w, h, config=c["config"], light=c["light"]) as r:
        r.load_volume(c["volume"])
        r.set_camera(c["camera"])
        r.set_transfer_functions(c["ctf"], c["otf"])
        for _ in range(max(args.warmup, 3) * 10):
            _native.check(lib.pvr_render_device(r._h, ctypes.c_void_p(out.data_ptr()), None, sptr))
        n_samples = r.last_sample_count()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(frames):
            _native.check(lib.pvr_render_device(r._h, ctypes.c_void_p(out.data_ptr()), None, sptr))
        b.record(stream)
        torch.cuda.synchronize()
        dev_ms = a.elapsed_time(b) / frames
        for _ in range(10):
            r.render()
        t = time.perf_counter()
        for _ in range(frames):
            r.set_camera(c["camera"])
            r.render()
        e2e_ms = 1000.0 * (time.perf_counter() - t) / frames
    res = {"ms_per_frame": dev_ms, "frames_per_s": 1000.0 / dev_ms, "e2e_frames_per_s": 1000.0 / e2e_ms,
           "samples_per_frame": n_samples,
           "config": "64^3 float32 double sphere, 256x256, balanced, directional light, linear opacity 0-0.1",
           "note": "L2-resident: a latency figure, not a bandwidth one"}
    if not args.skip_cpu:
        import oracle
        oracle.build()
        s = W.frame_inputs(c["volume"], c["camera"], c["light"], c["config"], rgba_lut(c["ctf"], c["otf"]),
                           w, h, c["value_scale"])
        oracle.render(s, want_float=False)
        reps = 10
        t = time.perf_counter()
        for _ in range(reps):
            oracle.render(s, want_float=False)
        cpu_ms = 1000.0 * (time.perf_counter() - t) / reps
        res["cpu_baseline"] = {"ms_per_frame": cpu_ms, "cores": oracle.max_threads(), "kind": "port",
                               "gpu_speedup_device": cpu_ms / dev_ms, "gpu_speedup_e2e": cpu_ms / e2e_ms}
    return res


def plain_section(args, torch):
    from pyvr_gb300 import VolumeRenderer, _native
    n_vol, res = args.plain_volume, args.plain_res
    scenes = make_scenes(tuple(args.storages.split(",")), n_vol, res)
    lib = _native.load()
    rend = {}
    from pyvr_gb300 import RenderConfig
    for dt, c in scenes.items():
        c["config"] = getattr(RenderConfig, args.plain_config)()
        r = VolumeRenderer(res, res, config=c["config"], light=c["light"])
        r.load_volume(c["volume"], value_scale=c["value_scale"])
        r.set_transfer_functions(c["ctf"], c["otf"])
        rend[dt] = r
    cams = next(iter(scenes.values()))["cameras"][:args.cameras]
    # an explicit stream: handle 0 (the legacy default stream) would mean
    # "the renderer's own stream" to the C ABI
    stream = torch.cuda.Stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)
    out = torch.empty(res * res * 4, dtype=torch.uint8, device="cuda")
    samples, shaded = {}, {}
    for dt, r in rend.items():
        for k, cam in enumerate(cams):
            r.set_camera(cam)
            _native.check(lib.pvr_render_device(r._h, ctypes.c_void_p(out.data_ptr()), None, sptr))
            samples[(dt, k)], shaded[(dt, k)] = r.last_sample_counts()

    def device_step(events=None):
        for dt, r in rend.items():
            for k, cam in enumerate(cams):
                r.set_camera(cam)
                if events is not None:
                    events.append((dt, k, torch.cuda.Event(enable_timing=True),
                                   torch.cuda.Event(enable_timing=True)))
                    events[-1][2].record(stream)
                _native.check(lib.pvr_render_device(r._h, ctypes.c_void_p(out.data_ptr()), None, sptr))
                if events is not None:
                    events[-1][3].record(stream)

    for _ in range(args.warmup):
        device_step()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    events = []
    t0.record(stream)
    for _ in range(args.steps):
        device_step(events)
    t1.record(stream)
    torch.cuda.synchronize()
    elapsed = t0.elapsed_time(t1) / 1000.0
    launch_ms = [(dt, k, a.elapsed_time(b)) for dt, k, a, b in events]
    e2e = None
    if not args.skip_e2e:
        for dt, r in rend.items():
            for cam in cams:
                r.set_camera(cam)
                r.render()
        torch.cuda.synchronize()
        te = time.perf_counter()
        for _ in range(args.steps):
            for dt, r in rend.items():
                for cam in cams:
                    r.set_camera(cam)
                    r.render()
        torch.cuda.synchronize()
        e2e = args.steps * len(rend) * len(cams) / (time.perf_counter() - te)
    frames = args.steps * len(rend) * len(cams)
    tot_bytes = sum(shaded[(dt, k)] * BYTES_PER_SAMPLE[dt] for dt, k, _ in launch_ms)
    tot_s = sum(ms for _, _, ms in launch_ms) / 1000.0
    peak, peak_kind = measured_peaks()
    per_dtype = {}
    for dt in rend:
        ms = [m for d, _, m in launch_ms if d == dt]
        by = sum(shaded[(d, k)] * BYTES_PER_SAMPLE[d] for d, k, _ in launch_ms if d == dt)
        # compulsory bytes: every voxel and its float32x3 normal read once, and
        # the image written once (an upper bound on what a frame must touch)
        data = scenes[dt]["volume"].data
        compulsory = data.size * (data.itemsize + 12) + res * res * 4
        per_dtype[dt] = {"avg_launch_ms": statistics.mean(ms), "gbs": by / (sum(ms) / 1000.0) / 1e9,
                         "samples_per_frame": statistics.mean(samples[(dt, k)] for k in range(len(cams))),
                         "compulsory_bytes_per_frame": compulsory,
                         "compulsory_gbs": compulsory / (statistics.mean(ms) / 1000.0) / 1e9}
    for r in rend.values():
        r.close()
    cpu = None
    if not args.skip_cpu:
        # the oracle on all host cores, one frame of camera 0 per storage
        import oracle
        from pyvr_gb300 import workloads as W
        from pyvr_gb300.renderer import rgba_lut
        oracle.build()
        cpu = {"cores": oracle.max_threads(), "kind": "port", "per_storage": {}}
        for dt, c in scenes.items():
            s = W.frame_inputs(c["volume"], cams[0], c["light"], c["config"], rgba_lut(c["ctf"], c["otf"]),
                               res, res, c["value_scale"])
            t = time.perf_counter()
            _, _, n = oracle.render(s, want_float=False)
            dt_s = time.perf_counter() - t
            cpu["per_storage"][dt] = {"ms_per_frame": 1000.0 * dt_s, "samples_per_s": n / dt_s,
                                      "gpu_speedup": dt_s / (per_dtype[dt]["avg_launch_ms"] / 1000.0)}
        cpu["sample"] = "one frame (camera 0) per storage"
    return {"frames_per_s": frames / elapsed, "e2e_frames_per_s": e2e,
            "ms_per_frame": 1000.0 * elapsed / frames,
            "samples_per_s": sum(samples[(dt, k)] for dt, k, _ in launch_ms) / elapsed,
            "roofline": march_roofline(sum(shaded[(dt, k)] for dt, k, _ in launch_ms), tot_s, None,
                                       PLAIN_WARP_INSTR_PER_SAMPLE, PLAIN_DRAM_BYTES_PER_SAMPLE, tot_bytes,
                                       torch, kernel="march_single_kernel", launches=len(launch_ms),
                                       per_storage=per_dtype,
                                       note="shaded samples over the summed CUDA-event times of the launches "
                                            "(one after the other on one stream); issue peak at the maximum "
                                            "SM clock", profile="profiles/march_single_kernel_256cube_1024px.md"),
            "gpu_launches": len(launch_ms), "cpu_baseline": cpu, "c1": c1_section(args, torch),
            "config": {"volume": f"{n_vol}^3 value noise seed 0", "storages": list(rend),
                       "cameras": len(cams), "resolution": f"{res}x{res}", "render_config": args.plain_config,
                       "frames_per_step": len(rend) * len(cams),
                       "l2": "inputs larger than L2 (208-256 MiB per storage)"}}


# ---------------------------------------------------------------------------

def serving_config(args):
    return {"workload": "serving: 32 resident volumes 128^3-512^3 u8/f16 (value noise, device normals), "
                        "Poisson stream 70% orbit 512^2 / 20% TF edit 512^2 / 5% 1024^2 high_quality "
                        "capture / 5% new-volume load, 40 GB budget, LRU",
            "step": "one second of the request stream at the sustained rate",
            "sustained": f"highest offered rate with p99 <= {P99_MS:.0f} ms over the 512^2 frames (orbit, TF "
                         f"edit, and new-volume load then render; captures reported beside) and completions >= 0.9x "
                         f"offered, found by an untimed sweep of {args.probe_s or args.steps:g}-second probes "
                         f"(doubling from {NOMINAL_RATE:.0f} req/s, then {args.refine} bisection probes)",
            "server": (f"continuous batching over {args.slots} launch slots (streams), "
                       f"up to {args.max_batch} requests and {args.batch_pixels} pixels per launch, "
                       f"linger {args.linger_us} us, {args.records} records, {args.arithmetic} arithmetic; "
                       "per-frame baseline: same runtime, one request per launch, each read back "
                       "before the next, a new volume loaded before anything that arrives after it"),
            "loads": (f"a pool of {args.serving_volumes + args.serving_extra} volumes whose records exceed the "
                      "40 GB budget; a load brings the volume out of the catalog longest (not resident), "
                      "uploads it from page-locked host memory (pvr_host_alloc) and lays it out with device normals; "
                      "LRU evicts"),
            "parallelism": f"replicas x{args.gpus}",
            "l2": "resident volumes (tens of GB) far exceed L2"}


def run_ours(args):
    import torch
    rank, world, local_rank = dist_env()
    torch.cuda.set_device(local_rank)
    from pyvr_gb300.batch import set_arithmetic, set_compact_records
    set_compact_records(args.records)
    set_arithmetic(args.arithmetic)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    if args.only == "requests":
        if rank == 0:
            print(json.dumps({"requests": requests_section(args, torch)}))
        return
    # the headline first, in a fresh process (no state of the other sections
    # -- their device memory, host threads, collected garbage -- around it)
    s = serving_section(args, torch) if args.only in ("all", "serving") else None

    def section(name, fn):
        if args.only not in ("all", name):
            return None
        gc.collect()
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        return fn(args, torch)

    plain = section("plain", plain_section)
    diff = section("diff", diff_section)
    batching = section("batching", batching_section)
    loaders = section("loaders", loaders_section)
    if s is None:
        if rank == 0:
            print(json.dumps({"plain": plain, "differentiation": diff, "batching_c3": batching,
                              "loaders": loaders}))
        return
    value, serial_value = s["value"], s["serial_value"]
    if world > 1:
        # replicas: each rank serves its own stream; the job's rate is all the
        # ranks' completed requests over the slowest rank's time
        from pyvr_gb300.replicas import job_rate
        n_srv, el_srv, n_ser, el_ser = s["counts"]
        value = job_rate(n_srv, el_srv, device="cuda")
        serial_value = job_rate(n_ser, el_ser, device="cuda")
    cpu = None
    if rank == 0 and not args.skip_cpu:
        # the same sample as the reference arm (--impl reference)
        c = reference_sample(args)
        cpu = {k: c[k] for k in ("value", "unit", "cores", "kind", "sample", "samples_per_s")}
    if rank == 0:
        srv = s["server"]
        att, satt = s["attempts"]["server"][-1], s["attempts"]["serial"][-1]
        # nested sections first, the headline's own keys last: the end of
        # the line is what a log tail keeps
        line = {"plain": plain, "batching_c3": batching, "differentiation": diff, "loaders": loaders,
                "nominal_400": s["nominal"],
                "probes": {"server": s["probes_server"], "serial": s["probes_serial"]},
                "timed_attempts": s["attempts"],
                "batching": {"batches": s["batches"], "mean_jobs_per_batch": s["mean_batch"],
                             "max_jobs_per_batch": s["max_batch"],
                             "summed_launch_time_over_wall": s["summed_launch_time_over_wall"],
                             "server": {"max_batch": args.max_batch, "slots": args.slots,
                                        "batch_pixels": args.batch_pixels, "linger_us": args.linger_us},
                             "lut_builds_timed": s["lut_builds"], "lut_hits": s["lut_hits"],
                             "lut_misses": s["lut_misses"]},
                "samples": {"inbox": s["inbox_samples"], "shaded": s["shaded_samples"],
                            "mean_inbox_per_request": s["mean_inbox_per_request"]},
                "pool": s["pool"], "roofline": s["roofline"], "cpu_baseline": cpu,
                "metric": "renders/s (batched server, mixed request stream, p99 of 512^2 frames <= 20 ms)",
                "value": value, "unit": "renders/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000.0,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": serving_config(args), "clocks": s["clocks"],
                "e2e": {"value": value, "unit": "renders/s", "h2d_bytes_per_step": s["h2d"],
                        "d2h_bytes_per_step": s["d2h"]},
                "gpu_launches": s["launches"],
                "latency_by_tag": s["by_tag"],
                "serial_per_frame": {"renders_per_s": serial_value, "p50_ms": s["serial_frames"].get("p50_ms"),
                                     "p99_ms": s["serial_frames"].get("p99_ms"),
                                     "p99_all_ms": s["serial"].get("p99_ms"), "sustained_offered": s["rate_serial"],
                                     "volume_loads": satt["volume_loads"], "evictions": satt["evictions"]},
                "timed_loads": {"load_requests": att["load_requests"], "volume_loads": att["volume_loads"],
                                "uploaded_bytes": att["uploaded_bytes"], "evictions": att["evictions"],
                                "over_budget": att["over_budget"], "alloc_retries": att["alloc_retries"],
                                "load_p50_ms": att["load_p50_ms"], "load_p99_ms": att["load_p99_ms"]},
                "roofline_issue_frac": s["roofline"]["frac"], "roofline_dram_frac": s["roofline"]["dram"]["frac"],
                "sustained_offered": s["rate_server"], "p99_all_ms": srv.get("p99_ms"),
                "p50_ms": s["server_frames"].get("p50_ms"), "p99_ms": s["server_frames"].get("p99_ms"),
                "server_over_serial": value / serial_value if serial_value else None}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def reference_sample(args) -> dict:
    """The reference's host path serving the request mix (ReferenceServer):
    a fresh workload (numpy value noise), ``--warmup`` untimed steps of one
    stream, then ``--steps`` timed steps of another, each at least
    ``--cpu-seconds / --steps`` seconds of host work.  Both the reference arm
    and the CPU baseline beside the headline report this same sample."""
    from pyvr_gb300 import workloads as W
    wl = W.ServingWorkload(n_volumes=args.serving_volumes, n_extra=args.serving_extra,
                           min_dim=args.serving_min_dim, max_dim=args.serving_max_dim, seed=0,
                           generator=lambda n, s: W.value_noise((n, n, n), s))
    per_step = max(1.0, args.cpu_seconds / max(1, args.steps))
    server = ReferenceServer()
    reference_serving_steps(wl, args.warmup, per_step, 800, server)
    steps, threads = reference_serving_steps(wl, args.steps, per_step, 900, server)
    reqs = sum(n for n, _, _, _ in steps)
    secs = sum(t for _, t, _, _ in steps)
    samples = sum(x for _, _, x, _ in steps)
    loads = sum(l for _, _, _, l in steps)
    value = reqs / secs if secs else 0.0
    return {"value": value, "unit": "renders/s", "cores": threads, "kind": "port",
            "sample": f"the reference's host path (float32 conversion and numpy normals for loads, Camera "
                      f"matrices, host LUTs) and the oracle on whole frames: {len(steps)} steps of the mix in "
                      f"stream order (catalog volumes {args.serving_min_dim}^3-{args.serving_max_dim}^3, 1024^2 "
                      f"captures, new-volume loads), each "
                      f">= {per_step:.1f} s of host work after {args.warmup} untimed steps; {reqs} requests "
                      f"({loads} loads) in {secs:.1f} s on {threads} threads",
            "samples_per_s": samples / secs if secs else 0.0,
            "steps": len(steps), "seconds": secs}


def run_reference(args):
    """The reference's own host path (no GPU, nothing of the pyvr_gb300 CUDA
    library): float32 conversion and numpy normals for new volumes, the
    Camera methods' matrices, host LUTs, and the CPU restatement of the
    shader (the oracle) on all host cores, serving the same request mix one
    request after another.  Each step is a bounded sample of the stream (at
    least --cpu-seconds / --steps seconds of host work, one second at least);
    the value is requests over the timed host seconds.  Volume data is
    generated (numpy) and the catalog volumes a request finds resident get
    their normals outside the timed work."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cpu = reference_sample(args)
    value = cpu["value"]
    line = {"impl": "reference", "metric": "renders/s (batched server, mixed request stream, p99 of 512^2 frames <= 20 ms)",
            "value": value, "unit": "renders/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * cpu["seconds"] / max(1, cpu["steps"]),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": serving_config(args),
            "cpu_baseline": {k: cpu[k] for k in ("kind", "cores", "value", "unit", "sample", "samples_per_s")},
            "e2e": {"value": value, "unit": "renders/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
