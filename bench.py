#!/usr/bin/env python
"""Benchmark of the pyvr ray-marching path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload ("plain at scale"): a 256^3 value-noise volume (seed 0) stored as
uint8 (read as UNORM), float16 and float32, each with float32 normals, 16
orbit cameras (azimuth 2*pi*k/16, elevation pi/6, distance 3), 1024x1024
RGBA8, RenderConfig.high_quality(), 8 seeded opacity points in [0, 0.3] and
a stand-in colour map.  One step renders all 48 frames (3 storages x 16
cameras).  Inputs (volume + normals, 208-256 MiB per storage) exceed the
129 MB L2.

value   : frames/s with the volume resident in HBM, device-timed (CUDA events)
e2e     : frames/s through the public API (set_camera + render() -> bytes,
          read back to host memory every frame)
roofline: the march kernel's algorithmic bytes (8 texels of the stored volume
          + 8 float32x3 normal texels per in-box sample) per launch over its
          event-timed duration, against the measured HBM copy bandwidth.
--impl reference: the CPU restatement of the reference shader (the oracle,
          OpenMP over all host cores) on bounded row bands of the same frames.
"""

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_SAMPLE = {"u8": 8 * 1 + 8 * 12, "f16": 8 * 2 + 8 * 12, "f32": 8 * 4 + 8 * 12}
DTYPES = ("u8", "f16", "f32")
RES = 1024
N_VOL = 256


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-rows", type=int, default=256, help="rows per CPU-baseline sample band")
    # smaller cases for profiling captures
    ap.add_argument("--storages", default=",".join(DTYPES))
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
    """nvidia-smi clocks/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu_index = gpu_index
        self.proc = None
        self.path = tempfile.mktemp(prefix="pvr_clocks_", suffix=".csv")

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9 or not parts[0].isdigit() or int(parts[0]) != self.gpu_index:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax = float(parts[2])
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def gpu_index(local_rank):
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    ids = [v for v in vis.split(",") if v.strip()]
    if ids and all(v.strip().isdigit() for v in ids) and local_rank < len(ids):
        return int(ids[local_rank])
    return local_rank


def make_scenes(storages=DTYPES):
    from pyvr_gb300 import workloads as W
    noise = W.config_scale_volume(N_VOL)
    return {dt: W.config_scale(dt, n=N_VOL, res=RES, noise=noise) for dt in storages}


def cpu_sample(scenes, rows, nthreads=0, cams=(0, 4, 8, 12)):
    """Time the oracle on a band of rows of the given frames; returns
    (seconds, in-box samples, threads)."""
    import oracle
    from pyvr_gb300 import workloads as W
    from pyvr_gb300.renderer import rgba_lut
    oracle.build()
    r0 = RES // 2 - rows // 2
    total_t, total_n = 0.0, 0
    for dt, c in scenes.items():
        lut = rgba_lut(c["ctf"], c["otf"])
        for k in cams:
            s = W.frame_inputs(c["volume"], c["cameras"][k], c["light"], c["config"], lut, RES,
                               RES, c["value_scale"])
            t = time.perf_counter()
            _, _, n = oracle.render(s, rows=(r0, r0 + rows), want_float=False, nthreads=nthreads)
            total_t += time.perf_counter() - t
            total_n += n
    return total_t, total_n, (nthreads or oracle.max_threads())


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    scenes = make_scenes()
    # samples of each full frame, for extrapolating band timings to frames/s:
    # the band's share of the frame's samples is estimated from the oracle
    # itself on a coarse (every 8th row) pass
    import oracle
    from pyvr_gb300 import workloads as W
    from pyvr_gb300.renderer import rgba_lut
    frame_samples = {}
    for dt, c in scenes.items():
        lut = rgba_lut(c["ctf"], c["otf"])
        s = W.frame_inputs(c["volume"], c["cameras"][3], c["light"], c["config"], lut, RES, RES,
                           c["value_scale"])
        tot = 0
        for r in range(0, RES, 16):
            tot += oracle.render(s, rows=(r, r + 1), want_float=False)[2]
        frame_samples[dt] = tot * 16
    times, rates = [], []
    for i in range(args.warmup + args.steps):
        t, n, threads = cpu_sample(scenes, args.cpu_rows)
        if i >= args.warmup:
            times.append(t)
            # frames/s: samples/s over the mean samples of one full frame
            rates.append(n / t / statistics.mean(frame_samples.values()))
    value = statistics.mean(rates)
    line = {"impl": "reference", "metric": "plain per-frame renders/s (256^3, 1024^2, high_quality)",
            "value": value, "unit": "renders/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * statistics.mean(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config_dict(args),
            "cpu_baseline": {"kind": "port", "cores": threads, "value": value, "unit": "renders/s",
                             "sample": f"rows {RES // 2 - args.cpu_rows // 2}..+{args.cpu_rows} of cameras 0,4,8,12, "
                                       f"each of u8/f16/f32, per step; frames/s = samples/s / samples per frame"},
            "e2e": {"value": value, "unit": "renders/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def config_dict(args):
    storages = args.storages.split(",")
    return {"workload": "plain_at_scale", "volume": f"{N_VOL}^3 value noise seed 0",
            "storages": storages, "cameras": args.cameras, "resolution": f"{RES}x{RES}",
            "render_config": "high_quality", "frames_per_step": args.cameras * len(storages),
            "parallelism": f"replicas x{args.gpus}", "l2": "inputs larger than L2 (208-256 MiB per storage)"}


def run_ours(args):
    import torch
    rank, world, local_rank = dist_env()
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    from pyvr_gb300 import VolumeRenderer, _native

    scenes = make_scenes(tuple(args.storages.split(",")))
    lib = _native.load()
    rend = {}
    for dt, c in scenes.items():
        r = VolumeRenderer(RES, RES, config=c["config"], light=c["light"])
        r.load_volume(c["volume"], value_scale=c["value_scale"])
        r.set_transfer_functions(c["ctf"], c["otf"])
        rend[dt] = r
    cams = next(iter(scenes.values()))["cameras"][:args.cameras]
    # an explicit stream: handle 0 (the legacy default stream) would mean
    # "the renderer's own stream" to the C ABI
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = ctypes.c_void_p(stream.cuda_stream)
    assert sptr.value
    out = torch.empty(RES * RES * 4, dtype=torch.uint8, device="cuda")

    # per-frame in-box and shaded sample counts (deterministic), from one
    # counted pass; the roofline counts the bytes of shaded samples only
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

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    for _ in range(args.warmup):
        device_step()
    clocks = ClockSampler(gpu_index(local_rank))
    clocks.start()
    barrier()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    events = []
    t0.record(stream)
    for _ in range(args.steps):
        device_step(events)
    t1.record(stream)
    barrier()
    clk = clocks.stop()
    elapsed = t0.elapsed_time(t1) / 1000.0
    launch_ms = [(dt, k, a.elapsed_time(b)) for dt, k, a, b in events]

    # end to end through the public API, host bytes back every frame
    e2e_elapsed = float("nan")
    if not args.skip_e2e:
        for dt, r in rend.items():
            for cam in cams:
                r.set_camera(cam)
                r.render()
        barrier()
        te = time.perf_counter()
        for _ in range(args.steps):
            for dt, r in rend.items():
                for cam in cams:
                    r.set_camera(cam)
                    r.render()
        barrier()
        e2e_elapsed = time.perf_counter() - te

    frames_per_step = len(rend) * len(cams)
    if world > 1:
        t = torch.tensor([elapsed, e2e_elapsed], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed, e2e_elapsed = t.tolist()
    value = world * args.steps * frames_per_step / elapsed
    e2e_value = (None if args.skip_e2e else
                 world * args.steps * frames_per_step / e2e_elapsed)

    # roofline of the march kernel (algorithmic bytes over event-timed launches)
    tot_bytes = sum(shaded[(dt, k)] * BYTES_PER_SAMPLE[dt] for dt, k, _ in launch_ms)
    tot_s = sum(ms for _, _, ms in launch_ms) / 1000.0
    achieved = tot_bytes / tot_s / 1e9
    peak, peak_kind = measured_peaks()
    tot_samples = sum(samples[(dt, k)] for dt, k, _ in launch_ms)
    per_dtype = {}
    for dt in rend:
        ms = [m for d, _, m in launch_ms if d == dt]
        by = sum(shaded[(d, k)] * BYTES_PER_SAMPLE[d] for d, k, _ in launch_ms if d == dt)
        per_dtype[dt] = {"avg_launch_ms": statistics.mean(ms),
                         "gbs": by / (sum(ms) / 1000.0) / 1e9,
                         "samples_per_frame": statistics.mean(samples[(dt, k)] for k in range(len(cams))),
                         "shaded_per_frame": statistics.mean(shaded[(dt, k)] for k in range(len(cams)))}

    cpu = None
    if rank == 0 and not args.skip_cpu:
        ct, cn, threads = cpu_sample(scenes, args.cpu_rows)
        mean_frame = statistics.mean(samples.values())
        cpu = {"value": cn / ct / mean_frame, "unit": "renders/s", "cores": threads, "kind": "port",
               "sample": f"oracle on rows {RES // 2 - args.cpu_rows // 2}..+{args.cpu_rows} of cameras 0,4,8,12 "
                         f"for u8/f16/f32 ({cn} samples in {ct:.1f} s); renders/s = samples/s / "
                         f"mean in-box samples per frame",
               "samples_per_s": cn / ct}
    for r in rend.values():
        r.close()
    if rank == 0:
        line = {"metric": "plain per-frame renders/s (256^3, 1024^2, high_quality)",
                "value": value, "unit": "renders/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000 * elapsed / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": config_dict(args),
                "samples_per_s": world * args.steps * (tot_samples / args.steps) / elapsed,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "peak_kind": peak_kind, "traffic": None,
                             "kernel": "march_kernel", "per_storage": per_dtype},
                "cpu_baseline": cpu, "clocks": clk,
                "e2e": {"value": e2e_value, "unit": "renders/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": frames_per_step * RES * RES * 4},
                "gpu_launches": len(launch_ms)}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
