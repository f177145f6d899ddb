"""Benchmark of the frame-stack compositing hot path on one GB300 (or N replicas).

Workload (one "step"): the HD stack of 64 frames of 1920x1080 RGB u8 (seeded gradient +
Gaussian noise sigma 4, three moving disks r in [10, 40]) composited six times, the settings
the configuration names for it: --threshold abs/0.05/0.2 with --outlier average, forward and
backward, --threshold rel/3/6 with --outlier average, and --mode darker / lighter.
Metric: megapixel-frames per second = 6 * 64 * 1920 * 1080 / 1e6 per step / time.

  value       device-resident frames, kernels only (CUDA events on the library's stream)
  e2e         the same step through cp_composite with the frames in pinned host memory:
              every step copies each composite's 64 frames host->device and the results back
  roofline    the outlier kernel: algorithmic bytes (n*P*C read + 2*P*C written) per launch /
              its mean launch time, against the measured HBM copy bandwidth
  cpu_baseline  the C++ restatement of the reference (oracle/) on a band of rows, all cores

--impl reference times the reference's CPU algorithm (the oracle restatement; the Rust
reference cannot be built here) on the same workload and prints its own line.
Under torchrun each rank runs the whole workload on its own GPU (replicas, weak scaling).
"""
import argparse
import ctypes as ct
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_FRAMES, W, H, C = 64, 1920, 1080, 3
VARIANTS = [
    ("abs/0.05/0.2 average", dict(mode="outlier", threshold="abs/0.05/0.2", outlier="average", background="first")),
    ("abs/0.05/0.2 forward", dict(mode="outlier", threshold="abs/0.05/0.2", outlier="forward", background="first")),
    ("abs/0.05/0.2 backward", dict(mode="outlier", threshold="abs/0.05/0.2", outlier="backward", background="first")),
    ("rel/3/6 average", dict(mode="outlier", threshold="rel/3/6", outlier="average", background="first")),
    ("darker", dict(mode="darker")),
    ("lighter", dict(mode="lighter")),
]
MPXF_PER_COMPOSITE = N_FRAMES * W * H / 1e6
ALGO_BYTES_OUTLIER = N_FRAMES * W * H * C + 2 * W * H * C   # frames read + composite + mask
ALGO_BYTES_SIMPLE = N_FRAMES * W * H * C + W * H * C
METRIC = "Mpx-frames/s"
CONFIG = {"workload": "64x1920x1080 RGB u8 stack, 6 composites per step (abs/0.05/0.2 "
                      "average|forward|backward, rel/3/6 average, darker, lighter), "
                      "background first",
          "frames": N_FRAMES, "width": W, "height": H, "channels": C,
          "l2": "inputs (398 MB per composite) exceed the 126 MB L2; no flush between steps"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def barrier_max(value):
    """Barrier + max over ranks (gloo on the host; no data-path collective)."""
    ws, _ = dist_env()
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier():
    ws, _ = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """SM clocks, power and clock-event reasons sampled every 10 ms during the timed region
    through NVML (libnvidia-ml, read-only queries); nvidia-smi at 200 ms if NVML is absent."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.nvml = None
        self.stop = threading.Event()
        self.samples = []   # (sm_mhz, max_mhz, power_w, reason_bits)
        self.lines = []

    def _nvml_handle(self):
        nv = ct.CDLL("libnvidia-ml.so.1")
        if nv.nvmlInit_v2() != 0:
            return None, None
        h = ct.c_void_p()
        try:
            import torch
            pr = torch.cuda.get_device_properties(self.gpu)
            bus = b"%08X:%02X:%02X.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
            if nv.nvmlDeviceGetHandleByPciBusId_v2(bus, ct.byref(h)) == 0:
                return nv, h
        except Exception:
            pass
        if nv.nvmlDeviceGetHandleByIndex_v2(ct.c_uint(self.gpu), ct.byref(h)) == 0:
            return nv, h
        return None, None

    def _poll(self, nv, h):
        reasons_fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nv.nvmlDeviceGetCurrentClocksThrottleReasons
        sm, mx, mw, bits = ct.c_uint(), ct.c_uint(), ct.c_uint(), ct.c_ulonglong()
        while not self.stop.is_set():
            if nv.nvmlDeviceGetClockInfo(h, 1, ct.byref(sm)) == 0:
                nv.nvmlDeviceGetMaxClockInfo(h, 1, ct.byref(mx))
                nv.nvmlDeviceGetPowerUsage(h, ct.byref(mw))
                reasons_fn(h, ct.byref(bits))
                self.samples.append((sm.value, mx.value, mw.value / 1e3, bits.value))
            self.stop.wait(0.01)

    def __enter__(self):
        try:
            nv, h = self._nvml_handle()
        except Exception:
            nv, h = None, None
        if nv is not None:
            self.nvml = nv
            self.t = threading.Thread(target=self._poll, args=(nv, h), daemon=True)
            self.t.start()
            deadline = time.time() + 2.0
            while not self.samples and time.time() < deadline:
                time.sleep(0.002)
            return self
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            deadline = time.time() + 5.0
            while not self.lines and time.time() < deadline:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        self.stop.set()
        if self.nvml is not None:
            self.t.join(timeout=2)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, power, reasons = [], None, [], set()
        for s, m, pw, bits in self.samples:
            sm.append(float(s))
            mx = float(m)
            power.append(pw)
            for b, nm in self.REASONS.items():
                if bits & b:
                    reasons.add(nm)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "power_w": statistics.median(power) if power else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "source": "nvml" if self.nvml is not None else "nvidia-smi"}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0}, "fallback"


def profiled_traffic():
    """DRAM bytes per launch of the outlier kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "k_composite_outlier_hd64.md")
    try:
        for line in open(path):
            if line.strip().startswith("dram_bytes_per_launch:"):
                return float(line.split(":")[1].split()[0])
    except Exception:
        pass
    return None


def cpu_band(rows):
    from chrono_photo_gb300 import example_data
    return example_data.hd_stack(seed=2, n=N_FRAMES, w=W, h=rows)


def cpu_sample(threads, frames, reps=1):
    """Reference CPU path (the oracle's C++ restatement of the reference) on a band of rows of
    the same stack: the six variants, `reps` times, on `threads` host threads.
    Returns (Mpx-frames/s, seconds, description)."""
    from chrono_photo_gb300 import make_params
    from oracle import oracle
    rows = frames.shape[1]
    keep = []
    params = [make_params(keep=keep, **kw) for _, kw in VARIANTS]
    t0 = time.perf_counter()
    for _ in range(reps):
        for p in params:
            oracle.composite(frames, p, threads=threads)
    dt = time.perf_counter() - t0
    mpxf = reps * len(VARIANTS) * N_FRAMES * W * rows / 1e6
    return mpxf / dt, dt, "%d x 6 variants on a 64x1920x%d band (%d rows of 1080), %d threads" % (
        reps, rows, rows, threads)


def run_reference(args):
    ws, rank = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    frames = cpu_band(160)   # one step: the six variants on 160 rows (~0.25 s on 16 cores)
    for _ in range(args.warmup):
        cpu_sample(threads, frames)
    t = 0.0
    for _ in range(args.steps):
        v, dt, desc = cpu_sample(threads, frames)
        t += dt
    value = args.steps * len(VARIANTS) * N_FRAMES * W * 160 / 1e6 / t
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * len(VARIANTS) * MPXF_PER_COMPOSITE / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded)", "config": CONFIG,
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import numpy as np
    import torch

    from chrono_photo_gb300 import _abi, example_data, make_params
    from chrono_photo_gb300.api import Context

    ws, rank = dist_env()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ctx = Context(local)
    lib = _abi.lib()
    h = ctx.handle
    frame_bytes = W * H * C
    # pinned host stack (e2e) and device-resident copy (kernel timing)
    host_ptr = ct.c_void_p()
    ctx.check(lib.cp_host_alloc(h, N_FRAMES * frame_bytes, ct.byref(host_ptr)))
    host = np.ctypeslib.as_array((ct.c_uint8 * (N_FRAMES * frame_bytes)).from_address(host_ptr.value))
    host = host.reshape(N_FRAMES, H, W, C)
    example_data.hd_stack(seed=2 + rank, out=host)
    dev = ctx.upload(host)
    out = ctx.alloc(frame_bytes)
    blend = ctx.alloc(frame_bytes)
    out_host = ct.c_void_p()
    blend_host = ct.c_void_p()
    ctx.check(lib.cp_host_alloc(h, frame_bytes, ct.byref(out_host)))
    ctx.check(lib.cp_host_alloc(h, frame_bytes, ct.byref(blend_host)))
    keep = []
    params = [make_params(keep=keep, **kw) for _, kw in VARIANTS]
    dstack = _abi.Stack(n=N_FRAMES, width=W, height=H, channels=C, base=dev,
                        frame_stride=frame_bytes)
    hstack = _abi.Stack(n=N_FRAMES, width=W, height=H, channels=C, base=host_ptr.value,
                        frame_stride=frame_bytes)
    stream = torch.cuda.ExternalStream(lib.cp_ctx_stream(h))

    def device_step(events=None):
        for i, p in enumerate(params):
            if events is not None:
                events[i][0].record(stream)
            rc = lib.cp_composite_device(h, ct.byref(dstack), ct.byref(p), out,
                                         blend if p.mode == 0 else None, None, None, None)
            ctx.check(rc, "cp_composite_device")
            if events is not None:
                events[i][1].record(stream)

    def e2e_step():
        for p in params:
            rc = lib.cp_composite(h, ct.byref(hstack), ct.byref(p), out_host.value,
                                  blend_host.value if p.mode == 0 else None, None, None)
            ctx.check(rc, "cp_composite")

    # ---- device-resident timing -------------------------------------------------------------
    for _ in range(args.warmup):
        device_step()
    ctx.synchronize()
    ev = [[[torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)]
           for _ in VARIANTS] for _ in range(args.steps)]
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        start.record(stream)
        for s in range(args.steps):
            device_step(ev[s])
        stop.record(stream)
        ctx.synchronize()
        torch.cuda.synchronize()
    barrier()
    ms = start.elapsed_time(stop)
    ms_max = barrier_max(ms)
    per_var = [statistics.mean(ev[s][i][0].elapsed_time(ev[s][i][1]) for s in range(args.steps))
               for i in range(len(VARIANTS))]
    value = ws * args.steps * len(VARIANTS) * MPXF_PER_COMPOSITE / (ms_max / 1e3)

    # ---- end to end through the host-memory entry point -------------------------------------
    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = barrier_max(time.perf_counter() - t0)
    e2e_value = ws * args.steps * len(VARIANTS) * MPXF_PER_COMPOSITE / e2e_s

    if rank != 0:
        return
    peaks, peak_kind = measured_peaks()
    outlier_ms = statistics.mean(per_var[:4])
    achieved = ALGO_BYTES_OUTLIER / (outlier_ms / 1e3) / 1e9
    traffic = profiled_traffic()
    cpu_v, cpu_dt, cpu_desc = cpu_sample(os.cpu_count() or 1, cpu_band(320), reps=3)
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded disk-over-gradient stacks)", "config": CONFIG,
        "variants_ms": {name: round(t, 4) for (name, _), t in zip(VARIANTS, per_var)},
        "e2e": {"value": e2e_value, "unit": METRIC,
                "h2d_bytes_per_step": len(VARIANTS) * N_FRAMES * frame_bytes,
                "d2h_bytes_per_step": (len(VARIANTS) + 4) * frame_bytes},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                     "kernel": "k_composite<3> (outlier)", "peak_kind": peak_kind},
        "cpu_baseline": {"value": cpu_v, "unit": METRIC, "cores": os.cpu_count(),
                         "kind": "port", "sample": cpu_desc},
        "clocks": clk.summary(),
        "gpu_launches": args.steps * len(VARIANTS),
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, _ = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    try:
        if args.impl == "reference":
            run_reference(args)
        else:
            run_gpu(args)
    finally:
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
