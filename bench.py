"""Benchmark of the frame-stack compositing hot path on one GB300 (or N replicas).

Workload (one "step"): the HD stack of 64 frames of 1920x1080 RGB u8 (seeded gradient +
Gaussian noise sigma 4, three moving disks r in [10, 40]) composited six times, the settings
the configuration names for it: --threshold abs/0.05/0.2 with --outlier average, forward and
backward, --threshold rel/3/6 with --outlier average, and --mode darker / lighter.
Metric: megapixel-frames per second = 6 * 64 * 1920 * 1080 / 1e6 per step / time.

  value       device-resident frames, kernels only (CUDA events on the library's stream): one
              cp_composite_device_multi call per step, one multi-setting launch that stages
              the stack once, shares its order statistics between the four outlier settings
              and folds darker / lighter on the same rows (device_single_calls: six
              cp_composite_device calls, one launch each)
  e2e         the same step from pinned host memory through cp_composite_multi: every step
              copies the 64 frames host->device once (band by band, overlapping the kernels:
              one multi-setting launch per band) and the six composites and four blend
              masks back
  e2e_single_calls  the step as six cp_composite calls (the one-setting drop-in), each
              copying the frames again
  roofline    the single-setting outlier kernel: algorithmic bytes (n*P*C read + 2*P*C
              written) per launch / its mean launch time, against the measured HBM copy
              bandwidth; roofline_multi the same for the multi-setting launch
  cpu_baseline  the C++ restatement of the reference (oracle/) on the same whole stack, two
              steps on all host threads
  batched     the batched half of the metric, against the plain kernel on the same work:
              batched.video (300 resident 1080p frames, 269 sliding windows of 32) and
              batched.serve (512 mixed jobs through the continuous-batching server, p50/p99
              latency); --no-batched leaves them out
  autotune    the launch configuration the autotuner chose per outlier setting (phase A
              layout, staging buffers, CTAs per SM) with the tuned and static times

--impl reference times the reference's CPU algorithm (the oracle restatement; the Rust
reference cannot be built here) on the same workload, the whole stack for every step, and
prints its own line; it loads the oracle's library only.
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


def profiled(key):
    """A per-launch figure (`dram_bytes_per_launch`, `warp_instructions_per_launch`) of the
    abs/average outlier launch from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "k_outlier_px_hd64.md")
    try:
        for line in open(path):
            if line.strip().startswith(key + ":"):
                return float(line.split(":")[1].split()[0])
    except Exception:
        pass
    return None


def example_data_module():
    """The seeded generators (chrono_photo_gb300/example_data.py, numpy only), loaded from
    their file so that the reference arm imports nothing else of the package."""
    import importlib.util
    path = os.path.join(ROOT, "chrono_photo_gb300", "example_data.py")
    spec = importlib.util.spec_from_file_location("cp_example_data", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def reference_settings():
    """The six settings as cp_params built by the oracle's pure-Python option parser."""
    from oracle import oracle
    return [oracle.params(**kw) for _, kw in VARIANTS]


def cpu_step(frames, settings, threads):
    """One step on the CPU: the reference's algorithm (the oracle's C++ restatement) for the
    six settings on the whole stack, `threads` host threads. Returns seconds."""
    from oracle import oracle
    t0 = time.perf_counter()
    for p in settings:
        oracle.composite(frames, p, threads=threads)
    return time.perf_counter() - t0


def run_reference(args):
    """The reference arm: the reference's CPU algorithm on the machine's host cores, the same
    64 x 1920x1080 stack and six settings per step as the GPU arm, `--warmup` untimed and
    `--steps` timed steps. Only the oracle's library is loaded (no library of the product)."""
    ws, rank = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    frames = example_data_module().hd_stack(seed=2)
    settings = reference_settings()
    for _ in range(args.warmup):
        cpu_step(frames, settings, threads)
    t = 0.0
    for _ in range(args.steps):
        t += cpu_step(frames, settings, threads)
    value = args.steps * len(VARIANTS) * MPXF_PER_COMPOSITE / t
    desc = ("the whole 64x1920x1080 stack, six settings per step, %d timed steps, %d threads"
            % (args.steps, threads))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t / args.steps,
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

    def e2e_single_calls():
        for p in params:
            rc = lib.cp_composite(h, ct.byref(hstack), ct.byref(p), out_host.value,
                                  blend_host.value if p.mode == 0 else None, None, None)
            ctx.check(rc, "cp_composite")

    # one cp_composite_multi call per step: the stack crosses the host link once, the six
    # composites and four blend masks come back into pinned memory
    nv = len(params)
    multi_ptr = ct.c_void_p()
    ctx.check(lib.cp_host_alloc(h, 2 * nv * frame_bytes, ct.byref(multi_ptr)))
    multi_params = (_abi.Params * nv)(*params)
    multi_outs = (ct.c_void_p * nv)(*[multi_ptr.value + i * frame_bytes for i in range(nv)])
    multi_blends = (ct.c_void_p * nv)(*[multi_ptr.value + (nv + i) * frame_bytes
                                        if p.mode == 0 else None for i, p in enumerate(params)])
    multi_warn = (ct.c_uint64 * nv)()

    def e2e_step():
        rc = lib.cp_composite_multi(h, ct.byref(hstack), multi_params, nv, multi_outs,
                                    multi_blends, multi_warn)
        ctx.check(rc, "cp_composite_multi")

    # the device-resident step as one cp_composite_device_multi call: one multi-setting
    # launch (cp_outlier_multi.cuh) stages the stack once, the four outlier settings share
    # its order statistics, darker and lighter fold the same staged rows
    dmo = [ctx.alloc(frame_bytes) for _ in range(nv)]
    dmb = [ctx.alloc(frame_bytes) if p.mode == 0 else None for p in params]
    dmulti_outs = (ct.c_void_p * nv)(*dmo)
    dmulti_blends = (ct.c_void_p * nv)(*dmb)
    n_outlier = sum(1 for p in params if p.mode == 0)

    def device_step_multi():
        rc = lib.cp_composite_device_multi(h, ct.byref(dstack), multi_params, nv, dmulti_outs,
                                           dmulti_blends, None, None)
        ctx.check(rc, "cp_composite_device_multi")

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
        ms = start.elapsed_time(stop)
        # the same step through cp_composite_device_multi, then its multi-setting launch alone
        for _ in range(args.warmup):
            device_step_multi()
        ctx.synchronize()
        barrier()
        torch.cuda.synchronize()
        launches0 = ct.c_uint64()
        ctx.check(lib.cp_ctx_launch_counts(h, ct.byref(launches0), None, None))
        start.record(stream)
        for _ in range(args.steps):
            device_step_multi()
        stop.record(stream)
        ctx.synchronize()
        torch.cuda.synchronize()
        ms_multi = start.elapsed_time(stop)
        launches1 = ct.c_uint64()
        ctx.check(lib.cp_ctx_launch_counts(h, ct.byref(launches1), None, None))
    barrier()
    ms_single_max = barrier_max(ms)
    ms_max = barrier_max(ms_multi)
    per_var = [statistics.mean(ev[s][i][0].elapsed_time(ev[s][i][1]) for s in range(args.steps))
               for i in range(len(VARIANTS))]
    value = ws * args.steps * len(VARIANTS) * MPXF_PER_COMPOSITE / (ms_max / 1e3)
    value_single = ws * args.steps * len(VARIANTS) * MPXF_PER_COMPOSITE / (ms_single_max / 1e3)
    for q in dmo + [q for q in dmb if q]:
        ctx.free(q)

    # ---- end to end through the host-memory entry point -------------------------------------
    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = barrier_max(time.perf_counter() - t0)
    e2e_value = ws * args.steps * len(VARIANTS) * MPXF_PER_COMPOSITE / e2e_s
    # the drop-in form: one cp_composite per setting, each uploading the stack again
    single_steps = max(1, min(args.steps, 20))
    e2e_single_calls()
    barrier()
    t0 = time.perf_counter()
    for _ in range(single_steps):
        e2e_single_calls()
    single_s = barrier_max(time.perf_counter() - t0)
    single_value = ws * single_steps * len(VARIANTS) * MPXF_PER_COMPOSITE / single_s

    if rank != 0:
        return
    peaks, peak_kind = measured_peaks()
    outlier_ms = statistics.mean(per_var[:4])
    # one multi-setting launch per step: the stack read once, composite + mask of each
    # outlier setting and the composite of darker / lighter written
    fused_ms = ms_max / args.steps
    multi_bytes = N_FRAMES * frame_bytes + (2 * n_outlier + (nv - n_outlier)) * frame_bytes
    achieved = ALGO_BYTES_OUTLIER / (outlier_ms / 1e3) / 1e9
    traffic = profiled("dram_bytes_per_launch")
    # the path is bound by instruction issue: the abs/average launch's warp instructions
    # (ncu) over its CUDA-event time, against 4 issues per clock on every SM
    instr = profiled("warp_instructions_per_launch")
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    clk_summary = clk.summary()
    sm_hz = (clk_summary["sm_mhz"] or 2070.0) * 1e6
    issue_peak = 4.0 * sms * sm_hz / 1e9
    issue = None
    if instr:
        ach = instr / (per_var[0] / 1e3) / 1e9
        issue = {"achieved": ach, "peak": issue_peak, "unit": "G warp instructions/s",
                 "frac": ach / issue_peak,
                 "kernel": "k_outlier_px<1, 2, 1, 2, 0, 2> (abs average)",
                 "instructions_per_launch": instr}
    # the reference's CPU algorithm on the same whole stack: two steps on all host threads
    cpu_threads = os.cpu_count() or 1
    cpu_settings = reference_settings()
    cpu_t = sum(cpu_step(host, cpu_settings, cpu_threads) for _ in range(2))
    cpu_v = 2 * len(VARIANTS) * MPXF_PER_COMPOSITE / cpu_t
    cpu_desc = "2 steps (six settings on the whole 64x1920x1080 stack), %d threads" % cpu_threads
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded disk-over-gradient stacks)", "config": CONFIG,
        "call": "one cp_composite_device_multi per step: one multi-setting launch stages "
                "the stack once; the four outlier settings share its order statistics, "
                "darker and lighter fold the same staged rows",
        "device_single_calls": {"value": value_single, "unit": METRIC,
                                "ms_per_step": ms_single_max / args.steps,
                                "call": "six cp_composite_device calls (one launch per "
                                        "setting)"},
        "variants_ms": {name: round(t, 4) for (name, _), t in zip(VARIANTS, per_var)},
        "e2e": {"value": e2e_value, "unit": METRIC,
                "h2d_bytes_per_step": N_FRAMES * frame_bytes,
                "d2h_bytes_per_step": (len(VARIANTS) + 4) * frame_bytes,
                "call": "cp_composite_multi: the stack from pinned host memory once per step, "
                        "six composites + four blend masks back"},
        "e2e_single_calls": {"value": single_value, "unit": METRIC, "steps": single_steps,
                             "h2d_bytes_per_step": len(VARIANTS) * N_FRAMES * frame_bytes,
                             "d2h_bytes_per_step": (len(VARIANTS) + 4) * frame_bytes,
                             "call": "six cp_composite calls (the drop-in for one "
                                     "OutlierProcessor / SimpleProcessor run each)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                     "kernel": "k_outlier_px (outlier, mean of the four settings)",
                     "peak_kind": peak_kind},
        "issue_roofline": issue,
        "roofline_multi": {"bound": "hbm", "achieved": multi_bytes / (fused_ms / 1e3) / 1e9,
                           "peak": peaks["hbm_gbs"], "unit": "GB/s",
                           "frac": multi_bytes / (fused_ms / 1e3) / 1e9 / peaks["hbm_gbs"],
                           "ms": fused_ms, "bytes": multi_bytes,
                           "kernel": "k_outlier_multi<2, true> (the six settings of a step)",
                           "note": "algorithmic bytes: the stack read once + the step's ten "
                                   "output images"},
        "cpu_baseline": {"value": cpu_v, "unit": METRIC, "cores": cpu_threads,
                         "kind": "port", "sample": cpu_desc},
        "clocks": clk_summary,
        # the library's own count of the kernels it launched in the timed region
        "gpu_launches": launches1.value - launches0.value,
        "autotune": tuning_report(ctx, lib, _abi),
    }
    if not args.no_batched:
        # the batched half of the metric: the sliding-window chrono-video and served mixed
        # jobs, each against the plain one-stack-per-launch kernel on the same work
        line["batched"] = {}
        for name, fn in (("video", video_workload), ("serve", serve_workload)):
            try:
                line["batched"][name] = fn(args, ctx, lib, _abi, local)
            except Exception as e:  # the headline line is printed in any case
                line["batched"][name] = {"error": "%s: %s" % (type(e).__name__, e)}
    print(json.dumps(line), flush=True)


def tuning_report(ctx, lib, _abi):
    """The launch configurations the autotuner chose for the outlier settings of this run
    (cp_ctx_tuning_report): per key the tuned and the static configuration's times, measured
    on the first launch of the warm-up or read from the tuning cache."""
    buf = ct.create_string_buffer(1 << 16)
    ctx.check(lib.cp_ctx_tuning_report(ctx.handle, buf, len(buf)), "cp_ctx_tuning_report")
    rows = json.loads(buf.value.decode())
    for r in rows:
        r["tuned_over_static"] = (r["static_ms"] / r["tuned_ms"]) if r["tuned_ms"] else None
    return {"keys": rows, "env": {k: os.environ.get(k) for k in ("CP_AUTOTUNE", "CP_PX_CONFIG")
                                  if os.environ.get(k) is not None}}


# ---- other configurations (--workload): their own JSON lines, not the headline ---------------
def _ctx_and_lib():
    import torch
    from chrono_photo_gb300 import _abi
    from chrono_photo_gb300.api import Context
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    return Context(local), _abi.lib(), _abi, local


def _pinned(ctx, lib, nbytes):
    import numpy as np
    ptr = ct.c_void_p()
    ctx.check(lib.cp_host_alloc(ctx.handle, nbytes, ct.byref(ptr)))
    return ptr.value, np.ctypeslib.as_array((ct.c_uint8 * nbytes).from_address(ptr.value))


def _time_device(ctx, lib, fn, steps, warmup):
    """Mean ms per call of fn() on the library's stream (CUDA events), after warm-up."""
    import torch
    for _ in range(warmup):
        fn()
    ctx.synchronize()
    stream = torch.cuda.ExternalStream(lib.cp_ctx_stream(ctx.handle))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def video_workload(args, ctx, lib, _abi, local, clk=None):
    """Chrono-video: 300 resident frames of 1920x1080 (--video-frames, --video-size; a smaller
    pool for profiling; brightness drift, one disk on a sine path, generated on the device),
    269 windows [f, f+32) with explicit index lists,
    abs/0.05/0.2 extreme, background first. Times one cp_composite_video_device call (the
    windows slide by one frame: the sliding-window kernel), the same call with every window
    on the general batched kernel (CP_VIDEO_SLIDING=0), and the plain kernel (one
    cp_composite_device launch per window); e2e uploads the pool from pinned host memory and
    reads every composite and mask back. Returns a dict."""
    import numpy as np
    from chrono_photo_gb300 import example_data, make_params
    n_pool, win = args.video_frames, 32
    VW, VH = (int(v) for v in args.video_size.lower().split("x"))
    nwin = n_pool - win + 1
    fb = VW * VH * C
    pool = example_data.video_stack_device(seed=3, n=n_pool, w=VW, h=VH)
    dev = pool.data_ptr()
    hptr, _ = _pinned(ctx, lib, n_pool * fb)
    ctx.check(lib.cp_memcpy_d2h(ctx.handle, hptr, dev, n_pool * fb, None))
    frame_ptrs = (ct.c_void_p * n_pool)(*[dev + i * fb for i in range(n_pool)])
    starts = np.arange(nwin, dtype=np.int64) * win
    lens = np.full(nwin, win, np.int32)
    idx = np.concatenate([np.arange(k, k + win, dtype=np.int32) for k in range(nwin)])
    outs_dev = ctx.alloc(2 * nwin * fb)
    outs = (ct.c_void_p * nwin)(*[outs_dev + k * fb for k in range(nwin)])
    blends = (ct.c_void_p * nwin)(*[outs_dev + (nwin + k) * fb for k in range(nwin)])
    keep = []
    p = make_params(keep=keep, mode="outlier", threshold="abs/0.05/0.2", outlier="extreme",
                    background="first")

    def call():
        ctx.check(lib.cp_composite_video_device(
            ctx.handle, frame_ptrs, n_pool, VW, VH, C, nwin, starts.ctypes.data_as(_abi.I64P),
            lens.ctypes.data_as(_abi.I32P), idx.ctypes.data_as(_abi.I32P), ct.byref(p), outs,
            blends, None, None), "cp_composite_video_device")

    steps = max(3, min(args.steps, 20))
    ms = _time_device(ctx, lib, call, steps, 3)
    os.environ["CP_VIDEO_SLIDING"] = "0"
    try:
        batched_ms = _time_device(ctx, lib, call, max(2, steps // 4), 2)
    finally:
        del os.environ["CP_VIDEO_SLIDING"]
    # the plain kernel on the same windows: one cp_composite_device launch per window
    wstacks = []
    for k in range(nwin):
        ptrs = (ct.c_void_p * win)(*[frame_ptrs[k + i] for i in range(win)])
        keep.append(ptrs)
        wstacks.append(_abi.Stack(n=win, width=VW, height=VH, channels=C,
                                  frames=ct.cast(ptrs, ct.POINTER(ct.c_void_p)), frame_offset=k))

    def plain():
        for k in range(nwin):
            ctx.check(lib.cp_composite_device(ctx.handle, ct.byref(wstacks[k]), ct.byref(p),
                                              outs[k], blends[k], None, None, None), "plain")
    plain_ms = _time_device(ctx, lib, plain, max(2, steps // 4), 2)
    # end to end: upload the pool from pinned memory, composite, read every window back
    optr, _ = _pinned(ctx, lib, 2 * nwin * fb)
    e2e_steps = max(2, min(steps, 5))

    def e2e():
        ctx.check(lib.cp_memcpy_h2d(ctx.handle, dev, hptr, n_pool * fb, None))
        call()
        ctx.check(lib.cp_memcpy_d2h(ctx.handle, optr, outs_dev, 2 * nwin * fb, None))
        ctx.synchronize()
    e2e()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    mpxf = nwin * win * VW * VH / 1e6
    unique = n_pool * fb + 2 * nwin * fb
    peaks, kind = measured_peaks()
    ach = unique / (ms / 1e3) / 1e9
    ctx.free(outs_dev)
    del pool
    return {
        "workload": "chrono-video: %d resident %dx%d RGB frames, %d windows of 32 at "
                    "stride 1, abs/0.05/0.2 extreme, background first" % (n_pool, VW, VH, nwin),
        "metric": METRIC, "value": mpxf / (ms / 1e3), "unit": METRIC, "ms_per_call": ms,
        "steps": steps, "kernel": "k_video_slide (windows sliding by one frame)",
        "batched_general": {"value": mpxf / (batched_ms / 1e3), "unit": METRIC,
                            "ms": batched_ms, "note": "every window recomputed by the "
                            "general persistent batched kernel (CP_VIDEO_SLIDING=0)"},
        "plain_kernel": {"value": mpxf / (plain_ms / 1e3), "unit": METRIC, "ms": plain_ms,
                         "note": "one single-stack launch per window"},
        "batched_over_plain": plain_ms / ms,
        "roofline": {"bound": "hbm", "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": ach / peaks["hbm_gbs"], "bytes": unique,
                     "note": "unique bytes: pool read once + composite and mask per window"},
        "e2e": {"value": mpxf / e2e_s, "unit": METRIC, "h2d_bytes_per_step": n_pool * fb,
                "d2h_bytes_per_step": 2 * nwin * fb},
        "data": "synthetic (seeded drift + sine-path disk, generated on the device)"}


def run_video(args):
    ctx, lib, _abi, local = _ctx_and_lib()
    with ClockSampler(local) as clk:
        res = video_workload(args, ctx, lib, _abi, local)
    res["clocks"] = clk.summary()
    print(json.dumps(res), flush=True)


SERVE_RES = [(320, 240), (1280, 720), (1920, 1080), (4000, 3000)]


def serve_workload(args, ctx, lib, _abi, local):
    """Mixed jobs through the continuous-batching server: 512 jobs, N ~ U{8..128},
    resolution ~ U{320x240, 1280x720, 1920x1080, 4000x3000}, outlier mode ~ U{extreme,
    average, first, last}, Poisson arrivals, 60 GB HBM budget. Job frames are drawn (by the
    job's seed) from 16 pinned host frames per resolution (generated on the device and read
    back), so the host side stays small; every job still uploads its own N frames. Returns a
    dict."""
    import numpy as np
    from chrono_photo_gb300 import example_data, make_params
    from chrono_photo_gb300.api import Server
    jobs = example_data.job_specs(seed=4, count=args.jobs)
    pool_n = 16
    pools = {}
    for (w, h) in SERVE_RES:
        ptr, arr = _pinned(ctx, lib, pool_n * w * h * C)
        arr = arr.reshape(pool_n, h, w, C)
        gen = example_data.stack_device(pool_n, w, h, sigma=3, n_disks=2, rmin=h / 40,
                                        rmax=h / 20, seed=4 + w)
        ctx.check(lib.cp_memcpy_d2h(ctx.handle, ptr, gen.data_ptr(), arr.nbytes, None))
        del gen
        pools[(w, h)] = (ptr, arr)
    mpx_job = [j["n"] * j["w"] * j["h"] / 1e6 for j in jobs]

    def frames_of(j):
        arr = pools[(j["w"], j["h"])][1]
        return [arr[(j["seed"] + i) % pool_n] for i in range(j["n"])]

    # kernel only: the same jobs with device-resident frames, 64 per batched launch
    dpool = {}
    dev_allocs = []
    for key, (ptr, arr) in pools.items():
        d = ctx.alloc(arr.nbytes)
        dev_allocs.append(d)
        ctx.check(lib.cp_memcpy_h2d(ctx.handle, d, ptr, arr.nbytes, None))
        dpool[key] = d
    keep = []
    params = [make_params(keep=keep, mode="outlier", threshold="abs/0.05/0.2",
                          outlier=j["outlier"], background="first", seed=j["seed"]) for j in jobs]
    batches = []
    for b0 in range(0, len(jobs), 64):
        bj = list(range(b0, min(b0 + 64, len(jobs))))
        stacks = (_abi.Stack * len(bj))()
        outs = (ct.c_void_p * len(bj))()
        for k, ji in enumerate(bj):
            j = jobs[ji]
            fb = j["w"] * j["h"] * C
            ptrs = (ct.c_void_p * j["n"])(*[dpool[(j["w"], j["h"])] + ((j["seed"] + i) % pool_n) * fb
                                            for i in range(j["n"])])
            keep.append(ptrs)
            stacks[k] = _abi.Stack(n=j["n"], width=j["w"], height=j["h"], channels=C,
                                   frames=ct.cast(ptrs, ct.POINTER(ct.c_void_p)))
            outs[k] = ctx.alloc(fb)
            dev_allocs.append(outs[k])
        prm = (_abi.Params * len(bj))(*[params[ji] for ji in bj])
        batches.append((stacks, prm, outs, len(bj)))

    def kernel_all():
        for stacks, prm, outs, nb in batches:
            ctx.check(lib.cp_composite_batch_device(ctx.handle, stacks, prm, nb, outs, None,
                                                    None, None), "batch")
    kernel_ms = _time_device(ctx, lib, kernel_all, max(1, args.steps // 50), 1)
    # the plain kernel on the same jobs: one single-stack launch per job
    flat = []
    for stacks, prm, outs, nb in batches:
        for k in range(nb):
            flat.append((stacks[k], prm[k], outs[k]))

    def plain_all():
        for st, pr, o in flat:
            ctx.check(lib.cp_composite_device(ctx.handle, ct.byref(st), ct.byref(pr), o, None,
                                              None, None, None), "plain")
    plain_ms = _time_device(ctx, lib, plain_all, max(1, args.steps // 50), 1)
    # where batching pays: the small (320x240) jobs alone, batched in one launch vs one each
    small = [i for i, j in enumerate(jobs) if j["w"] * j["h"] <= 320 * 240]
    s_st = (_abi.Stack * len(small))(*[flat[i][0] for i in small])
    s_pr = (_abi.Params * len(small))(*[flat[i][1] for i in small])
    s_out = (ct.c_void_p * len(small))(*[flat[i][2] for i in small])
    small_mpxf = sum(mpx_job[i] for i in small)

    def small_batched():
        ctx.check(lib.cp_composite_batch_device(ctx.handle, s_st, s_pr, len(small), s_out, None,
                                                None, None), "small batch")

    def small_plain():
        for i in small:
            st, pr, o = flat[i]
            ctx.check(lib.cp_composite_device(ctx.handle, ct.byref(st), ct.byref(pr), o, None,
                                              None, None, None), "small plain")
    small_b_ms = _time_device(ctx, lib, small_batched, 20, 2) if small else 0.0
    small_p_ms = _time_device(ctx, lib, small_plain, 20, 2) if small else 0.0
    total_mpxf = sum(mpx_job)
    kernel_rate = total_mpxf / (kernel_ms / 1e3)
    # served: Poisson arrivals, mean inter-arrival = 0.5 x the mean kernel-only job time
    mean_gap = 0.5 * (kernel_ms / 1e3) / len(jobs)
    rng = np.random.default_rng(4)
    gaps = rng.exponential(mean_gap, size=len(jobs))
    with Server(ctx, hbm_budget=60 << 30, max_inflight=8) as srv:
        warm = srv.submit(frames_of(jobs[0]), params=params[0])
        srv.wait(warm)
        ids = []
        t0 = time.perf_counter()
        t_next = t0
        for j, g, prm in zip(jobs, gaps, params):
            t_next += g
            while time.perf_counter() < t_next:
                pass
            ids.append(srv.submit(frames_of(j), params=prm))
        res = [srv.wait(i) for i in ids]
        wall = max(r["done_s"] for r in res) - min(r["submit_s"] for r in res)
    lat = np.array([r["done_s"] - r["submit_s"] for r in res]) * 1e3
    bad = sum(1 for r in res if r["status"] != 0)
    bad_status = {}
    for r in res:
        if r["status"] != 0:
            bad_status[str(r["status"])] = bad_status.get(str(r["status"]), 0) + 1
    h2d = sum(j["n"] * j["w"] * j["h"] * C for j in jobs)
    for d in dev_allocs:
        ctx.free(d)
    return {
        "workload": "serve", "metric": METRIC, "value": total_mpxf / wall, "unit": METRIC,
        "jobs": len(jobs), "failed": bad, "failed_status": bad_status, "wall_s": wall,
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "max": float(lat.max())},
        "arrival_mean_gap_ms": mean_gap * 1e3,
        "kernel_only": {"value": kernel_rate, "unit": METRIC, "ms_all_jobs": kernel_ms},
        "plain_kernel": {"value": total_mpxf / (plain_ms / 1e3), "unit": METRIC,
                         "ms_all_jobs": plain_ms, "note": "one single-stack launch per job"},
        "batched_over_plain": plain_ms / kernel_ms,
        "small_jobs": {"jobs": len(small), "batched_ms": small_b_ms, "plain_ms": small_p_ms,
                       "batched": small_mpxf / (small_b_ms / 1e3) if small_b_ms else None,
                       "plain": small_mpxf / (small_p_ms / 1e3) if small_p_ms else None,
                       "batched_over_plain": small_p_ms / small_b_ms if small_b_ms else None,
                       "note": "the 320x240 jobs: one batched launch vs one launch per job"},
        "e2e": {"value": total_mpxf / wall, "unit": METRIC, "h2d_bytes_total": h2d,
                "d2h_bytes_total": 2 * sum(j["w"] * j["h"] * C for j in jobs)},
        "dtype": "u8", "data": "synthetic (seeded; frames drawn from 16 per resolution)",
        "config": {"budget_gb": 60, "max_inflight": 8, "settings": "abs/0.05/0.2, background first"}}


def run_serve(args):
    ctx, lib, _abi, local = _ctx_and_lib()
    with ClockSampler(local) as clk:
        res = serve_workload(args, ctx, lib, _abi, local)
    res["clocks"] = clk.summary()
    print(json.dumps(res), flush=True)


def run_shake(args):
    """Camera shake on 100 frames of 6000x4000: the offset search (4 anchors, radius 32,
    search radius 20) and the composite of the cropped stack (abs/0.05/0.2 extreme)."""
    import numpy as np
    from chrono_photo_gb300 import example_data, make_params
    ctx, lib, _abi, local = _ctx_and_lib()
    n, w, h, r, s = 100, 6000, 4000, 32, 20
    frames, shifts = example_data.shake_stack_device(n, w, h, 12, seed=5)
    fb = w * h * C
    base = frames.data_ptr()
    ptrs = (ct.c_void_p * n)(*[base + i * fb for i in range(n)])
    anchors = np.array([[1000, 800], [5000, 800], [1000, 3200], [5000, 3200]], np.int32)
    offs = np.zeros((n, 2), np.int32)

    def analyze():
        ctx.check(lib.cp_shake_analyze_device(ctx.handle, ptrs, n, w, h, C,
                                              anchors.ctypes.data_as(_abi.I32P), len(anchors), r,
                                              s, offs.ctypes.data_as(_abi.I32P), None), "shake")
    with ClockSampler(local) as clk:
        shake_ms = _time_device(ctx, lib, analyze, max(1, args.steps // 20), 2)
    expect = shifts[0] - shifts
    offsets_ok = bool((offs == expect).all())
    has_crop = ct.c_int32()
    crops = np.zeros((n, 4), np.int32)   # per frame (x, y, width, height)
    ctx.check(lib.cp_crop_create(offs.ctypes.data_as(_abi.I32P), n, w, h, ct.byref(has_crop),
                                 crops.ctypes.data_as(_abi.I32P)), "crop")
    origins = np.ascontiguousarray(crops[:, :2])
    cw, ch = (int(crops[0, 2]), int(crops[0, 3])) if has_crop.value else (w, h)
    keep = []
    p = make_params(keep=keep, mode="outlier", threshold="abs/0.05/0.2", outlier="extreme",
                    background="first")
    stack = _abi.Stack(n=n, width=cw, height=ch, channels=C,
                       frames=ct.cast(ptrs, ct.POINTER(ct.c_void_p)),
                       crop=origins.ctypes.data_as(_abi.I32P) if has_crop.value else None,
                       src_width=w, src_height=h)
    out = ctx.alloc(cw * ch * C)
    blend = ctx.alloc(cw * ch * C)

    def comp():
        ctx.check(lib.cp_composite_device(ctx.handle, ct.byref(stack), ct.byref(p), out, blend,
                                          None, None, None), "composite")
    comp_ms = _time_device(ctx, lib, comp, max(1, args.steps // 20), 2)
    terms = (n - 1) * len(anchors) * (2 * s + 1) ** 2 * (2 * r + 1) ** 2 * C
    mpxf = n * cw * ch / 1e6
    peaks, kind = measured_peaks()
    algo = n * cw * ch * C + 2 * cw * ch * C
    print(json.dumps({
        "workload": "shake", "metric": METRIC, "value": mpxf / (comp_ms / 1e3), "unit": METRIC,
        "composite_ms": comp_ms, "crop": [cw, ch], "has_crop": int(has_crop.value),
        "shake": {"ms": shake_ms, "G_ssd_terms_per_s": terms / (shake_ms / 1e3) / 1e9,
                  "offsets_match_translation": offsets_ok},
        "roofline": {"bound": "hbm", "achieved": algo / (comp_ms / 1e3) / 1e9,
                     "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": algo / (comp_ms / 1e3) / 1e9 / peaks["hbm_gbs"]},
        "dtype": "u8", "data": "synthetic (seeded, generated on the device)",
        "config": {"frames": n, "width": w, "height": h, "anchors": anchors.tolist(),
                   "anchor_radius": r, "search_radius": s},
        "clocks": clk.summary()}), flush=True)


def run_ingest(args):
    """Frame ingest: the HD stack (64 x 1920x1080 RGB) as files -> composite, the work the
    reference does per frame inside its slicing loop (src/streams.rs:63-70).

    value: JPEG frames/s. The frames written as baseline JPEG at quality 95 (the quality of
    the reference's example frames, src/util/create_example_data.rs:56), read on host
    threads and decoded by nvJPEG (the GPU's JPEG engines) straight into device memory by
    cp_load_jpeg_device. Also: files -> composite (decode, then cp_composite_device,
    abs/0.05/0.2 average, and the composite and blend mask copied back), files -> files (the
    composite and mask written as JPEG by cp_save_jpeg, src/main.rs:542-556), the decode to
    host memory (cp_load_jpeg), and the same with PNG files (cp_load_png on all host
    threads, then cp_composite from pinned memory; outputs by cp_save_png)."""
    import shutil
    import tempfile
    import numpy as np
    from chrono_photo_gb300 import example_data, make_params
    ctx, lib, _abi, local = _ctx_and_lib()
    fb = W * H * C
    frames = example_data.hd_stack(seed=2)
    tmp = tempfile.mkdtemp(prefix="cp_ingest_")
    steps = max(1, min(args.steps, 5))
    threads = os.cpu_count() or 1
    keep = []
    p = make_params(keep=keep, mode="outlier", threshold="abs/0.05/0.2", outlier="average",
                    background="first")
    try:
        # ---- JPEG ---------------------------------------------------------------------------
        t0 = time.perf_counter()
        jpaths = []
        for i in range(N_FRAMES):
            jp = os.path.join(tmp, "image-%05d.jpg" % i)
            ctx.check(lib.cp_save_jpeg(ctx.handle, jp.encode(), frames[i].ctypes.data, W, H, C,
                                       95, 0, 0), "cp_save_jpeg")
            jpaths.append(jp)
        t_jenc_frames = time.perf_counter() - t0
        jbytes = sum(os.path.getsize(q) for q in jpaths)
        jarr = (ct.c_char_p * N_FRAMES)(*[q.encode() for q in jpaths])
        stride = (fb + 15) // 16 * 16
        dev = ctx.alloc(N_FRAMES * stride + 16)
        out_d, blend_d = ctx.alloc(fb), ctx.alloc(fb)
        optr, _ = _pinned(ctx, lib, 2 * fb)
        stack = _abi.Stack(n=N_FRAMES, width=W, height=H, channels=C, base=dev,
                           frame_stride=stride)

        def jdecode():
            ctx.check(lib.cp_load_jpeg_device(ctx.handle, jarr, N_FRAMES, threads, dev, stride,
                                              W, H, C), "cp_load_jpeg_device")

        def jcomposite():
            ctx.check(lib.cp_composite_device(ctx.handle, ct.byref(stack), ct.byref(p), out_d,
                                              blend_d, None, None, None), "cp_composite_device")
            ctx.check(lib.cp_memcpy_d2h(ctx.handle, optr, out_d, fb, None), "d2h")
            ctx.check(lib.cp_memcpy_d2h(ctx.handle, optr + fb, blend_d, fb, None), "d2h")

        jdecode()
        jcomposite()
        # decoded frames against the sources (JPEG is lossy: the quantisation error)
        raw = ctx.download(dev, (stride,))[:fb].reshape(H, W, C)
        jerr = np.abs(raw.astype(np.int16) - frames[0].astype(np.int16))
        t_dec = t_comp = 0.0
        with ClockSampler(local) as clk:
            for _ in range(steps):
                t0 = time.perf_counter()
                jdecode()
                t1 = time.perf_counter()
                jcomposite()
                t2 = time.perf_counter()
                t_dec += t1 - t0
                t_comp += t2 - t1
        t_dec /= steps
        t_comp /= steps
        t0 = time.perf_counter()
        for k, name in enumerate(("composite.jpg", "blend.jpg")):
            ctx.check(lib.cp_save_jpeg(ctx.handle, os.path.join(tmp, name).encode(),
                                       optr + k * fb, W, H, C, 95, 0, 0), "cp_save_jpeg")
        t_jenc = time.perf_counter() - t0
        hptr, host = _pinned(ctx, lib, N_FRAMES * fb)
        ctx.check(lib.cp_load_jpeg(ctx.handle, jarr, N_FRAMES, threads, hptr, fb, W, H, C))
        t0 = time.perf_counter()
        for _ in range(steps):
            ctx.check(lib.cp_load_jpeg(ctx.handle, jarr, N_FRAMES, threads, hptr, fb, W, H, C),
                      "cp_load_jpeg")
        t_jhost = (time.perf_counter() - t0) / steps
        for q in (dev, out_d, blend_d):
            ctx.free(q)

        # ---- PNG ----------------------------------------------------------------------------
        paths = example_data.write_pngs(frames, tmp, level=6, threads=threads)
        file_bytes = sum(os.path.getsize(q) for q in paths)
        host = host.reshape(N_FRAMES, H, W, C)
        arr = (ct.c_char_p * N_FRAMES)(*[q.encode() for q in paths])

        def decode(nthreads, n=N_FRAMES):
            ctx.check(lib.cp_load_png(ctx.handle, arr, n, nthreads, hptr, fb, W, H, C),
                      "cp_load_png")
        decode(threads)
        exact = bool(np.array_equal(host, frames))
        hstack = _abi.Stack(n=N_FRAMES, width=W, height=H, channels=C, base=hptr,
                            frame_stride=fb)

        def composite():
            ctx.check(lib.cp_composite(ctx.handle, ct.byref(hstack), ct.byref(p), optr,
                                       optr + fb, None, None), "cp_composite")
        composite()
        p_dec = p_comp = 0.0
        for _ in range(steps):
            t0 = time.perf_counter()
            decode(threads)
            t1 = time.perf_counter()
            composite()
            t2 = time.perf_counter()
            p_dec += t1 - t0
            p_comp += t2 - t1
        p_dec /= steps
        p_comp /= steps
        n1 = 8
        decode(1, n1)
        t0 = time.perf_counter()
        decode(1, n1)
        t_one = (time.perf_counter() - t0) / n1
        t0 = time.perf_counter()
        for k, name in enumerate(("composite.png", "blend.png")):
            ctx.check(lib.cp_save_png(ctx.handle, os.path.join(tmp, name).encode(),
                                      optr + k * fb, W, H, C, -1, 0), "cp_save_png")
        t_enc = time.perf_counter() - t0
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    print(json.dumps({
        "workload": "ingest", "metric": "frames/s", "value": N_FRAMES / t_dec, "unit": "frames/s",
        "format": "jpeg", "threads": threads,
        "decode_ms_per_stack": 1e3 * t_dec, "decoded_MB_per_s": N_FRAMES * fb / t_dec / 1e6,
        "decoder": "nvJPEG batched decode (JPEG engines), file reads on host threads, frames "
                   "written to device memory",
        "decode_error_vs_source": {"max": int(jerr.max()), "mean": float(jerr.mean()),
                                   "note": "frame 0; the JPEG quantisation error at quality 95"},
        "files_to_composite": {"value": MPXF_PER_COMPOSITE / (t_dec + t_comp), "unit": METRIC,
                               "decode_ms": 1e3 * t_dec, "composite_ms": 1e3 * t_comp,
                               "note": "cp_load_jpeg_device, then cp_composite_device and the "
                                       "composite and mask copied to pinned memory"},
        "encode_ms": 1e3 * t_jenc,
        "files_to_files": {"value": MPXF_PER_COMPOSITE / (t_dec + t_comp + t_jenc),
                           "unit": METRIC,
                           "note": "the above plus cp_save_jpeg of composite and mask at "
                                   "quality 95 (each on all host threads), in sequence"},
        "decode_to_host": {"value": N_FRAMES / t_jhost, "unit": "frames/s",
                           "note": "cp_load_jpeg: decoded on the device, copied to pinned "
                                   "host memory"},
        "frame_encode_ms": 1e3 * t_jenc_frames / N_FRAMES,
        "png": {"value": N_FRAMES / p_dec, "unit": "frames/s", "decoded_exact": exact,
                "decode_ms_per_stack": 1e3 * p_dec,
                "one_thread_frames_per_s": 1.0 / t_one,
                "files_to_composite": {"value": MPXF_PER_COMPOSITE / (p_dec + p_comp),
                                       "unit": METRIC, "decode_ms": 1e3 * p_dec,
                                       "composite_e2e_ms": 1e3 * p_comp},
                "encode_ms": 1e3 * t_enc,
                "files_to_files": {"value": MPXF_PER_COMPOSITE / (p_dec + p_comp + t_enc),
                                   "unit": METRIC},
                "note": "cp_load_png on all host threads into pinned memory, then cp_composite "
                        "(H2D, kernel, D2H); outputs by cp_save_png",
                "config": {"png": "8-bit RGB, Paeth filter, zlib level 6",
                           "compressed_MB_per_frame": file_bytes / N_FRAMES / 1e6}},
        "steps": steps, "dtype": "u8", "data": "synthetic (seeded HD stack written as JPEG "
                                               "and PNG)",
        "config": {"frames": N_FRAMES, "width": W, "height": H, "channels": C,
                   "jpeg": "baseline, 4:4:4, quality 95, restart interval of one MCU row",
                   "compressed_MB_per_frame": jbytes / N_FRAMES / 1e6},
        "clocks": clk.summary()}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="hd",
                    choices=["hd", "video", "serve", "shake", "ingest"],
                    help="hd (default): the headline line; the others print their own lines")
    ap.add_argument("--jobs", type=int, default=512, help="serve: number of jobs")
    ap.add_argument("--video-frames", type=int, default=300,
                    help="video: frames in the resident pool (windows of 32 slide over it)")
    ap.add_argument("--video-size", default="1920x1080", help="video: frame size WxH")
    ap.add_argument("--no-batched", action="store_true",
                    help="hd: leave out the video and serve sub-objects of the headline line")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, _ = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    try:
        if args.impl == "reference":
            run_reference(args)
        elif args.workload == "video":
            run_video(args)
        elif args.workload == "serve":
            run_serve(args)
        elif args.workload == "shake":
            run_shake(args)
        elif args.workload == "ingest":
            run_ingest(args)
        else:
            run_gpu(args)
    finally:
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
