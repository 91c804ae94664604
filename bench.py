"""Benchmark: vectorial RS (VRS) propagation of 2048 x 2048 fields on one GB300.

Workload: 2048^2 grid over a 4 mm window (space(2 mm, 2048)), 633 nm; a
radially polarised source (Ex = x/w e^{-rho^2/w^2}, Ey = y/w e^{-rho^2/w^2},
w = 1 mm) behind a per-pixel LCD retarder (eta, theta uniform in [0, 2 pi))
and a linear polarizer at one random angle; Ez derived; z drawn from
{1, 5, 10, 20} cm.  One step propagates a batch of B fields (default 8).

Arms:
  default            libxlgb kernels; `value` = fields/s with inputs resident in
                     HBM; `e2e` = the same through the public API with pinned
                     host buffers copied in and the propagated fields copied out.
  --impl reference   the FP64 CPU restatement of the reference algorithm (the
                     reference itself is pure jax, which is not installable on
                     these machines) on all host cores, one field per step.

Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 2048
HALF_WIDTH = 2000.0          # um, space(2 mm, 2048)
WAVELENGTH = 0.633           # um
WAIST = 1000.0               # um
Z_SET = (1e4, 5e4, 1e5, 2e5)  # um
METRIC = "2048² VRS fields/s"
SERVE_MAX_LAUNCH_MS = 4.0   # the serving tuner's latency bound per batched launch
E2E_STREAMS = 3   # end-to-end pipeline depth (2: 1547, 3: 1677, 4: 1651 fields/s measured)
WORKLOAD = ("VRS 2048x2048 complex64, 4 mm window, 633 nm, radially polarised source w=1 mm, "
            "per-pixel LCD (eta, theta) + linear polarizer fused, Ez derived, z in {1,5,10,20} cm")


def make_inputs(batch, seed=1000):
    """Seeded synthetic inputs for `batch` fields (float64 host arrays)."""
    x = np.linspace(-HALF_WIDTH, HALF_WIDTH, N)
    X, Y = np.meshgrid(x, x)
    g = np.exp(-(X ** 2 + Y ** 2) / WAIST ** 2)
    Ex = (X / WAIST) * g
    Ey = (Y / WAIST) * g
    rng = np.random.default_rng(seed)
    eta = rng.uniform(0, 2 * np.pi, (batch, N, N)).astype(np.float32)
    theta = rng.uniform(0, 2 * np.pi, (batch, N, N)).astype(np.float32)
    alpha = float(rng.uniform(0, np.pi))
    zs = [Z_SET[i % len(Z_SET)] for i in range(batch)]
    return x, Ex, Ey, eta, theta, alpha, zs


class ClockSampler:
    """nvidia-smi clock / throttle sampling (every 100 ms) around the timed
    region; summary() keeps the samples taken between mark_start() and
    mark_end() (the nearest ones if the region is shorter than one interval)."""

    QUERY = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.3)
        except (OSError, ValueError):
            self.proc = None
        return self

    def mark_start(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    @staticmethod
    def _epoch(stamp):
        import datetime
        for fmt in ("%Y/%m/%d %H:%M:%S.%f", "%Y/%m/%d %H:%M:%S"):
            try:
                return datetime.datetime.strptime(stamp.strip(), fmt).timestamp()
            except ValueError:
                continue
        return None

    def summary(self):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        samples = []
        for ln in getattr(self, "lines", []):
            f = [v.strip() for v in ln.split(",")]
            if len(f) < 10:
                continue
            try:
                samples.append((self._epoch(f[0]), float(f[2]), float(f[3]), f[6:10]))
            except ValueError:
                continue
        inside = [smp for smp in samples if smp[0] is not None and self.t0 is not None and
                  self.t0 <= smp[0] <= self.t1]
        if not inside and samples and self.t0 is not None:   # region shorter than the interval
            mid = 0.5 * (self.t0 + self.t1)
            inside = sorted((smp for smp in samples if smp[0] is not None), key=lambda smp: abs(smp[0] - mid))[:2]
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        reasons = set()
        for smp in inside:
            for nm, v in zip(names, smp[3]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(smp[1] for smp in inside), "sm_max_mhz": inside[-1][2],
                "reasons": sorted(reasons), "samples": len(inside)}


# DRAM bytes (read + write) per 2048^2 VRS field of each pass, measured by
# ncu (dram__bytes_read.sum + dram__bytes_write.sum, one replay pass).  The
# column pass's figure is from a capture of this benchmark's own 8-field
# launch (4 distances, so pairs of fields share a transfer spectrum) with
# NCU_TRAFFIC_COMMAND below; the row passes' from a batch-2 capture (--batch 2)
# scaled per field (every field is an independent slice of those launches).
# The column-pass variants move the same bytes (within 2 % at batch 2).
NCU_TRAFFIC_PER_FIELD = {"rs_rows_fwd": 276.15e6, "rs_cols_conv": 478.88e6, "rs_rows_inv": 283.60e6}
# Warp instructions per 2048^2 VRS field of the column pass, by kernel variant
# (ncu smsp__inst_executed.sum of one launch of the batch-2 case, halved; the
# instruction stream does not depend on the batch): NCU_INST_COMMAND below
# with V = 8 and 10.  The pass's issue ceiling is 4 warp instructions per
# cycle per SM (one per scheduler).
NCU_COL_INST_PER_FIELD = {8: 303.87e6 / 2, 10: 314.38e6 / 2}
NCU_INST_COMMAND = ("ncu --metrics smsp__inst_executed.sum --clock-control none -k regex:rs_cols -s 4 -c 1 "
                    "python bench.py --steps 2 --warmup 3 --batch 2 --no-cpu-baseline --no-fwd-bwd --no-serving "
                    "--no-parity --col-variant V")
NCU_TRAFFIC_COMMAND = ("ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum "
                       "--clock-control none -k regex:rs_cols -s 1 -c 1 python bench.py --steps 10 --warmup 3 "
                       "--no-cpu-baseline --no-fwd-bwd --no-serving")


def host_link_rates(dev, nbytes=256 << 20, reps=2, trials=5):
    """Copy rates (GB/s) between pinned host memory and the device: each
    direction alone and both at once on two streams; the best of ``trials``
    timings of ``reps`` copies each (the link is shared with the rest of the
    machine, so a single timing can catch a slow spell)."""
    import torch
    d = torch.empty(nbytes // 8, dtype=torch.complex64, device=dev)
    d2 = torch.empty_like(d)
    h = torch.empty(nbytes // 8, dtype=torch.complex64).pin_memory()
    h2 = torch.empty_like(h).pin_memory()
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def rate(fn, moved):
        fn()
        torch.cuda.synchronize()
        best = 0.0
        for _ in range(trials):
            t0 = time.perf_counter()
            for _ in range(reps):
                fn()
            torch.cuda.synchronize()
            best = max(best, moved * reps / (time.perf_counter() - t0) / 1e9)
        return best

    def both():
        with torch.cuda.stream(s1):
            h.copy_(d, non_blocking=True)
        with torch.cuda.stream(s2):
            d2.copy_(h2, non_blocking=True)
        s1.synchronize()
        s2.synchronize()

    return {"d2h_gbs": rate(lambda: h.copy_(d, non_blocking=True), nbytes),
            "h2d_gbs": rate(lambda: d.copy_(h, non_blocking=True), nbytes),
            "duplex_gbs": rate(both, 2 * nbytes)}


def cpu_vrs_field(ref, x, Ex, Ey, eta, theta, alpha, z):
    """One field of the workload through the FP64 CPU restatement."""
    ax, ay = ref.lcd(Ex, Ey, eta.astype(np.float64), theta.astype(np.float64))
    ax, ay = ref.linear_polarizer(ax, ay, alpha)
    return ref.vrs_propagate(ax, ay, x, x, WAVELENGTH, z)


def run_reference(args, budget_s=150.0):
    """The reference algorithm on the host cores, one field per step.  A CPU
    field takes over a second, so the timed steps are capped at about
    `budget_s` of work (at least 5; about 100 fields at 1.4 s each, the
    sample size planned for the 2048^2 propagators); the line reports how
    many were timed."""
    from oracle import xlumina_ref as ref
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:      # under torchrun rank 0 alone runs the CPU reference
        return
    x, Ex, Ey, eta, theta, alpha, zs = make_inputs(1)
    t_w = time.perf_counter()
    for _ in range(args.warmup):
        cpu_vrs_field(ref, x, Ex, Ey, eta[0], theta[0], alpha, zs[0])
    per_field = (time.perf_counter() - t_w) / max(1, args.warmup)
    steps = max(5, min(args.steps, int(budget_s / max(per_field, 1e-3))))
    times = []
    t0 = time.perf_counter()
    for i in range(steps):
        ts = time.perf_counter()
        cpu_vrs_field(ref, x, Ex, Ey, eta[0], theta[0], alpha, Z_SET[i % len(Z_SET)])
        times.append(time.perf_counter() - ts)
    dt = time.perf_counter() - t0
    v = steps / dt
    cores = ref.WORKERS
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "fields/s", "n_gpus": args.gpus,
            "steps": steps, "steps_requested": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic", "config": {"workload": WORKLOAD, "batch": 1},
            "ms_per_field_p50": 1e3 * float(np.percentile(times, 50)),
            "ms_per_field_p99": 1e3 * float(np.percentile(times, 99)),
            "cpu_baseline": {"value": v, "unit": "fields/s", "cores": cores, "kind": "port",
                             "sample": f"{steps} fields, one per step (capped at about {budget_s:.0f} s of work), "
                                       f"scipy.fft with {cores} workers"},
            "e2e": {"value": v, "unit": "fields/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def cpu_baseline_sample(seconds=20.0):
    from oracle import xlumina_ref as ref
    x, Ex, Ey, eta, theta, alpha, zs = make_inputs(1)
    cpu_vrs_field(ref, x, Ex, Ey, eta[0], theta[0], alpha, zs[0])  # warm-up (FFT plans, page-in)
    n = 0
    t0 = time.perf_counter()
    while True:
        cpu_vrs_field(ref, x, Ex, Ey, eta[0], theta[0], alpha, Z_SET[n % len(Z_SET)])
        n += 1
        dt = time.perf_counter() - t0
        if dt > seconds or n >= 8:
            break
    return {"value": n / dt, "unit": "fields/s", "cores": ref.WORKERS, "kind": "port",
            "sample": f"{n} fields of the same workload (FP64 numpy/scipy restatement, "
                      f"scipy.fft workers={ref.WORKERS})"}


# ---- replicas: under torchrun every rank runs the whole workload on its own
# GPU (fields share nothing, so there is no data-path collective); timing is
# bracketed by barriers and the whole-job rate is the units of all ranks over
# the slowest rank's time.

def dist_context():
    """(rank, world size, local rank) of this process; initialises the process
    group of a torchrun launch (NCCL with GPUs, gloo without)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0
    import torch
    import torch.distributed as dist
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if not dist.is_initialized():
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
    return dist.get_rank(), dist.get_world_size(), local


def replica_barrier():
    import torch
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        if torch.cuda.is_available():
            torch.cuda.synchronize()
        dist.barrier()


def reduce_replicas(seconds, units):
    """(the slowest rank's seconds, the units of all ranks)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(seconds), float(units)
    dev = torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else torch.device("cpu")
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    u = torch.tensor([float(units)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def run_gpu(args):
    import torch

    from xlumina_gb300 import engine
    from xlumina_gb300 import optical_elements as oe
    from xlumina_gb300 import vectorized_optics as vo

    rank, world, local = dist_context()
    if world != args.gpus:
        print(json.dumps({"error": f"--gpus {args.gpus} but {world} process(es): launch one process per GPU"}))
        sys.exit(2)
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    B = args.batch
    x, Ex, Ey, eta, theta, alpha, zs = make_inputs(B)
    Ex_d = torch.as_tensor(Ex, dtype=torch.complex64, device=dev).expand(B, N, N).contiguous()
    Ey_d = torch.as_tensor(Ey, dtype=torch.complex64, device=dev).expand(B, N, N).contiguous()
    eta_d = torch.as_tensor(eta, device=dev)
    theta_d = torch.as_tensor(theta, device=dev)
    pre = [engine.op_lcd(eta_d, theta_d), engine.op_lp(alpha)]
    call = engine.RsCall([Ex_d, Ey_d], x, x, WAVELENGTH, zs, vector=True, pre=pre)
    stream = torch.cuda.current_stream()

    # warm-up (transfer spectra are built here, once per distinct z)
    for _ in range(args.warmup):
        for s in range(3):
            call.stage(s)
    torch.cuda.synchronize()
    # the column pass's kernel variant, chosen by measurement on this launch
    from xlumina_gb300 import _lib
    from xlumina_gb300.autotune import VariantTuner, cuda_event_timer
    col_logp = engine.rs_logq(N, N) + 1
    if args.col_variant is None:
        tuned = VariantTuner(repeats=5).best_variant(_lib.XL_PASS_RS_COLS, col_logp,
                                                      cuda_event_timer(lambda: call.stage(1)), force=True)
    else:   # a fixed variant (profiling one kernel)
        _lib.check(engine.lib().xl_set_kernel_variant(_lib.XL_PASS_RS_COLS, col_logp, args.col_variant))
        tuned = {"variant": args.col_variant, "ms": {}}
    for s in range(3):
        call.stage(s)
    torch.cuda.synchronize()

    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        replica_barrier()
        torch.cuda.synchronize()
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        clk.mark_start()
        t_start.record(stream)
        for k in range(args.steps):
            ev[k][0].record(stream)
            for s in range(3):
                call.stage(s)
                ev[k][s + 1].record(stream)
        t_end.record(stream)
        torch.cuda.synchronize()
        replica_barrier()
        clk.mark_end()
    total_s, fields = reduce_replicas(t_start.elapsed_time(t_end) / 1e3, B * args.steps)
    step_ms = np.asarray([ev[k][0].elapsed_time(ev[k][3]) for k in range(args.steps)])
    # the timed output against the FP64 oracle: fields 0 (z = 1 cm) and 3 (z = 20 cm)
    # of the last timed step (rank 0)
    parity = None
    if rank == 0 and not args.no_parity:
        from oracle import xlumina_ref as ref
        parity = {"what": "fields of the last timed step against the FP64 oracle (complex64 Ex, Ey, Ez)"}
        for b in (0, 3):
            exp = cpu_vrs_field(ref, x, Ex, Ey, eta[b], theta[b], alpha, zs[b])
            errs = [_rel_l2(call.outs[c][b].cpu().numpy(), exp[c]) for c in range(3)]
            parity[f"field{b}_z{zs[b] / 1e4:g}cm"] = dict(zip(("Ex", "Ey", "Ez"), errs))
        parity["max"] = max(max(v.values()) for k, v in parity.items() if k.startswith("field"))
    total_ms = total_s * 1e3
    stage_ms = [sum(ev[k][s].elapsed_time(ev[k][s + 1]) for k in range(args.steps)) / args.steps
                for s in range(3)]
    value = fields / total_s

    # roofline: algorithmic bytes per launch (B fields), per stage
    n2 = N * N
    alg = [72 * n2 * B, 128 * n2 * B, 72 * n2 * B]
    names = ["rs_rows_fwd", "rs_cols_conv", "rs_rows_inv"]
    dom = int(np.argmax(stage_ms))
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    achieved = alg[dom] / (stage_ms[dom] / 1e3) / 1e9
    pipe_gbs = sum(alg) / (sum(stage_ms) / 1e3) / 1e9

    # plain path: one public-API call per field, no batching
    src = vo.VectorizedLight(x, x, WAVELENGTH)
    src.Ex = Ex_d[0]
    src.Ey = Ey_d[0]
    for _ in range(2):
        oe.linear_polarizer(oe.LCD(src, eta_d[0], theta_d[0]), alpha).VRS_propagation(zs[0])
    torch.cuda.synchronize()
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    nplain = 2 * B
    for i in range(nplain):
        light = oe.linear_polarizer(oe.LCD(src, eta_d[i % B], theta_d[i % B]), alpha)
        out, _ = light.VRS_propagation(zs[i % B])
    p1.record(stream)
    torch.cuda.synchronize()
    plain = nplain / (p0.elapsed_time(p1) / 1e3)

    # end to end through the public API: pinned host buffers in, propagated fields out.
    # A step's inputs are the source (one Ex, Ey plane, shared by the batch: the
    # workload is one source through B random LCD masks) and the B mask planes;
    # its result is the B propagated fields (Ex, Ey, Ez).  Steps rotate over
    # E2E_STREAMS streams with their own pinned buffers, so the copies of one
    # step overlap the kernels and copies of the others.
    streams = [torch.cuda.Stream() for _ in range(E2E_STREAMS)]
    hosts = []
    for _ in streams:
        hosts.append(dict(
            Ex=torch.as_tensor(Ex.astype(np.complex64)[None]).pin_memory(),
            Ey=torch.as_tensor(Ey.astype(np.complex64)[None]).pin_memory(),
            eta=torch.as_tensor(eta).pin_memory(), theta=torch.as_tensor(theta).pin_memory(),
            out=[torch.empty((B, N, N), dtype=torch.complex64).pin_memory() for _ in range(3)]))
    zarr = np.asarray(zs)

    def e2e_step(i):
        h = hosts[i % E2E_STREAMS]
        with torch.cuda.stream(streams[i % E2E_STREAMS]):
            light = vo.VectorizedLight(x, x, WAVELENGTH)
            light.Ex = h["Ex"].to(dev, non_blocking=True).expand(B, N, N)
            light.Ey = h["Ey"].to(dev, non_blocking=True).expand(B, N, N)
            e_ = h["eta"].to(dev, non_blocking=True)
            t_ = h["theta"].to(dev, non_blocking=True)
            out, _ = oe.linear_polarizer(oe.LCD(light, e_, t_), alpha).VRS_propagation(zarr)
            for hb, d in zip(h["out"], (out.Ex, out.Ey, out.Ez)):
                hb.copy_(d, non_blocking=True)

    for i in range(E2E_STREAMS):
        e2e_step(i)
    torch.cuda.synchronize()
    # three consecutive timed segments of ke steps; the median is reported (the
    # host link is shared with the rest of the machine and a single segment
    # can catch a slow spell)
    ke = max(4, args.steps // 2)
    segments = []
    for _ in range(3):
        replica_barrier()
        t0 = time.perf_counter()
        for i in range(ke):
            streams[i % E2E_STREAMS].synchronize()   # the stream's host buffers are free again
            e2e_step(i)
        torch.cuda.synchronize()
        e2e_s, e2e_fields = reduce_replicas(time.perf_counter() - t0, B * ke)
        segments.append(e2e_fields / e2e_s)
    e2e = float(np.median(segments))
    h2d = (hosts[0]["Ex"].numel() + hosts[0]["Ey"].numel()) * 8 + \
        (hosts[0]["eta"].numel() + hosts[0]["theta"].numel()) * 4
    d2h = sum(hb.numel() for hb in hosts[0]["out"]) * 8
    link = host_link_rates(dev)
    # the fields/s the copies alone allow: each direction at its own rate, and
    # both together at the duplex rate
    link_s = max(d2h / (link["d2h_gbs"] * 1e9), h2d / (link["h2d_gbs"] * 1e9),
                 (d2h + h2d) / (link["duplex_gbs"] * 1e9))
    link["bound_fields_per_s"] = B / link_s

    # the column pass against its instruction-issue ceiling: warp instructions
    # per launch (ncu, per variant) over the SMs' issue rate at the SM clock
    # sampled while the timed region ran
    clocks = clk.summary()
    inst = NCU_COL_INST_PER_FIELD.get(int(tuned["variant"]))
    issue_roofline = None
    if inst is not None and clocks.get("sm_mhz"):
        n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
        ipeak = n_sm * 4 * float(clocks["sm_mhz"]) * 1e6
        iach = inst * B / (stage_ms[1] / 1e3)
        issue_roofline = {"bound": "instruction issue", "kernel": "rs_cols_conv", "variant": int(tuned["variant"]),
                          "achieved": iach, "peak": ipeak, "unit": "warp instructions/s", "frac": iach / ipeak,
                          "instructions_per_launch": inst * B,
                          "source": "ncu smsp__inst_executed.sum per field x fields per launch: " + NCU_INST_COMMAND,
                          "peak_how": "%d SMs x 4 schedulers x the median SM clock of the timed region" % n_sm}

    line = {
        "metric": METRIC, "value": value, "unit": "fields/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "batch": B, "fields_per_step": B * world,
                   "parallelism": "replicas x%d (no data-path collective)" % world,
                   "l2": "inputs larger than L2 (%.2f GB of fields and masks per step)" %
                         ((Ex_d.numel() + Ey_d.numel()) * 8 / 1e9 + (eta_d.numel() + theta_d.numel()) * 4 / 1e9)},
        "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": (NCU_TRAFFIC_PER_FIELD[names[dom]] * B
                                 if NCU_TRAFFIC_PER_FIELD[names[dom]] is not None else None),
                     "traffic_source": "ncu capture of this benchmark's own 8-field launch, "
                                       "dram__bytes_read.sum + dram__bytes_write.sum: " + NCU_TRAFFIC_COMMAND,
                     "peak_source": peak_src,
                     "alg_bytes_per_launch": alg[dom], "ms_per_launch": stage_ms[dom]},
        "issue_roofline": issue_roofline,
        "rel_l2": parity,
        "latency": {"step_ms_p50": float(np.percentile(step_ms, 50)),
                    "step_ms_p99": float(np.percentile(step_ms, 99)),
                    "ms_per_field_p50": float(np.percentile(step_ms / B, 50)),
                    "ms_per_field_p99": float(np.percentile(step_ms / B, 99)),
                    "how": "CUDA events around each timed step of B fields; a field's latency is its step's"},
        "stages_ms": dict(zip(names, stage_ms)),
        "column_pass_variant": {"chosen": tuned["variant"], "transform_length": 1 << col_logp,
                                "ms_per_launch": {str(k): v for k, v in tuned["ms"].items()},
                                "variants": "0 one line per thread; 1 two lines per thread (packed FP32), "
                                            "pairs interleaved in warps; 2 packed, pairs in barrier groups; "
                                            "3 one line per thread with L2 prefetch; 4 packed interleaved "
                                            "with L2 and register prefetch; 5 one line per thread, two "
                                            "barrier groups; 6 one line per thread, two CTAs per SM; 7 as 5 with "
                                            "the groups started half a component apart; 8 one line per thread, "
                                            "persistent (the library's default at 4096 points); 9 (4096 "
                                            "points) radix-64, 64 elements per thread, one exchange per "
                                            "transform; 10 (4096 points) as 8, each unit's spectrum values "
                                            "kept in Tensor Memory for its second and third components"},
        "pipeline_roofline": {"alg_bytes_per_field": 272 * n2, "achieved": pipe_gbs, "frac": pipe_gbs / peak},
        "plain_path": {"value": plain, "unit": "fields/s", "how": "one VRS_propagation call per field"},
        "e2e": {"value": e2e, "unit": "fields/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "segments": segments, "steps_per_segment": ke,
                "host_link": dict(link, how="pinned-memory copies of 256 MiB, one stream per direction, "
                                            "timed outside the timed region, best of 5 timings; bound = B / "
                                            "the longest of the step's copies at these rates")},
        "gpu_launches": 3 * args.steps,
        "clocks": clocks,
        "spectrum_builds": engine.SPECTRA.builds,
    }
    if world > 1:   # the single-GPU sections below are not replicated
        if rank == 0:
            print(json.dumps(line))
        return
    if not args.no_fwd_bwd:
        del call, Ex_d, Ey_d, eta_d, theta_d, hosts
        torch.cuda.empty_cache()
        line["czt_high_na"] = run_czt()
        torch.cuda.empty_cache()
        line["rs_plain_1024"] = run_rs_plain_config()
        torch.cuda.empty_cache()
        line["fwd_bwd"] = run_fwd_bwd()
        torch.cuda.empty_cache()
        line["hybrid_sharp_focus"] = run_hybrid()
    if not args.no_serving:
        line["uneven_batch"] = run_uneven()
        line["serving"] = run_serving(args.serve_requests)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample(args.cpu_seconds)
    print(json.dumps(line))


def run_czt(batch=8, steps=20, warmup=3, check=True):
    """The high-NA objective-lens focus (VCZT_objective_lens, optical_elements.py:600-638):
    2048^2 (Ex, Ey) behind a per-pixel LCD and sSLM -> lens -> 1024^2 focal ROI
    (Ex, Ey, Ez), forward, `batch` fields per launch; per-kernel times from
    CUDA events on the launching stream."""
    import torch

    from xlumina_gb300 import engine, toolbox
    n, m = 2048, 1024
    x, y = toolbox.space(2700.0, n)
    xo, yo = toolbox.space(1.0, m)
    f, r = 3000.0, 2700.0
    rng = np.random.default_rng(7000)
    X, Y = np.meshgrid(x, y)
    src = np.exp(-(X ** 2 + Y ** 2) / 1500.0 ** 2).astype(np.complex64)
    ex = torch.as_tensor(src, device="cuda").expand(batch, n, n)
    ey = torch.zeros((n, n), dtype=torch.complex64, device="cuda").expand(batch, n, n)
    eta = torch.as_tensor(rng.uniform(0, 2 * np.pi, (n, n)).astype(np.float32), device="cuda")
    theta = torch.as_tensor(rng.uniform(0, 2 * np.pi, (n, n)).astype(np.float32), device="cuda")
    alpha = torch.as_tensor(rng.uniform(0, 2 * np.pi, (batch, n, n)).astype(np.float32), device="cuda")
    phi = torch.as_tensor(rng.uniform(0, 2 * np.pi, (batch, n, n)).astype(np.float32), device="cuda")
    lens_op, s_max = engine.op_high_na(x, y, r, f)
    pre = [engine.op_lcd(eta, theta), engine.op_sslm(alpha, phi), lens_op]
    call = engine.CztCall([ex, ey], x, y, 0.650, 0.0, xo, yo, "high_na", pre=pre, lens=(r, f, s_max))
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        call.stage(0)
        call.stage(1)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3 * steps)]
    for k in range(steps):
        ev[3 * k].record(stream)
        call.stage(0)
        ev[3 * k + 1].record(stream)
        call.stage(1)
        ev[3 * k + 2].record(stream)
    torch.cuda.synchronize()
    rows = sum(ev[3 * k].elapsed_time(ev[3 * k + 1]) for k in range(steps)) / steps
    cols = sum(ev[3 * k + 1].elapsed_time(ev[3 * k + 2]) for k in range(steps)) / steps
    # algorithmic bytes per field: rows read Ex, Ey 16 n^2 (shared by the batch), the sSLM
    # planes 8 n^2 (per field), LCD planes 8 n^2 and lens coefficients 24 n^2 (shared), and
    # write 3 n m complex64; columns read 3 n m and write 3 m^2
    rows_b = 8 * n * n + 3 * n * m * 8 + (16 + 8 + 24) * n * n / batch
    cols_b = 3 * n * m * 8 + 3 * m * m * 8
    err = None
    if check:   # field 0 of the last timed launch against the FP64 oracle
        from oracle import xlumina_ref as ref
        ax, ay = ref.lcd(src.astype(np.complex128), np.zeros((n, n)), eta.cpu().numpy().astype(np.float64),
                         theta.cpu().numpy().astype(np.float64))
        ax, ay = ref.sslm(ax, ay, alpha[0].cpu().numpy().astype(np.float64), phi[0].cpu().numpy().astype(np.float64))
        exp = ref.vczt_objective_lens(ax, ay, x, y, 0.650, r, f, xo, yo)
        err = max(_rel_l2(call.outs[c][0].cpu().numpy(), exp[c]) for c in range(3))
    return {"workload": "high-NA focus 2048^2 -> 1024^2 ROI (2 um), LCD + sSLM + lens fused, Ez derived, forward",
            "rel_l2": err,
            "batch": batch, "fields_per_s": batch / ((rows + cols) / 1e3),
            "czt_rows_ms": rows, "czt_cols_ms": cols,
            "czt_rows_gbs": batch * rows_b / (rows / 1e3) / 1e9, "czt_cols_gbs": batch * cols_b / (cols / 1e3) / 1e9}


def _time_steps(fn, steps, warmup):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(steps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / 1e3 / steps


def _rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def oracle_four_f_intensity(t, b):
    """Table b of a FourFTable through the FP64 oracle: its normalised output intensity."""
    from oracle import xlumina_ref as ref
    inp, _, p1, p2 = t.entry(b)
    u = ref.slm(inp, p1)[0]
    u = ref.rs_propagate(u, t.x, t.y, t.wavelength, t.f)
    u = u * ref.lens_mask(t.x, t.y, t.wavelength, t.lens_r, (t.f, t.f))
    u = ref.czt(u, t.x, t.y, t.wavelength, t.f, t.xo, t.yo)
    u = ref.slm(u, p2)[0]
    I = np.abs(ref.czt(u, t.xo, t.yo, t.wavelength, t.f, t.xo, t.yo)) ** 2
    return I / np.sum(I)


def oracle_high_na_intensity(t, b):
    """Table b of a HighNATable through the FP64 oracle: its focal |Ez|^2."""
    from oracle import xlumina_ref as ref
    eta, theta, alpha, phi = t.entry(b)
    Ex = t.Ex.cpu().numpy().astype(np.complex128)
    ax, ay = ref.lcd(Ex, np.zeros_like(Ex), eta, theta)
    ax, ay = ref.sslm(ax, ay, alpha, phi)
    return np.abs(ref.vczt_objective_lens(ax, ay, t.x, t.y, t.wavelength, t.r, t.f, t.xo, t.yo)[2]) ** 2


def _peak_step_bytes(step):
    """Device memory in use at the peak of one step, above what was allocated before it."""
    import torch
    torch.cuda.synchronize()
    base = torch.cuda.memory_allocated()
    torch.cuda.reset_peak_memory_stats()
    step()
    torch.cuda.synchronize()
    return int(torch.cuda.max_memory_allocated() - base)


def run_fwd_bwd(steps=10, warmup=3):
    """fwd+bwd optimisation steps through the hand-written adjoints: the batched
    form (one step over the whole batch, eager and replayed from a captured
    CUDA graph) and the plain form (one table or field per call).  Each row
    states the rel-L2 of one timed table's output against the FP64 oracle."""
    import torch

    from xlumina_gb300.plans import CapturedStep
    from xlumina_gb300.tables import FourFTable, HighNATable, VrsLcdTable
    out = {}

    def captured_rate(make, nsteps):
        t = make()
        cs = CapturedStep(t)
        dt = _time_steps(cs, nsteps, 2)
        del cs, t
        torch.cuda.empty_cache()
        return 1.0 / dt

    tv = VrsLcdTable()
    dt = _time_steps(tv.step, steps, warmup)
    single = lambda i=[0]: tv.step(slice(i[0] % tv.B, i[0] % tv.B + 1))  # noqa: E731
    dt1 = _time_steps(single, tv.B, 2)
    B = tv.B
    del tv
    torch.cuda.empty_cache()
    cap = captured_rate(lambda: VrsLcdTable(capturable=True), steps)
    out["vrs"] = {"workload": "VRS 2048^2, 8 fields, per-field LCD (eta, theta) + LP, z = 5 cm, "
                              "intensity MSE vs per-field targets, AdamW",
                  "steps_per_s": 1.0 / dt, "fields_per_s": B / dt, "captured_steps_per_s": cap,
                  "captured_fields_per_s": B * cap, "plain_fields_per_s": 1.0 / dt1, "batch": B}

    t4 = FourFTable()
    dt = _time_steps(t4.step, steps, warmup)
    single = lambda i=[0]: t4.step(tables=slice(i[0] % t4.B, i[0] % t4.B + 1))  # noqa: E731
    dt1 = _time_steps(single, t4.B, 2)
    B = t4.B
    with torch.no_grad():
        err4 = _rel_l2(t4.intensities()[0].cpu().numpy(), oracle_four_f_intensity(t4, 0))
    del t4
    torch.cuda.empty_cache()
    cap = captured_rate(lambda: FourFTable(capturable=True), steps)
    out["four_f"] = {"workload": "4f step, 16 independent tables (own seed: input mask, 10 % binary target, "
                                 "SLM1 1024^2 and SLM2 512^2 phases U[-pi, pi)), 1024^2 -> RS 25 cm -> lens -> "
                                 "CZT 512^2 ROI -> SLM2 -> CZT, 532 nm, normalised intensity MSE, AdamW",
                     "steps_per_s": 1.0 / dt, "tables_per_s": B / dt, "captured_steps_per_s": cap,
                     "captured_tables_per_s": B * cap, "plain_tables_per_s": 1.0 / dt1, "batch": B,
                     "rel_l2": {"what": "table 0's normalised output intensity after the timed steps, "
                                        "against the FP64 oracle", "value": err4}}

    # high-NA: the configured form keeps no focal field for the backward
    # (activation checkpointing: the focus is recomputed); the row also times
    # the form that keeps them, with each form's peak memory
    hrow = {}
    for ck in (True, False):
        th = HighNATable(checkpoint=ck)
        dt = _time_steps(th.step, max(2, steps // 2), 2)
        peak = _peak_step_bytes(th.step)
        if ck:
            with torch.no_grad():
                errh = _rel_l2(th._spot_intensity()[0].cpu().numpy(), oracle_high_na_intensity(th, 0))
        B = th.B
        del th
        torch.cuda.empty_cache()
        hrow[ck] = (dt, peak)
    cap = captured_rate(lambda: HighNATable(capturable=True, checkpoint=True), max(2, steps // 2))
    out["high_na"] = {"workload": "high-NA step, 32 tables with their own per-pixel LCD (eta, theta) and sSLM "
                                  "(alpha, phi) planes U[0, 2 pi), 2048^2 -> VCZT objective lens (NA 0.9, f 3 mm) "
                                  "-> 1024^2 focal ROI (2 um), 650 nm, Ez spot loss, AdamW, activation "
                                  "checkpointing of the focal fields",
                      "steps_per_s": 1.0 / hrow[True][0], "tables_per_s": B / hrow[True][0],
                      "captured_steps_per_s": cap, "captured_tables_per_s": B * cap, "batch": B,
                      "peak_step_bytes": hrow[True][1],
                      "without_checkpointing": {"steps_per_s": 1.0 / hrow[False][0],
                                                "peak_step_bytes": hrow[False][1]},
                      "rel_l2": {"what": "table 0's focal |Ez|^2 after the timed steps, against the FP64 oracle",
                                 "value": errh}}
    torch.cuda.empty_cache()
    return out


def run_rs_plain_config(batch=16, steps=20, warmup=3, seed=0):
    """Scalar RS at 1024^2 (the reference's plain propagation case): 2 mm
    window, 650 nm, Gaussian w0 = 200 um behind a per-field SLM phase
    U[-pi, pi), z = 5 cm.  Batched (one call for `batch` fields, inputs
    resident in HBM) and plain (one RS_propagation call per field)."""
    import torch

    from oracle import xlumina_ref as ref
    from xlumina_gb300 import engine
    from xlumina_gb300 import optical_elements as oe
    from xlumina_gb300 import wave_optics as wo
    n, wl, z = 1024, 0.650, 5.0e4
    x, y = ref.space(1000.0, n)
    src = wo.LightSource(x, y, wl)
    src.gaussian_beam(w0=(200.0, 200.0), E0=1)
    rng = np.random.default_rng(seed)
    ph = torch.as_tensor(rng.uniform(-np.pi, np.pi, (batch, n, n)).astype(np.float32), device="cuda")
    field = src.field.expand(batch, n, n)
    call = engine.RsCall([field], x, y, wl, z, vector=False, pre=[engine.op_phase(ph)])
    dt = _time_steps(call.run, steps, warmup)
    light = wo.ScalarLight(x, y, wl)
    light.field = src.field

    def plain(i=[0]):
        k = i[0] % batch
        i[0] += 1
        oe.SLM(light, ph[k], n)[0].RS_propagation(z)
    dtp = _time_steps(plain, 2 * batch, 3)
    alg = (112 + 4) * n * n          # bytes per field (4N^2: the phase mask)
    exp = ref.rs_propagate(ref.slm(ref.gaussian_beam(x, y, wl, (200.0, 200.0)), ph[0].cpu().numpy())[0],
                           x, y, wl, z)
    err = _rel_l2(call.outs[0][0].cpu().numpy(), exp)
    return {"rel_l2": err, "workload": "scalar RS 1024^2, 2 mm window, 650 nm, Gaussian w0 200 um, per-field SLM phase, z = 5 cm",
            "batch": batch, "fields_per_s": batch / dt, "plain_fields_per_s": 1.0 / dtp,
            "pipeline_gbs": batch * alg / dt / 1e9, "alg_bytes_per_field": alg}


def run_hybrid(steps=5, warmup=2):
    """The hybrid sharp-focus discovery step (9 splitters, 16 VRS and 6
    objective-lens focuses at 1024^2, every distance, angle, LCD setting and
    phase mask trainable): fwd + bwd + AdamW per step."""
    import torch

    from xlumina_gb300.plans import CapturedStep
    from xlumina_gb300.tables import SharpFocusTable
    t = SharpFocusTable()
    dt = _time_steps(t.step, steps, warmup)
    del t
    torch.cuda.empty_cache()
    t = SharpFocusTable(capturable=True)
    cs = CapturedStep(t)
    dtc = _time_steps(cs, steps, 2)
    del cs, t
    torch.cuda.empty_cache()
    return {"workload": "hybrid_setup_sharp_focus 1024^2 (2.5 mm, 635 nm) -> 6 x VCZT objective lens 400^2 "
                        "(10 um, NA 0.9), softmin(vectorized_loss_hybrid), AdamW over 29 parameters",
            "steps_per_s": 1.0 / dt, "ms_per_step": dt * 1e3, "captured_steps_per_s": 1.0 / dtc,
            "captured_ms_per_step": dtc * 1e3}


def run_uneven(reps=20, seed=6000):
    """Many setups of uneven size: 48 scalar RS at 256^2, 12 VRS at 512^2 and
    4 scalar RS at 1024^2, each with its own SLM phase mask and distance.
    Three forms: one public-API call per setup; one batched call per size
    group (a distance per batch entry); and the grouped calls captured in one
    CUDA graph, replayed with a single launch."""
    import torch

    from xlumina_gb300 import engine, toolbox
    from xlumina_gb300.plans import CapturedPlan
    rng = np.random.default_rng(seed)
    groups = [("rs", 256, 48), ("vrs", 512, 12), ("rs", 1024, 4)]
    data = []
    for kind, n, cnt in groups:
        x, y = toolbox.space(1000.0 * n / 1024, n)
        comps = 1 if kind == "rs" else 2
        f = torch.as_tensor((rng.standard_normal((comps, cnt, n, n)) + 1j * rng.standard_normal((comps, cnt, n, n)))
                            .astype(np.complex64), device="cuda")
        ph = torch.as_tensor(rng.uniform(-np.pi, np.pi, (cnt, n, n)).astype(np.float32), device="cuda")
        zs = list(rng.choice([1e4, 2e4, 5e4, 1e5], cnt))
        data.append((kind, n, cnt, x, y, f, ph, zs))
    n_setups = sum(c for _, _, c in groups)

    def one_by_one():
        for kind, n, cnt, x, y, f, ph, zs in data:
            for i in range(cnt):
                engine.rs_propagate([f[c, i] for c in range(f.shape[0])], x, y, 0.6, zs[i], kind == "vrs",
                                    pre=[engine.op_phase(ph[i])] if kind == "rs" else
                                    [engine.op_sslm(ph[i], ph[i])])

    def grouped():
        outs = []
        for kind, n, cnt, x, y, f, ph, zs in data:
            outs += engine.rs_propagate([f[c] for c in range(f.shape[0])], x, y, 0.6, zs, kind == "vrs",
                                        pre=[engine.op_phase(ph)] if kind == "rs" else [engine.op_sslm(ph, ph)])
        return outs

    res = {"workload": "uneven setups: 48 RS 256^2 + 12 VRS 512^2 + 4 RS 1024^2, per-setup SLM masks and distances",
           "setups": n_setups}
    dt = _time_steps(one_by_one, reps, 3)
    res["one_call_per_setup_setups_per_s"] = n_setups / dt
    dt = _time_steps(grouped, reps, 3)
    res["grouped_setups_per_s"] = n_setups / dt
    plan = CapturedPlan(grouped)
    dt = _time_steps(plan.replay, reps, 3)
    res["captured_graph_setups_per_s"] = n_setups / dt
    del plan
    torch.cuda.empty_cache()
    return res


def run_serving(n_req=10000, seed=4000):
    """Poisson stream of mixed requests (sizes 256..2048 with weights .4/.3/.2/.1; RS, VRS, CZT
    or an SLM-phase gradient; z uniform in [1, 20] cm) through the continuous-batching server,
    against the plain path (one call per request, in order)."""
    import threading

    import torch

    from xlumina_gb300 import toolbox
    from xlumina_gb300.serving import Request, Server, run_batch
    rng = np.random.default_rng(seed)
    sizes = np.array([256, 512, 1024, 2048])
    kinds = ["rs", "vrs", "czt", "grad"]
    pool = {}
    for n in sizes:
        g = torch.Generator(device="cuda").manual_seed(int(n))
        f = lambda: torch.randn((int(n), int(n)), dtype=torch.complex64, device="cuda", generator=g)  # noqa: E731
        x, y = toolbox.space(2000.0 * n / 2048, int(n))
        xo, yo = toolbox.space(200.0 * n / 2048, int(n) // 2)
        pool[int(n)] = dict(f=[f(), f()], x=x, y=y, xo=xo, yo=yo,
                            ph=torch.rand((int(n), int(n)), device="cuda", generator=g) * 6.2832 - 3.1416,
                            tgt=torch.rand((int(n), int(n)), device="cuda", generator=g))

    def make(i):
        n = int(rng.choice(sizes, p=[0.4, 0.3, 0.2, 0.1]))
        k = kinds[int(rng.integers(4))]
        z = float(rng.uniform(1e4, 2e5))
        p = pool[n]
        if k == "czt":
            return Request(k, [p["f"][0]], p["x"], p["y"], 0.633, z, xout=p["xo"], yout=p["yo"])
        if k == "grad":
            return Request(k, [p["f"][0]], p["x"], p["y"], 0.633, z, phase=p["ph"], target=p["tgt"])
        return Request(k, p["f"][:1 if k == "rs" else 2], p["x"], p["y"], 0.633, z)

    # plain path: one call per request, each waited for
    n_plain = min(600, n_req)
    plain_reqs = [make(i) for i in range(n_plain)]
    for r in plain_reqs[:20]:
        run_batch([r])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lat = []
    for r in plain_reqs:
        t1 = time.perf_counter()
        run_batch([r])
        torch.cuda.synchronize()
        lat.append(time.perf_counter() - t1)
    plain_rate = n_plain / (time.perf_counter() - t0)

    reqs = [make(i) for i in range(n_req)]
    from xlumina_gb300.autotune import BatchTuner
    examples = {}
    for r in reqs:
        examples.setdefault((r.kind, len(r.x)), r)

    def serve(max_launch_ms, rate=None):
        """Tune, measure the capacity with a saturating burst, then serve the
        Poisson stream at ``rate`` (default 80 % of that capacity).  Each run
        serves fresh copies of the requests (a request's future completes once)."""
        import dataclasses
        import gc
        from concurrent.futures import Future
        # start from a settled process: collect and freeze the objects the
        # earlier sections left (so that garbage collections during the run
        # do not walk them), and return the allocator's unused blocks
        gc.collect()
        gc.freeze()
        torch.cuda.empty_cache()
        stream = [dataclasses.replace(r, future=Future()) for r in reqs]
        srv = Server(hbm_budget_bytes=150e9, max_batch=16, streams=2,
                     tuner=BatchTuner(candidates=(1, 2, 4, 8, 16), repeats=2), max_launch_ms=max_launch_ms)
        t_tune = time.perf_counter()
        packing = srv.tune(list(examples.values()))
        t_tune = time.perf_counter() - t_tune
        n_sat = min(3000, n_req)
        sat_reqs = [make(i) for i in range(n_sat)]
        t0 = time.perf_counter()
        sat = [srv.submit(r) for r in sat_reqs]
        for f in sat:
            f.result(timeout=600)
        capacity = n_sat / (time.perf_counter() - t0)
        srv.reset_stats()
        offered = 0.8 * capacity if rate is None else min(rate, 0.8 * capacity)
        # the same arrival pattern for every run (scaled to its rate), so that
        # runs at the same offered rate see the same bursts
        gaps = np.random.default_rng(seed + 1).exponential(1.0, n_req) / offered
        futs = [None] * n_req

        def client():
            t = time.perf_counter()
            for i, r in enumerate(stream):
                t += gaps[i]
                d = t - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                futs[i] = srv.submit(r)

        t0 = time.perf_counter()
        th = threading.Thread(target=client)
        th.start()
        th.join()
        for f in futs:
            f.result(timeout=600)
        wall = time.perf_counter() - t0
        srv.close()
        gc.unfreeze()
        st = srv.stats()
        return {"capacity_req_per_s": capacity, "offered_req_per_s": offered, "served_req_per_s": n_req / wall,
                "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_batch": st["mean_batch"],
                "batch_packing": {f"{k[0]} {k[1]}^2": v for k, v in packing.items()}, "tuning_s": t_tune}

    thr = serve(None)
    bounded = serve(SERVE_MAX_LAUNCH_MS, rate=thr["offered_req_per_s"])
    out = {"workload": "10,000 Poisson requests, sizes 256/512/1024/2048 (.4/.3/.2/.1), RS/VRS/CZT/grad, "
                       "z U[1,20] cm, HBM budget 150 GB",
           "requests": n_req, "offered_load": "80 % of the saturated capacity"}
    out.update(thr)
    out["latency_bounded"] = dict(bounded, max_launch_ms=SERVE_MAX_LAUNCH_MS,
                                  how="batch sizes whose launch takes at most max_launch_ms, same offered rate "
                                      "(or 80 % of this capacity if lower)")
    out.update({"plain_req_per_s": plain_rate, "plain_p50_ms": float(np.percentile(np.asarray(lat) * 1e3, 50)),
                "plain_p99_ms": float(np.percentile(np.asarray(lat) * 1e3, 99))})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--impl", default="xlgb", choices=["xlgb", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fwd-bwd", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=10000)
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--col-variant", type=int, default=None,
                    help="use this column-pass kernel variant instead of measuring them all")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle checks of the timed outputs")
    ap.add_argument("--czt-cols-variant", type=int, default=None,
                    help="use this chirp-z column-pass kernel variant (all transform lengths)")
    ap.add_argument("--step-batch", type=int, default=None,
                    help="tables per step for --only highna_step / fourf_step (default: the workload's)")
    ap.add_argument("--czt-rows-variant", type=int, default=None,
                    help="use this chirp-z row-pass kernel variant (all transform lengths)")
    ap.add_argument("--only", choices=["czt", "hybrid", "rs1024", "highna_step", "fourf_step", "serving"], default=None,
                    help="run one section alone (for profiling): czt = the high-NA focus, "
                         "hybrid = the sharp-focus discovery step")
    args = ap.parse_args()
    for pass_name, v in (("XL_PASS_CZT_ROWS", args.czt_rows_variant), ("XL_PASS_CZT_COLS", args.czt_cols_variant)):
        if v is None:
            continue
        from xlumina_gb300 import _lib, engine
        pid = getattr(_lib, pass_name)
        for lg in range(5, 14):   # every transform length that has the variant
            if v < engine.lib().xl_kernel_variant_count(pid, lg):
                _lib.check(engine.lib().xl_set_kernel_variant(pid, lg, v))
    if args.only == "czt":
        print(json.dumps({"czt_high_na": run_czt(batch=args.batch, steps=args.steps, warmup=args.warmup,
                                                  check=False)}))
        return
    if args.only == "hybrid":
        print(json.dumps({"hybrid_sharp_focus": run_hybrid(steps=args.steps, warmup=args.warmup)}))
        return
    if args.only in ("highna_step", "fourf_step"):
        import torch

        from xlumina_gb300.tables import FourFTable, HighNATable
        kw = {"batch": args.step_batch} if args.step_batch else {}
        t = HighNATable(checkpoint=True, **kw) if args.only == "highna_step" else FourFTable(**kw)
        dt = _time_steps(t.step, args.steps, args.warmup)
        torch.cuda.synchronize()
        print(json.dumps({args.only: {"steps_per_s": 1.0 / dt, "tables_per_s": t.B / dt, "batch": t.B}}))
        return
    if args.only == "rs1024":
        print(json.dumps({"rs_plain_1024": run_rs_plain_config(steps=args.steps, warmup=args.warmup)}))
        return
    if args.only == "serving":
        print(json.dumps({"serving": run_serving()}))
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
