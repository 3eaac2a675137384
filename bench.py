#!/usr/bin/env python
"""Benchmark of the GB300 segment-attenuation sweep: prints ONE JSON line on rank 0.

A step is one forward sweep (moc_attenuate_fwd) over the whole workload: every segment
of every track, every energy group. The default workload is the reference's default
problem size (-s 50000000 -e 128): 50,000,000 segments x 128 groups, 100,000 tracks,
10,000 regions x 5 fine axial intervals, seeded synthetic inputs (the reference reads
no dataset; it draws random inputs itself).

  value        segment*group attenuations per second, inputs resident in HBM, CUDA
               events around each sweep call on the launching stream, L2 flushed
               (256 MiB write) between steps
  e2e          the same metric through moc_attenuate_fwd_host on page-locked host
               arrays: every step moves all inputs in and psi + fine_flux out over the
               host link (the sweep reads the mapped descriptors and psi in place, the
               tables are copied up, the tallies are added into fine_flux in place)
  roofline     the sweep kernel against its binding resource (L2: row gathers +
               tally reductions), with the HBM fraction beside it
  cpu_baseline the reference sweep restated in C (OpenMP over tracks, per-cell locks,
               the reference's gnu flags), on a bounded sample of the same workload
  forms        the precision, batching and differentiation forms beside the plain sweep
  tracks       track generation (the step before the sweep): ray tracing a 17 x 17
               assembly into 58.5M segment descriptors, segments/s, with the oracle's
               CPU tracer timed beside it
  transport    the power iteration around the sweep (the step after): the traced
               assembly swept both ways at 128 groups, source update and eigenvalue,
               time per iteration, with the oracle's source update timed beside it

--impl reference times that CPU reference arm alone (all host threads), as the
reference's own path for this workload.
--peaks runs the roofline microbenchmarks and writes profiles/peaks_gb300.json.

Multi-GPU: the sweep runs on one GPU; with torchrun every rank runs its own replica of
the workload (no collective in the data path) and the slowest rank sets the time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "simplemoc-kernel_gb300")
sys.path.insert(0, PKG)

METRIC = "segment·group attenuations/s, plain FP32 vs chosen form at ≤1e-5 rel err, %HBM"
UNIT = "segment·group attenuations/s"
PEAKS_FILE = os.path.join(ROOT, "profiles", "peaks_gb300.json")
MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")

# Algorithmic L2 bytes per segment*group of the plain FP32 sweep: the cell block
# (sigT, q0, q1*mu, q2*mu2) 16 B + the segment descriptor 9 B / G gathered, and the tally
# 4 B reduced. FP32 instructions per segment*group of the plain arithmetic (25, counted
# from attenuate<> in csrc/moc_sweep.cu) and MUFU operations (ex2 + rcp).
FP32_OPS_PER_UNIT = 25
MUFU_OPS_PER_UNIT = 2


def l2_bytes_per_unit(I: int, G: int) -> dict:
    return {"gather": 16.0 + 9.0 / G, "reduce": 4.0}


def hbm_compulsory_bytes(hp) -> float:
    """Bytes a sweep must move to or from HBM at least once: descriptors, offsets, psi in
    and out, sigT and source (read by the block pass), cell blocks written and read,
    fine_flux read and written."""
    S, T, Gs, R, I = hp.S, hp.T, hp.Gs, hp.R, hp.I
    return (9.0 * S + 8.0 * (T + 1) + 2 * 4.0 * T * Gs + 4.0 * R * Gs + 4.0 * R * I * Gs
            + 2 * 16.0 * R * I * Gs + 2 * 4.0 * R * I * Gs)


# --precision: the form the timed steps sweep (the headline is the plain FP32 form; the
# others exist for profiling a precision form on the same harness)
PRECISION_ARG = {"fp32": "MOC_PREC_FP32", "fp32_stable": "MOC_PREC_FP32_STABLE",
                 "bf16": "MOC_PREC_BF16", "fp16": "MOC_PREC_FP16"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms while running; the
    constructor returns once the first sample is written, so the timed region that
    follows is covered from its start."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        if self.p is not None:
            t0 = time.time()
            while time.time() - t0 < 5.0 and self.p.poll() is None:
                self.f.flush()
                if os.path.getsize(self.f.name) > 0:
                    break
                time.sleep(0.02)
            # count only what is sampled from here on
            self.skip = len(open(self.f.name).read().strip().splitlines())
        else:
            self.skip = 0

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        rows = rows[self.skip:] or rows
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, r[4:8]):
                if v.strip().lower() in ("active", "1"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(workload, sample_tracks: int, steps: int, warmup: int,
                 table_points: int = 0) -> dict:
    """The CPU reference arm (oracle/_build/cpu_bench) on a bounded sample."""
    exe = os.path.join(ROOT, "oracle", "_build", "cpu_bench")
    if not os.path.exists(exe):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"], check=True)
    args = [exe] + workload.cpu_bench_args() + [
        "--sample-tracks", str(sample_tracks), "--steps", str(steps), "--warmup", str(warmup)]
    if table_points:
        args += ["--table", str(table_points), "10.0"]
    out = subprocess.run(args, capture_output=True, text=True, check=True).stdout
    r = json.loads(out.strip().splitlines()[-1])
    r["sample"] = (f"first {r['sample_tracks']} of {workload.tracks} tracks "
                   f"({r['sample_segments']} segments x {r['groups']} groups), "
                   f"{steps} timed passes after {warmup} warm-up")
    return r


# Roofline peaks measured by this process (run_peaks after the timed steps); they take
# precedence over the committed profiles/peaks_gb300.json.
IN_RUN_PEAKS: dict = {}


def load_peaks() -> dict:
    peaks = {}
    if os.path.exists(MEASURED_PEAKS):
        with open(MEASURED_PEAKS) as f:
            m = json.load(f)
        peaks["hbm_gbs"] = m.get("hbm_gbs")
        peaks["hbm_source"] = "MEASURED_PEAKS.json (measured copy bandwidth)"
    else:
        peaks["hbm_gbs"] = 6800.0
        peaks["hbm_source"] = "fallback 6.8 TB/s"
    if os.path.exists(PEAKS_FILE):
        with open(PEAKS_FILE) as f:
            peaks.update(json.load(f))
        peaks["peaks_measured"] = "by bench.py --peaks (profiles/peaks_gb300.json)"
    if IN_RUN_PEAKS:
        peaks.update(IN_RUN_PEAKS)
        peaks["peaks_measured"] = "in this run (csrc/moc_peaks.cu after the timed steps)"
    return peaks


def run_peaks() -> dict:
    """The roofline microbenchmarks (csrc/moc_peaks.cu) on GPU 0, with the SM clock sampled
    by nvidia-smi while they run and the date of the run."""
    lib = C.CDLL(os.path.join(PKG, "_build", "libmocpeaks.so"))
    lib.mocpeak_run.restype = C.c_int
    res = (C.c_double * 14)()
    clocks = ClockSampler(0)
    rc = lib.mocpeak_run(res, 14)
    clk = clocks.stop()
    if rc:
        raise RuntimeError(f"mocpeak_run failed: {rc}")
    out = {"l2_stream_read_gbs": res[0], "l2_row_gather_hashed_gbs": res[1],
           "l2_row_reduce_hashed_gbs": res[2], "fp32_fma_tflops": res[3],
           "mufu_ex2_gops": res[4], "hbm_read_gbs": res[5], "l2_row_gather_gbs": res[6],
           "l2_row_reduce_gbs": res[7], "l2_mix_gbs": res[8], "fp64_fma_tflops": res[9],
           "l2_wide_gather_gbs": res[10], "l2_wide_reduce_gbs": res[11],
           "l2_wide_mix_gbs": res[12], "fp32_fma2_tflops": res[13],
           "mix": "four random 512-byte row gathers per 512-byte red.v4 row reduction "
                  "(the sweep's 16 B gathered : 4 B reduced per segment*group)",
           "wide_mix": "the sweep's shape at its most parallel: eight streams per warp, each a "
                       "random 1 KB row read with one 256-bit load per lane and a random "
                       "256-byte row reduced with red.v2 (16 B : 4 B per segment*group), best "
                       "of 8, 16 and 24 warps per SM",
           "how": "simplemoc-kernel_gb300/csrc/moc_peaks.cu via bench.py --peaks: "
                  "CUDA events, mean of 5 launches after 1 warm-up",
           "clocks": clk, "date": time.strftime("%Y-%m-%d %H:%M:%S UTC", time.gmtime())}
    return out


def reference_arm(args, workload):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    r = cpu_baseline(workload, args.cpu_sample_tracks, args.steps, args.warmup,
                     args.table_points if args.exp == "table" else 0)
    line = {
        "impl": "reference", "metric": METRIC, "value": r["value"], "unit": UNIT,
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r["s_per_step"] * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 generator, same inputs as the GPU arm)",
        "config": config_of(args, workload),
        "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": r["cores"],
                         "kind": "port", "sample": r["sample"], "compiler": r["compiler"]},
        "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def config_of(args, w) -> dict:
    return {"workload": w.name, "segments": w.segments, "groups": w.groups,
            "tracks": w.tracks, "regions": w.regions, "intervals": w.intervals,
            "exp_mode": args.exp,
            "form": ("plain FP32 (reference computation, drop-in)" if args.precision == "fp32"
                     else f"precision form {args.precision} (FP32 tallies)"),
            "l2": "flushed between steps (256 MiB write); 0.5 GB of descriptors per step "
                  "exceeds L2", "parallelism": "replicas only (one sweep per GPU)"}


def reference_bytes_per_unit(I: int, G: int) -> float:
    """L2 bytes per segment*group of the reference's own access pattern: sigT 4 B, the
    source rows the axial fit reads (two at the first and last interval, three inside:
    4 (2*2 + 3*(I-2)) / I B), the tally 4 B, and an 8-byte descriptor per segment (8/G).
    At I = 5, G = 128: 18.46 B."""
    return 4.0 + 4.0 * (2 * 2 + 3 * (I - 2)) / I + 4.0 + 8.0 / G


TRAFFIC_FILE = os.path.join(ROOT, "profiles", "sweep_fwd_50M_g128_traffic.json")


def sweep_roofline(hp, sweep_ms: float, prep_ms: float, split_ms: float) -> dict:
    """The sweep kernel against the measured peaks. achieved = algorithmic L2 bytes per
    launch / the kernel's mean event time, in two byte models: the reference's access
    pattern (18.46 B per segment*group at 50M x 128) and this layout's (the 16-byte cell
    block + descriptors + the 4-byte tally, 20.07 B). peak = the stronger of the two
    measured gather+reduction mixes (profiles/peaks_gb300.json, bench.py --peaks). The other
    resources (FP32, MUFU, HBM) are timed at their measured peaks; the largest binds."""
    peaks = load_peaks()
    units = float(hp.S) * hp.G
    sweep_s = sweep_ms * 1e-3
    per = l2_bytes_per_unit(hp.I, hp.G)
    layout_b = per["gather"] + per["reduce"]
    ref_b = reference_bytes_per_unit(hp.I, hp.G)
    roof = {"bound": "l2", "unit": "GB/s",
            "achieved": ref_b * units / sweep_s / 1e9,
            "algorithmic_bytes_per_unit": ref_b,
            "bytes_model": "the reference's access pattern: sigT + the fit's source rows + "
                           "tally + descriptor (18.46 B per segment*group at 50M x 128)",
            "achieved_layout": layout_b * units / sweep_s / 1e9,
            "layout_bytes_per_unit": layout_b,
            "units_per_launch": units, "sweep_ms": sweep_ms, "prep_ms": prep_ms,
            "split_ms": split_ms, "traffic": None}
    mixes = {k: peaks[k] for k in ("l2_mix_gbs", "l2_wide_mix_gbs") if peaks.get(k)}
    terms = {}
    if mixes:
        key = max(mixes, key=mixes.get)
        roof["peak"] = mixes[key]
        roof["peak_source"] = (f"{key}, measured {peaks.get('peaks_measured')} on "
                               f"{peaks.get('date', 'an undated run')} at SM clock "
                               f"{peaks.get('clocks', {}).get('sm_mhz')} MHz")
        roof["frac"] = roof["achieved"] / roof["peak"]
        roof["frac_layout"] = roof["achieved_layout"] / roof["peak"]
        terms["l2"] = ref_b * units / (roof["peak"] * 1e9) * 1e3
        fp32 = max(peaks.get("fp32_fma_tflops", 0.0), peaks.get("fp32_fma2_tflops", 0.0))
        terms["fp32"] = FP32_OPS_PER_UNIT * units / (fp32 * 1e12 / 2) * 1e3
        terms["mufu"] = MUFU_OPS_PER_UNIT * units / (peaks["mufu_ex2_gops"] * 1e9) * 1e3
    else:
        roof["peak"] = None
        roof["frac"] = None
    hbm_bytes = hbm_compulsory_bytes(hp)
    terms["hbm"] = hbm_bytes / (peaks["hbm_gbs"] * 1e9) * 1e3
    roof["terms_ms"] = terms
    binding = max(terms, key=terms.get)
    roof["binding_term"] = binding
    roof["binding_frac"] = terms[binding] / sweep_ms
    roof["hbm"] = {"compulsory_bytes": hbm_bytes, "achieved_gbs": hbm_bytes / sweep_s / 1e9,
                   "peak_gbs": peaks["hbm_gbs"], "frac": hbm_bytes / sweep_s / 1e9 / peaks["hbm_gbs"],
                   "peak_source": peaks["hbm_source"]}
    if os.path.exists(TRAFFIC_FILE) and hp.S == 50_000_000 and hp.G == 128:
        with open(TRAFFIC_FILE) as f:
            tr = json.load(f)
        roof["traffic"] = tr.get("dram_bytes_per_launch")
        roof["traffic_source"] = {k: tr.get(k) for k in ("kernel", "captured", "command",
                                                         "lts_bytes_per_launch")}
    return roof


def plain_timing(h, dp, hp, opts, steps: int, flush, stream) -> dict:
    """A plain-form sweep timed as the headline is: 3 warm-up calls, then `steps` calls each
    after an L2 flush, CUDA events around each call on its stream, the sweep kernel's own
    events inside the library."""
    import torch

    units = float(hp.S) * hp.G
    for _ in range(3):
        h.fwd(dp, opts, stream)
    if h.synchronize(stream):
        raise RuntimeError("device error")
    step_ms, sweep_ms = [], []
    for _ in range(steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        h.fwd(dp, opts, stream)
        e1.record(stream)
        t = h.timings()
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        sweep_ms.append(t.sweep_ms)
    if h.synchronize(stream):
        raise RuntimeError("device error")
    ms = statistics.mean(step_ms)
    return {"segments": hp.S, "groups": hp.G, "tracks": hp.T, "regions": hp.R,
            "ms_per_step": ms, "sweep_ms": statistics.mean(sweep_ms),
            "value": units / (ms * 1e-3), "unit": UNIT, "steps": steps}


def gpu_arm(args, workload):
    import numpy as np
    import torch

    import mocatt

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    hp = mocatt.generate(workload)
    dp = mocatt.DeviceProblem(hp, dev)
    h = mocatt.Handle(local)
    kw = dict(profile=1, precision=getattr(mocatt, PRECISION_ARG[args.precision]))
    if args.exp == "table":
        kw.update(exp_mode=mocatt.MOC_EXP_TABLE, table_points=args.table_points, table_max=10.0)
    opts = mocatt.default_opts(**kw)
    stream = torch.cuda.current_stream(dev)
    units = float(hp.S) * hp.G
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    for _ in range(args.warmup):
        h.fwd(dp, opts, stream)
    torch.cuda.synchronize(dev)
    if h.synchronize(stream):
        raise RuntimeError("device error during warm-up")

    gpu_index = local
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis and vis.split(",")[local].strip().isdigit():
        gpu_index = int(vis.split(",")[local])
    clocks = ClockSampler(gpu_index)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    step_ms, sweep_ms, prep_ms, split_ms = [], [], [], []
    launches = 0
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        h.fwd(dp, opts, stream)
        e1.record(stream)
        t = h.timings()  # waits for this step's kernels
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        sweep_ms.append(t.sweep_ms)
        prep_ms.append(t.prep_ms)
        split_ms.append(t.split_ms)
        launches += t.launches
    torch.cuda.synchronize(dev)
    if ws > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    if h.synchronize(stream):
        raise RuntimeError("device error during the timed steps")
    total_ms = float(sum(step_ms))
    if ws > 1:
        tt = torch.tensor([total_ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(tt.item())
    value = ws * units * args.steps / (total_ms * 1e-3)

    # ---- end to end through the host entry point, page-locked host arrays ----------
    e2e = None
    if not args.no_e2e:
        pinned = hp.copy()
        for name in mocatt.DeviceProblem.NAMES:
            a = getattr(hp, name)
            t_ = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
            setattr(pinned, name, t_.numpy())
        h2d = sum(getattr(pinned, n).nbytes for n in mocatt.DeviceProblem.NAMES)
        d2h = pinned.psi.nbytes + pinned.fine_flux.nbytes
        e2e_steps = max(1, min(args.steps, 5))
        h.fwd_host(pinned, opts)  # warm-up (sizes the device copies once)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            h.fwd_host(pinned, opts)
        e2e_s = (time.perf_counter() - t0) / e2e_steps
        e2e = {"value": ws * units / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
               "call": "moc_attenuate_fwd_host on page-locked host arrays, returns synced: "
                       "the arrays are mapped, so the sweep reads descriptors, offsets "
                       "and psi in place over the host link and writes psi back there; "
                       "sigT and source are copied up first; the tallies start at zero "
                       "on the device and a last pass adds them into the mapped "
                       "fine_flux in place"}

    if rank != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return

    # ---- roofline of the sweep kernel, against peaks measured now --------------------
    if not args.no_peaks_run:
        try:
            IN_RUN_PEAKS.update(run_peaks())
        except (OSError, RuntimeError) as e:
            print(f"warning: roofline microbenchmarks failed ({e}); using the committed "
                  f"peaks", file=sys.stderr)
    roof = sweep_roofline(hp, statistics.mean(sweep_ms), statistics.mean(prep_ms),
                          statistics.mean(split_ms))

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 generator; the reference draws random inputs "
                "itself and reads no dataset)",
        "config": config_of(args, workload), "roofline": roof, "e2e": e2e,
        "gpu_launches": launches, "clocks": clk,
    }
    if ws == 1 and args.exp == "full" and args.precision == "fp32" and not args.no_extra:
        # the other plain-form lines: the table exp mode on this workload, and the
        # reference's CPU-sized problem (1M segments x 64 groups)
        def table_line():
            r = plain_timing(h, dp, hp, mocatt.default_opts(
                profile=1, exp_mode=mocatt.MOC_EXP_TABLE, table_points=args.table_points,
                table_max=10.0), args.steps, flush, stream)
            r.update(workload=workload.name, exp_mode="table", table_points=args.table_points,
                     table_max=10.0)
            return r

        def small_line():
            small = mocatt.generate(mocatt.WORKLOADS["sweep_1M_g64"])
            sdp = mocatt.DeviceProblem(small, dev)
            r = plain_timing(h, sdp, small, mocatt.default_opts(profile=1), args.steps, flush,
                             stream)
            r.update(workload="sweep_1M_g64", exp_mode="full")
            return r

        optional_section(line, "table", table_line)
        optional_section(line, "sweep_1M_g64", small_line)
    if not args.no_forms and ws == 1:
        optional_section(line, "forms",
                         lambda: forms_section(h, dp, hp, statistics.mean(sweep_ms)))
    if not args.no_tracks and ws == 1:
        optional_section(line, "tracks", lambda: tracks_section(h))
        optional_section(line, "transport", lambda: transport_section(h))
    if not args.no_cpu_baseline and ws == 1:
        def cpu_line():
            r = cpu_baseline(workload, args.cpu_sample_tracks, 3, 1,
                             args.table_points if args.exp == "table" else 0)
            return {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": "port",
                    "sample": r["sample"], "compiler": r["compiler"]}

        optional_section(line, "cpu_baseline", cpu_line)
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def optional_section(line: dict, key: str, fn) -> None:
    """line[key] = fn(); a section beside the headline that fails records its error there
    (and on stderr) instead of costing the whole line."""
    try:
        line[key] = fn()
    except Exception as e:  # noqa: BLE001 - any failure of an optional section
        msg = f"{type(e).__name__}: {e}"
        print(f"warning: bench section {key} failed: {msg}", file=sys.stderr)
        line[key] = {"error": msg[:400]}


def _time_fwd(h, dp, opts, reps=3):
    """Median device time of prep + split passes + sweep + finish over reps calls (after
    one warm-up)."""
    h.fwd(dp, opts)
    ts = []
    for _ in range(reps):
        h.fwd(dp, opts)
        t = h.timings()
        ts.append(t.prep_ms + t.split_ms + t.sweep_ms + t.finish_ms)
    if h.synchronize():
        raise RuntimeError("device error")
    return statistics.median(ts)


def _adjoint_vs_forward(h, dp, opts, fwd_ms, reps=3):
    """Median device time of moc_attenuate_adj (every pass: cell blocks, split, recording,
    reverse, finish) on a problem, against one forward sweep of it (fwd_ms)."""
    import torch

    w = torch.randn_like(dp.fine_flux)
    v = torch.randn_like(dp.psi)
    h.adj(dp, w, v, opts)
    ts = []
    for _ in range(reps):
        h.adj(dp, w, v, opts)
        t = h.timings()
        ts.append(t.prep_ms + t.split_ms + t.sweep_ms + t.finish_ms)
    if h.synchronize():
        raise RuntimeError("device error in the adjoint")
    adj = statistics.median(ts)
    return {"segments": int(dp.S), "groups": int(dp.G), "forward_ms": fwd_ms,
            "adjoint_ms": adj, "ratio": adj / fwd_ms}


# The precision forms and the workload they are graded and timed on: the wide-tau inputs
# (sigT ~ logU(1e-3, 20), ds ~ U(1e-3, 2), tau over ~[1e-6, 40]) at 50M segments x 128
# groups. Their accuracy is measured in the same run against the FP64 oracle (on the values
# each form stores) on the first FORMS_SAMPLE_TRACKS tracks swept as a problem of their own;
# tests/test_forms_gpu.py grades the whole workload.
FORMS_WORKLOAD = "widetau_50M_g128"
FORMS_SAMPLE_TRACKS = 10_000
PRECISION_FORMS = {
    "plain_fp32": ("MOC_PREC_FP32", "MOC_TALLY_ATOMIC_FP32"),
    "fp32_stable": ("MOC_PREC_FP32_STABLE", "MOC_TALLY_ATOMIC_FP32"),
    "fp32_stable_compensated": ("MOC_PREC_FP32_STABLE", "MOC_TALLY_COMPENSATED"),
    "fp32_stable_fp64": ("MOC_PREC_FP32_STABLE", "MOC_TALLY_FP64"),
    "bf16_stable": ("MOC_PREC_BF16", "MOC_TALLY_ATOMIC_FP32"),
    "bf16_stable_compensated": ("MOC_PREC_BF16", "MOC_TALLY_COMPENSATED"),
    "fp16_stable": ("MOC_PREC_FP16", "MOC_TALLY_ATOMIC_FP32"),
}
# The rule that picks chosen_form: normwise relative error <= 1e-5 for psi and for
# fine_flux, against the FP64 oracle on the stored values.
FORMS_TOL = 1e-5


def _form_errors(hp, psi, ff, ref) -> dict:
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import parity

    out = {}
    G = hp.G
    for name, x, r in (("psi", psi, ref["psi"]), ("fine_flux", ff, ref["ff"])):
        mx, rms = parity.rel_err(x[:, :G], r[:, :G])
        d = x[:, :G].astype(np.float64) - r[:, :G]
        out[name] = {"max_rel": mx, "rms_rel": rms,
                     "normwise": float(np.linalg.norm(d) / np.linalg.norm(r[:, :G]))}
    return out


def precision_section(h) -> dict:
    """The precision forms on the wide-tau workload: every form timed on the full workload
    (all passes, median of 3 after a warm-up), its error measured in this run on a track
    sample against the FP64 oracle (test infrastructure, here only as the checker), and the
    chosen form: the fastest non-plain form that meets the rule."""
    import torch

    import mocatt

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    w = mocatt.WORKLOADS[FORMS_WORKLOAD]
    whp = mocatt.generate(w)
    wdp = mocatt.DeviceProblem(whp)
    units = float(whp.S) * whp.G
    forms = {n: (getattr(mocatt, p), getattr(mocatt, t)) for n, (p, t) in PRECISION_FORMS.items()}
    out = {"workload": FORMS_WORKLOAD, "segments": whp.S, "groups": whp.G, "tracks": whp.T,
           "regions": whp.R}
    times = {n: _time_fwd(h, wdp, mocatt.default_opts(profile=1, precision=p, tally=t))
             for n, (p, t) in forms.items()}
    del wdp
    torch.cuda.empty_cache()

    sub = whp.subset_tracks(range(min(FORMS_SAMPLE_TRACKS, whp.T)))
    sdp = mocatt.DeviceProblem(sub)
    psi0 = sdp.psi.clone()
    results = {}
    for n, (p, t) in forms.items():
        sdp.psi.copy_(psi0)
        sdp.fine_flux.zero_()
        h.fwd(sdp, mocatt.default_opts(precision=p, tally=t))
        if h.synchronize():
            raise RuntimeError(f"device error in form {n}")
        results[n] = (sdp.to_host("psi"), sdp.to_host("fine_flux"))
    del sdp
    threads = os.cpu_count() or 1
    kind = {mocatt.MOC_PREC_FP32: mocatt.MOC_PREC_FP32_STABLE,
            mocatt.MOC_PREC_FP32_STABLE: mocatt.MOC_PREC_FP32_STABLE,
            mocatt.MOC_PREC_BF16: mocatt.MOC_PREC_BF16, mocatt.MOC_PREC_FP16: mocatt.MOC_PREC_FP16}
    errors = {}
    for storage in sorted(set(kind.values())):
        qp, coef = oracle.quantized_inputs(sub, storage)
        ref = oracle.fwd_fp64_coef(qp, coef, threads=threads)
        for n, (p, _) in forms.items():
            if kind[p] == storage:
                errors[n] = _form_errors(sub, *results[n], ref)
        del ref
    t_plain = times["plain_fp32"]
    precision = {}
    for n in forms:
        e = errors[n]
        ok = e["psi"]["normwise"] <= FORMS_TOL and e["fine_flux"]["normwise"] <= FORMS_TOL
        precision[n] = {"ms": times[n], "value": units / (times[n] * 1e-3),
                        "speed_vs_plain": t_plain / times[n], "error": e, "meets_rule": ok}
    ok = [n for n in precision if n != "plain_fp32" and precision[n]["meets_rule"]]
    out["forms"] = precision
    out["chosen_form"] = max(ok, key=lambda n: precision[n]["value"]) if ok else None
    out["chosen_rule"] = ("normwise <= 1e-5: the fastest precision form whose psi and "
                          "fine_flux normwise relative errors are <= 1e-5 against the FP64 "
                          "oracle on the values it stores (RMS and maximum relative errors "
                          "are reported beside them, not part of the rule)")
    out["error_sample"] = (f"the first {sub.T} of {whp.T} tracks ({sub.S} segments x {sub.G} "
                           f"groups) swept as a problem of their own, FP64 oracle on {threads} "
                           f"host threads; the whole workload is graded by "
                           f"tests/test_forms_gpu.py")
    return out


def forms_section(h, dp, hp, plain_sweep_ms) -> dict:
    """The three forms beside the plain sweep, timed on this GPU: the precision forms on
    their own wide-tau workload at full size, with their accuracy measured in this run
    (precision_section), the adjoint's cost relative to one forward sweep, and the batching
    form against one launch per problem."""
    import ctypes as C

    import torch

    import mocatt

    out = {"precision": precision_section(h)}
    plain = mocatt.default_opts(profile=1)
    t_plain = _time_fwd(h, dp, plain)

    # adjoint: on the bench problem (50M x 128, the size the adjoint's cost target is
    # stated at), on the gradient-check workload (5,000 lognormal tracks, ~2M segments,
    # G = 64) and on the reference's CPU-sized problem (1M x 64)
    out["adjoint"] = {"sweep_50M_g128": _adjoint_vs_forward(h, dp, plain, t_plain)}
    for name in ("adjoint_2M_g64", "sweep_1M_g64"):
        ahp = mocatt.generate(mocatt.WORKLOADS[name])
        adp = mocatt.DeviceProblem(ahp)
        out["adjoint"][name] = _adjoint_vs_forward(h, adp, plain, _time_fwd(h, adp, plain, 7),
                                                   7)
        del adp

    # batching: three problems (G = 16, 70, 128), one graph-captured launch
    bh = [mocatt.generate(mocatt.WORKLOADS[n])
          for n in ("batch_20k_g16", "batch_20k_g70", "batch_20k_g128")]
    bdp = [mocatt.DeviceProblem(x) for x in bh]
    t_single = sum(_time_fwd(h, d, plain) for d in bdp)
    arr = (mocatt.MocProblem * 3)(*[d.c_struct() for d in bdp])
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    res = mocatt.MocTuneResult()
    h.check(mocatt.lib().moc_autotune_batch(h.ptr, arr, 3, C.byref(plain), sp, C.byref(res)))
    h.check(mocatt.lib().moc_attenuate_fwd_batch(h.ptr, arr, 3, C.byref(plain), sp))
    bt = []
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        h.check(mocatt.lib().moc_attenuate_fwd_batch(h.ptr, arr, 3, C.byref(plain), sp))
        e1.record(stream)
        e1.synchronize()
        bt.append(e0.elapsed_time(e1))
    if h.synchronize():
        raise RuntimeError("device error")
    t_batch = statistics.median(bt)
    bunits = sum(float(x.S) * x.G for x in bh)
    out["batching"] = {"problems": [{"G": x.G, "tracks": x.T, "segments": x.S} for x in bh],
                       "one_launch_ms": t_batch, "three_calls_ms": t_single,
                       "value": bunits / (t_batch * 1e-3), "speedup": t_single / t_batch,
                       "tuned": {"vec": res.vec, "warps_per_block": res.warps_per_block,
                                 "tracks_per_block": res.tracks_per_block}}
    return out


# Track generation (include/moc_tracks.h): a 17 x 17 assembly 200 cm tall, 3 fuel rings,
# 40 axial source regions of 5 fine intervals; 8 azimuths x 4 polar bins, 0.1 cm radial
# and 2 cm axial track spacing: 747,024 tracks, 58.5M segments.
TRACKS_GEOMETRY = dict(nx=17, ny=17, n_rings=3, n_axial=40, n_intervals=5, pitch=1.26,
                       fuel_radius=0.54, height=200.0)
TRACKS_QUADRATURE = dict(n_azim=8, n_polar=4, spacing=0.1, axial_spacing=2.0)
# FP64 arithmetic instructions per segment of the walk (DADD 11.49 + DMUL 12.52 + DFMA
# 1.67, thread level), from ncu's instruction counters on this workload
# (profiles/trace_walk_assembly_58M_ncu.md). The FP64 pipe issues one of them per slot
# whatever its kind, so the peak is the measured DFMA instruction rate.
TRACE_FP64_INST_PER_SEGMENT = 25.68


def tracks_section(h, reps: int = 5) -> dict:
    """moc_trace_count + moc_trace_segments on the assembly workload, CUDA events around
    the pair (their host synchronisations included), median of reps after one warm-up;
    the oracle's OpenMP tracer timed on this host beside it."""
    import numpy as np
    import torch

    import mocatt

    g = mocatt.geometry(**TRACKS_GEOMETRY)
    q = mocatt.quadrature(**TRACKS_QUADRATURE)
    plan = mocatt.tracks_plan(g, q)
    T = len(plan)
    d = torch.from_numpy(plan.view(np.uint8)).cuda()
    off, reg, itv, ds = h.trace(g, d, T)
    if h.synchronize():
        raise RuntimeError("device error in track generation")
    S = int(off[-1].item())
    L = mocatt.lib()
    st = torch.cuda.current_stream()
    n = C.c_int64()
    ts = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        h.check(L.moc_trace_count(h.ptr, C.byref(g), d.data_ptr(), T, off.data_ptr(),
                                  C.byref(n), C.c_void_p(st.cuda_stream)))
        h.check(L.moc_trace_segments(h.ptr, C.byref(g), d.data_ptr(), T, off.data_ptr(),
                                     reg.data_ptr(), itv.data_ptr(), ds.data_ptr(),
                                     C.c_void_p(st.cuda_stream)))
        e1.record(st)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    if h.synchronize() or n.value != S:
        raise RuntimeError("track generation changed between calls")
    ms = float(np.median(ts))
    out = {"workload": "assembly_17x17_58M", "geometry": TRACKS_GEOMETRY,
           "quadrature": TRACKS_QUADRATURE, "tracks": T, "segments": S,
           "ms": ms, "value": S / (ms * 1e-3), "unit": "segments/s",
           "timed": "moc_trace_count + moc_trace_segments (bounds, one walk, scans, "
                    "compaction, two host synchronisations), CUDA events, median of "
                    f"{reps} after 1 warm-up",
           "parity": "bit for bit against the oracle's sort-all-crossings tracer "
                     "(tests/test_tracks_gpu.py)"}
    peaks = load_peaks()
    if peaks.get("fp64_fma_tflops"):
        ach = TRACE_FP64_INST_PER_SEGMENT * S / (ms * 1e-3) / 1e9
        peak = peaks["fp64_fma_tflops"] * 1e3 / 2  # DFMA instructions per second
        out["roofline"] = {"bound": "fp64 pipe", "unit": "G FP64 instructions/s",
                           "achieved": ach, "peak": peak, "frac": ach / peak,
                           "inst_per_segment": TRACE_FP64_INST_PER_SEGMENT,
                           "peak_source": "profiles/peaks_gb300.json fp64_fma_tflops / 2 "
                                          "(bench.py --peaks, csrc/moc_peaks.cu)",
                           "time": "the whole timed pair, not the walk kernel alone"}
    # the CPU arm: the oracle (test infrastructure), here only as the timed baseline
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    threads = os.cpu_count() or 1
    oracle.trace_count_omp(g, plan[: min(T, 20000)], threads)  # warm-up
    t0 = time.perf_counter()
    n_cpu = oracle.trace_count_omp(g, plan, threads)
    cpu_s = time.perf_counter() - t0
    if n_cpu != S:
        raise RuntimeError(f"oracle counts {n_cpu} segments, the GPU {S}")
    out["cpu_baseline"] = {"value": S / cpu_s, "unit": "segments/s", "cores": threads,
                           "kind": "port",
                           "sample": "the whole plan (the reference has no tracer: the "
                                     "oracle's tracer, OpenMP over tracks, counting)"}
    return out


def transport_section(h, iterations: int = 10) -> dict:
    """The power iteration around the sweep (include/moc_transport.h) on the traced
    assembly, both directions, 128 groups, 4 synthetic materials, flat sources, vacuum
    boundaries: moc_power_iteration timed with CUDA events (its per-iteration host
    synchronisation included) after 2 warm-up iterations; the sweep and the source update
    timed apart; the oracle's FP32 source update timed on this host beside it."""
    import numpy as np
    import torch

    import mocatt

    G = 128
    g = mocatt.geometry(**TRACKS_GEOMETRY)
    q = mocatt.quadrature(both_directions=1, **TRACKS_QUADRATURE)
    plan = mocatt.tracks_plan(g, q)
    d = torch.from_numpy(plan.view(np.uint8)).cuda()
    off, reg, itv, ds = h.trace(g, d, len(plan))
    T, S = len(plan), int(off[-1].item())
    R, I = mocatt.geometry_regions(g), g.n_intervals
    xs = mocatt.synth_xs(4, G)
    dxs = mocatt.DeviceXS(xs)
    mat = mocatt.geometry_materials(g)
    vol = mocatt.geometry_volumes(g)
    dmat, dvol = torch.from_numpy(mat).cuda(), torch.from_numpy(vol).cuda()
    ff = torch.zeros((R * I, xs.Gs), device="cuda")
    ff[:, :G] = dvol[:, None].float()
    dp = mocatt.DeviceProblem.from_tensors(
        R, I, G, xs.Gs, T, S, track_offsets=off, seg_region=reg, seg_interval=itv, seg_ds=ds,
        sigT=h.region_sigT(dxs, dmat), source=torch.zeros_like(ff), fine_flux=ff,
        psi=torch.zeros((T, xs.Gs), device="cuda"))
    opts = mocatt.default_opts(weight=mocatt.tracks_weight(q), zin=0.0, mu=0.0, mu2=0.0)
    k, _ = h.power_iteration(dp, opts, dxs, dmat, dvol, 1.0, 2)
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    k, it = h.power_iteration(dp, opts, dxs, dmat, dvol, k, iterations)
    e1.record(st)
    e1.synchronize()
    ms_it = e0.elapsed_time(e1) / it
    popts = mocatt.default_opts(weight=mocatt.tracks_weight(q), zin=0.0, mu=0.0, mu2=0.0,
                                profile=1)
    sweep = _time_fwd(h, dp, popts)
    e0.record(st)
    for _ in range(5):
        h.source_update(dxs, dmat, I, dvol, dp.fine_flux, k)
    e1.record(st)
    e1.synchronize()
    upd_ms = e0.elapsed_time(e1) / 5
    if h.synchronize():
        raise RuntimeError("device error in the power iteration")
    cells = R * I
    flops = 2.0 * G * (G + 1) * cells  # the scattering and fission chains
    peaks = load_peaks()
    out = {"workload": "assembly_17x17_both_directions_g128", "tracks": T, "segments": S,
           "groups": G, "cells": cells, "materials": xs.M, "iterations": it, "k": k,
           "ms_per_iteration": ms_it, "value": 1e3 / ms_it, "unit": "power iterations/s",
           "attenuations_per_s": S * G / (ms_it * 1e-3),
           "sweep_ms": sweep, "source_update_ms": upd_ms,
           "timed": "moc_power_iteration over the iterations (psi and tally resets, sweep, "
                    "source update, one host synchronisation each), CUDA events",
           "parity": "source update bit for bit against the oracle's FP32 restatement; "
                     "iteration against the oracle's (tests/test_transport_gpu.py)"}
    if peaks.get("fp32_fma_tflops"):
        ach = flops / (upd_ms * 1e-3) / 1e12
        out["source_update_roofline"] = {
            "bound": "fp32", "unit": "TFLOP/s", "achieved": ach,
            "peak": peaks["fp32_fma_tflops"], "frac": ach / peaks["fp32_fma_tflops"],
            "flops_per_cell": 2.0 * G * (G + 1),
            "peak_source": "profiles/peaks_gb300.json fp32_fma_tflops"}
    # the CPU arm: the oracle's source update (test infrastructure), one thread, on the
    # first 20,000 cells of the same tallies
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    n = min(cells, 20000)
    nreg = (n + I - 1) // I
    tally = dp.fine_flux[: nreg * I].cpu().numpy()
    t0 = time.perf_counter()
    oracle.source_update(xs, mat[:nreg], nreg, I, vol[: nreg * I], tally, k)
    cpu_s = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": nreg * I / cpu_s, "unit": "cells/s (source update)",
                           "gpu_value": cells / (upd_ms * 1e-3), "cores": 1, "kind": "port",
                           "sample": f"the oracle's FP32 source update of the first "
                                     f"{nreg * I} of {cells} cells, 128 groups"}
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mine", choices=["mine", "reference"])
    ap.add_argument("--workload", default="sweep_50M_g128")
    ap.add_argument("--exp", default="full", choices=["full", "table"])
    ap.add_argument("--precision", default="fp32", choices=sorted(PRECISION_ARG),
                    help="the form the timed steps sweep (default: the plain FP32 form)")
    ap.add_argument("--table-points", type=int, default=10_000)
    ap.add_argument("--cpu-sample-tracks", type=int, default=20_000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg")
    ap.add_argument("--no-tracks", action="store_true",
                    help="skip the track-generation line")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the precision / adjoint / batching measurements")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the table-mode and 1M x 64 lines")
    ap.add_argument("--no-peaks-run", action="store_true",
                    help="take the roofline peaks from profiles/peaks_gb300.json instead "
                         "of measuring them after the timed steps")
    ap.add_argument("--segments", type=int, default=0,
                    help="override the workload's segment count (smaller profiling cases)")
    ap.add_argument("--tracks", type=int, default=0, help="override the track count")
    ap.add_argument("--peaks", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "mine" and not args.peaks:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)

    import mocatt

    workload = mocatt.WORKLOADS[args.workload]
    if args.segments:
        workload = workload.with_(segments=args.segments)
    if args.tracks:
        workload = workload.with_(tracks=args.tracks)
    if args.peaks:
        out = run_peaks()
        os.makedirs(os.path.dirname(PEAKS_FILE), exist_ok=True)
        with open(PEAKS_FILE, "w") as f:
            json.dump(out, f, indent=1)
        print(json.dumps(out))
        return
    if args.impl == "reference":
        reference_arm(args, workload)
    else:
        gpu_arm(args, workload)


if __name__ == "__main__":
    main()
