"""Benchmark: Earth LUT rebuilds per second on one GB300.

Workload (one "step"): a batched rebuild of B Earth atmospheres with the
reference's default LUT shape (transmittance 256x64, scattering NU 8 x MU_S 32
x MU 128 x R 32 = 256x128x32 RGBA, irradiance 64x16), 4 scattering orders,
3 wavelengths (680/550/440 nm), combined scattering textures, FP32 -- the
Earth parameters of atmosphere/demo/demo.cc:188-284 with max sun zenith 102
degrees.  A batch of B >= 4 (64 MB of LUTs and temporaries per instance) is
several times larger than the 129 MB L2, so no explicit L2 flush is needed
between steps.

Rank 0 prints one compact JSON line (the headline figures); the full record
(per-pass times, parity, the mixed batch, serving, the other configurations)
goes to stderr as one line starting with "detail: " and, when ATMO_BENCH_OUT
names a directory, to bench_detail.json there.  Reported:
  value          batched rebuilds/s (device-timed with CUDA events),
  e2e            the same through the public C API with host buffers: every
                 step's atmosphere parameters go host->device and all its LUTs
                 come back device->host into pinned memory inside the timed
                 region (two batches alternate, so a step's read-back overlaps
                 the next step's rebuilds),
  single_and_plain  single-rebuild p50 / p99 latency (fast path), the plain
                 per-texel kernels' rebuilds/s and the batched / plain ratio,
  roofline       the scattering-density kernel (the dominant one) against this
                 GPU's FP32 FMA throughput measured in the same run: the FP32
                 operations the kernel executes per direction sample (ncu SASS
                 op counters) x samples / launch time; the reference
                 algorithm's operation count (tests/golden/flops_config0.json)
                 over the same time is reported apart, as algorithmic_tflops,
  parity         per-LUT max / p99 relative error of the benchmarked LUTs at
                 the FP64 reference's committed sampled texels,
  configs        the spectral-precision (15 wavelengths, FP16 LUTs) and the
                 high-resolution (8 orders) rebuilds: device-timed ms and
                 error against the FP64 GPU oracle's committed sampled texels,
  batched_mixed  256 seeded planets of uneven LUT shapes ({half, default,
                 double-R}) and 2-6 orders in one batched pass sequence,
  serving        a short seeded Poisson stream (2000 req/s, 10% rebuilds of
                 such planets, 90% shading of 1920x1080 pinhole views with the
                 three render functions) through atmo_server: p50/p99 latency
                 per request type, split into queue and run time,
  cpu_baseline   one whole, unsampled rebuild by the FP64 CPU oracle (the
                 reference's CPU algorithm restated), all host threads.

--impl reference times the reference's CPU algorithm (the oracle port of
atmosphere/reference/model.cc + functions.glsl) on the host cores instead:
every warm-up and timed step is one whole, unsampled rebuild.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Earth LUT rebuilds/s batched vs plain on 1 GB300 @<=1e-3 vs FP64; p99 ms"
UNIT = "rebuilds/s"
WORKLOAD = ("Earth LUT rebuild, 256x64/256x128x32/64x16 RGBA FP32, 4 orders, 3 wavelengths, "
            "combined")
# FP32 operations per direction sample that the fast scattering-density kernel
# executes, from ncu's SASS op counters over one launch (an FMA counts 2, a
# packed FP32x2 instruction 2 or 4): order 2 evaluates single scattering with
# its phase functions, higher orders one radiance table (one merged sky +
# ground table on the rows that hit the ground).
DENSITY_FLOPS_PER_SAMPLE = {2: 48.9, 3: 20.1}
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one density
# launch over 16 default-shape Earth instances, from a one-pass ncu capture of
# the batch-16 rebuild (python -m precomputed_atmospheric_scattering_gb300.
# profile_case --batch 16): order 2 read 67.8 MB + wrote 207.4 MB, orders 3
# and 4 read 36.0 MB + wrote 207.5 MB.
DENSITY_DRAM_BYTES_B16 = {2: 275.27e6, 3: 243.53e6}
# Bytes a density launch must move per default-shape Earth instance: the
# previous order's mu rows that its 16 theta samples interpolate (484 unique
# rows of the 4,096 per instance, 1.98 MB per species; two species at order
# 2) and the 16.8 MB delta-density LUT it writes.  The measured bytes fall
# below this because the last ~60 MB of writes are still dirty in the 129 MB
# L2 when a launch ends (they are written back during the next one).
DENSITY_COMPULSORY_BYTES = {2: 2 * 1982464 + 16777216, 3: 1982464 + 16777216}
# The reference algorithm's operation counts of this workload, frozen from the
# oracle's counting build (tests/golden/make_flops.py): adds and muls of the
# shader arithmetic per direction sample of each density launch, and per
# rebuild.
FLOPS_CONFIG0 = os.path.join(ROOT, "tests", "golden", "flops_config0.json")


def hbm_peak():
    """(GB/s, source): the measured copy bandwidth of the GB300s, else
    the recipe's fallback figure."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (measured)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "6.8 TB/s (fallback: MEASURED_PEAKS.json absent)"


def reference_flops():
    with open(FLOPS_CONFIG0) as f:
        d = json.load(f)
    per_sample = {l["order"]: l["flops_per_unit"] for l in d["counts"]["launches"]
                  if l["pass"] == "scattering_density"}
    return per_sample, d["counts"]["total"]["flops"]


def rnd(x, digits=4):
    """x rounded to `digits` significant digits (floats in nested values)."""
    if isinstance(x, float):
        return float("%.*g" % (digits, x)) if math.isfinite(x) else None
    if isinstance(x, dict):
        return {k: rnd(v, digits) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [rnd(v, digits) for v in x]
    return x


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--warm-seconds", type=float, default=8.0,
                   help="keep running untimed steps (at least --warmup) until the GPU has "
                        "been busy this long: a GPU that starts idle runs the L1-bound "
                        "kernels ~3%% slower for its first seconds")
    p.add_argument("--batch", type=int, default=16, help="atmospheres per batched step")
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-serving", action="store_true",
                   help="skip the mixed-batch and serving measurements")
    p.add_argument("--serving-seconds", type=float, default=3.0)
    return p.parse_args()


def replica_rate(local_seconds, local_units, world, device=None):
    """Whole-job rate of independent replicas: the units every rank processed
    over the slowest rank's time (max over ranks; no data-path collective,
    only this reduction of the timings)."""
    if world <= 1:
        return local_units / local_seconds, local_seconds
    import torch
    import torch.distributed as dist
    t = torch.tensor([local_seconds, local_units], dtype=torch.float64, device=device)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t[1].item()) / float(mx[0].item()), float(mx[0].item())


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (FP64 restatement of the reference CPU model).
# ---------------------------------------------------------------------------
def cpu_rebuild_seconds(threads=0, by_rows=False):
    """(wall seconds, per-pass seconds) of one whole, unsampled rebuild by the
    FP64 oracle.  by_rows: the threads take whole rows and r-slices (the
    reference CPU driver's partition) instead of 64-texel blocks."""
    from oracle import oracle as O
    O.build()
    import ctypes as C
    atm = O.earth_atmosphere()
    shp = O.shape(*O.DEFAULT_SHAPE)
    sec = np.zeros(6)
    t0 = time.perf_counter()
    rc = O.lib().oracle_time_precompute_partitioned(C.byref(atm), C.byref(shp), 4, 1,
                                                    threads, int(by_rows),
                                                    sec.ctypes.data_as(O.dp))
    wall = time.perf_counter() - t0
    if rc != 0:
        raise RuntimeError("oracle timing failed")
    return wall, sec


def cpu_baseline_entry():
    cores = os.cpu_count() or 1
    wall, sec = cpu_rebuild_seconds()
    rows_wall, _ = cpu_rebuild_seconds(by_rows=True)
    return {"value": 1.0 / wall, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "one whole unsampled FP64 oracle rebuild, %d threads: %.1f s"
                      % (cores, wall),
            "reference_partition_rebuilds_per_s": 1.0 / rows_wall,
            "pass_seconds": [round(x, 3) for x in sec]}


def run_reference(args):
    """The reference's CPU algorithm (the FP64 oracle port of
    atmosphere/reference/model.cc + functions.glsl) with every host thread:
    each warm-up and each timed step is one whole, unsampled rebuild."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    t_warm = time.perf_counter()
    for _ in range(args.warmup):
        cpu_rebuild_seconds()
    warm_s = time.perf_counter() - t_warm
    walls = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        wall, _ = cpu_rebuild_seconds()
        walls.append(wall)
    total = time.perf_counter() - t0
    value = args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "batch": 1, "orders": 4,
                   "implementation": "CPU oracle port of atmosphere/reference/model.cc "
                                     "(FP64, all host threads, 64-texel blocks)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "every step one whole, unsampled rebuild; %d warm-up "
                                   "rebuilds (%.0f s), %d timed (%.0f s, min %.1f s, max "
                                   "%.1f s per rebuild)" % (args.warmup, warm_s, args.steps,
                                                            total, min(walls), max(walls))},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(rnd(line, 6)), flush=True)


# ---------------------------------------------------------------------------
# GPU measurement.
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        # The raw samples (the JSON line carries their summary).
        out_dir = os.environ.get("ATMO_BENCH_OUT") or tempfile.gettempdir()
        self.path = os.path.join(out_dir, "clocks_bench_%d.csv" % gpu_index)
        self.gpu = gpu_index

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        try:
            rows = [l.split(",") for l in open(self.path).read().strip().splitlines()]
        except Exception:
            return None
        rows = [[x.strip() for x in r] for r in rows if len(r) >= 9]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i - 5] for r in rows for i in range(5, 9)
                          if r[i].lower() in ("active", "1")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def run_gpu(args):
    import torch
    import precomputed_atmospheric_scattering_gb300 as atmo
    from precomputed_atmospheric_scattering_gb300 import workloads as W

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    atmo.build()
    atmo.lib()
    B = args.batch
    shape = W.DEFAULT
    atms = [W.earth() for _ in range(B)]
    # Block shapes of the row-restructured kernels, timed on this GPU.
    tuning = atmo.autotune(atms[0], shape, 4).as_dict()
    batch = atmo.Batch(atms, [shape] * B, 4, combined=True)
    kernels_per_step = batch.kernel_count()
    stream = torch.cuda.current_stream()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # --- device-timed batched rebuilds -------------------------------------
    t_warm, warm_steps = time.perf_counter(), 0
    while warm_steps < args.warmup or time.perf_counter() - t_warm < args.warm_seconds:
        batch.run(stream)
        torch.cuda.synchronize()
        warm_steps += 1
    warm_s = time.perf_counter() - t_warm
    barrier()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local) as clocks:
        ev[0].record(stream)
        for k in range(args.steps):
            batch.run(stream)
            ev[k + 1].record(stream)
        barrier()
    step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    value, total_s = replica_rate(sum(step_ms) / 1000.0, B * args.steps, world,
                                  device="cuda" if world > 1 else None)

    # --- end to end through the C API with host buffers ---------------------
    # Every step sets its atmospheres (host -> device with the run) and reads
    # all LUTs back into pinned host memory.  Two batches alternate so that the
    # read-back of step k (on a copy stream) overlaps the rebuilds of step k+1.
    kinds = [atmo.LUT_TRANSMITTANCE, atmo.LUT_SCATTERING, atmo.LUT_IRRADIANCE]
    views = [batch.lut_view(0, k) for k in kinds]
    sizes = [v.width * v.height * v.depth * 16 for v in views]
    batches = [batch, atmo.Batch(atms, [shape] * B, 4, combined=True)]
    host = [[[torch.empty(sz // 4, dtype=torch.float32).pin_memory() for sz in sizes]
             for _ in range(B)] for _ in range(2)]
    import ctypes as C
    h2d = B * C.sizeof(atmo.Atmosphere)
    d2h = B * sum(sizes)
    copy_stream = torch.cuda.Stream()
    ran = [torch.cuda.Event(), torch.cuda.Event()]
    copied = [None, None]

    def e2e_step(k):
        slot = k % 2
        b = batches[slot]
        if copied[slot] is not None:
            stream.wait_event(copied[slot])      # its LUTs were read back
        for i in range(B):
            b.set_atmosphere(i, atms[i])
        b.run(stream)
        ran[slot].record(stream)
        copy_stream.wait_event(ran[slot])
        for i in range(B):
            for kind, buf, nb in zip(kinds, host[slot][i], sizes):
                b.copy_lut(i, kind, buf.data_ptr(), nb, copy_stream)
        copied[slot] = torch.cuda.Event()
        copied[slot].record(copy_stream)

    e2e_step(0)
    e2e_step(1)
    copy_stream.synchronize()
    barrier()
    e2e_steps = max(4, args.steps)
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        e2e_step(k)
    copy_stream.synchronize()
    barrier()
    e2e_value, _ = replica_rate(time.perf_counter() - t0, B * e2e_steps, world,
                                device="cuda" if world > 1 else None)
    del batches[1]

    # --- single-instance latency (fast) and the plain path ------------------
    single = atmo.Batch([atms[0]], [shape], 4, combined=True)
    lat = []
    for _ in range(args.warmup):
        single.run(stream)
    for _ in range(max(args.steps, 10)):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        single.run(stream)
        b.record(stream)
        b.synchronize()
        lat.append(a.elapsed_time(b))
    lat.sort()
    p50 = lat[len(lat) // 2]
    p99 = lat[min(len(lat) - 1, int(math.ceil(0.99 * len(lat))) - 1)]
    plain_ms = time_plain(atmo, W, torch, stream, args)
    # The single rebuild's kernels timed one by one (no graph): their sum
    # against the graph replay's p50 is the cost of the launch boundaries.
    single_passes = single.time_passes(stream)
    launch_gaps = {"graph_p50_ms": p50,
                   "sum_of_kernels_ms": sum(ms for _, _, ms in single_passes),
                   "kernels": len(single_passes)}

    # --- error of the benchmarked LUTs against the FP64 reference ------------
    parity = parity_entry(atmo, W, batch, torch)

    # --- roofline of the scattering-density kernel ---------------------------
    peak = atmo.measure_fp32_peak()
    roof, passes_ms = roofline_entry(batch, B, peak, stream, value / world)
    del batch, single
    torch.cuda.empty_cache()

    # --- the spectral-precision and high-resolution configurations ----------
    configs = {"spectral_fp16": run_spectral(atmo, W, torch, stream),
               "hires_8_orders": run_hires(atmo, W, torch, stream)}
    torch.cuda.empty_cache()

    # --- mixed batch (uneven shapes and order counts) and serving -----------
    mixed = run_mixed_batch(atmo, W, torch, stream) if not args.no_serving else None
    serving = half_rate = None
    if not args.no_serving:
        serving = run_serving(atmo, W, torch, args.serving_seconds, rebuild_alone_ms=p50)
        # The same stream at half the rate: the tail against the offered load.
        half_rate = run_serving(atmo, W, torch, args.serving_seconds, rate=1000.0,
                                rebuild_alone_ms=p50)

    clk = clocks.summary()
    if rank != 0:
        return
    single_plain = {"single_p50_ms": p50, "single_p99_ms": p99,
             "plain_rebuilds_per_s": 1000.0 / plain_ms,
             "batched_vs_plain": value / (1000.0 / plain_ms) / world}
    cpu = cpu_baseline_entry() if not args.no_cpu_baseline else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: the reference demo's Earth",
        "single_and_plain": single_plain,
        "config": {"workload": WORKLOAD, "batch": B, "orders": 4,
                   "parallelism": "replicas (independent batches "
                   "per GPU)" if world > 1 else "single GPU",
                   "l2": "no flush: step working set %d MB > 129 MB L2" % (B * 64)},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": kernels_per_step * args.steps,
        "clocks": {k: v for k, v in (clk or {}).items() if k != "samples"} or None,
        "roofline": {k: roof[k] for k in ("bound", "kernel", "achieved", "peak", "unit", "frac",
                                          "traffic", "dram_frac", "share_of_step",
                                          "algorithmic_tflops")},
    }
    if cpu:
        line["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
    line["parity_max"] = {k[0].upper(): parity[k]["max"] for k in (
        "transmittance", "scattering", "irradiance") if k in parity}
    line["configs_ms"] = {k: v.get("ms") for k, v in configs.items()}
    if serving:
        line["serving_p50_p99_ms"] = {
            "rebuild": [serving["rebuild_ms"]["p50"], serving["rebuild_ms"]["p99"]],
            "shade": [serving["shade_ms"]["p50"], serving["shade_ms"]["p99"]]}
    detail = {"config": {"lut_shape": list(shape), "tuning": tuning,
                         "warm_up": {"steps": warm_steps, "seconds": round(warm_s, 2)}},
              "single_and_plain": single_plain, "launch_gaps": launch_gaps, "roofline": roof,
              "passes_ms": passes_ms,
              "parity": parity, "configs": configs, "batched_mixed": mixed,
              "serving": serving, "serving_half_rate": half_rate, "cpu_baseline": cpu}
    detail = rnd(detail, 6)
    print("detail: " + json.dumps(detail), file=sys.stderr, flush=True)
    out_dir = os.environ.get("ATMO_BENCH_OUT")
    if out_dir:
        os.makedirs(out_dir, exist_ok=True)
        with open(os.path.join(out_dir, "bench_detail.json"), "w") as f:
            json.dump(detail, f, indent=1)
    print(json.dumps(rnd(line)), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def time_plain(atmo, W, torch, stream, args):
    """One rebuild with the plain per-texel kernels (atmo_precompute, plain
    path) into device buffers, CUDA-event timed (median of 3)."""
    s = atmo.LutShape(*W.DEFAULT)
    T = torch.zeros((64, 256, 4), device="cuda")
    S = torch.zeros((32, 128, 256, 4), device="cuda")
    I = torch.zeros((16, 64, 4), device="cuda")
    atm = W.earth()
    atmo.precompute(atm, s, 4, T, S, None, I, path=atmo.PATH_PLAIN, stream=stream)
    out = []
    for _ in range(3):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        atmo.precompute(atm, s, 4, T, S, None, I, path=atmo.PATH_PLAIN, stream=stream)
        b.record(stream)
        b.synchronize()
        out.append(a.elapsed_time(b))
    return sorted(out)[1]


def roofline_entry(batch, B, peak, stream, rebuilds_per_s):
    """The density kernel's FP32 roofline: executed FLOPs per second over the
    measured FP32 FMA peak; its DRAM bytes against the compulsory ones."""
    passes = batch.time_passes(stream)
    dens = [(o, ms) for name, o, ms in passes if name == "scattering_density"]
    total = sum(ms for _, _, ms in passes)
    # One launch covers B instances x 1,048,576 texels x 512 directions.
    samples = B * 1048576 * 512
    dens_ms = sum(ms for _, ms in dens)
    executed = sum(DENSITY_FLOPS_PER_SAMPLE[min(o, 3)] * samples for o, _ in dens)
    achieved = executed / (dens_ms * 1e-3) / 1e12
    ref_per_sample, ref_rebuild = reference_flops()
    algorithmic = sum(ref_per_sample[min(o, 3)] * samples for o, _ in dens)
    scale = B / 16.0
    measured = [DENSITY_DRAM_BYTES_B16[min(o, 3)] for o, _ in dens]
    traffic = (sum(measured) * scale / len(dens)) if all(m is not None for m in measured) \
        else None
    compulsory = sum(DENSITY_COMPULSORY_BYTES[min(o, 3)] * B for o, _ in dens) / len(dens)
    hbm, _ = hbm_peak()
    launch_s = dens_ms / len(dens) * 1e-3
    roof = {"bound": "fp32", "kernel": "k_density_fast",
            "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "peak_source": "measured FP32 FMA rate",
            "traffic": traffic, "compulsory_bytes": compulsory,
            "dram_frac": (traffic / launch_s / 1e9 / hbm) if traffic else None,
            "avg_launch_ms": dens_ms / len(dens), "share_of_step": dens_ms / total,
            "algorithmic_tflops": algorithmic / (dens_ms * 1e-3) / 1e12}
    passes_ms = {n + ("" if o == 0 else str(o)): round(ms, 4) for n, o, ms in passes}
    return roof, passes_ms


GOLDEN = os.path.join(ROOT, "tests", "golden", "earth_default.npz")
PARITY_FLOOR = 1e-6        # relative-error floor, x the channel's largest value


def parity_entry(atmo, W, batch, torch):
    """Per-LUT relative error of instance 0 of the benchmarked batch against
    the FP64 reference values committed in tests/golden/earth_default.npz
    (the reference's own functions.glsl built as FP64 C++; sampled texels:
    every 7th transmittance, every 61st scattering texel, all irradiance)."""
    g = np.load(GOLDEN)
    a = W.earth()
    fields = [*a.solar_irradiance, a.sun_angular_radius, a.bottom_radius, a.top_radius]
    if not np.allclose(g["atmosphere"][:6], fields, rtol=1e-12) or \
            tuple(g["shape"]) != W.DEFAULT or int(g["orders"]) != 4:
        return {"unavailable": "golden atmosphere differs from the benchmarked one"}
    torch.cuda.synchronize()
    out = {}
    for name, kind, idx, ch in (("transmittance", atmo.LUT_TRANSMITTANCE, "transmittance_index", 3),
                                ("scattering", atmo.LUT_SCATTERING, "scattering_index", 4),
                                ("irradiance", atmo.LUT_IRRADIANCE, None, 3)):
        got = batch.read(0, kind).reshape(-1, 4).astype(np.float64)
        ref = g[name].reshape(-1, 4).astype(np.float64)
        if idx is not None:
            got = got[g[idx]]
        got, ref = got[:, :ch], ref[:, :ch]
        floor = PARITY_FLOOR * np.maximum(np.abs(ref).max(axis=0), 1e-300)
        rel = np.abs(got - ref) / np.maximum(np.abs(ref), floor)
        out[name] = {"max": float(rel.max()), "p99": float(np.quantile(rel, 0.99)),
                     "texels": int(ref.shape[0])}
    out["reference"] = ("FP64 reference build (functions.glsl as C++), tests/golden/"
                        "earth_default.npz; relative error, floor 1e-6 x channel max")
    out["tolerance"] = {"transmittance": 1e-4, "scattering": 1e-3, "irradiance": 1e-3}
    return out


SPECTRAL_GOLDEN = os.path.join(ROOT, "tests", "golden", "spectral_default.npz")
HIRES_GOLDEN = os.path.join(ROOT, "tests", "golden", "hires_earth.npz")


def sampled_error(got, ref, idx=None, channels=3):
    """(max, p99) relative error of got (float32 RGBA texels) at the golden
    texels, with a floor of 1e-6 x the channel's and the texel's largest
    value (the sRGB channels of the spectral configuration can be
    cancellations of terms as large as the texel's largest channel)."""
    g = np.asarray(got, np.float64).reshape(-1, 4)
    if idx is not None:
        g = g[idx]
    r = np.asarray(ref, np.float64).reshape(-1, 4)[:, :channels]
    g = g[:, :channels]
    floor = np.maximum(PARITY_FLOOR * np.maximum(np.abs(r).max(axis=0), 1e-300),
                       PARITY_FLOOR * np.abs(r).max(axis=1, keepdims=True))
    rel = np.abs(g - r) / np.maximum(np.abs(r), floor)
    return float(rel.max()), float(np.quantile(rel, 0.99))


def time_events(torch, stream, fn, reps=3):
    """Median CUDA-event time (ms) of fn() on `stream` over reps runs."""
    out = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        out.append(a.elapsed_time(b))
    return sorted(out)[len(out) // 2]


def run_spectral(atmo, W, torch, stream):
    """The spectral-precision configuration: 15 wavelengths in 5 groups of 3,
    FP16 LUTs, the reference's default shape, 4 orders, through Model.Init;
    error against the FP64 GPU oracle's committed sampled texels (bound:
    1e-4 / 1e-3 plus FP16's 2^-11 on the stored scattering values)."""
    m = W.spectral_earth_model(W.DEFAULT)
    m.Init(4, stream=stream)
    ms = time_events(torch, stream, lambda: m.Init(4, stream=stream, synchronize=False))
    out = {"ms": ms, "wavelengths": 15, "groups": 5, "storage": "fp16"}
    if os.path.exists(SPECTRAL_GOLDEN):
        g = np.load(SPECTRAL_GOLDEN)
        errs = {"T": sampled_error(m.transmittance(), g["transmittance"],
                                   g["transmittance_index"]),
                "S": sampled_error(m.scattering(), g["scattering"], g["scattering_index"]),
                "M": sampled_error(m.single_mie_scattering(), g["single_mie"],
                                   g["scattering_index"]),
                "I": sampled_error(m.irradiance(), g["irradiance"])}
        out["max_err"] = {k: v[0] for k, v in errs.items()}
        out["p99_err"] = {k: v[1] for k, v in errs.items()}
        out["reference"] = "FP64 GPU oracle, tests/golden/spectral_default.npz"
    del m
    return out


def run_hires(atmo, W, torch, stream):
    """The high-resolution configuration: scattering NU16 x MU_S64 x MU256 x
    R64, transmittance 512x128, irradiance 128x32, 8 orders, one instance,
    replayed as a CUDA graph; error against the FP64 GPU oracle's committed
    sampled texels."""
    b = atmo.Batch([W.hires_earth()], [W.HIRES], 8, combined=True)
    b.run(stream)
    ms = time_events(torch, stream, lambda: b.run(stream))
    out = {"ms": ms, "orders": 8, "kernels": b.kernel_count()}
    if os.path.exists(HIRES_GOLDEN):
        torch.cuda.synchronize()
        g = np.load(HIRES_GOLDEN)
        errs = {"T": sampled_error(b.read(0, atmo.LUT_TRANSMITTANCE), g["transmittance"],
                                   g["transmittance_index"]),
                "S": sampled_error(b.read(0, atmo.LUT_SCATTERING), g["scattering"],
                                   g["scattering_index"], channels=4),
                "I": sampled_error(b.read(0, atmo.LUT_IRRADIANCE), g["irradiance"])}
        out["max_err"] = {k: v[0] for k, v in errs.items()}
        out["p99_err"] = {k: v[1] for k, v in errs.items()}
        out["reference"] = "FP64 GPU oracle, tests/golden/hires_earth.npz"
    del b
    return out


def run_mixed_batch(atmo, W, torch, stream, n=256, seed=3):
    """The batched configuration: n seeded planets with shapes from {half,
    default, double-R} and 2-6 orders in one pass sequence (CUDA graph)."""
    rng = np.random.default_rng(seed)
    reqs = [W.random_rebuild(rng) for _ in range(n)]
    tunings = {name: atmo.autotune(W.earth(), shape, 4).as_dict()
               for name, shape in (("half", W.HALF), ("default", W.DEFAULT),
                                   ("double_r", W.DOUBLE_R))}
    b = atmo.Batch([a for a, _, _ in reqs], [s for _, s, _ in reqs], [o for _, _, o in reqs])
    b.run(stream)
    torch.cuda.synchronize()
    times = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.run(stream)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = sorted(times)[1]
    out = {"instances": n, "ms": ms, "rebuilds_per_s": n / (ms * 1e-3),
           "kernels_per_run": b.kernel_count(),
           "shapes": {"half": sum(s == W.HALF for _, s, _ in reqs),
                      "default": sum(s == W.DEFAULT for _, s, _ in reqs),
                      "double_r": sum(s == W.DOUBLE_R for _, s, _ in reqs)},
           "mean_orders": float(np.mean([o for _, _, o in reqs])), "tunings": tunings}
    del b
    torch.cuda.empty_cache()
    return out


def ticket_split(info):
    """A request's latency split: queue (submission to admission: budget,
    instance rows, batching window), launch (admission to its first kernel's
    enqueue), device (GPU time of the launches it took part in) and the rest
    (waiting on the GPU behind other work)."""
    d = {"total": info.latency_ms, "queue": info.queue_ms,
         "launch": max(info.launch_ms - info.queue_ms, 0.0) if info.launch_ms >= 0 else 0.0,
         "device": max(info.device_ms, 0.0), "rounds": info.rounds}
    d["wait"] = max(d["total"] - d["queue"] - d["launch"] - d["device"], 0.0)
    return d


def latency_breakdown(lat, split, pct):
    """p50 / p99 of a request type's latency, and the mean split of the
    requests at or above the p99 against that of all requests."""
    out = {"p50": pct(lat, 0.5), "p99": pct(lat, 0.99), "n": len(lat)}
    if not split:
        return out
    keys = ("queue", "launch", "device", "wait", "rounds")
    p99 = out["p99"]
    tail = [d for d in split if d["total"] >= p99] or split
    out["mean_split"] = {k: float(np.mean([d[k] for d in split])) for k in keys}
    out["p99_tail_split"] = {k: float(np.mean([d[k] for d in tail])) for k in keys}
    out["queue_p50_p99"] = [pct([d["queue"] for d in split], 0.5),
                            pct([d["queue"] for d in split], 0.99)]
    out["device_p50_p99"] = [pct([d["device"] for d in split], 0.5),
                             pct([d["device"] for d in split], 0.99)]
    return out


def run_serving(atmo, W, torch, seconds, rate=2000.0, rebuild_fraction=0.1, seed=4,
                pool=16, max_shades_in_flight=0, rebuild_alone_ms=None):
    """The serving configuration: a seeded Poisson stream of rebuild requests
    (planets as in the batched configuration) and shading requests (the three
    render functions over a 1920x1080 pinhole view, FOV 50 degrees) against
    resident LUT sets, through atmo_server under a 120 GiB budget.  Also: the
    GPU time of one shading request run alone, and the offered GPU load
    (requests/s x their lone GPU time)."""
    rng = np.random.default_rng(seed)
    srv = atmo.Server(max_shades_in_flight=max_shades_in_flight)
    radius = {}
    earth_id = srv.submit_rebuild(W.earth(), W.DEFAULT, 4)
    srv.wait(earth_id)
    radius[earth_id] = 6360.0
    ready = [earth_id]
    H, Wd = 1080, 1920
    depth = torch.from_numpy(rng.uniform(0.1, 100.0, size=H * Wd).astype(np.float32)).cuda()
    sky = [torch.empty((H, Wd, 4), device="cuda") for _ in range(pool)]
    shaded = [torch.empty((H, Wd, 4), device="cuda") for _ in range(pool)]
    slot_ticket = [None] * pool
    # Warm-up shading (module load, first launches).
    for j in range(4):
        t = srv.submit_shade(earth_id, W.random_view(rng, 6360.0), depth, sky[j], shaded[j])
        srv.wait(t)
        srv.release_ticket(t)
    # One shading request alone, on the default stream (CUDA events, median of 5).
    lone = srv.lut_set(earth_id)
    stream = torch.cuda.current_stream()
    lone_view = W.random_view(np.random.default_rng(0), 6360.0)
    lone.shade_view(lone_view, depth, stream=stream)
    shade_alone_ms = time_events(torch, stream,
                                 lambda: lone.shade_view(lone_view, depth, stream=stream), reps=5)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * seconds * 1.2) + 16))
    arrivals = arrivals[arrivals < seconds]
    building, records, kinds = [], [], []
    nslot = 0
    t0 = time.perf_counter()
    for ta in arrivals:
        now = time.perf_counter() - t0
        if ta > now:
            time.sleep(ta - now)
        if building:
            # Newly built sets join the shading targets.
            still = []
            for tk in building:
                if srv.poll(tk).state == atmo.Server.DONE:
                    ready.append(tk)
                else:
                    still.append(tk)
            building = still
        if rng.random() < rebuild_fraction:
            a, shape, orders = W.random_rebuild(rng)
            tk = srv.submit_rebuild(a, shape, orders)
            radius[tk] = a.bottom_radius
            building.append(tk)
            records.append(("rebuild", tk, time.perf_counter() - t0))
            kinds.append((tuple(shape), orders, a))
        else:
            set_id = ready[int(rng.integers(0, len(ready)))]
            j = nslot % pool
            nslot += 1
            if slot_ticket[j] is not None:
                srv.wait(slot_ticket[j], 120000)
            tk = srv.submit_shade(set_id, W.random_view(rng, radius[set_id]), depth, sky[j],
                                  shaded[j])
            slot_ticket[j] = tk
            records.append(("shade", tk, time.perf_counter() - t0))
    submit_end = time.perf_counter() - t0
    lat = {"rebuild": [], "shade": []}
    split = {"rebuild": [], "shade": []}
    end = 0.0
    failed = 0
    for kind, tk, ts in records:
        try:
            info = srv.wait(tk, 300000)
        except atmo.AtmoError:
            failed += 1
            continue
        lat[kind].append(info.latency_ms)
        split[kind].append(ticket_split(info))
        end = max(end, ts + info.latency_ms * 1e-3)
    st = srv.stats()
    srv.close()
    # Each rebuild's own GPU time alone (one instance of its LUT shape and
    # order count, CUDA-graph replay, median of 3): the spread of the work
    # itself, beside the latencies.
    lone = {}
    for shape, orders, a in kinds:
        if (shape, orders) not in lone:
            b = atmo.Batch([a], [shape], orders)
            b.run(stream)
            lone[(shape, orders)] = time_events(torch, stream, lambda: b.run(stream))
            del b
    lone_ms = sorted(lone[(shape, orders)] for shape, orders, _ in kinds)

    def pct(xs, q):
        xs = sorted(xs)
        return xs[min(len(xs) - 1, max(0, int(math.ceil(q * len(xs))) - 1))] if xs else None

    done = len(lat["rebuild"]) + len(lat["shade"])
    return {
        "offered_rate": rate, "seconds": seconds, "submitted": len(records),
        "submit_seconds": submit_end, "completed": done, "failed": failed,
        "throughput_req_per_s": done / end if end > 0 else None,
        "rebuilds_per_s": len(lat["rebuild"]) / end if end > 0 else None,
        "shades_per_s": len(lat["shade"]) / end if end > 0 else None,
        "rebuild_ms": latency_breakdown(lat["rebuild"], split["rebuild"], pct),
        "shade_ms": latency_breakdown(lat["shade"], split["shade"], pct),
        "view": "1920x1080, FOV 50 deg: GetSkyRadiance, GetSkyRadianceToPoint and "
                "GetSunAndSkyIrradiance per pixel",
        "max_shades_in_flight": max_shades_in_flight,
        "shade_alone_ms": shade_alone_ms,
        "rebuild_alone_ms": {"p50": pct(lone_ms, 0.5), "p99": pct(lone_ms, 0.99),
                             "mean": float(np.mean(lone_ms)) if lone_ms else None},
        "offered_gpu_load": (rate * (1.0 - rebuild_fraction) * shade_alone_ms +
                             rate * rebuild_fraction *
                             (float(np.mean(lone_ms)) if lone_ms else (rebuild_alone_ms or 0.0))
                             ) / 1000.0,
        "server": {"rounds": st.rounds, "kernels": st.kernels, "evictions": st.evictions,
                   "resident_sets": st.resident_sets, "used_gb": st.used_bytes / 2 ** 30,
                   "budget_gb": st.budget_bytes / 2 ** 30},
    }


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
