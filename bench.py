"""Benchmark: Earth LUT rebuilds per second on one GB300.

Workload (one "step"): a batched rebuild of B Earth atmospheres with the
reference's default LUT shape (transmittance 256x64, scattering NU 8 x MU_S 32
x MU 128 x R 32 = 256x128x32 RGBA, irradiance 64x16), 4 scattering orders,
3 wavelengths (680/550/440 nm), combined scattering textures, FP32 -- the
Earth parameters of atmosphere/demo/demo.cc:188-284 with max sun zenith 102
degrees.  Every instance's working set (64 MB) exceeds nothing in L2 on its
own, and a batch of B >= 4 is several times larger than the 129 MB L2, so no
explicit L2 flush is needed between steps.

Reported (one JSON line on rank 0):
  value          batched rebuilds/s (device-timed with CUDA events),
  e2e            the same through the public C API with host buffers: the
                 atmosphere parameters go host->device and every LUT comes
                 back device->host into pinned memory inside the timed region,
  single_rebuild p50/p99 latency of one Model.Init (fast path) and the plain
                 path's rebuilds/s,
  roofline       the scattering-density kernel against this GPU's FP32 FMA
                 throughput measured in the same run,
  cpu_baseline   the FP64 CPU oracle on a bounded sample, all host threads.

--impl reference times the reference's CPU algorithm (the oracle port of
atmosphere/reference/model.cc + functions.glsl) on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Earth LUT rebuilds/s batched vs plain on 1 GB300 @<=1e-3 vs FP64; p99 ms"
UNIT = "rebuilds/s"
WORKLOAD = ("Earth atmosphere LUT rebuild, 256x64 / 256x128x32 / 64x16 RGBA FP32, "
            "4 scattering orders, 3 wavelengths, combined textures")
# FP32 operations per density direction sample of the fast kernel's inner
# loop (counted from the kernel's arithmetic, FMA = 2).
DENSITY_FLOPS_PER_SAMPLE = 46.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--batch", type=int, default=16, help="atmospheres per batched step")
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (FP64 restatement of the reference CPU model).
# ---------------------------------------------------------------------------
def cpu_rebuild_seconds(stride=16, threads=0):
    from oracle import oracle as O
    O.build()
    import ctypes as C
    atm = O.earth_atmosphere()
    shp = O.shape(*O.DEFAULT_SHAPE)
    sec = np.zeros(6)
    t0 = time.perf_counter()
    rc = O.lib().oracle_time_precompute_sample(C.byref(atm), C.byref(shp), 4, stride, threads,
                                               sec.ctypes.data_as(O.dp))
    wall = time.perf_counter() - t0
    if rc != 0:
        raise RuntimeError("oracle timing failed")
    # Density and multiple scattering ran on every stride-th texel: scale them.
    full = sec[0] + sec[1] + sec[2] + sec[4] + (sec[3] + sec[5]) * stride
    return full, wall, sec


def cpu_baseline_entry(stride=16):
    cores = os.cpu_count() or 1
    full, wall, sec = cpu_rebuild_seconds(stride)
    return {"value": 1.0 / full, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": ("one config-0 Earth rebuild (4 orders) by the FP64 oracle with %d threads; "
                       "transmittance, irradiance and single scattering in full, scattering "
                       "density and multiple scattering on every %dth texel and scaled x%d "
                       "(%.1f s of CPU wall time, extrapolated rebuild %.1f s)"
                       % (cores, stride, stride, wall, full))}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    stride = 64
    for _ in range(args.warmup):
        pass  # the CPU path has no warm-up state beyond the first call below
    t0 = time.perf_counter()
    totals = []
    for _ in range(args.steps):
        full, _, _ = cpu_rebuild_seconds(stride)
        totals.append(full)
    wall = time.perf_counter() - t0
    value = len(totals) / sum(totals)
    cores = os.cpu_count() or 1
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * sum(totals) / len(totals), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "batch": 1, "implementation":
                   "CPU oracle port of atmosphere/reference/model.cc (FP64, all host threads)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "per step: one rebuild with density/multiple scattering on "
                                   "every %dth texel, scaled; %.1f s wall for %d steps"
                                   % (stride, wall, args.steps)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU measurement.
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", "clocks_bench_%d.csv" % gpu_index)
        self.gpu = gpu_index

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
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


def earth_atmospheres(O, n):
    return [O.earth_atmosphere() for _ in range(n)]


def run_gpu(args):
    import torch
    import precomputed_atmospheric_scattering_gb300 as atmo
    from oracle import oracle as O

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    atmo.build()
    atmo.lib()
    B = args.batch
    shape = O.DEFAULT_SHAPE
    atms = earth_atmospheres(O, B)
    batch = atmo.Batch(atms, [shape] * B, 4, combined=True)
    kernels_per_step = batch.kernel_count()
    stream = torch.cuda.current_stream()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # --- device-timed batched rebuilds -------------------------------------
    for _ in range(args.warmup):
        batch.run(stream)
    barrier()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local) as clocks:
        ev[0].record(stream)
        for k in range(args.steps):
            batch.run(stream)
            ev[k + 1].record(stream)
        barrier()
    step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    total_s = sum(step_ms) / 1000.0
    if world > 1:
        t = torch.tensor([total_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_s = float(t.item())
    value = B * args.steps * world / total_s

    # --- end to end through the C API with host buffers ---------------------
    kinds = [atmo.LUT_TRANSMITTANCE, atmo.LUT_SCATTERING, atmo.LUT_IRRADIANCE]
    views = [batch.lut_view(0, k) for k in kinds]
    sizes = [v.width * v.height * v.depth * 16 for v in views]
    host = [[torch.empty(s // 4, dtype=torch.float32).pin_memory() for s in sizes]
            for _ in range(B)]
    import ctypes as C
    L = atmo.lib()
    h2d = B * C.sizeof(atmo.Atmosphere)
    d2h = B * sum(sizes)

    def e2e_step():
        for i in range(B):
            batch.set_atmosphere(i, atms[i])
        batch.run(stream)
        for i in range(B):
            for k, buf, nb in zip(kinds, host[i], sizes):
                st = L.atmo_batch_read_lut(batch._h, i, k, C.cast(buf.data_ptr(),
                                           C.POINTER(C.c_float)), nb)
                if st != 0:
                    raise RuntimeError(L.atmo_last_error().decode())
    e2e_step()
    barrier()
    e2e_steps = max(3, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_value = B * e2e_steps * world / e2e_s

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
    plain_ms = time_plain(atmo, O, torch, stream, args)

    # --- roofline of the scattering-density kernel ---------------------------
    peak = density_roofline(atmo, O, torch, stream)
    roof = roofline_entry(batch, B, peak, stream)

    clk = clocks.summary()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: Earth parameters of the reference demo (no dataset)",
        "config": {"workload": WORKLOAD, "batch": B, "orders": 4,
                   "lut_shape": list(shape), "parallelism": "replicas (independent batches "
                   "per GPU)" if world > 1 else "single GPU",
                   "l2": "no flush: each step's working set (%d MB) exceeds the 129 MB L2"
                         % (B * 64)},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "single_rebuild": {"p50_ms": p50, "p99_ms": p99, "fast_rebuilds_per_s": 1000.0 / p50,
                           "plain_ms": plain_ms, "plain_rebuilds_per_s": 1000.0 / plain_ms,
                           "batched_vs_plain": value / (1000.0 / plain_ms) / world},
        "roofline": roof,
        "gpu_launches": kernels_per_step * args.steps,
        "clocks": clk,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_entry()
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def time_plain(atmo, O, torch, stream, args):
    """One rebuild with the plain per-texel kernels (atmo_precompute, plain
    path) into device buffers, CUDA-event timed (median of 3)."""
    s = atmo.LutShape(*O.DEFAULT_SHAPE)
    T = torch.zeros((64, 256, 4), device="cuda")
    S = torch.zeros((32, 128, 256, 4), device="cuda")
    I = torch.zeros((16, 64, 4), device="cuda")
    atm = O.earth_atmosphere()
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


def density_roofline(atmo, O, torch, stream):
    """The scattering-density kernel of one batched step against this GPU's
    FP32 FMA throughput (measured here): launches timed with CUDA events on
    the launching stream (a non-graph run of the same batch)."""
    peak = atmo.measure_fp32_peak()
    return peak


def roofline_entry(batch, B, peak, stream):
    passes = batch.time_passes(stream)
    dens = [ms for name, _, ms in passes if name == "scattering_density"]
    total = sum(ms for _, _, ms in passes)
    # One launch covers B instances x 1,048,576 texels x 512 directions.
    samples = B * 1048576 * 512
    avg = sum(dens) / len(dens)
    achieved = DENSITY_FLOPS_PER_SAMPLE * samples / (avg * 1e-3) / 1e12
    return {"bound": "fp32", "kernel": "scattering density",
            "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "traffic": None,
            "peak_source": "FP32 FMA throughput measured in this run by atmo_measure_fp32_peak "
                           "(MEASURED_PEAKS.json holds only HBM and bf16 tensor peaks)",
            "avg_launch_ms": avg, "launches_per_step": len(dens),
            "share_of_step": sum(dens) / total, "flops_per_sample": DENSITY_FLOPS_PER_SAMPLE,
            "passes_ms": {n + ("" if o == 0 else str(o)): round(ms, 4)
                          for n, o, ms in passes}}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
