"""Runs a fixed batched precomputation for profiling (e.g. under ncu):
B Earth atmospheres of one LUT shape, `runs` times; with --shade N, then N
shading requests (the three render functions over a 1920x1080 pinhole view)
on instance 0's LUT set.

    python -m precomputed_atmospheric_scattering_gb300.profile_case --batch 4
"""
import argparse

from . import Batch, lib, synchronize_stream
from . import workloads as W

SHAPES = {"default": W.DEFAULT, "half": W.HALF, "double_r": W.DOUBLE_R, "hires": W.HIRES,
          "medium": (128, 32, 8, 32, 16, 8, 32, 8)}


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--batch", type=int, default=4)
    p.add_argument("--shape", default="default", choices=sorted(SHAPES))
    p.add_argument("--orders", type=int, default=4)
    p.add_argument("--runs", type=int, default=1)
    p.add_argument("--no-graph", action="store_true", help="launch the passes directly")
    p.add_argument("--shade", type=int, default=0, help="1920x1080 shading requests afterwards")
    a = p.parse_args()
    lib()
    b = Batch([W.earth() for _ in range(a.batch)], [SHAPES[a.shape]] * a.batch, a.orders)
    if a.no_graph:
        for _ in range(a.runs):
            passes = b.time_passes()
        for name, order, ms in passes:
            print("%-22s %2d %9.4f ms" % (name, order, ms))
    else:
        for _ in range(a.runs):
            b.run()
    synchronize_stream()
    if a.shade:
        import numpy as np
        import torch
        rng = np.random.default_rng(4)
        depth = torch.from_numpy(rng.uniform(0.1, 100.0, 1920 * 1080).astype(np.float32)).cuda()
        lut = b.lut_set(0)
        for _ in range(a.shade):
            lut.shade_view(W.random_view(rng, 6360.0), depth)
        torch.cuda.synchronize()
    print("ok: %d kernels per run" % b.kernel_count())


if __name__ == "__main__":
    main()
