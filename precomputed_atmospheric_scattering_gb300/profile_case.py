"""Runs a fixed batched precomputation for profiling (e.g. under ncu):
B Earth atmospheres of one LUT shape, `runs` times.

    python -m precomputed_atmospheric_scattering_gb300.profile_case --batch 4
"""
import argparse
import math

from . import Atmosphere, Batch, lib, synchronize_stream

SHAPES = {"default": (256, 64, 32, 128, 32, 8, 64, 16),
          "medium": (128, 32, 8, 32, 16, 8, 32, 8),
          "hires": (512, 128, 64, 256, 64, 16, 128, 32)}


def earth(mie_g=0.8, albedo=0.1):
    """Earth at 680/550/440 nm in km (atmosphere/demo/demo.cc:188-284)."""
    a = Atmosphere()
    lam = (680.0, 550.0, 440.0)
    for i, l in enumerate(lam):
        a.solar_irradiance[i] = 1.5
        a.rayleigh_scattering[i] = 1.24062e-6 * (l * 1e-3) ** -4 * 1000.0
        a.mie_scattering[i] = 5.328e-3 / 1200.0 * 1000.0 * 0.9
        a.mie_extinction[i] = 5.328e-3 / 1200.0 * 1000.0
        a.absorption_extinction[i] = 300.0 * 2.687e20 / 15000.0 * {
            680.0: 1.209e-25, 550.0: 3.5e-25, 440.0: 1.582e-26}[l] * 1000.0
        a.ground_albedo[i] = albedo
    a.sun_angular_radius = 0.00935 / 2.0
    a.bottom_radius, a.top_radius = 6360.0, 6420.0
    a.rayleigh_density.layers[1].exp_term = 1.0
    a.rayleigh_density.layers[1].exp_scale = -1.0 / 8.0
    a.mie_density.layers[1].exp_term = 1.0
    a.mie_density.layers[1].exp_scale = -1.0 / 1.2
    a.absorption_density.layers[0].width = 25.0
    a.absorption_density.layers[0].linear_term = 1.0 / 15.0
    a.absorption_density.layers[0].constant_term = -2.0 / 3.0
    a.absorption_density.layers[1].linear_term = -1.0 / 15.0
    a.absorption_density.layers[1].constant_term = 8.0 / 3.0
    a.mie_phase_function_g = mie_g
    a.mu_s_min = math.cos(math.radians(102.0))
    return a


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--batch", type=int, default=4)
    p.add_argument("--shape", default="default", choices=sorted(SHAPES))
    p.add_argument("--orders", type=int, default=4)
    p.add_argument("--runs", type=int, default=1)
    p.add_argument("--no-graph", action="store_true", help="launch the passes directly")
    a = p.parse_args()
    lib()
    b = Batch([earth()] * a.batch, [SHAPES[a.shape]] * a.batch, a.orders)
    if a.no_graph:
        for _ in range(a.runs):
            b.time_passes()
    else:
        for _ in range(a.runs):
            b.run()
    synchronize_stream()
    print("ok: %d kernels per run" % b.kernel_count())


if __name__ == "__main__":
    main()
