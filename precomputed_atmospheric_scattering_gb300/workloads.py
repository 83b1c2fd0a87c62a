"""Synthetic workloads of the measurements: the Earth atmosphere of the
reference's demo, seeded planets over the batched-rebuild ranges, the LUT
shapes of the configurations and pinhole views of the serving workload.
Parameters are in km (length_unit_in_meters = 1000), 3 wavelengths
(680 / 550 / 440 nm)."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import Atmosphere, DensityProfileLayer, Model, PinholeView

DEFAULT = (256, 64, 32, 128, 32, 8, 64, 16)      # atmosphere/constants.h:47-61
HALF = (128, 32, 16, 64, 16, 4, 32, 8)           # every size halved
DOUBLE_R = (256, 64, 64, 128, 32, 8, 64, 16)     # twice the r slices
HIRES = (512, 128, 64, 256, 64, 16, 128, 32)     # NU16 x MU_S64 x MU256 x R64
LAMBDAS = (680.0, 550.0, 440.0)


def _layer(p, i, width=0.0, exp_term=0.0, exp_scale=0.0, linear_term=0.0, constant_term=0.0):
    l = p.layers[i]
    l.width, l.exp_term, l.exp_scale = width, exp_term, exp_scale
    l.linear_term, l.constant_term = linear_term, constant_term


def earth(mie_g=0.8, albedo=0.1, ozone=True, max_sun_zenith_deg=102.0) -> Atmosphere:
    """The Earth of atmosphere/demo/demo.cc:188-284 with a constant solar
    spectrum of 1.5 W/m^2/nm."""
    a = Atmosphere()
    xs = {680.0: 1.209e-25, 550.0: 3.5e-25, 440.0: 1.582e-26}   # ozone cross sections, m^2
    for i, l in enumerate(LAMBDAS):
        a.solar_irradiance[i] = 1.5
        a.rayleigh_scattering[i] = 1.24062e-6 * (l * 1e-3) ** -4 * 1000.0
        a.mie_scattering[i] = 5.328e-3 / 1200.0 * 1000.0 * 0.9
        a.mie_extinction[i] = 5.328e-3 / 1200.0 * 1000.0
        a.absorption_extinction[i] = (300.0 * 2.687e20 / 15000.0 * xs[l] * 1000.0
                                      if ozone else 0.0)
        a.ground_albedo[i] = albedo
    a.sun_angular_radius = 0.00935 / 2.0
    a.bottom_radius, a.top_radius = 6360.0, 6420.0
    _layer(a.rayleigh_density, 1, exp_term=1.0, exp_scale=-1.0 / 8.0)
    _layer(a.mie_density, 1, exp_term=1.0, exp_scale=-1.0 / 1.2)
    _layer(a.absorption_density, 0, width=25.0, linear_term=1.0 / 15.0, constant_term=-2.0 / 3.0)
    _layer(a.absorption_density, 1, linear_term=-1.0 / 15.0, constant_term=8.0 / 3.0)
    a.mie_phase_function_g = mie_g
    a.mu_s_min = math.cos(math.radians(max_sun_zenith_deg))
    return a


def random_planet(rng) -> Atmosphere:
    """Uniform draws over the batched-rebuild ranges: bottom radius
    3000-7000 km, thickness 40-120 km, Rayleigh scale height 5-15 km and
    beta x0.2-5 of Earth, Mie beta_s 1e-6-5e-5 /m (extinction 1.1 beta_s),
    scale height 0.5-3 km, g 0.6-0.9, ozone on/off, albedo 0-0.5."""
    a = earth()
    rb = rng.uniform(3000.0, 7000.0)
    a.bottom_radius, a.top_radius = rb, rb + rng.uniform(40.0, 120.0)
    scale = rng.uniform(0.2, 5.0)
    mie_s = rng.uniform(1e-6, 5e-5) * 1000.0
    ozone = rng.random() < 0.5
    albedo = rng.uniform(0.0, 0.5)
    for i in range(3):
        a.rayleigh_scattering[i] *= scale
        a.mie_scattering[i] = mie_s
        a.mie_extinction[i] = 1.1 * mie_s
        if not ozone:
            a.absorption_extinction[i] = 0.0
        a.ground_albedo[i] = albedo
    _layer(a.rayleigh_density, 1, exp_term=1.0, exp_scale=-1.0 / rng.uniform(5.0, 15.0))
    _layer(a.mie_density, 1, exp_term=1.0, exp_scale=-1.0 / rng.uniform(0.5, 3.0))
    a.mie_phase_function_g = rng.uniform(0.6, 0.9)
    return a


def random_rebuild(rng):
    """(atmosphere, shape, orders) of a batched / served rebuild request:
    shape from {half, default, double-R}, 2-6 scattering orders."""
    shape = (HALF, DEFAULT, DOUBLE_R)[int(rng.integers(0, 3))]
    return random_planet(rng), shape, int(rng.integers(2, 7))


def _unit(rng):
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


def random_view(rng, bottom_radius, width=1920, height=1080, fov_deg=50.0) -> PinholeView:
    """A pinhole view of the serving workload: camera altitude 0-100 km,
    view and sun directions uniform on the sphere."""
    cam = _unit(rng) * (bottom_radius + rng.uniform(0.0, 100.0))
    fwd = _unit(rng)
    right = np.cross(fwd, _unit(rng))
    right /= np.linalg.norm(right)
    up = np.cross(right, fwd)
    v = PinholeView()
    for name, x in (("camera", cam), ("right", right), ("up", up), ("forward", fwd),
                    ("sun_direction", _unit(rng)), ("albedo", (0.1, 0.1, 0.1))):
        setattr(v, name, (C.c_float * 3)(*x))
    v.fov_y = math.radians(fov_deg)
    v.width, v.height = width, height
    return v


def smooth_solar_spectrum(seed, wavelengths):
    """A seeded smooth solar spectrum in [1, 2] W/m^2/nm at `wavelengths`
    (nm): 1.5 plus four random sines over 360-830 nm, clipped."""
    rng = np.random.default_rng(seed)
    x = (np.asarray(wavelengths, np.float64) - 360.0) / 470.0
    s = 1.5 + sum(rng.uniform(0.05, 0.12) * np.sin(2 * np.pi * rng.uniform(0.5, 3.0) * x +
                                                   rng.uniform(0, 2 * np.pi)) for _ in range(4))
    return np.clip(s, 1.0, 2.0)


# Ozone absorption cross sections (m^2) at 360, 370, ..., 830 nm.
OZONE_CROSS_SECTION_10NM = np.array([
    1.18e-27, 2.182e-28, 2.818e-28, 6.636e-28, 1.527e-27, 2.763e-27, 5.52e-27, 8.451e-27,
    1.582e-26, 2.316e-26, 3.669e-26, 4.924e-26, 7.752e-26, 9.016e-26, 1.48e-25, 1.602e-25,
    2.139e-25, 2.755e-25, 3.091e-25, 3.5e-25, 4.266e-25, 4.672e-25, 4.398e-25, 4.701e-25,
    5.019e-25, 4.305e-25, 3.74e-25, 3.215e-25, 2.662e-25, 2.238e-25, 1.852e-25, 1.473e-25,
    1.209e-25, 9.423e-26, 7.455e-26, 6.566e-26, 5.105e-26, 4.15e-26, 4.228e-26, 3.237e-26,
    2.451e-26, 2.801e-26, 2.534e-26, 1.624e-26, 1.465e-26, 2.078e-26, 1.383e-26, 7.105e-27])


def spectral_earth_model(shape=None, seed=1, num_precomputed_wavelengths=15,
                         combine_scattering_textures=False, half_precision=True) -> Model:
    """The spectral-precision configuration: the demo's Earth tabulated every
    10 nm over 360-830 nm with a seeded smooth solar spectrum, 15 precomputed
    wavelengths (5 groups of 3), FP16 LUT storage, separate single-Mie LUT."""
    w = np.arange(360.0, 831.0, 10.0)
    lam = w * 1e-3
    mie = 5.328e-3 / 1200.0 * np.ones_like(w)
    L = DensityProfileLayer
    return Model(w, smooth_solar_spectrum(seed, w), 0.00935 / 2.0, 6360e3, 6420e3,
                 [L(0.0, 1.0, -1.0 / 8000.0, 0.0, 0.0)], 1.24062e-6 * lam ** -4,
                 [L(0.0, 1.0, -1.0 / 1200.0, 0.0, 0.0)], mie * 0.9, mie, 0.8,
                 [L(25000.0, 0.0, 0.0, 1.0 / 15000.0, -2.0 / 3.0),
                  L(0.0, 0.0, 0.0, -1.0 / 15000.0, 8.0 / 3.0)],
                 300.0 * 2.687e20 / 15000.0 * OZONE_CROSS_SECTION_10NM, np.full_like(w, 0.1),
                 102.0 / 180.0 * math.pi, 1000.0, num_precomputed_wavelengths,
                 combine_scattering_textures, half_precision, lut_shape=shape)


def hires_earth() -> Atmosphere:
    """The high-resolution configuration's atmosphere: the demo's Earth with
    Mie g = 0.76 and ground albedo 0.3 (LUT shape HIRES, 8 orders)."""
    return earth(mie_g=0.76, albedo=0.3)
