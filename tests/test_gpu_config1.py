"""The spectral-precision configuration: 15 precomputed wavelengths (5 groups
of 3 over 360-830 nm, atmosphere/model.cc:914-963), a seeded smooth solar
spectrum in [1, 2] W/m^2/nm tabulated every 10 nm, LUTs stored in FP16
(half_precision = true), luminance through the CIE 1931 tables.  Every
texel is compared with the FP64 oracle's composition of the same five groups
(the CPU oracle at the medium shape, the FP64 GPU oracle at the reference's
default shape); the bound is the FP32 tolerance plus FP16's rounding of the
stored value, with a floor of 1e-6 of the texel's largest channel for the
sRGB channels that are cancellations.  The per-LUT relative and absolute
errors are printed (pytest -s)."""
import math

import numpy as np
import pytest

from parity import FLOOR, TOL_IRRADIANCE, TOL_SCATTERING, TOL_TRANSMITTANCE
from test_gpu_parity import oracle_luminance_model

pytestmark = pytest.mark.gpu


def smooth_solar_spectrum(seed, wavelengths):
    rng = np.random.default_rng(seed)
    x = (wavelengths - 360.0) / 470.0
    s = 1.5 + sum(rng.uniform(0.05, 0.12) * np.sin(2 * np.pi * rng.uniform(0.5, 3.0) * x +
                                                   rng.uniform(0, 2 * np.pi)) for _ in range(4))
    return np.clip(s, 1.0, 2.0)


def config1_model(atmo, shape):
    w = np.arange(360.0, 831.0, 10.0)
    lam = w * 1e-3
    mie = 5.328e-3 / 1200.0 * np.ones_like(w)
    # Ozone absorption cross sections (m^2) at 360, 370, ..., 830 nm.
    xs = np.array([1.18e-27, 2.182e-28, 2.818e-28, 6.636e-28, 1.527e-27, 2.763e-27, 5.52e-27,
                   8.451e-27, 1.582e-26, 2.316e-26, 3.669e-26, 4.924e-26, 7.752e-26, 9.016e-26,
                   1.48e-25, 1.602e-25, 2.139e-25, 2.755e-25, 3.091e-25, 3.5e-25, 4.266e-25,
                   4.672e-25, 4.398e-25, 4.701e-25, 5.019e-25, 4.305e-25, 3.74e-25, 3.215e-25,
                   2.662e-25, 2.238e-25, 1.852e-25, 1.473e-25, 1.209e-25, 9.423e-26, 7.455e-26,
                   6.566e-26, 5.105e-26, 4.15e-26, 4.228e-26, 3.237e-26, 2.451e-26, 2.801e-26,
                   2.534e-26, 1.624e-26, 1.465e-26, 2.078e-26, 1.383e-26, 7.105e-27])
    L = atmo.DensityProfileLayer
    return atmo.Model(w, smooth_solar_spectrum(1, w), 0.00935 / 2.0, 6360e3, 6420e3,
                      [L(0.0, 1.0, -1.0 / 8000.0, 0.0, 0.0)], 1.24062e-6 * lam ** -4,
                      [L(0.0, 1.0, -1.0 / 1200.0, 0.0, 0.0)], mie * 0.9, mie, 0.8,
                      [L(25000.0, 0.0, 0.0, 1.0 / 15000.0, -2.0 / 3.0),
                       L(0.0, 0.0, 0.0, -1.0 / 15000.0, 8.0 / 3.0)],
                      300.0 * 2.687e20 / 15000.0 * xs, np.full_like(w, 0.1),
                      102.0 / 180.0 * math.pi, 1000.0, 15, False, True, lut_shape=shape)


def report(name, got, ref, tol, fp16, channels=3):
    g = np.asarray(got, np.float64)[..., :channels].reshape(-1, channels)
    r = np.asarray(ref, np.float64)[..., :channels].reshape(-1, channels)
    floor = FLOOR * np.maximum(np.abs(r).max(axis=0), 1e-300)
    rel = np.abs(g - r) / np.maximum(np.abs(r), floor)
    abs_err = np.abs(g - r)
    print("config 1 %-13s max rel %.3g  p99 rel %.3g  max abs %.3g" % (
        name, rel.max(), np.quantile(rel, 0.99), abs_err.max()))
    # FP16 storage adds one rounding: 2^-11 relative, 2^-25 absolute (subnormal).
    # The outputs are sRGB (XYZ -> sRGB has negative coefficients): a channel
    # can be a cancellation of terms as large as the texel's largest channel,
    # and its FP32 error scales with those terms, hence a floor of 1e-6 of the
    # texel's largest channel beside the channel's own.
    texel = FLOOR * np.abs(r).max(axis=1, keepdims=True)
    bound = (tol + (2.0 ** -11 if fp16 else 0.0)) * np.maximum(np.abs(r), floor) + \
        (2.0 ** -25 if fp16 else 0.0) + texel
    bad = np.abs(g - r) > bound
    assert not bad.any(), "%s: %d texels over the bound (max rel %.3g)" % (
        name, int(bad.sum()), rel.max())


def test_config1_fifteen_wavelengths_fp16_vs_oracle(atmo, oracle):
    shape = oracle.MEDIUM_SHAPE
    m = config1_model(atmo, shape)
    m.Init(4)
    assert m.lut_view(atmo.LUT_SCATTERING).dtype == 1     # FP16 scattering
    ref = oracle_luminance_model(oracle, m, 4, shape)
    report("transmittance", m.transmittance(), ref.transmittance, TOL_TRANSMITTANCE, False)
    report("scattering", m.scattering(), ref.scattering, TOL_SCATTERING, True)
    report("single_mie", m.single_mie_scattering(), ref.single_mie, TOL_SCATTERING, True)
    report("irradiance", m.irradiance(), ref.irradiance, TOL_IRRADIANCE, False)


def test_config1_default_shape_vs_gpu_oracle(atmo, oracle):
    """The same at the reference's default LUT sizes (1,048,576 scattering
    texels per group), against the FP64 GPU oracle's composition."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    shape = atmo.DEFAULT_SHAPE
    m = config1_model(atmo, shape)
    m.Init(4)
    ref = oracle_luminance_model(oracle, m, 4, shape, precompute=oracle.gpu_precompute)
    report("transmittance", m.transmittance(), ref.transmittance, TOL_TRANSMITTANCE, False)
    report("scattering", m.scattering(), ref.scattering, TOL_SCATTERING, True)
    report("single_mie", m.single_mie_scattering(), ref.single_mie, TOL_SCATTERING, True)
    report("irradiance", m.irradiance(), ref.irradiance, TOL_IRRADIANCE, False)
