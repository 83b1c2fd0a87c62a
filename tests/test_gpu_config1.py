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

import numpy as np
import pytest

from parity import FLOOR, TOL_IRRADIANCE, TOL_SCATTERING, TOL_TRANSMITTANCE
from test_gpu_parity import oracle_luminance_model

pytestmark = pytest.mark.gpu


def config1_model(atmo, shape):
    from precomputed_atmospheric_scattering_gb300 import workloads as W
    return W.spectral_earth_model(shape)


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
