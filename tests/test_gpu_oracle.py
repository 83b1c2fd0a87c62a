"""The FP64 GPU oracle (oracle/atmo_oracle_gpu.cu: the CPU oracle's texel
evaluators compiled as device code, one thread per texel) against the CPU
oracle, before it stands in for the CPU oracle at sizes the CPU cannot
evaluate in test time.  Both run the same FP64 arithmetic in the same order
without FMA contraction; only the device's sin / cos / exp / pow (within 2
ulp, glibc's within 1) differ.  Measured on the Earth atmosphere: ~1e-15 for
transmittance, up to 3e-9 for scattering (the roundings grow through the
orders and lookups), up to 1.4e-9 for irradiance; the bar is 1e-8 per texel
(relative, floor 1e-6 of the channel maximum), 1e5 times below the FP32
tolerances it stands in for."""
import numpy as np
import pytest

from parity import rel_err

pytestmark = pytest.mark.gpu

TOL_ORACLES = 1e-8


@pytest.fixture(scope="module")
def gpu(oracle):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return oracle


def agree(name, a, b, channels):
    mx, _ = rel_err(a, b, channels)
    print("%-14s max rel %.3g" % (name, mx))
    assert mx <= TOL_ORACLES, (name, mx)


@pytest.mark.parametrize("combined", [True, False], ids=["combined", "separate"])
@pytest.mark.parametrize("shape", ["SMALL_SHAPE", "MEDIUM_SHAPE"])
def test_gpu_oracle_equals_cpu_oracle(gpu, shape, combined):
    O = gpu
    shp = getattr(O, shape)
    atm = O.earth_atmosphere(mie_g=0.7, ground_albedo=0.3)
    cpu = O.precompute(atm, shp, 4, combined=combined)
    dev = O.gpu_precompute(atm, shp, 4, combined=combined)
    agree("transmittance", dev.transmittance, cpu.transmittance, 3)
    agree("scattering", dev.scattering, cpu.scattering, 4 if combined else 3)
    if not combined:
        agree("single_mie", dev.single_mie, cpu.single_mie, 3)
    agree("irradiance", dev.irradiance, cpu.irradiance, 3)


def test_gpu_oracle_blends_a_luminance_group(gpu):
    """A second wavelength group: luminance matrix and blending into the
    first group's LUTs (model.cc:1082-1083), as the 15-wavelength models do."""
    O = gpu
    shp = O.SMALL_SHAPE
    atm = O.earth_atmosphere()
    lum = np.array([0.3, 0.2, 0.1, 0.05, 0.6, 0.1, 0.0, 0.1, 0.9])
    cpu = O.precompute(atm, shp, 3, lum=lum, blend=True, combined=False,
                       out=O.precompute(atm, shp, 3, combined=False))
    dev = O.gpu_precompute(atm, shp, 3, lum=lum, blend=True, combined=False,
                           out=O.precompute(atm, shp, 3, combined=False))
    agree("scattering", dev.scattering, cpu.scattering, 3)
    agree("single_mie", dev.single_mie, cpu.single_mie, 3)
    agree("irradiance", dev.irradiance, cpu.irradiance, 3)
