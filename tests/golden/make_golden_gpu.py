"""Generates the golden fixtures of the two GPU-only configurations from the
FP64 GPU oracle (oracle/atmo_oracle_gpu.cu: the CPU oracle's evaluators as
device code, pinned to the CPU oracle within 1e-8 by tests/test_gpu_oracle.py).
Needs a CUDA device; run on the GPU host and commit the outputs.

Fixtures (numpy .npz, float32 values with their flat texel indices):
  spectral_default.npz  the spectral-precision configuration (15 wavelengths in
                        5 groups, seeded smooth solar spectrum, the reference's
                        default LUT shape, 4 orders, separate single-Mie LUT):
                        the luminance-mode LUTs composed from the five groups
                        (atmosphere/model.cc:914-963) -- every 7th transmittance
                        texel, every 61st scattering and single-Mie texel, all
                        irradiance texels.
  hires_earth.npz       the high-resolution configuration (transmittance
                        512x128, scattering NU16 x MU_S64 x MU256 x R64,
                        irradiance 128x32, 8 orders, Earth with Mie g = 0.76 and
                        ground albedo 0.3, combined textures) -- every 17th
                        transmittance texel, every 4099th scattering texel, all
                        irradiance texels.

Run:  python tests/golden/make_golden_gpu.py      (~2 minutes on a GB300)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle as O  # noqa: E402
from golden.make_golden import atm_fields  # noqa: E402


def sampled(lut, stride):
    flat = np.asarray(lut, np.float64).reshape(-1, 4)
    idx = np.arange(0, flat.shape[0], stride, dtype=np.int64)
    return flat[idx].astype(np.float32), idx


def main():
    import precomputed_atmospheric_scattering_gb300 as atmo
    from precomputed_atmospheric_scattering_gb300 import workloads as W
    from test_gpu_parity import oracle_luminance_model

    O.build()
    atmo.build()

    m = W.spectral_earth_model(W.DEFAULT)
    ref = oracle_luminance_model(O, m, 4, W.DEFAULT, precompute=O.gpu_precompute)
    t, ti = sampled(ref.transmittance, 7)
    s, si = sampled(ref.scattering, 61)
    mie, _ = sampled(ref.single_mie, 61)
    np.savez_compressed(os.path.join(HERE, "spectral_default.npz"),
                        wavelengths=np.arange(360.0, 831.0, 10.0),
                        solar_irradiance=W.smooth_solar_spectrum(1, np.arange(360.0, 831.0, 10.0)),
                        shape=np.array(W.DEFAULT), orders=4, combined=0, seed=1,
                        transmittance=t, transmittance_index=ti, scattering=s,
                        scattering_index=si, single_mie=mie,
                        irradiance=np.asarray(ref.irradiance, np.float32).reshape(-1, 4))

    atm = O.Atmosphere.from_buffer_copy(bytes(W.hires_earth()))
    ref = O.gpu_precompute(atm, W.HIRES, 8, combined=True)
    t, ti = sampled(ref.transmittance, 17)
    s, si = sampled(ref.scattering, 4099)
    np.savez_compressed(os.path.join(HERE, "hires_earth.npz"), atmosphere=atm_fields(atm),
                        shape=np.array(W.HIRES), orders=8, combined=1,
                        transmittance=t, transmittance_index=ti, scattering=s,
                        scattering_index=si,
                        irradiance=np.asarray(ref.irradiance, np.float32).reshape(-1, 4))
    print("wrote spectral_default.npz and hires_earth.npz")


if __name__ == "__main__":
    main()
