"""Generates the golden LUT fixtures in this directory from the reference's
own atmosphere/functions.glsl, compiled as C++ in double precision over
oracle/ref/ref_shim.h (oracle/_ref/libatmo_ref.so, built by `make -C oracle/ref`
where the reference sources are present).

Fixtures (numpy .npz):
  earth_small.npz     Earth atmosphere, LUT shape 64x16 / R4 MU16 MU_S8 NU4 /
                      16x4, 4 orders, combined textures: full float64 LUTs.
  toy_small.npz       the functions_test.cc fixture planet, same shape, 3 orders,
                      separate single-Mie texture: full float64 LUTs.
  earth_medium.npz    Earth, 128x32 / R8 MU32 MU_S16 NU8 / 32x8, 4 orders,
                      separate single-Mie texture: full float32 LUTs.
  earth_default.npz   Earth, the reference's default shape (256x64 /
                      R32 MU128 MU_S32 NU8 / 64x16), 4 orders, combined: all of
                      the irradiance LUT, every 7th transmittance texel and
                      every 61st scattering texel, as float32, with the flat
                      texel indices.

Run:  python tests/golden/make_golden.py      (several minutes: the default
shape is a full CPU precomputation of the reference)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402


def atm_fields(atm):
    return np.array([
        *atm.solar_irradiance, atm.sun_angular_radius, atm.bottom_radius, atm.top_radius,
        *[getattr(atm.rayleigh_density.layers[i], f) for i in range(2)
          for f in ("width", "exp_term", "exp_scale", "linear_term", "constant_term")],
        *atm.rayleigh_scattering,
        *[getattr(atm.mie_density.layers[i], f) for i in range(2)
          for f in ("width", "exp_term", "exp_scale", "linear_term", "constant_term")],
        *atm.mie_scattering, *atm.mie_extinction, atm.mie_phase_function_g,
        *[getattr(atm.absorption_density.layers[i], f) for i in range(2)
          for f in ("width", "exp_term", "exp_scale", "linear_term", "constant_term")],
        *atm.absorption_extinction, *atm.ground_albedo, atm.mu_s_min])


def run(atm, shp, orders, combined):
    return O.precompute(atm, shp, orders, combined=combined, use_reference=True)


def main():
    O.build()
    if O.ref_lib() is None:
        raise SystemExit("the reference build oracle/_ref/libatmo_ref.so is missing")
    earth = O.earth_atmosphere()
    toy = O.toy_atmosphere()

    luts = run(earth, O.SMALL_SHAPE, 4, True)
    np.savez_compressed(os.path.join(HERE, "earth_small.npz"), atmosphere=atm_fields(earth),
                        shape=np.array(O.SMALL_SHAPE), orders=4, combined=1,
                        transmittance=luts.transmittance, scattering=luts.scattering,
                        irradiance=luts.irradiance)

    luts = run(toy, O.SMALL_SHAPE, 3, False)
    np.savez_compressed(os.path.join(HERE, "toy_small.npz"), atmosphere=atm_fields(toy),
                        shape=np.array(O.SMALL_SHAPE), orders=3, combined=0,
                        transmittance=luts.transmittance, scattering=luts.scattering,
                        single_mie=luts.single_mie, irradiance=luts.irradiance)

    luts = run(earth, O.MEDIUM_SHAPE, 4, False)
    f32 = np.float32
    np.savez_compressed(os.path.join(HERE, "earth_medium.npz"), atmosphere=atm_fields(earth),
                        shape=np.array(O.MEDIUM_SHAPE), orders=4, combined=0,
                        transmittance=luts.transmittance.astype(f32),
                        scattering=luts.scattering.astype(f32),
                        single_mie=luts.single_mie.astype(f32),
                        irradiance=luts.irradiance.astype(f32))

    luts = run(earth, O.DEFAULT_SHAPE, 4, True)
    t_flat = luts.transmittance.reshape(-1, 4)
    s_flat = luts.scattering.reshape(-1, 4)
    t_idx = np.arange(0, t_flat.shape[0], 7)
    s_idx = np.arange(0, s_flat.shape[0], 61)
    np.savez_compressed(os.path.join(HERE, "earth_default.npz"), atmosphere=atm_fields(earth),
                        shape=np.array(O.DEFAULT_SHAPE), orders=4, combined=1,
                        transmittance_index=t_idx, transmittance=t_flat[t_idx].astype(f32),
                        scattering_index=s_idx, scattering=s_flat[s_idx].astype(f32),
                        irradiance=luts.irradiance.astype(f32))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
