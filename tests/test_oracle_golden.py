"""Pins the oracle restatement (oracle/atmo_oracle.cc) to the reference's own
atmosphere/functions.glsl: against the golden LUT fixtures generated from the
reference compiled as C++ (tests/golden/make_golden.py), and, where that build
is present (oracle/_ref), against it directly."""
import ctypes as C
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def atmosphere_from_fields(O, f):
    f = list(f)
    take = lambda n: [f.pop(0) for _ in range(n)]  # noqa: E731
    def prof():
        v = take(10)
        return O.profile(O.layer(*v[:5]), O.layer(*v[5:]))
    a = O.Atmosphere()
    a.solar_irradiance = (C.c_double * 3)(*take(3))
    a.sun_angular_radius, a.bottom_radius, a.top_radius = take(3)
    a.rayleigh_density = prof()
    a.rayleigh_scattering = (C.c_double * 3)(*take(3))
    a.mie_density = prof()
    a.mie_scattering = (C.c_double * 3)(*take(3))
    a.mie_extinction = (C.c_double * 3)(*take(3))
    (a.mie_phase_function_g,) = take(1)
    a.absorption_density = prof()
    a.absorption_extinction = (C.c_double * 3)(*take(3))
    a.ground_albedo = (C.c_double * 3)(*take(3))
    (a.mu_s_min,) = take(1)
    assert not f
    return a


@pytest.mark.parametrize("name", ["earth_small.npz", "toy_small.npz"])
def test_oracle_matches_reference_bitwise_small(oracle, name):
    g = load(name)
    atm = atmosphere_from_fields(oracle, g["atmosphere"])
    luts = oracle.precompute(atm, tuple(g["shape"]), int(g["orders"]),
                             combined=bool(g["combined"]))
    np.testing.assert_array_equal(luts.transmittance, g["transmittance"])
    np.testing.assert_array_equal(luts.scattering, g["scattering"])
    np.testing.assert_array_equal(luts.irradiance, g["irradiance"])
    if "single_mie" in g:
        np.testing.assert_array_equal(luts.single_mie, g["single_mie"])


def test_oracle_matches_reference_medium(oracle):
    g = load("earth_medium.npz")
    atm = atmosphere_from_fields(oracle, g["atmosphere"])
    luts = oracle.precompute(atm, tuple(g["shape"]), int(g["orders"]), combined=False)
    for k in ("transmittance", "scattering", "single_mie", "irradiance"):
        np.testing.assert_allclose(getattr(luts, k).astype(np.float32), g[k], rtol=1e-6,
                                   atol=1e-30)


def test_golden_default_shape_fixture_is_consistent(oracle):
    """The sampled default-shape fixture covers every irradiance texel and is
    finite and non-negative (its full check is the GPU parity test)."""
    g = load("earth_default.npz")
    assert tuple(g["shape"]) == oracle.DEFAULT_SHAPE
    assert g["irradiance"].shape == (16, 64, 4)
    for k in ("transmittance", "scattering", "irradiance"):
        assert np.all(np.isfinite(g[k])) and np.all(g[k][..., :3] >= 0)
    assert np.all(g["transmittance"][:, :3] <= 1.0)


def test_oracle_against_reference_build(oracle):
    """Direct comparison with the reference's functions.glsl compiled here
    (skipped where the reference sources are not present)."""
    if oracle.ref_lib() is None:
        pytest.skip("reference build oracle/_ref not present on this machine")
    wide_nu = (64, 16, 4, 16, 8, 128, 16, 4)   # 128 nu nodes: lookups far from column 0
    for shp in (oracle.SMALL_SHAPE, oracle.MEDIUM_SHAPE, wide_nu):
        for combined in ((True,) if shp == wide_nu else (True, False)):
            atm = oracle.earth_atmosphere(mie_g=0.7, ground_albedo=0.3)
            a = oracle.precompute(atm, shp, 3, combined=combined)
            b = oracle.precompute(atm, shp, 3, combined=combined, use_reference=True)
            for k in ("transmittance", "scattering", "single_mie", "irradiance"):
                np.testing.assert_array_equal(getattr(a, k), getattr(b, k))


def test_oracle_render_functions_against_reference_build(oracle):
    """GetSkyRadiance / GetSkyRadianceToPoint / GetSunAndSkyIrradiance of the
    restatement against the reference's (non-combined layout)."""
    R = oracle.ref_lib()
    if R is None:
        pytest.skip("reference build oracle/_ref not present on this machine")
    L = oracle.lib()
    shp = oracle.shape(*oracle.SMALL_SHAPE)
    atm = oracle.earth_atmosphere()
    luts = oracle.precompute(atm, shp, 4, combined=False)
    dp = oracle.dp
    T, S, M, I = (x.ctypes.data_as(dp) for x in (luts.transmittance, luts.scattering,
                                                 luts.single_mie, luts.irradiance))
    rng = np.random.default_rng(7)
    by = C.byref
    for _ in range(50):
        cam = np.array([0.0, 0.0, 6360.0 + rng.uniform(0.0, 100.0)])
        v = rng.normal(size=3); v /= np.linalg.norm(v)
        sun = rng.normal(size=3); sun /= np.linalg.norm(sun)
        pt = cam + v * rng.uniform(0.1, 50.0)
        pt *= max(1.0, 6360.5 / np.linalg.norm(pt))
        shadow = float(rng.choice([0.0, rng.uniform(0.0, 5.0)]))
        for fo, fr, x in ((L.oracle_sky_radiance, R.ref_sky_radiance, v),
                          (L.oracle_sky_radiance_to_point, R.ref_sky_radiance_to_point, pt)):
            o1, t1, o2, t2 = (np.zeros(3) for _ in range(4))
            fo(by(atm), by(shp), T, S, M, 0, cam.ctypes.data_as(dp), x.ctypes.data_as(dp),
               shadow, sun.ctypes.data_as(dp), o1.ctypes.data_as(dp), t1.ctypes.data_as(dp))
            fr(by(atm), by(shp), T, S, M, cam.ctypes.data_as(dp), x.ctypes.data_as(dp), shadow,
               sun.ctypes.data_as(dp), o2.ctypes.data_as(dp), t2.ctypes.data_as(dp))
            np.testing.assert_array_equal(o1, o2)
            np.testing.assert_array_equal(t1, t2)
        n = rng.normal(size=3); n /= np.linalg.norm(n)
        a1, b1, a2, b2 = (np.zeros(3) for _ in range(4))
        L.oracle_sun_and_sky_irradiance(by(atm), by(shp), T, I, pt.ctypes.data_as(dp),
                                        n.ctypes.data_as(dp), sun.ctypes.data_as(dp),
                                        a1.ctypes.data_as(dp), b1.ctypes.data_as(dp))
        R.ref_sun_and_sky_irradiance(by(atm), by(shp), T, I, pt.ctypes.data_as(dp),
                                     n.ctypes.data_as(dp), sun.ctypes.data_as(dp),
                                     a2.ctypes.data_as(dp), b2.ctypes.data_as(dp))
        np.testing.assert_array_equal(a1, a2)
        np.testing.assert_array_equal(b1, b2)
