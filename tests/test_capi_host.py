"""CPU tests of the boundary: libatmo_gb300.so loads and exports every entry
point include/atmo/atmo.h declares, and the host-side logic of the Model
(parameter conversion of atmosphere/model.cc:613-745, wavelength groups,
luminance factors, GLSL header, validation) agrees with the oracle.  No
compute kernel runs here."""
import ctypes as C
import math
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "atmo", "atmo.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(atmo_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(atmo):
    syms = declared_symbols()
    assert len(syms) >= 25
    L = C.CDLL(atmo.LIB_PATH)
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    assert L.atmo_abi_version() == 3


def earth_model(atmo, n_lambda=3, combined=True, half=False, shape=None):
    w = np.arange(360.0, 831.0, 10.0)
    lam = w * 1e-3
    mie = 5.328e-3 / 1200.0 * np.ones_like(w)
    xs = np.array([1.18e-27, 2.182e-28, 2.818e-28, 6.636e-28, 1.527e-27, 2.763e-27, 5.52e-27,
                   8.451e-27, 1.582e-26, 2.316e-26, 3.669e-26, 4.924e-26, 7.752e-26, 9.016e-26,
                   1.48e-25, 1.602e-25, 2.139e-25, 2.755e-25, 3.091e-25, 3.5e-25, 4.266e-25,
                   4.672e-25, 4.398e-25, 4.701e-25, 5.019e-25, 4.305e-25, 3.74e-25, 3.215e-25,
                   2.662e-25, 2.238e-25, 1.852e-25, 1.473e-25, 1.209e-25, 9.423e-26, 7.455e-26,
                   6.566e-26, 5.105e-26, 4.15e-26, 4.228e-26, 3.237e-26, 2.451e-26, 2.801e-26,
                   2.534e-26, 1.624e-26, 1.465e-26, 2.078e-26, 1.383e-26, 7.105e-27])
    ozone = 300.0 * 2.687e20 / 15000.0 * xs
    L = atmo.DensityProfileLayer
    return atmo.Model(w, np.full_like(w, 1.5), 0.00935 / 2.0, 6360e3, 6420e3,
                      [L(0.0, 1.0, -1.0 / 8000.0, 0.0, 0.0)], 1.24062e-6 * lam ** -4,
                      [L(0.0, 1.0, -1.0 / 1200.0, 0.0, 0.0)], mie * 0.9, mie, 0.8,
                      [L(25000.0, 0.0, 0.0, 1.0 / 15000.0, -2.0 / 3.0),
                       L(0.0, 0.0, 0.0, -1.0 / 15000.0, 8.0 / 3.0)], ozone,
                      np.full_like(w, 0.1), 102.0 / 180.0 * math.pi, 1000.0, n_lambda, combined,
                      half, lut_shape=shape)


def test_model_parameter_conversion_matches_reference_rules(atmo, oracle):
    m = earth_model(atmo)
    a = m.atmosphere_at()
    # std::to_string rounding (model.cc:636-666): 6 decimals in length units.
    assert list(a.rayleigh_scattering) == [0.005802, 0.013558, 0.0331]
    assert list(a.absorption_extinction) == [0.00065, 0.001881, 0.000085]
    assert a.mu_s_min == -0.207912
    assert a.bottom_radius == 6360.0 and a.top_radius == 6420.0
    assert a.mie_density.layers[1].exp_scale == -0.833333
    assert a.absorption_density.layers[0].width == 25.0
    assert a.absorption_density.layers[0].constant_term == -0.666667
    # Profiles given with one layer are padded in front (model.cc:676-690).
    assert a.rayleigh_density.layers[0].width == 0 and a.rayleigh_density.layers[0].exp_term == 0
    m.set_exact_parameters(True)
    e = m.atmosphere_at()
    ref = oracle.earth_atmosphere()
    np.testing.assert_allclose(list(e.rayleigh_scattering), list(ref.rayleigh_scattering),
                               rtol=1e-12)
    np.testing.assert_allclose(list(e.absorption_extinction), list(ref.absorption_extinction),
                               rtol=1e-12)
    assert abs(e.mu_s_min - ref.mu_s_min) < 1e-15


def test_interpolation_between_wavelength_samples(atmo, oracle):
    m = earth_model(atmo)
    m.set_exact_parameters(True)
    w = np.arange(360.0, 831.0, 10.0)
    ray = 1.24062e-6 * (w * 1e-3) ** -4
    lam = (365.0, 512.5, 829.0)
    a = m.atmosphere_at(lam)
    for i, l in enumerate(lam):
        exp = oracle.lib().oracle_interpolate(w.ctypes.data_as(oracle.dp),
                                              ray.ctypes.data_as(oracle.dp), len(w), l)
        assert abs(a.rayleigh_scattering[i] - exp * 1000.0) < 1e-15


def test_luminance_factors_match_oracle(atmo, oracle):
    m = earth_model(atmo)
    sky, sun = m.luminance_factors()
    w = np.arange(360.0, 831.0, 10.0)
    sol = np.full_like(w, 1.5)
    k = np.zeros(3)
    oracle.lib().oracle_radiance_to_luminance_factors(w.ctypes.data_as(oracle.dp),
                                                      sol.ctypes.data_as(oracle.dp), len(w),
                                                      -3.0, k.ctypes.data_as(oracle.dp))
    np.testing.assert_allclose(sky, k, rtol=1e-12)
    oracle.lib().oracle_radiance_to_luminance_factors(w.ctypes.data_as(oracle.dp),
                                                      sol.ctypes.data_as(oracle.dp), len(w),
                                                      0.0, k.ctypes.data_as(oracle.dp))
    np.testing.assert_allclose(sun, k, rtol=1e-12)
    # Precomputed-illuminance mode uses MAX_LUMINOUS_EFFICACY (model.cc:663-673).
    sky15, _ = earth_model(atmo, n_lambda=15).luminance_factors()
    assert sky15 == (683.0, 683.0, 683.0)


def test_convert_spectrum_to_linear_srgb_matches_oracle(atmo, oracle):
    w = np.arange(360.0, 831.0, 10.0)
    s = 1.0 + 0.5 * np.sin(w / 40.0)
    got = atmo.Model.ConvertSpectrumToLinearSrgb(w, s)
    exp = np.zeros(3)
    oracle.lib().oracle_convert_spectrum_to_linear_srgb(w.ctypes.data_as(oracle.dp),
                                                        s.ctypes.data_as(oracle.dp), len(w),
                                                        exp.ctypes.data_as(oracle.dp))
    np.testing.assert_allclose(got, exp, rtol=1e-12)


def reference_glsl_header(w, solar, sun_angular_radius, bottom, top, ray_layers, ray_sca,
                          mie_layers, mie_sca, mie_ext, g, abs_layers, abs_ext, albedo,
                          max_sun_zenith, unit, n_lambda, combined, shape, sky_k, sun_k):
    """A restatement of the reference's GLSL header factory
    (atmosphere/model.cc:636-744) for lambdas = kLambdaR/G/B, with the two
    GLSL files it splices in (definitions.glsl, functions.glsl) replaced by
    the marker lines the library writes in their place.  std::to_string of a
    double is printf's "%f"."""
    def interpolate(values, lam):            # atmosphere/model.cc:535-552
        if lam < w[0]:
            return values[0]
        for i in range(len(w) - 1):
            if lam < w[i + 1]:
                u = (lam - w[i]) / (w[i + 1] - w[i])
                return values[i] * (1.0 - u) + values[i + 1] * u
        return values[-1]

    f = lambda x: "%f" % x                   # noqa: E731
    lambdas = (680.0, 550.0, 440.0)

    def to_string(v, scale):
        return "vec3(" + ",".join(f(interpolate(v, l) * scale) for l in lambdas) + ")"

    def layer(x):
        width, exp_term, exp_scale, linear_term, constant_term = x
        return "DensityProfileLayer(%s,%s,%s,%s,%s)" % (
            f(width / unit), f(exp_term), f(exp_scale * unit), f(linear_term * unit),
            f(constant_term))

    def profile(layers):
        layers = [(0.0, 0.0, 0.0, 0.0, 0.0)] * (2 - len(layers)) + list(layers)
        return "DensityProfile(DensityProfileLayer[2](" + layer(layers[0]) + "," + \
            layer(layers[1]) + "))"

    tw, th, sr, smu, smus, snu, iw, ih = shape
    return ("#version 330\n#define IN(x) const in x\n#define OUT(x) out x\n"
            "#define TEMPLATE(x)\n#define TEMPLATE_ARGUMENT(x)\n#define assert(x)\n"
            "const int TRANSMITTANCE_TEXTURE_WIDTH = %d;\n"
            "const int TRANSMITTANCE_TEXTURE_HEIGHT = %d;\n"
            "const int SCATTERING_TEXTURE_R_SIZE = %d;\n"
            "const int SCATTERING_TEXTURE_MU_SIZE = %d;\n"
            "const int SCATTERING_TEXTURE_MU_S_SIZE = %d;\n"
            "const int SCATTERING_TEXTURE_NU_SIZE = %d;\n"
            "const int IRRADIANCE_TEXTURE_WIDTH = %d;\n"
            "const int IRRADIANCE_TEXTURE_HEIGHT = %d;\n" % (tw, th, sr, smu, smus, snu, iw, ih) +
            ("#define COMBINED_SCATTERING_TEXTURES\n" if combined else "") +
            "// <atmosphere/definitions.glsl of the reference goes here>\n" +
            "const AtmosphereParameters ATMOSPHERE = AtmosphereParameters(\n" +
            to_string(solar, 1.0) + ",\n" + f(sun_angular_radius) + ",\n" +
            f(bottom / unit) + ",\n" + f(top / unit) + ",\n" + profile(ray_layers) + ",\n" +
            to_string(ray_sca, unit) + ",\n" + profile(mie_layers) + ",\n" +
            to_string(mie_sca, unit) + ",\n" + to_string(mie_ext, unit) + ",\n" + f(g) + ",\n" +
            profile(abs_layers) + ",\n" + to_string(abs_ext, unit) + ",\n" +
            to_string(albedo, 1.0) + ",\n" + f(math.cos(max_sun_zenith)) + ");\n" +
            "const vec3 SKY_SPECTRAL_RADIANCE_TO_LUMINANCE = vec3(%s,%s,%s);\n" % tuple(
                f(x) for x in sky_k) +
            "const vec3 SUN_SPECTRAL_RADIANCE_TO_LUMINANCE = vec3(%s,%s,%s);\n" % tuple(
                f(x) for x in sun_k) +
            "// <atmosphere/functions.glsl of the reference goes here>\n")


@pytest.mark.parametrize("n_lambda,combined", [(3, True), (15, False)])
def test_shader_source_header_is_the_reference_header(atmo, oracle, n_lambda, combined):
    """The generated header, byte for byte, against the restatement of
    model.cc:636-744 for the same constructor arguments (3 wavelengths with
    combined textures: the radiance API; 15 wavelengths with a separate
    single-Mie texture: precomputed luminance, SKY_..._TO_LUMINANCE = 683)."""
    w = np.arange(360.0, 831.0, 10.0)
    lam = w * 1e-3
    mie = 5.328e-3 / 1200.0 * np.ones_like(w)
    m = earth_model(atmo, n_lambda=n_lambda, combined=combined)
    solar = np.full_like(w, 1.5)
    sun_k = np.zeros(3)
    L = oracle.lib()
    L.oracle_radiance_to_luminance_factors(w.ctypes.data_as(oracle.dp),
                                           solar.ctypes.data_as(oracle.dp), len(w), 0.0,
                                           sun_k.ctypes.data_as(oracle.dp))
    if n_lambda > 3:
        sky_k = np.full(3, 683.0)
    else:
        sky_k = np.zeros(3)
        L.oracle_radiance_to_luminance_factors(w.ctypes.data_as(oracle.dp),
                                               solar.ctypes.data_as(oracle.dp), len(w), -3.0,
                                               sky_k.ctypes.data_as(oracle.dp))
    xs = np.array([1.18e-27, 2.182e-28, 2.818e-28, 6.636e-28, 1.527e-27, 2.763e-27, 5.52e-27,
                   8.451e-27, 1.582e-26, 2.316e-26, 3.669e-26, 4.924e-26, 7.752e-26, 9.016e-26,
                   1.48e-25, 1.602e-25, 2.139e-25, 2.755e-25, 3.091e-25, 3.5e-25, 4.266e-25,
                   4.672e-25, 4.398e-25, 4.701e-25, 5.019e-25, 4.305e-25, 3.74e-25, 3.215e-25,
                   2.662e-25, 2.238e-25, 1.852e-25, 1.473e-25, 1.209e-25, 9.423e-26, 7.455e-26,
                   6.566e-26, 5.105e-26, 4.15e-26, 4.228e-26, 3.237e-26, 2.451e-26, 2.801e-26,
                   2.534e-26, 1.624e-26, 1.465e-26, 2.078e-26, 1.383e-26, 7.105e-27])
    want = reference_glsl_header(
        list(w), list(solar), 0.00935 / 2.0, 6360e3, 6420e3, [(0.0, 1.0, -1.0 / 8000.0, 0.0, 0.0)],
        list(1.24062e-6 * lam ** -4), [(0.0, 1.0, -1.0 / 1200.0, 0.0, 0.0)], list(mie * 0.9),
        list(mie), 0.8, [(25000.0, 0.0, 0.0, 1.0 / 15000.0, -2.0 / 3.0),
                         (0.0, 0.0, 0.0, -1.0 / 15000.0, 8.0 / 3.0)],
        list(300.0 * 2.687e20 / 15000.0 * xs), list(np.full_like(w, 0.1)),
        102.0 / 180.0 * math.pi, 1000.0, n_lambda, combined, atmo.DEFAULT_SHAPE, sky_k, sun_k)
    src = m.shader()
    assert src[:len(want)] == want
    # Then the API shader of model.cc:221-281 (the radiance API only below 4
    # precomputed wavelengths).
    api = src[len(want):]
    assert api.startswith("#define RADIANCE_API_ENABLED\n") == (n_lambda <= 3)
    for fn in ("GetSolarLuminance", "GetSkyLuminance", "GetSkyLuminanceToPoint",
               "GetSunAndSkyIlluminance"):
        assert fn + "(" in api
    # The radiance functions sit between #ifdef RADIANCE_API_ENABLED and #endif.
    guarded = api[api.index("#ifdef RADIANCE_API_ENABLED\n"):api.index("#endif\n")]
    for fn in ("GetSolarRadiance", "GetSkyRadiance", "GetSkyRadianceToPoint",
               "GetSunAndSkyIrradiance"):
        assert fn + "(" in guarded


def test_set_program_uniforms_is_unavailable(atmo):
    m = earth_model(atmo)
    with pytest.raises(atmo.Unavailable):
        m.SetProgramUniforms(1, 0, 1, 2)


@pytest.mark.parametrize("bad", ["nan", "top_below_bottom", "layers", "shape", "g"])
def test_invalid_parameters_are_rejected(atmo, bad):
    w = np.array([400.0, 500.0, 600.0, 700.0])
    L = atmo.DensityProfileLayer
    args = dict(wavelengths=w, solar_irradiance=np.ones(4), sun_angular_radius=0.004675,
                bottom_radius=6360e3, top_radius=6420e3,
                rayleigh_density=[L(0, 1, -1 / 8000.0, 0, 0)],
                rayleigh_scattering=np.full(4, 1e-5), mie_density=[L(0, 1, -1 / 1200.0, 0, 0)],
                mie_scattering=np.full(4, 4e-6), mie_extinction=np.full(4, 4.4e-6),
                mie_phase_function_g=0.8, absorption_density=[], absorption_extinction=np.zeros(4),
                ground_albedo=np.full(4, 0.1), max_sun_zenith_angle=2.0,
                length_unit_in_meters=1000.0, num_precomputed_wavelengths=3,
                combine_scattering_textures=True, half_precision=False)
    if bad == "nan":
        args["rayleigh_scattering"] = np.array([1e-5, np.nan, 1e-5, 1e-5])
    elif bad == "top_below_bottom":
        args["top_radius"] = 6000e3
    elif bad == "layers":
        args["mie_density"] = [L(), L(), L()]
    elif bad == "shape":
        args["lut_shape"] = (256, 64, 32, 127, 32, 8, 64, 16)
    elif bad == "g":
        args["mie_phase_function_g"] = 1.0
    with pytest.raises(atmo.AtmoError) as e:
        atmo.Model(**args)
    assert e.value.status == atmo.INVALID_ARG


def test_luminance_groups_of_fifteen_wavelengths(atmo):
    """model.cc:915-924: 5 groups at 360 + (3i + {0.5, 1.5, 2.5}) * 470 / 15."""
    m = earth_model(atmo, n_lambda=15)
    m.set_exact_parameters(True)
    d = 470.0 / 15.0
    for i in range(5):
        lam = [360.0 + (3 * i + k + 0.5) * d for k in range(3)]
        a = m.atmosphere_at(lam)
        assert all(np.isfinite(list(a.rayleigh_scattering)))
