"""Known-answer tests of the CUDA passes, independent of the oracle.

atmosphere/reference/functions_test.cc:1130-1344 checks the order loop's
integrators against closed forms on inputs that make the integrals
analytic: uniform incident radiance, uniform ground irradiance, uniform
scattering density, unit transmittance.  Here the same inputs go, through
the C ABI's atmo_run_pass, into the CUDA kernels of both paths (the
restructured fast kernels: merged sky + ground tables, saturating lookups,
staged lines; and the plain per-texel kernels), on the functions_test.cc
fixture planet at the reference's default LUT shape, and EVERY texel of the
output is compared with the closed form:

* scattering density with uniform radiance L (order 3: delta multiple
  scattering) = the scattering coefficient x L -- functions_test.cc:1155-1180;
  at order 2 (single Rayleigh or single Mie = L; the fixture's Mie phase
  function with g = 0 is the Rayleigh one, P(nu) = 3 (1 + nu^2) / (16 pi)) the
  incident radiance is L P(nu_1), and the integral of P(nu_1) P(nu_2) over
  the sphere is 3 (26 + 2 nu^2) / (320 pi), nu the texel's own (the sphere
  integral of (a.w)^2 (b.w)^2 is 4 pi (1 + 2 (a.b)^2) / 15);
* scattering density with no radiance, uniform ground irradiance E and unit
  transmittance, at the bottom radius = (beta_R + beta_M) x albedo x E /
  (2 pi) -- :1182-1199 (which checks the horizontal direction; at r = R_b every
  direction's ground directions are exactly the lower hemisphere, whose
  phase integral is 1/2 for both phase functions);
* multiple scattering with uniform density j and unit transmittance = j x the
  distance to the nearest atmosphere boundary -- :1202-1235;
* indirect irradiance with uniform radiance L = pi x L -- :1325-1344.

Bars.  The density and indirect quadratures (16 x 32 midpoint directions, 16
x 64 hemisphere directions) integrate the phase functions and cos(theta)
with their own error: the density sums are 1.0012-1.0024 x the exact
integral (1.0024 at mu = +-1; 1.0009-1.0035 for the order-2 product of phase
functions), the hemisphere sum 1.0016082 x pi.  So the density texels must
lie in [1, 1.0025] (order 2: [1, 1.0035]) x the closed form (the reference
allows 2e-3 at its test point, where the quadrature gives 1.0012-1.0016),
the indirect texels within 1e-5 of 1.0016082 x pi L (and 1e-2 of pi L, the
reference's bar), the multiple-scattering texels within 1e-5 of j x d (the
trapezoid of a constant is exact)."""
import math

import numpy as np
import pytest

SHAPE = (256, 64, 32, 128, 32, 8, 64, 16)     # the reference's default sizes
KM = 1000.0
BETA_R, BETA_M = 0.001 / KM, 0.0015 / KM
HR, HM = 60.0 * KM, 30.0 * KM
RB, RT = 1000.0 * KM, 1500.0 * KM
ALBEDO = 0.1
HEMISPHERE_SUM = 1.0016081890839748   # sum of cos sin dtheta dphi over the 16 x 64 grid / pi


@pytest.fixture(scope="module")
def torch():
    import torch as t
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def toy(oracle):
    """The functions_test.cc fixture planet (Mie phase function g = 0)."""
    a = oracle.toy_atmosphere()
    assert a.mie_phase_function_g == 0.0
    return a


def luts(torch, fill=None):
    """Device LUTs of the default shape: T, delta R, delta M, delta I,
    delta J, S, I (fill: {name: value} for uniform RGB, alpha 1)."""
    tw, th, sr, smu, smus, snu, iw, ih = SHAPE
    dev = torch.device("cuda")
    s_shape = (sr, smu, snu * smus, 4)
    out = {"transmittance": torch.ones((th, tw, 4), device=dev),
           "delta_rayleigh": torch.zeros(s_shape, device=dev),
           "delta_mie": torch.zeros(s_shape, device=dev),
           "delta_irradiance": torch.zeros((ih, iw, 4), device=dev),
           "delta_density": torch.full(s_shape, -1.0, device=dev),
           "scattering": torch.zeros(s_shape, device=dev),
           "irradiance": torch.zeros((ih, iw, 4), device=dev)}
    for k, v in (fill or {}).items():
        out[k][..., :3] = v
        out[k][..., 3] = 1.0
    return out


def slice_altitudes():
    """Altitude of each r-slice's texel centre: rho = H k / (R - 1)
    (GetRMuMuSNuFromScatteringTextureUvwz's inverse mapping at a centre)."""
    sr = SHAPE[2]
    H = math.sqrt(RT * RT - RB * RB)
    rho = H * np.arange(sr) / (sr - 1)
    return np.sqrt(rho * rho + RB * RB) - RB


def ray_lengths():
    """[R][MU] distance from each texel's point to the nearest atmosphere
    boundary along its ray, from the texel-centre mapping of r and mu
    (functions.glsl:837-890)."""
    sr, smu = SHAPE[2], SHAPE[3]
    n = smu // 2
    H = math.sqrt(RT * RT - RB * RB)
    d = np.zeros((sr, smu))
    for k in range(sr):
        rho = H * k / (sr - 1)
        r = math.sqrt(rho * rho + RB * RB)
        for j in range(smu):
            if j < n:   # rays to the ground
                d_min, d_max = r - RB, rho
                d[k, j] = d_min + (d_max - d_min) * (n - 1 - j) / (n - 1)
            else:
                d_min, d_max = RT - r, rho + H
                d[k, j] = d_min + (d_max - d_min) * (j - n) / (n - 1)
    return d


def texel_nu():
    """[R][MU][NU * MU_S] nu of every scattering texel: the node's
    2 n / (NU - 1) - 1 clamped to the range mu and mu_s allow
    (functions.glsl:837-926 at texel centres), vectorised."""
    _, _, sr, smu, smus, snu, _, _ = SHAPE
    n2 = smu // 2
    H = math.sqrt(RT * RT - RB * RB)
    rho = H * np.arange(sr)[:, None] / (sr - 1)
    r = np.sqrt(rho * rho + RB * RB)
    j = np.arange(smu)[None, :]
    with np.errstate(divide="ignore", invalid="ignore"):
        dg = (r - RB) + (rho - (r - RB)) * (n2 - 1 - j) / (n2 - 1)
        ds = (RT - r) + (rho + H - (RT - r)) * (j - n2) / (n2 - 1)
        mu_g = np.where(dg == 0, -1.0, np.clip(-(rho * rho + dg * dg) / (2 * r * dg), -1, 1))
        mu_s_ = np.where(ds == 0, 1.0, np.clip((H * H - rho * rho - ds * ds) / (2 * r * ds),
                                               -1, 1))
    mu = np.where(j < n2, mu_g, mu_s_)                                  # [R][MU]
    x = np.arange(smus) / (smus - 1)
    d_min, d_max = RT - RB, H
    D = RB + RT                          # distance to the top from R_b at mu_s_min = -1
    A = (D - d_min) / (d_max - d_min)
    a = (A - x * A) / (1.0 + x * A)
    d = d_min + np.minimum(a, A) * (d_max - d_min)
    mus = np.where(d == 0, 1.0, np.clip((H * H - d * d) / (2 * RB * d), -1, 1))   # [MU_S]
    nu_node = np.clip(2.0 * np.arange(snu) / (snu - 1) - 1.0, -1, 1)             # [NU]
    m = mu[:, :, None, None]
    ms = mus[None, None, None, :]
    half = np.sqrt(np.maximum((1 - m * m) * (1 - ms * ms), 0.0))
    nu = np.clip(nu_node[None, None, :, None], m * ms - half, m * ms + half)
    return nu.reshape(sr, smu, snu * smus)


def test_texel_geometry_helper_matches_the_oracle(oracle):
    """The vectorised texel-centre mapping above against the oracle's
    (GetRMuMuSNuFromScatteringTextureFragCoord) on sampled texels."""
    import ctypes as C
    nu = texel_nu()
    L = oracle.lib()
    atm = toy(oracle)
    shp = oracle.shape(*SHAPE)
    rng = np.random.default_rng(5)
    for _ in range(500):
        z, y, x = (int(rng.integers(0, n)) for n in nu.shape)
        frag = (C.c_double * 3)(x + 0.5, y + 0.5, z + 0.5)
        out = (C.c_double * 4)()
        g = C.c_int()
        L.oracle_rmumusnu_from_frag_coord(C.byref(atm), C.byref(shp), frag, out, C.byref(g))
        assert abs(out[3] - nu[z, y, x]) <= 1e-9, (z, y, x, out[3], nu[z, y, x])


def ratio_to(got, expected_per_slice):
    g = got[..., 0].double().cpu().numpy()             # first wavelength only
    return g / np.asarray(expected_per_slice)[:, None, None]


PATHS = pytest.mark.parametrize("path_name", ["fast", "plain"])


def path_of(atmo, name):
    return atmo.PATH_FAST if name == "fast" else atmo.PATH_PLAIN


def assert_quadrature_ratio(ratio, what, hi=1.0025):
    assert np.isfinite(ratio).all(), what
    lo_, hi_ = float(ratio.min()), float(ratio.max())
    assert 1.0 - 1e-5 <= lo_ and hi_ <= hi, "%s: ratio to the closed form in [%.6f, %.6f]" % (
        what, lo_, hi_)


@pytest.mark.gpu
@PATHS
def test_density_uniform_multiple_scattering(atmo, oracle, torch, path_name):
    """Order 3, delta multiple scattering = L in every direction, no ground
    irradiance: J = (beta_R rho_R(h) + beta_M rho_M(h)) L at every texel."""
    L = 13.0
    b = luts(torch, {"delta_rayleigh": L})
    atmo.run_pass(toy(oracle), SHAPE, atmo.PASS_SCATTERING_DENSITY, 3,
                  path_of(atmo, path_name), **b)
    torch.cuda.synchronize()
    h = slice_altitudes()
    expected = (BETA_R * np.exp(-h / HR) + BETA_M * np.exp(-h / HM)) * L
    assert_quadrature_ratio(ratio_to(b["delta_density"], expected), "order-3 density")


@pytest.mark.gpu
@PATHS
@pytest.mark.parametrize("species", ["delta_rayleigh", "delta_mie"])
def test_density_order2_uniform_single_scattering(atmo, oracle, torch, path_name, species):
    """Order 2, single Rayleigh or single Mie = L (the other 0): the incident
    radiance is L P(nu_1), and J = (beta_R rho_R + beta_M rho_M) L x
    3 (26 + 2 nu^2) / (320 pi) at every texel (nu: the texel's own)."""
    L = 13.0
    b = luts(torch, {species: L})
    atmo.run_pass(toy(oracle), SHAPE, atmo.PASS_SCATTERING_DENSITY, 2,
                  path_of(atmo, path_name), **b)
    torch.cuda.synchronize()
    h = slice_altitudes()
    beta = BETA_R * np.exp(-h / HR) + BETA_M * np.exp(-h / HM)
    nu = texel_nu()
    expected = beta[:, None, None] * L * 3.0 * (26.0 + 2.0 * nu * nu) / (320.0 * math.pi)
    ratio = b["delta_density"][..., 0].double().cpu().numpy() / expected
    assert_quadrature_ratio(ratio, "order-2 density (%s)" % species, hi=1.0035)


@pytest.mark.gpu
@PATHS
@pytest.mark.parametrize("order", [2, 3])
def test_density_uniform_ground_irradiance(atmo, oracle, torch, path_name, order):
    """No radiance, ground irradiance E everywhere, unit transmittance: at
    the bottom radius every texel gets (beta_R + beta_M) albedo E / (2 pi)
    from the ground (the ground term of order 2 and the merged sky + ground
    tables above it)."""
    E = 13.0
    b = luts(torch, {"delta_irradiance": E})
    atmo.run_pass(toy(oracle), SHAPE, atmo.PASS_SCATTERING_DENSITY, order,
                  path_of(atmo, path_name), **b)
    torch.cuda.synchronize()
    expected = (BETA_R + BETA_M) * ALBEDO * E / (2.0 * math.pi)
    ratio = b["delta_density"][0, ..., 0].double().cpu().numpy() / expected
    assert_quadrature_ratio(ratio, "order-%d ground term at r = R_b" % order)
    # Above the ground fewer directions see it: less, never more.
    above = b["delta_density"][1:, ..., 0].double().cpu().numpy() / expected
    assert np.isfinite(above).all() and above.max() <= 1.0025 and above.min() >= 0.0


@pytest.mark.gpu
@PATHS
def test_multiple_scattering_uniform_density(atmo, oracle, torch, path_name):
    """Scattering density j everywhere, unit transmittance: delta multiple
    scattering = j x the ray's length to the nearest boundary, every texel."""
    j = 0.17
    b = luts(torch, {"delta_density": j})
    atmo.run_pass(toy(oracle), SHAPE, atmo.PASS_MULTIPLE_SCATTERING, 2,
                  path_of(atmo, path_name), **b)
    torch.cuda.synchronize()
    got = b["delta_rayleigh"][..., 0].double().cpu().numpy()
    want = np.broadcast_to(j * ray_lengths()[:, :, None], got.shape)
    zero = want == 0.0          # ground rays at the bottom radius have no length
    assert np.all(got[zero] == 0.0)
    rel = np.abs(got[~zero] - want[~zero]) / want[~zero]
    assert np.isfinite(rel).all() and float(rel.max()) <= 1e-5, float(rel.max())


@pytest.mark.gpu
@PATHS
def test_indirect_irradiance_uniform_radiance(atmo, oracle, torch, path_name):
    """Radiance L in every direction (delta multiple scattering, order 2): the
    irradiance is pi L at every texel (the hemisphere grid's own sum, 1.0016082
    pi, to 1e-5; the reference's bar is 1e-2 of pi L), added to the
    irradiance accumulator."""
    L = 1.0
    b = luts(torch, {"delta_rayleigh": L})
    b["irradiance"][..., :3] = 0.5
    atmo.run_pass(toy(oracle), SHAPE, atmo.PASS_INDIRECT_IRRADIANCE, 2,
                  path_of(atmo, path_name), **b)
    torch.cuda.synchronize()
    dI = b["delta_irradiance"][..., 0].double().cpu().numpy()
    assert float(np.abs(dI / (math.pi * L) - 1.0).max()) <= 1e-2
    assert float(np.abs(dI / (math.pi * L * HEMISPHERE_SUM) - 1.0).max()) <= 1e-5
    acc = b["irradiance"][..., 0].double().cpu().numpy()
    assert np.allclose(acc, 0.5 + dI, rtol=1e-6, atol=0)


@pytest.mark.gpu
def test_run_pass_rejects_missing_buffers(atmo, oracle, torch):
    b = luts(torch)
    del b["delta_density"]
    with pytest.raises(atmo.AtmoError) as e:
        atmo.run_pass(toy(oracle), SHAPE, atmo.PASS_SCATTERING_DENSITY, 3, **b)
    assert e.value.status == atmo.INVALID_ARG
