"""GPU parity of the CUDA precomputation against the FP64 oracle and the golden
fixtures of the reference (tests/golden/), through the C ABI.

Tolerances (tests/parity.py): per-texel relative error <= 1e-4 for the
transmittance LUT and <= 1e-3 for scattering, single-Mie and irradiance, with
an absolute floor at 1e-6 of each channel's maximum."""
import ctypes as C
import math
import os

import numpy as np
import pytest

from parity import (TOL_IRRADIANCE, TOL_SCATTERING, TOL_TRANSMITTANCE, check, check_masked,
                    robust_masks)
from test_capi_host import earth_model

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def torch():
    import torch as t
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def gpu_precompute(atmo, torch, atm, shape, orders, combined=True, path=0, lum=None,
                   blend=False, init=None):
    """atmo_precompute into fresh device buffers; returns host float32 LUTs."""
    s = atmo.LutShape.of(shape)
    W = s.scattering_nu * s.scattering_mu_s
    dev = torch.device("cuda")
    T = torch.zeros((s.transmittance_height, s.transmittance_width, 4), device=dev)
    S = torch.zeros((s.scattering_r, s.scattering_mu, W, 4), device=dev)
    M = torch.zeros_like(S)
    I = torch.zeros((s.irradiance_height, s.irradiance_width, 4), device=dev)
    if init is not None:
        for t, v in zip((T, S, M, I), init):
            t.copy_(torch.from_numpy(np.ascontiguousarray(v, np.float32)))
    atmo.precompute(atm, s, orders, T, S, None if combined else M, I, lum=lum, blend=blend,
                    combined=combined, path=path)
    torch.cuda.synchronize()
    return [x.cpu().numpy() for x in (T, S, M, I)]


def compare(oracle_luts, gpu, combined, report=None):
    T, S, M, I = gpu
    check("transmittance", T, oracle_luts.transmittance, TOL_TRANSMITTANCE, report=report)
    check("scattering", S, oracle_luts.scattering, TOL_SCATTERING,
          channels=4 if combined else 3, report=report)
    if not combined:
        check("single_mie", M, oracle_luts.single_mie, TOL_SCATTERING, report=report)
    check("irradiance", I, oracle_luts.irradiance, TOL_IRRADIANCE, report=report)


@pytest.mark.parametrize("path", [0, 1], ids=["fast", "plain"])
@pytest.mark.parametrize("combined", [True, False], ids=["combined", "separate"])
def test_small_shape_earth_vs_oracle(atmo, oracle, torch, path, combined):
    atm = oracle.earth_atmosphere()
    ref = oracle.precompute(atm, oracle.SMALL_SHAPE, 4, combined=combined)
    gpu = gpu_precompute(atmo, torch, atm, oracle.SMALL_SHAPE, 4, combined, path)
    compare(ref, gpu, combined)


def compare_robust(oracle, atm, shape, orders, gpu, combined, report=None):
    ref, masks = robust_masks(oracle, atm, shape, orders, combined)
    T, S, M, I = gpu
    check_masked("transmittance", T, ref.transmittance, TOL_TRANSMITTANCE,
                 masks["transmittance"], report=report)
    check_masked("scattering", S, ref.scattering, TOL_SCATTERING, masks["scattering"],
                 channels=4 if combined else 3, report=report)
    if not combined:
        check_masked("single_mie", M, ref.single_mie, TOL_SCATTERING, masks["single_mie"],
                     report=report)
    check_masked("irradiance", I, ref.irradiance, TOL_IRRADIANCE, masks["irradiance"],
                 report=report)


@pytest.mark.parametrize("path", [0, 1], ids=["fast", "plain"])
@pytest.mark.parametrize("nu", [2, 33, 38, 128])
def test_extreme_nu_sizes_vs_oracle(atmo, oracle, torch, nu, path):
    """NU = 2: the density kernel's staged rows are two nodes between their
    end entries; NU = 33: odd, so (n + u_mu_s) / NU is inexact in FP32 and
    the lookups must keep the within-block coordinate apart from the block;
    NU = 38, 128: the density tables exceed 48 KB per block and the fast path
    hands the density pass to the plain kernel, and the column coordinates of
    the 4D lookups reach 1024.  Every texel, no mask."""
    shape = (64, 16, 4, 16, 8, nu, 16, 4)
    atm = oracle.earth_atmosphere()
    ref = oracle.precompute(atm, shape, 4, combined=True)
    compare(ref, gpu_precompute(atmo, torch, atm, shape, 4, True, path), True)


@pytest.mark.parametrize("path", [0, 1], ids=["fast", "plain"])
@pytest.mark.parametrize("orders", [1, 2, 12])
def test_minimal_shape_vs_oracle(atmo, oracle, torch, orders, path):
    """The smallest shape the C ABI accepts (every size 2, MU = 4: one texel
    row per ray half, transmittance and irradiance of 2 x 2 texels), for one
    order, two, and twelve (the long tail of many small orders)."""
    shape = (2, 2, 2, 4, 2, 2, 2, 2)
    atm = oracle.earth_atmosphere()
    ref = oracle.precompute(atm, shape, orders, combined=False)
    compare(ref, gpu_precompute(atmo, torch, atm, shape, orders, False, path), False)


@pytest.mark.parametrize("path", [0, 1], ids=["fast", "plain"])
def test_odd_sizes_vs_oracle(atmo, oracle, torch, path):
    """Odd sizes everywhere but MU (which must be even): transmittance 33 x 9,
    scattering R 5 x MU 14 x MU_S 5 x NU 3 (line width W = 15), irradiance
    17 x 5."""
    shape = (33, 9, 5, 14, 5, 3, 17, 5)
    atm = oracle.earth_atmosphere()
    ref = oracle.precompute(atm, shape, 4, combined=True)
    compare(ref, gpu_precompute(atmo, torch, atm, shape, 4, True, path), True)


def density_merge_need_and_room(shape, rb, rt):
    """The fast density kernel's merged ground tables above order 2: the
    host's budget estimate (DensityMergeNeed: the worst r-slice's sum over
    its ground rows of (NU + 1) J entries of 32 bytes) and the room a block
    has for them (99 KB minus DensityBaseSmem), as atmo_fast.cu computes
    them."""
    _, _, sr, _, _, nu, iw, _ = shape
    h = math.sqrt(rt * rt - rb * rb)
    k1, kg = (nu - 1) / (2.0 * nu), (iw - 1) / (2.0 * iw)
    worst = 0
    for k in range(sr):
        rho = h * k / max(sr - 1, 1)
        r = math.sqrt(rho * rho + rb * rb)
        entries = 0
        for l in range(16):
            mu = math.cos((l + 0.5) * math.pi / 16)
            disc = r * r * (mu * mu - 1.0) + rb * rb
            if mu >= 0.0 or disc < 0.0:
                continue
            gs = kg * (-r * mu - math.sqrt(disc)) / (rb * k1)
            entries += (nu + 1) * min(int(math.floor(gs * iw)) + 3, iw + 1)
        worst = max(worst, entries)
    base = 16 * (nu + 1) * 32 + (iw + 1) * 32 + (16 * nu + iw) * 16 + 16 * 32 + 16
    return worst * 32, 99 * 1024 - base


@pytest.mark.parametrize("path", [0, 1], ids=["fast", "plain"])
def test_partially_merged_ground_tables_vs_oracle(atmo, oracle, torch, path):
    """A small planet under a thick atmosphere (3000 km, 120 km) with a wide
    irradiance row (256 texels): the grazing ground rays reach many
    irradiance entries, so above order 2 the merged sky + ground tables of
    the top r-slices exceed a block's shared memory.  The first ground rows
    (in theta order) get merged tables; the rest keep the separate sky and
    ground lookups, in the same block."""
    shape = (64, 16, 4, 16, 8, 16, 256, 4)
    need, room = density_merge_need_and_room(shape, 3000.0, 3120.0)
    assert need > room > 0, (need, room)
    atm = oracle.earth_atmosphere()
    atm.bottom_radius, atm.top_radius = 3000.0, 3120.0
    gpu = gpu_precompute(atmo, torch, atm, shape, 4, True, path)
    compare_robust(oracle, atm, shape, 4, gpu, True)


@pytest.mark.parametrize("shape", [(64, 16, 2, 4, 16, 128, 16, 4), (2048, 4, 4, 16, 8, 8, 16, 4)],
                         ids=["line_2048", "transmittance_2048"])
def test_wide_lines_vs_oracle(atmo, oracle, torch, shape):
    """The fast path with passes too wide for its restructured kernels: a
    2048-column scattering line (NU 128 x MU_S 16) exceeds the single- and
    multiple-scattering kernels' 1024 columns (and NU 128 the density tables'
    48 KB), and a 2048-texel transmittance row exceeds single scattering's
    48 KB of line buffers.  Those passes run the plain kernels, the others
    the fast ones.  Every texel, no mask."""
    atm = oracle.earth_atmosphere()
    ref = oracle.precompute(atm, shape, 4, combined=True)
    compare(ref, gpu_precompute(atmo, torch, atm, shape, 4, True, 0), True)


@pytest.mark.parametrize("path", [0, 1], ids=["fast", "plain"])
@pytest.mark.parametrize("combined", [True, False], ids=["combined", "separate"])
def test_default_shape_every_texel_vs_gpu_oracle(atmo, oracle, torch, path, combined):
    """Config 0 (Earth, the reference's default LUT sizes, 4 orders): every
    texel against the FP64 GPU oracle (the golden test above samples texels
    of the reference build's own LUTs)."""
    atm = oracle.earth_atmosphere()
    shape = atmo.DEFAULT_SHAPE
    ref = oracle.gpu_precompute(atm, shape, 4, combined=combined)
    compare(ref, gpu_precompute(atmo, torch, atm, shape, 4, combined, path), combined)


def test_double_r_random_atmospheres_vs_gpu_oracle(atmo, oracle, torch):
    """Random planets of the batched configuration at its largest size
    (double-R: 256 x 64 / R 64 x MU 128 x MU_S 32 x NU 8 / 64 x 16), 2 and 6
    orders, every texel where the FP64 values are not rounding-dominated
    (masks from the FP64 GPU oracle)."""
    from precomputed_atmospheric_scattering_gb300.workloads import DOUBLE_R
    rng = np.random.default_rng(77)
    for orders in (2, 6):
        atm = random_atmosphere(oracle, rng)
        ref, masks = robust_masks(oracle, atm, DOUBLE_R, orders, False,
                                  precompute=oracle.gpu_precompute)
        T, S, M, I = gpu_precompute(atmo, torch, atm, DOUBLE_R, orders, False, 0)
        check_masked("transmittance", T, ref.transmittance, TOL_TRANSMITTANCE,
                     masks["transmittance"])
        check_masked("scattering", S, ref.scattering, TOL_SCATTERING, masks["scattering"])
        check_masked("single_mie", M, ref.single_mie, TOL_SCATTERING, masks["single_mie"])
        check_masked("irradiance", I, ref.irradiance, TOL_IRRADIANCE, masks["irradiance"])


@pytest.mark.parametrize("path", [0, 1], ids=["fast", "plain"])
def test_medium_shape_random_atmospheres_vs_oracle(atmo, oracle, torch, path):
    """Non-Earth planets: seeded draws over the batched-rebuild ranges, compared
    on the texels where the FP64 reference is not rounding-dominated."""
    rng = np.random.default_rng(1234)
    for trial in range(2):
        atm = random_atmosphere(oracle, rng)
        orders = int(rng.integers(2, 5))
        gpu = gpu_precompute(atmo, torch, atm, oracle.MEDIUM_SHAPE, orders, False, path)
        compare_robust(oracle, atm, oracle.MEDIUM_SHAPE, orders, gpu, False)


def random_atmosphere(O, rng):
    """Parameters drawn uniformly from the batched-rebuild ranges: bottom
    radius 3000-7000 km, thickness 40-120 km, Rayleigh H 5-15 km and beta x0.2-5
    of Earth, Mie beta_s 1e-6-5e-5 /m (ext 1.1x), H 0.5-3 km, g 0.6-0.9, ozone
    on/off, albedo 0-0.5; in km."""
    rb = rng.uniform(3000.0, 7000.0)
    thick = rng.uniform(40.0, 120.0)
    hr = rng.uniform(5.0, 15.0)
    scale = rng.uniform(0.2, 5.0)
    ray = [1.24062e-6 * (l * 1e-3) ** -4 * 1000.0 * scale for l in (680.0, 550.0, 440.0)]
    mie_s = rng.uniform(1e-6, 5e-5) * 1000.0
    hm = rng.uniform(0.5, 3.0)
    ozone = rng.random() < 0.5
    oz = [v * 1000.0 if ozone else 0.0 for v in (0.650e-6, 1.881e-6, 0.085e-6)]
    return O.atmosphere(
        solar_irradiance=1.5, sun_angular_radius=0.004675, bottom_radius=rb,
        top_radius=rb + thick,
        rayleigh_density=O.profile(O.layer(0.0, 1.0, -1.0 / hr, 0.0, 0.0)),
        rayleigh_scattering=ray,
        mie_density=O.profile(O.layer(0.0, 1.0, -1.0 / hm, 0.0, 0.0)),
        mie_scattering=mie_s, mie_extinction=1.1 * mie_s,
        mie_phase_function_g=rng.uniform(0.6, 0.9),
        absorption_density=O.profile(O.layer(25.0, 0.0, 0.0, 1.0 / 15.0, -2.0 / 3.0),
                                     O.layer(0.0, 0.0, 0.0, -1.0 / 15.0, 8.0 / 3.0)),
        absorption_extinction=oz, ground_albedo=rng.uniform(0.0, 0.5),
        mu_s_min=np.cos(np.deg2rad(102.0)))


def golden_atmosphere(oracle, g):
    from test_oracle_golden import atmosphere_from_fields
    return atmosphere_from_fields(oracle, g["atmosphere"])


def test_medium_shape_vs_reference_golden(atmo, oracle, torch):
    g = np.load(os.path.join(GOLDEN, "earth_medium.npz"))
    atm = golden_atmosphere(oracle, g)
    T, S, M, I = gpu_precompute(atmo, torch, atm, tuple(g["shape"]), int(g["orders"]), False)
    check("transmittance", T, g["transmittance"], TOL_TRANSMITTANCE)
    check("scattering", S, g["scattering"], TOL_SCATTERING)
    check("single_mie", M, g["single_mie"], TOL_SCATTERING)
    check("irradiance", I, g["irradiance"], TOL_IRRADIANCE)


@pytest.mark.parametrize("path", [0, 1], ids=["fast", "plain"])
def test_default_shape_earth_vs_reference_golden(atmo, oracle, torch, path):
    """Config 0 (Earth, 256x64 / 8x32x128x32 / 64x16, 4 orders, combined) against
    the reference's own LUT values at sampled texels."""
    g = np.load(os.path.join(GOLDEN, "earth_default.npz"))
    atm = golden_atmosphere(oracle, g)
    T, S, M, I = gpu_precompute(atmo, torch, atm, tuple(g["shape"]), 4, True, path)
    check("transmittance", T.reshape(-1, 4)[g["transmittance_index"]], g["transmittance"],
          TOL_TRANSMITTANCE)
    check("scattering", S.reshape(-1, 4)[g["scattering_index"]], g["scattering"],
          TOL_SCATTERING, channels=4)
    check("irradiance", I, g["irradiance"], TOL_IRRADIANCE)


def test_toy_planet_golden(atmo, oracle, torch):
    g = np.load(os.path.join(GOLDEN, "toy_small.npz"))
    atm = golden_atmosphere(oracle, g)
    T, S, M, I = gpu_precompute(atmo, torch, atm, tuple(g["shape"]), int(g["orders"]), False)
    check("transmittance", T, g["transmittance"], TOL_TRANSMITTANCE)
    check("scattering", S, g["scattering"], TOL_SCATTERING)
    check("single_mie", M, g["single_mie"], TOL_SCATTERING)
    check("irradiance", I, g["irradiance"], TOL_IRRADIANCE)


def test_fast_and_plain_paths_agree(atmo, oracle, torch):
    atm = oracle.earth_atmosphere(mie_g=0.76, ground_albedo=0.3)
    a = gpu_precompute(atmo, torch, atm, oracle.MEDIUM_SHAPE, 5, True, 0)
    b = gpu_precompute(atmo, torch, atm, oracle.MEDIUM_SHAPE, 5, True, 1)
    for x, y in zip(a, b):
        check("fast vs plain", x, y, 1e-4, channels=4)


def test_blend_accumulates_like_second_wavelength_group(atmo, oracle, torch):
    atm = oracle.earth_atmosphere()
    lum = np.array([0.3, 0.1, 0.0, 0.05, 0.6, 0.1, 0.0, 0.1, 0.9])
    base = oracle.precompute(atm, oracle.SMALL_SHAPE, 3, combined=False)
    ref = oracle.precompute(atm, oracle.SMALL_SHAPE, 3, lum=lum, blend=True, combined=False,
                            out=oracle.precompute(atm, oracle.SMALL_SHAPE, 3, combined=False))
    init = [base.transmittance, base.scattering, base.single_mie, base.irradiance]
    gpu = gpu_precompute(atmo, torch, atm, oracle.SMALL_SHAPE, 3, False, 0, lum=lum,
                         blend=True, init=init)
    compare(ref, gpu, False)


def test_model_init_earth_matches_oracle(atmo, oracle):
    """The drop-in Model (spectral parameters, Init) against the oracle run on
    the model's own 3-wavelength parameters."""
    m = earth_model(atmo, shape=oracle.SMALL_SHAPE)
    m.Init(4)
    a = m.atmosphere_at()
    atm = oracle.Atmosphere.from_buffer_copy(bytes(a))
    ref = oracle.precompute(atm, oracle.SMALL_SHAPE, 4, combined=True)
    compare(ref, [m.transmittance(), m.scattering(), None, m.irradiance()], True)
    # Init again (CUDA-graph replay) gives the same LUTs.
    s1 = m.scattering()
    m.Init(4)
    np.testing.assert_array_equal(s1, m.scattering())


def test_model_half_precision(atmo, oracle):
    m32 = earth_model(atmo, shape=oracle.SMALL_SHAPE, combined=False)
    m16 = earth_model(atmo, shape=oracle.SMALL_SHAPE, combined=False, half=True)
    m32.Init(4)
    m16.Init(4)
    assert m16.lut_view(atmo.LUT_SCATTERING).dtype == 1
    # FP16 storage: one round-to-nearest, at most 2^-11 relative for normal
    # values and 2^-25 absolute in FP16's subnormal range.
    for name, a, b in (("scattering", m16.scattering(), m32.scattering()),
                       ("single mie", m16.single_mie_scattering(),
                        m32.single_mie_scattering())):
        a, b = a[..., :3].astype(np.float64), b[..., :3].astype(np.float64)
        assert np.all(np.abs(a - b) <= 2.0 ** -11 * np.abs(b) + 2.0 ** -25), name
    np.testing.assert_array_equal(m16.transmittance(), m32.transmittance())


def oracle_luminance_model(oracle, m, orders, shape, precompute=None):
    """atmosphere/model.cc:914-963 with the oracle: 3-wavelength groups, the
    CIE luminance_from_radiance matrices, blending, then the transmittance at
    680/550/440 nm (precompute: oracle.precompute, or oracle.gpu_precompute
    for shapes too large for the CPU)."""
    precompute = precompute or oracle.precompute
    n = (m.num_precomputed_wavelengths + 2) // 3
    dl = (830.0 - 360.0) / (3 * n)
    luts = None
    xyz = [3.2406, -1.5372, -0.4986, -0.9689, 1.8758, 0.0415, 0.0557, -0.2040, 1.0570]
    L = oracle.lib()
    for i in range(n):
        lam = [360.0 + (3 * i + k + 0.5) * dl for k in range(3)]
        lum = np.zeros(9)
        for row in range(3):
            for col in range(3):
                x, y, z = (L.oracle_cie_table_value(lam[col], c) for c in (1, 2, 3))
                lum[row * 3 + col] = np.float32(
                    (xyz[row * 3] * x + xyz[row * 3 + 1] * y + xyz[row * 3 + 2] * z) * dl)
        atm = oracle.Atmosphere.from_buffer_copy(bytes(m.atmosphere_at(lam)))
        luts = precompute(atm, shape, orders, lum=lum, blend=i > 0,
                          combined=m.combine_scattering_textures, out=luts)
    atm = oracle.Atmosphere.from_buffer_copy(bytes(m.atmosphere_at()))
    t = precompute(atm, shape, 1, combined=True)
    luts.transmittance[...] = t.transmittance
    return luts


def test_model_luminance_fifteen_wavelengths(atmo, oracle):
    """Precomputed-illuminance mode (15 wavelengths, 5 groups, blend, final
    transmittance recompute) against the oracle composition."""
    m = earth_model(atmo, n_lambda=15, combined=False, shape=oracle.SMALL_SHAPE)
    m.Init(4)
    ref = oracle_luminance_model(oracle, m, 4, oracle.SMALL_SHAPE)
    compare(ref, [m.transmittance(), m.scattering(), m.single_mie_scattering(),
                  m.irradiance()], False)


def test_precompute_rejects_bad_arguments(atmo, oracle, torch):
    atm = oracle.earth_atmosphere()
    atm.top_radius = atm.bottom_radius - 1.0
    with pytest.raises(atmo.AtmoError) as e:
        gpu_precompute(atmo, torch, atm, oracle.SMALL_SHAPE, 4)
    assert e.value.status == atmo.INVALID_ARG
