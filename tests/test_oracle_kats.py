"""Known-answer tests of the CPU oracle: the unit tests of the reference's
atmosphere/reference/functions_test.cc:321-1478, restated against the oracle's
restatement of atmosphere/functions.glsl (same fixture planet, same analytic
answers, same tolerances, kEpsilon = 1e-3)."""
import ctypes as C
import math

import numpy as np
import pytest

kEpsilon = 1e-3
km = 1000.0
kSolarIrradiance = 123.0
kBottomRadius = 1000.0 * km
kTopRadius = 1500.0 * km
kRayleighScaleHeight = 60.0 * km
kMieScaleHeight = 30.0 * km
kRayleighScattering = 0.001 / km
kMieScattering = 0.0015 / km
kMieExtinction = 0.002 / km
kGroundAlbedo = 0.1
DEFAULT = (256, 64, 32, 128, 32, 8, 64, 16)


def cos_horizon(r):
    # functions_test.cc:70-73
    return -math.sqrt(1.0 - (kBottomRadius / r) ** 2)


@pytest.fixture
def O(oracle):
    return oracle


@pytest.fixture
def atm(oracle):
    return oracle.toy_atmosphere()


@pytest.fixture
def shp(oracle):
    return oracle.shape(*DEFAULT)


def set_uniform(O, a):
    # functions_test.cc:1522-1532 (SetUniformAtmosphere)
    a.rayleigh_density = O.profile(O.layer(), O.layer(0, 0, 0, 0, 1.0))
    a.mie_density = O.profile(O.layer(), O.layer(0, 0, 0, 0, 1.0))
    a.absorption_density = O.profile()


def remove_aerosols(a):
    a.mie_scattering = (C.c_double * 3)(0, 0, 0)
    a.mie_extinction = (C.c_double * 3)(0, 0, 0)


def by(x):
    return C.byref(x)


def dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def full_transmittance_texture(O, a, s):
    """All texels of the transmittance texture (the lazy texture of
    functions_test.cc:82-117, evaluated eagerly)."""
    n = s.t_size
    idx = np.arange(n, dtype=np.int64)
    out = np.zeros((n, 4))
    O.lib().oracle_eval_texels(0, by(a), by(s), None, None, None, None, None, None, 0, n,
                               idx.ctypes.data_as(C.POINTER(C.c_longlong)), dp(out), None, 0)
    return out


def test_distance_to_top_atmosphere_boundary(O, atm):
    # functions_test.cc:321-334
    r = kBottomRadius * 0.2 + kTopRadius * 0.8
    L = O.lib()
    assert abs(L.oracle_distance_to_top(by(atm), r, 1.0) - (kTopRadius - r)) < 1.0
    assert abs(L.oracle_distance_to_top(by(atm), r, 0.0) -
               math.sqrt(kTopRadius ** 2 - r * r)) < 1.0


def test_ray_intersects_ground(O, atm):
    # functions_test.cc:343-352
    r = kBottomRadius * 0.9 + kTopRadius * 0.1
    mu_h = cos_horizon(r)
    L = O.lib()
    assert not L.oracle_ray_intersects_ground(by(atm), r, 1.0)
    assert not L.oracle_ray_intersects_ground(by(atm), r, mu_h + kEpsilon)
    assert L.oracle_ray_intersects_ground(by(atm), r, mu_h - kEpsilon)
    assert L.oracle_ray_intersects_ground(by(atm), r, -1.0)


def test_compute_optical_length_to_top_atmosphere_boundary(O, atm):
    # functions_test.cc:370-389
    r = kBottomRadius * 0.2 + kTopRadius * 0.8
    h_r, h_top = r - kBottomRadius, kTopRadius - kBottomRadius
    K = kRayleighScaleHeight
    L = O.lib()
    expected = K * (math.exp(-h_r / K) - math.exp(-h_top / K))
    assert abs(L.oracle_optical_length(by(atm), by(atm.rayleigh_density), r, 1.0) -
               expected) < 1.0
    set_uniform(O, atm)
    assert abs(L.oracle_optical_length(by(atm), by(atm.rayleigh_density), r, 0.0) -
               math.sqrt(kTopRadius ** 2 - r * r)) < 1.0


def test_get_profile_density(O):
    # functions_test.cc:396-419
    L = O.lib()
    p = O.profile(O.layer(), O.layer(0, 1.0, -1.0 / km, 0, 0))
    assert L.oracle_profile_density(by(p), 2.0 * km) == math.exp(-2.0)
    p = O.profile(O.layer(), O.layer(0, 0, 0, -0.5 / km, 1.0))
    assert L.oracle_profile_density(by(p), 0.0) == 1.0
    assert L.oracle_profile_density(by(p), 1.0 * km) == 0.5
    assert L.oracle_profile_density(by(p), 3.0 * km) == 0.0
    p = O.profile(O.layer(25 * km, 0, 0, 1.0 / (15 * km), -2.0 / 3.0),
                  O.layer(0, 0, 0, -1.0 / (15 * km), 8.0 / 3.0))
    assert L.oracle_profile_density(by(p), 0.0) == 0.0
    assert abs(L.oracle_profile_density(by(p), 10 * km)) < kEpsilon
    assert abs(L.oracle_profile_density(by(p), 25 * km) - 1.0) < kEpsilon
    assert abs(L.oracle_profile_density(by(p), 40 * km)) < kEpsilon
    assert L.oracle_profile_density(by(p), 50 * km) == 0.0


def test_compute_transmittance_to_top_atmosphere_boundary(O, atm):
    # functions_test.cc:433-469
    L = O.lib()
    r = kBottomRadius * 0.2 + kTopRadius * 0.8
    h_r, h_top = r - kBottomRadius, kTopRadius - kBottomRadius
    ray = kRayleighScattering * kRayleighScaleHeight * (
        math.exp(-h_r / kRayleighScaleHeight) - math.exp(-h_top / kRayleighScaleHeight))
    mie = kMieExtinction * kMieScaleHeight * (
        math.exp(-h_r / kMieScaleHeight) - math.exp(-h_top / kMieScaleHeight))
    assert abs(O.v3(L.oracle_transmittance_to_top, by(atm), r, 1.0)[0] -
               math.exp(-(ray + mie))) < kEpsilon
    atm.rayleigh_density = O.profile()
    atm.mie_density = O.profile()
    atm.absorption_density = O.profile(O.layer(25 * km, 0, 0, 1.0 / (15 * km), -2.0 / 3.0),
                                       O.layer(0, 0, 0, -1.0 / (15 * km), 8.0 / 3.0))
    atm.absorption_extinction = (C.c_double * 3)(0.02 / km, 0, 0)
    assert abs(O.v3(L.oracle_transmittance_to_top, by(atm), kBottomRadius, 1.0)[0] -
               math.exp(-0.02 * 15.0)) < kEpsilon
    set_uniform(O, atm)
    remove_aerosols(atm)
    assert abs(O.v3(L.oracle_transmittance_to_top, by(atm), r, 0.0)[0] -
               math.exp(-kRayleighScattering * math.sqrt(kTopRadius ** 2 - r * r))) < kEpsilon


def test_get_texture_coord_from_unit_range(O):
    # functions_test.cc:479-489
    L = O.lib()
    assert abs(L.oracle_tex_coord_from_unit_range(0.0, 10) - 0.5 / 10) < kEpsilon
    assert abs(L.oracle_tex_coord_from_unit_range(1.0, 10) - 9.5 / 10) < kEpsilon
    assert abs(L.oracle_unit_range_from_tex_coord(0.5 / 10, 10)) < kEpsilon
    assert abs(L.oracle_unit_range_from_tex_coord(9.5 / 10, 10) - 1.0) < kEpsilon
    assert abs(L.oracle_unit_range_from_tex_coord(
        L.oracle_tex_coord_from_unit_range(1.0 / 3.0, 10), 10) - 1.0 / 3.0) < kEpsilon


def test_get_transmittance_texture_uv_from_rmu(O, atm, shp):
    # functions_test.cc:497-522
    L = O.lib()
    W, H = shp.transmittance_width, shp.transmittance_height
    uv = np.zeros(2)
    L.oracle_transmittance_uv_from_rmu(by(atm), by(shp), kTopRadius, 1.0, dp(uv))
    assert abs(uv[0] - 0.5 / W) < kEpsilon and abs(uv[1] - (1 - 0.5 / H)) < kEpsilon
    L.oracle_transmittance_uv_from_rmu(by(atm), by(shp), kTopRadius, cos_horizon(kTopRadius),
                                       dp(uv))
    assert abs(uv[0] - (1 - 0.5 / W)) < kEpsilon and abs(uv[1] - (1 - 0.5 / H)) < kEpsilon
    L.oracle_transmittance_uv_from_rmu(by(atm), by(shp), kBottomRadius, 1.0, dp(uv))
    assert abs(uv[0] - 0.5 / W) < kEpsilon and abs(uv[1] - 0.5 / H) < kEpsilon
    L.oracle_transmittance_uv_from_rmu(by(atm), by(shp), kBottomRadius, 0.0, dp(uv))
    assert abs(uv[0] - (1 - 0.5 / W)) < kEpsilon and abs(uv[1] - 0.5 / H) < kEpsilon


def test_get_rmu_from_transmittance_texture_uv(O, atm, shp):
    # functions_test.cc:532-574
    L = O.lib()
    W, H = shp.transmittance_width, shp.transmittance_height
    r, mu = C.c_double(), C.c_double()

    def rmu(u, v):
        L.oracle_rmu_from_transmittance_uv(by(atm), by(shp), u, v, by(r), by(mu))
        return r.value, mu.value
    a, b = rmu(0.5 / W, 1 - 0.5 / H)
    assert abs(a - kTopRadius) < 1.0 and abs(b - 1.0) < kEpsilon
    a, b = rmu(1 - 0.5 / W, 1 - 0.5 / H)
    assert abs(a - kTopRadius) < 1.0 and abs(b - cos_horizon(kTopRadius)) < kEpsilon
    a, b = rmu(0.5 / W, 0.5 / H)
    assert abs(a - kBottomRadius) < 1.0 and abs(b - 1.0) < kEpsilon
    a, b = rmu(1 - 0.5 / W, 0.5 / H)
    assert abs(a - kBottomRadius) < 1.0 and abs(b) < kEpsilon
    uv = np.zeros(2)
    r0 = kBottomRadius * 0.2 + kTopRadius * 0.8
    L.oracle_transmittance_uv_from_rmu(by(atm), by(shp), r0, 0.25, dp(uv))
    a, b = rmu(uv[0], uv[1])
    assert abs(a - r0) < 1.0 and abs(b - 0.25) < kEpsilon


def test_get_transmittance_to_top_atmosphere_boundary(O, atm, shp):
    # functions_test.cc:583-595
    L = O.lib()
    T = full_transmittance_texture(O, atm, shp)
    r, mu = kBottomRadius * 0.2 + kTopRadius * 0.8, 0.4
    direct = O.v3(L.oracle_transmittance_to_top, by(atm), r, mu)[0]
    lookup = O.v3(L.oracle_lookup_transmittance_to_top, by(atm), by(shp), dp(T), r, mu)[0]
    assert abs(direct - lookup) < kEpsilon


def test_compute_and_get_transmittance(O, atm, shp):
    # functions_test.cc:605-631
    L = O.lib()
    set_uniform(O, atm)
    remove_aerosols(atm)
    T = full_transmittance_texture(O, atm, shp)
    r = kBottomRadius * 0.2 + kTopRadius * 0.8
    d = (kTopRadius - kBottomRadius) * 0.1
    expected = math.exp(-kRayleighScattering * d)
    for r0, mu, g in ((kBottomRadius, 0.0, 0), (r, 0.7, 0),
                      (r, -0.7, L.oracle_ray_intersects_ground(by(atm), r, -0.7))):
        got = O.v3(L.oracle_lookup_transmittance, by(atm), by(shp), dp(T), r0, mu, d, g)[0]
        assert abs(got - expected) < kEpsilon


def test_compute_single_scattering_integrand(O, atm, shp):
    # functions_test.cc:676-755
    L = O.lib()
    T = full_transmittance_texture(O, atm, shp)
    h_top = kTopRadius - kBottomRadius
    h = h_top / 2.0
    ray, mie = np.zeros(3), np.zeros(3)
    L.oracle_single_scattering_integrand(by(atm), by(shp), dp(T), kBottomRadius, 1.0, 1.0, 1.0,
                                         h, 0, dp(ray), dp(mie))
    ro = kRayleighScattering * kRayleighScaleHeight * (1 - math.exp(-h_top / kRayleighScaleHeight))
    mo = kMieExtinction * kMieScaleHeight * (1 - math.exp(-h_top / kMieScaleHeight))
    assert abs(ray[0] - math.exp(-ro - mo) * math.exp(-h / kRayleighScaleHeight)) < kEpsilon
    assert abs(mie[0] - math.exp(-ro - mo) * math.exp(-h / kMieScaleHeight)) < kEpsilon
    L.oracle_single_scattering_integrand(by(atm), by(shp), dp(T), kTopRadius, -1.0, 1.0, -1.0,
                                         h, 1, dp(ray), dp(mie))
    ro = 2 * kRayleighScattering * kRayleighScaleHeight * (
        math.exp(-h / kRayleighScaleHeight) - math.exp(-h_top / kRayleighScaleHeight))
    mo = 2 * kMieExtinction * kMieScaleHeight * (
        math.exp(-h / kMieScaleHeight) - math.exp(-h_top / kMieScaleHeight))
    assert abs(ray[0] - math.exp(-ro - mo) * math.exp(-h / kRayleighScaleHeight)) < kEpsilon
    assert abs(mie[0] - math.exp(-ro - mo) * math.exp(-h / kMieScaleHeight)) < kEpsilon
    set_uniform(O, atm)
    remove_aerosols(atm)
    T = full_transmittance_texture(O, atm, shp)
    L.oracle_single_scattering_integrand(by(atm), by(shp), dp(T), kBottomRadius, 0.0, 0.0, 1.0,
                                         50.0 * km, 0, dp(ray), dp(mie))
    ro = kRayleighScattering * math.sqrt(kTopRadius ** 2 - kBottomRadius ** 2)
    assert abs(ray[0] - math.exp(-ro)) < kEpsilon


def test_distance_to_nearest_atmosphere_boundary(O, atm):
    # functions_test.cc:764-788
    L = O.lib()
    r = kBottomRadius * 0.2 + kTopRadius * 0.8
    g = lambda mu: L.oracle_ray_intersects_ground(by(atm), r, mu)  # noqa: E731
    assert abs(L.oracle_distance_to_nearest(by(atm), r, 1.0, g(1.0)) - (kTopRadius - r)) < 1
    assert abs(L.oracle_distance_to_nearest(by(atm), r, 0.0, g(0.0)) -
               math.sqrt(kTopRadius ** 2 - r * r)) < 1
    assert abs(L.oracle_distance_to_nearest(by(atm), r, -1.0, g(-1.0)) -
               (r - kBottomRadius)) < 1


def test_compute_single_scattering(O, atm, shp):
    # functions_test.cc:818-862 (relative errors of about 1%)
    L = O.lib()
    T = full_transmittance_texture(O, atm, shp)
    h_top = kTopRadius - kBottomRadius
    ray, mie = np.zeros(3), np.zeros(3)
    L.oracle_single_scattering(by(atm), by(shp), dp(T), kBottomRadius, 1.0, 1.0, 1.0, 0,
                               dp(ray), dp(mie))
    ro = kRayleighScattering * kRayleighScaleHeight * (1 - math.exp(-h_top / kRayleighScaleHeight))
    mo = kMieExtinction * kMieScaleHeight * (1 - math.exp(-h_top / kMieScaleHeight))
    assert abs(ray[0] / (kSolarIrradiance * ro * math.exp(-ro - mo)) - 1) < 10 * kEpsilon
    assert abs(mie[0] / (kSolarIrradiance * mo * kMieScattering / kMieExtinction *
                         math.exp(-ro - mo)) - 1) < 10 * kEpsilon
    remove_aerosols(atm)
    T = full_transmittance_texture(O, atm, shp)
    L.oracle_single_scattering(by(atm), by(shp), dp(T), kTopRadius, -1.0, 1.0, -1.0, 1,
                               dp(ray), dp(mie))
    expected = kSolarIrradiance * 0.5 * (1 - math.exp(
        -2 * kRayleighScaleHeight * kRayleighScattering *
        (1 - math.exp(-h_top / kRayleighScaleHeight))))
    assert abs(ray[0] / expected - 1) < 2 * kEpsilon
    assert abs(mie[0]) < kEpsilon


def test_phase_functions(O):
    # functions_test.cc:865-879
    L = O.lib()
    N = 100
    ri = mi = 0.0
    for i in range(N):
        theta = (i + 0.5) * math.pi / N
        dw = math.sin(theta) * (math.pi / N) * (2 * math.pi)
        ri += L.oracle_rayleigh_phase(math.cos(theta)) * dw
        mi += L.oracle_mie_phase(0.8, math.cos(theta)) * dw
    assert abs(ri - 1) < 2 * kEpsilon and abs(mi - 1) < 2 * kEpsilon


def uvwz(O, atm, shp, r, mu, mu_s, nu, g):
    out = np.zeros(4)
    O.lib().oracle_scattering_uvwz(by(atm), by(shp), r, mu, mu_s, nu, g, dp(out))
    return out


def test_get_scattering_texture_uvwz_from_rmumusnu(O, atm, shp):
    # functions_test.cc:888-947
    R, MU, MU_S = shp.scattering_r, shp.scattering_mu, shp.scattering_mu_s
    assert abs(uvwz(O, atm, shp, kBottomRadius, 0, 0, 0, 0)[3] - 0.5 / R) < kEpsilon
    assert abs(uvwz(O, atm, shp, kTopRadius, 0, 0, 0, 0)[3] - (1 - 0.5 / R)) < kEpsilon
    r = (kTopRadius + kBottomRadius) / 2
    mu = cos_horizon(r)
    assert abs(uvwz(O, atm, shp, r, mu, 0, 0, 1)[2] - 0.5 / MU) < kEpsilon
    assert abs(uvwz(O, atm, shp, r, mu, 0, 0, 0)[2] - (1 - 0.5 / MU)) < kEpsilon
    assert uvwz(O, atm, shp, r, -1.0, 0, 0, 1)[2] < 0.5
    assert uvwz(O, atm, shp, r, 1.0, 0, 0, 0)[2] > 0.5
    for rr in (kBottomRadius, kTopRadius):
        assert abs(uvwz(O, atm, shp, rr, 0, -1, 0, 0)[1] - 0.5 / MU_S) < kEpsilon
        assert abs(uvwz(O, atm, shp, rr, 0, 1, 0, 0)[1] - (1 - 0.5 / MU_S)) < kEpsilon
    assert abs(uvwz(O, atm, shp, kBottomRadius, 0, 0, -1, 0)[0]) < kEpsilon
    assert abs(uvwz(O, atm, shp, kBottomRadius, 0, 0, 1, 0)[0] - 1) < kEpsilon


def test_get_rmumusnu_from_scattering_texture_uvwz(O, atm, shp):
    # functions_test.cc:957-1060
    R, MU, MU_S = shp.scattering_r, shp.scattering_mu, shp.scattering_mu_s
    L = O.lib()
    g = C.c_int()

    def inv(u):
        out = np.zeros(4)
        L.oracle_rmumusnu_from_uvwz(by(atm), by(shp), dp(np.asarray(u, float)), dp(out), by(g))
        return out, g.value
    (r, mu, mu_s, nu), _ = inv([0, 0.5 / MU_S, 0.5 / MU, 0.5 / R])
    assert abs(r - kBottomRadius) < 1
    (r, mu, mu_s, nu), _ = inv([0, 0.5 / MU_S, 0.5 / MU, 1 - 0.5 / R])
    assert abs(r - kTopRadius) < 1
    (r, mu, mu_s, nu), gr = inv([0, 0.5 / MU_S, 0.5 / MU + kEpsilon, 0.5])
    mh = cos_horizon(r)
    assert abs(mu - mh) < kEpsilon and mu <= mh and gr
    (r, mu, mu_s, nu), gr = inv([0, 0.5 / MU_S, 1 - 0.5 / MU - kEpsilon, 0.5])
    assert abs(mu - mh) < 5 * kEpsilon and mu >= mh and not gr
    (r, mu, mu_s, nu), _ = inv([0, 0.5 / MU_S, 0.5 / MU, 0.5 / R])
    assert abs(mu_s + 1) < kEpsilon and abs(nu + 1) < kEpsilon
    (r, mu, mu_s, nu), _ = inv([0, 1 - 0.5 / MU_S, 0.5 / MU, 0.5 / R])
    assert abs(mu_s - 1) < kEpsilon
    (r, mu, mu_s, nu), _ = inv([1, 0.5 / MU_S, 0.5 / MU, 0.5 / R])
    assert abs(nu - 1) < kEpsilon
    for rr, mu0, mus0, nu0, g0 in ((kBottomRadius, -1, 1, -1, 1), (kTopRadius, -1, 1, -1, 1),
                                   ((kBottomRadius + kTopRadius) / 2, 0.2, 0.3, 0.4, 0)):
        (r, mu, mu_s, nu), gr = inv(uvwz(O, atm, shp, rr, mu0, mus0, nu0, g0))
        assert abs(r - rr) < 1
        assert abs(mu - mu0) < kEpsilon and abs(mu_s - mus0) < kEpsilon
        assert abs(nu - nu0) < kEpsilon and gr == g0


def lazy_single_scattering(O, atm, shp, T, points):
    """Single-scattering textures holding exactly the texels the lookups at
    `points` read (the lazy textures of functions_test.cc:124-165)."""
    L = O.lib()
    idx = set()
    for (r, mu, mu_s, nu, g) in points:
        taps = np.zeros(16, np.int32)
        w = np.zeros(16)
        L.oracle_scattering_taps(by(atm), by(shp), r, mu, mu_s, nu, g,
                                 taps.ctypes.data_as(C.POINTER(C.c_int)), dp(w))
        idx.update(int(t) for t in taps)
    idx = np.array(sorted(idx), np.int64)
    ray = np.zeros((len(idx), 4))
    mie = np.zeros((len(idx), 4))
    L.oracle_eval_texels(2, by(atm), by(shp), dp(T), None, None, None, None, None, 0, len(idx),
                         idx.ctypes.data_as(C.POINTER(C.c_longlong)), dp(ray), dp(mie), 0)
    SR = np.zeros((shp.s_size, 4))
    SM = np.zeros((shp.s_size, 4))
    SR[idx] = ray
    SM[idx] = mie
    return SR, SM


def test_compute_and_get_single_scattering(O, atm, shp):
    # functions_test.cc:1069-1139 (6-8% error allowed at the horizontal ray)
    L = O.lib()
    T = full_transmittance_texture(O, atm, shp)
    mu_h = cos_horizon(kTopRadius)
    cases = [(kBottomRadius, 1.0, 1.0, 1.0, 0, kEpsilon),
             (kTopRadius, -1.0, 1.0, -1.0, 1, kEpsilon),
             (kBottomRadius, 0.0, 0.0, 0.0, 0, 1e-1),
             (kTopRadius, mu_h, 1.0, mu_h, 0, kEpsilon)]
    SR, SM = lazy_single_scattering(O, atm, shp, T, [c[:5] for c in cases])
    for r, mu, mu_s, nu, g, tol in cases:
        got_r = O.v3(L.oracle_lookup_scattering, by(atm), by(shp), dp(SR), r, mu, mu_s, nu, g)
        got_m = O.v3(L.oracle_lookup_scattering, by(atm), by(shp), dp(SM), r, mu, mu_s, nu, g)
        er, em = np.zeros(3), np.zeros(3)
        L.oracle_single_scattering(by(atm), by(shp), dp(T), r, mu, mu_s, nu, g, dp(er), dp(em))
        assert abs(got_r[0] / er[0] - 1) < tol
        assert abs(got_m[0] / em[0] - 1) < tol


def const_tex(n, value):
    t = np.zeros((n, 4))
    t[:, :3] = value
    return t


def test_compute_scattering_density(O, atm, shp):
    # functions_test.cc:1155-1200
    L = O.lib()
    T1 = const_tex(shp.t_size, 1.0)
    S0 = const_tex(shp.s_size, 0.0)
    Sk = const_tex(shp.s_size, 13.0)
    I0 = const_tex(shp.i_size, 0.0)
    out = np.zeros(3)
    L.oracle_scattering_density(by(atm), by(shp), dp(T1), dp(S0), dp(S0), dp(Sk), dp(I0),
                                kBottomRadius, 0.0, 0.0, 1.0, 3, dp(out))
    expected = (kRayleighScattering + kMieScattering) * 13.0
    assert abs(out[0] / expected - 1) < 2 * kEpsilon
    Ik = const_tex(shp.i_size, 13.0)
    L.oracle_scattering_density(by(atm), by(shp), dp(T1), dp(S0), dp(S0), dp(S0), dp(Ik),
                                kBottomRadius, 0.0, 0.0, 1.0, 3, dp(out))
    expected = (kRayleighScattering + kMieScattering) * kGroundAlbedo / (2 * math.pi) * 13.0
    assert abs(out[0] / expected - 1) < 2 * kEpsilon


def test_compute_multiple_scattering(O, atm, shp):
    # functions_test.cc:1211-1235
    L = O.lib()
    T1 = const_tex(shp.t_size, 1.0)
    J = const_tex(shp.s_size, 0.17)
    r = kBottomRadius * 0.2 + kTopRadius * 0.8
    got = O.v3(L.oracle_multiple_scattering, by(atm), by(shp), dp(T1), dp(J), r, -1.0, 1.0,
               -1.0, 1)[0]
    assert abs(got - 0.17 * (r - kBottomRadius)) < 0.17 * (r - kBottomRadius) * kEpsilon
    mu = cos_horizon(kTopRadius)
    dh = math.sqrt(kTopRadius ** 2 - kBottomRadius ** 2)
    got = O.v3(L.oracle_multiple_scattering, by(atm), by(shp), dp(T1), dp(J), kTopRadius, mu,
               1.0, mu, 1)[0]
    assert abs(got - 0.17 * dh) < 0.17 * dh * kEpsilon


def lazy_texels(O, atm, shp, kind, T, SR, SM, SMulti, I, J, order, points):
    L = O.lib()
    idx = set()
    for (r, mu, mu_s, nu, g) in points:
        taps = np.zeros(16, np.int32)
        w = np.zeros(16)
        L.oracle_scattering_taps(by(atm), by(shp), r, mu, mu_s, nu, g,
                                 taps.ctypes.data_as(C.POINTER(C.c_int)), dp(w))
        idx.update(int(t) for t in taps)
    idx = np.array(sorted(idx), np.int64)
    vals = np.zeros((len(idx), 4))
    p = lambda a: dp(a) if a is not None else None  # noqa: E731
    L.oracle_eval_texels(kind, by(atm), by(shp), p(T), p(SR), p(SM), p(SMulti), p(I), p(J),
                         order, len(idx), idx.ctypes.data_as(C.POINTER(C.c_longlong)), dp(vals),
                         None, 0)
    out = np.zeros((shp.s_size, 4))
    out[idx] = vals
    return out


def test_compute_and_get_scattering_density(O, atm, shp):
    # functions_test.cc:1244-1290
    L = O.lib()
    T1 = const_tex(shp.t_size, 1.0)
    S0 = const_tex(shp.s_size, 0.0)
    pt = [(kBottomRadius, 0.0, 0.0, 1.0, 0)]
    J = lazy_texels(O, atm, shp, 3, T1, S0, S0, const_tex(shp.s_size, 13.0),
                    const_tex(shp.i_size, 0.0), None, 3, pt)
    got = O.v3(L.oracle_lookup_scattering, by(atm), by(shp), dp(J), *pt[0])[0]
    assert abs(got / ((kRayleighScattering + kMieScattering) * 13.0) - 1) < 2 * kEpsilon
    J = lazy_texels(O, atm, shp, 3, T1, S0, S0, S0, const_tex(shp.i_size, 13.0), None, 3, pt)
    got = O.v3(L.oracle_lookup_scattering, by(atm), by(shp), dp(J), *pt[0])[0]
    expected = (kRayleighScattering + kMieScattering) * kGroundAlbedo / (2 * math.pi) * 13.0
    assert abs(got / expected - 1) < 2 * kEpsilon


def test_compute_and_get_multiple_scattering(O, atm, shp):
    # functions_test.cc:1299-1323
    L = O.lib()
    T1 = const_tex(shp.t_size, 1.0)
    J = const_tex(shp.s_size, 0.17)
    r = kBottomRadius * 0.2 + kTopRadius * 0.8
    mu = cos_horizon(kTopRadius)
    dh = math.sqrt(kTopRadius ** 2 - kBottomRadius ** 2)
    pts = [(r, -1.0, 1.0, -1.0, 1), (kTopRadius, mu, 1.0, mu, 1)]
    M = lazy_texels(O, atm, shp, 5, T1, None, None, None, None, J, 0, pts)
    got = O.v3(L.oracle_lookup_scattering, by(atm), by(shp), dp(M), *pts[0])[0]
    exp0 = 0.17 * (r - kBottomRadius)
    assert abs(got - exp0) < exp0 * kEpsilon
    got = O.v3(L.oracle_lookup_scattering, by(atm), by(shp), dp(M), *pts[1])[0]
    assert abs(got - 0.17 * dh) < 0.17 * dh * kEpsilon


def test_compute_indirect_irradiance(O, atm, shp):
    # functions_test.cc:1325-1344 (about 1%)
    L = O.lib()
    S0 = const_tex(shp.s_size, 0.0)
    S1 = const_tex(shp.s_size, 1.0)
    got = O.v3(L.oracle_indirect_irradiance, by(atm), by(shp), dp(S0), dp(S0), dp(S1),
               kBottomRadius, 1.0, 2)[0]
    assert abs(got - math.pi) < 10 * kEpsilon


def test_get_irradiance_texture_uv_from_rmus(O, atm, shp):
    # functions_test.cc:1346-1370
    L = O.lib()
    W, H = shp.irradiance_width, shp.irradiance_height
    uv = np.zeros(2)
    L.oracle_irradiance_uv_from_rmus(by(atm), by(shp), kBottomRadius, 0.0, dp(uv))
    assert abs(uv[1] - 0.5 / H) < kEpsilon
    L.oracle_irradiance_uv_from_rmus(by(atm), by(shp), kTopRadius, 0.0, dp(uv))
    assert abs(uv[1] - (1 - 0.5 / H)) < kEpsilon
    L.oracle_irradiance_uv_from_rmus(by(atm), by(shp), kBottomRadius, -1.0, dp(uv))
    assert abs(uv[0] - 0.5 / W) < kEpsilon
    L.oracle_irradiance_uv_from_rmus(by(atm), by(shp), kBottomRadius, 1.0, dp(uv))
    assert abs(uv[0] - (1 - 0.5 / W)) < kEpsilon


def test_get_rmus_from_irradiance_texture_uv(O, atm, shp):
    # functions_test.cc:1379-1406
    L = O.lib()
    W, H = shp.irradiance_width, shp.irradiance_height
    r, mu_s = C.c_double(), C.c_double()
    L.oracle_rmus_from_irradiance_uv(by(atm), by(shp), 0.5 / W, 0.5 / H, by(r), by(mu_s))
    assert abs(r.value - kBottomRadius) < 1 and abs(mu_s.value + 1) < kEpsilon
    L.oracle_rmus_from_irradiance_uv(by(atm), by(shp), 0.5 / W, 1 - 0.5 / H, by(r), by(mu_s))
    assert abs(r.value - kTopRadius) < 1
    L.oracle_rmus_from_irradiance_uv(by(atm), by(shp), 1 - 0.5 / W, 0.5 / H, by(r), by(mu_s))
    assert abs(mu_s.value - 1) < kEpsilon


def test_compute_and_get_irradiance(O, atm, shp):
    # functions_test.cc:1408-1478: a fake multiple-scattering texture whose
    # value encodes the texel coordinates.
    L = O.lib()
    S0 = const_tex(shp.s_size, 0.0)
    W, H, D = shp.s_width, shp.scattering_mu, shp.scattering_r
    x, y, z = np.meshgrid(np.arange(W), np.arange(H), np.arange(D), indexing="ij")
    v = z + D * (y + H * x)
    fake = np.zeros((D, H, W, 4))
    fake[..., :3] = np.transpose(v, (2, 1, 0))[..., None]
    fake = fake.reshape(-1, 4)
    r = kBottomRadius * 0.8 + kTopRadius * 0.2
    mu_s = 0.25
    n = shp.i_size
    idx = np.arange(n, dtype=np.int64)
    I = np.zeros((n, 4))
    L.oracle_eval_texels(4, by(atm), by(shp), None, dp(S0), dp(S0), dp(fake), None, None, 2, n,
                         idx.ctypes.data_as(C.POINTER(C.c_longlong)), dp(I), None, 0)
    lookup = O.v3(L.oracle_lookup_irradiance, by(atm), by(shp), dp(I), r, mu_s)[0]
    direct = O.v3(L.oracle_indirect_irradiance, by(atm), by(shp), dp(S0), dp(S0), dp(fake), r,
                  mu_s, 2)[0]
    assert abs(lookup / direct - 1) < kEpsilon
    other = O.v3(L.oracle_indirect_irradiance, by(atm), by(shp), dp(S0), dp(S0), dp(fake), r,
                 0.5, 2)[0]
    assert abs(lookup / other - 1) >= kEpsilon
