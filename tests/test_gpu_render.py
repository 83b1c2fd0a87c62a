"""Render-time queries (GetSkyRadiance, GetSkyRadianceToPoint,
GetSunAndSkyIrradiance, GetSolarRadiance: atmosphere/functions.glsl:1633-1896
behind the API of atmosphere/model.cc:221-281) on GPU-precomputed LUTs,
against the FP64 oracle's restatement of the same functions fed the same
LUT texels.

Queries follow the serving workload: cameras at 0-100 km altitude, view and
sun directions uniform on the sphere, points 0.1-100 km along the view ray,
shadow lengths 0 or up to 5 km.  Parity is checked on the queries the
reference's formulas are made for: the shaded point inside the atmosphere
and the segment from the camera to it above the ground (cameras above the
atmosphere included).  Outside that domain the reference evaluates its ray-
sphere distances with square roots of negative discriminants clamped to 0;
there the kernels only have to return finite values.  A query is compared only where the oracle is
continuous and well conditioned: a query whose oracle value moves by more
than half the tolerance when its directions turn by ~2e-6 rad and its positions
move by ~1 m (a few times what FP32 resolves)
sits on a discontinuity or a steep edge of the reference itself (the ground /
sky switch of the mu mapping at the horizon, the edge of the sun disc), where
FP32 and FP64 inputs legitimately give different values."""
import ctypes as C

import numpy as np
import pytest

from parity import FLOOR, TOL_SCATTERING
from test_capi_host import earth_model

pytestmark = pytest.mark.gpu

TOL_RENDER = TOL_SCATTERING      # per-query relative error, floor FLOOR x max
# GetSkyRadianceToPoint is S(camera) - T S(point): for short segments the
# difference is much smaller than its terms, and FP32 lookups carry errors
# relative to the terms.  Its error is bounded by TOL_RENDER |result| +
# TOL_TERMS |GetSkyRadiance along the same ray| (the first term, as radiance).
TOL_TERMS = 1e-4
# The sky irradiance is I(r, mu_s) (1 + n.p / r) / 2; the factor cancels for
# normals pointing down, so its FP32 error is a few ulp of I, not of the
# product.
TOL_FACTOR = 1e-6
ROBUST_STEP = 3e-7               # direction perturbation (rad) of the robustness mask
ROBUST_POSITION = 3e-7           # per-component position perturbation, relative
                                 # (~2 m at 6400 km; FP32 resolves ~0.4 m there)
ROBUST_THRESHOLD = 0.5 * TOL_SCATTERING   # oracle change that marks a steep spot


@pytest.fixture(scope="module")
def torch():
    import torch as t
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def draw_queries(rng, n, rb):
    cam = unit(rng, n) * (rb + rng.uniform(0.0, 100.0, size=(n, 1)))
    view = unit(rng, n)
    sun = unit(rng, n)
    depth = rng.uniform(0.1, 100.0, size=(n, 1))
    point = cam + view * depth
    normal = unit(rng, n)
    shadow = np.where(rng.random(n) < 0.5, 0.0, rng.uniform(0.0, 5.0, size=n))
    return cam, view, sun, point, normal, shadow, depth[:, 0]


def in_domain(q, rb, rt):
    """Point inside the atmosphere shell, camera-to-point segment above ground."""
    cam, view, _, point, _, _, depth = q
    rp = np.linalg.norm(point, axis=1)
    rmu = np.sum(cam * view, axis=1)
    r2 = np.sum(cam * cam, axis=1)
    disc = rmu * rmu - (r2 - rb * rb)
    t_ground = -rmu - np.sqrt(np.maximum(disc, 0.0))
    hits = (disc >= 0.0) & (t_ground > 0.0) & (t_ground < depth)
    return (rp >= rb) & (rp <= rt) & ~hits


def as_f32(q):
    """The queries as the kernels receive them (float32)."""
    return tuple(np.asarray(x, np.float32).astype(np.float64) for x in q)


def make_queries(rng, n, rb, rt=None, domain=True):
    if not domain:
        return as_f32(draw_queries(rng, n, rb)[:6])
    parts = [[] for _ in range(6)]
    count = 0
    while count < n:
        q = draw_queries(rng, 4 * n, rb)
        keep = in_domain(q, rb, rt if rt is not None else rb + 60.0)
        for p, x in zip(parts, q[:6]):
            p.append(x[keep])
        count += int(keep.sum())
    return as_f32(tuple(np.concatenate(p)[:n] for p in parts))


class OracleRender:
    """The oracle's render functions over LUTs read back from the GPU."""

    def __init__(self, oracle, atm, shape, T, S, M, I, combined):
        self.O = oracle
        self.L = oracle.lib()
        self.atm = oracle.Atmosphere.from_buffer_copy(bytes(atm))
        self.shp = oracle.shape(*shape)
        self.arrays = [np.ascontiguousarray(x, np.float64) for x in (T, S, M, I)]
        dp = oracle.dp
        self.T, self.S, self.M, self.I = (a.ctypes.data_as(dp) for a in self.arrays)
        self.combined = int(combined)

    def _p(self, v):
        return np.ascontiguousarray(v, np.float64).ctypes.data_as(self.O.dp)

    def sky(self, cam, view, shadow, sun):
        o, t = np.zeros(3), np.zeros(3)
        self.L.oracle_sky_radiance(C.byref(self.atm), C.byref(self.shp), self.T, self.S, self.M,
                                   self.combined, self._p(cam), self._p(view), float(shadow),
                                   self._p(sun), self._p(o), self._p(t))
        return o, t

    def to_point(self, cam, point, shadow, sun):
        o, t = np.zeros(3), np.zeros(3)
        self.L.oracle_sky_radiance_to_point(C.byref(self.atm), C.byref(self.shp), self.T,
                                            self.S, self.M, self.combined, self._p(cam),
                                            self._p(point), float(shadow), self._p(sun),
                                            self._p(o), self._p(t))
        return o, t

    def sun_sky(self, point, normal, sun):
        a, b = np.zeros(3), np.zeros(3)
        self.L.oracle_sun_and_sky_irradiance(C.byref(self.atm), C.byref(self.shp), self.T,
                                             self.I, self._p(point), self._p(normal),
                                             self._p(sun), self._p(a), self._p(b))
        return a, b


def oracle_outputs(ref, q, rng, perturb, position=ROBUST_POSITION):
    cam, view, sun, point, normal, shadow = q
    n = len(cam)
    outs = {k: np.zeros((n, 3)) for k in ("sky", "sky_t", "pt", "pt_t", "sun", "skyirr")}
    def turn(u):
        u = u + rng.normal(size=3) * ROBUST_STEP
        return u / np.linalg.norm(u)

    def move(x):
        return x + rng.normal(size=3) * position * np.linalg.norm(x)

    for i in range(n):
        c, v, p, s, nm = cam[i], view[i], point[i], sun[i], normal[i]
        if perturb:
            c, p = move(c), move(p)
            v, s, nm = turn(v), turn(s), turn(nm)
        outs["sky"][i], outs["sky_t"][i] = ref.sky(c, v, shadow[i], s)
        outs["pt"][i], outs["pt_t"][i] = ref.to_point(c, p, shadow[i], s)
        outs["sun"][i], outs["skyirr"][i] = ref.sun_sky(p, nm, s)
    return outs


def gpu_outputs(torch, lut_set, q):
    cam, view, sun, point, normal, shadow = (
        torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda() for x in q)
    sky, sky_t = lut_set.sky_radiance(cam, view, sun, shadow)
    pt, pt_t = lut_set.sky_radiance_to_point(cam, point, sun, shadow)
    su, sk = lut_set.sun_and_sky_irradiance(point, normal, sun)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy().astype(np.float64) for k, v in
            (("sky", sky), ("sky_t", sky_t), ("pt", pt), ("pt_t", pt_t), ("sun", su),
             ("skyirr", sk))}


def compare(ref_out, pert_out, gpu_out, what, terms=None, factor=None, min_robust=0.85):
    bad = []
    for k in ref_out:
        o, g, p = ref_out[k], gpu_out[k], pert_out[k]
        floor = np.full_like(o, FLOOR * max(np.abs(o).max(), 1e-30))
        if k == "pt" and terms is not None:
            floor = np.maximum(floor, TOL_TERMS / TOL_RENDER * np.abs(terms))
        if k == "skyirr" and factor is not None:
            floor = np.maximum(floor, TOL_FACTOR / TOL_RENDER * np.abs(o) /
                               np.maximum(factor, 1e-30)[:, None])
        robust = np.all(np.abs(p - o) <= ROBUST_THRESHOLD * np.maximum(np.abs(o), floor),
                        axis=1)
        rel = np.abs(g - o) / np.maximum(np.abs(o), floor)
        worst = rel[robust].max() if robust.any() else 0.0
        assert robust.mean() > min_robust, (what, k, robust.mean())
        assert np.all(np.isfinite(g)), (what, k)
        i = int(np.argmax(np.where(robust[:, None], rel, 0.0)) // 3)
        print("%s %-7s worst %.3g at %d (%d robust of %d)" % (what, k, worst, i,
                                                              robust.sum(), len(o)))
        if worst > TOL_RENDER:
            bad.append((k, float(worst), i))
    assert not bad, (what, bad)


def run_case(atmo, oracle, torch, model_or_set, atm, shape, T, S, M, I, combined, seed, n=400):
    rng = np.random.default_rng(seed)
    q = make_queries(rng, n, atm.bottom_radius, atm.top_radius)
    ref = OracleRender(oracle, atm, shape, T, S, M, I, combined)
    ref_out = oracle_outputs(ref, q, rng, False)
    pert_out = oracle_outputs(ref, q, rng, True)
    gpu_out = gpu_outputs(torch, model_or_set, q)
    # The first term of GetSkyRadianceToPoint: the radiance of the whole ray.
    cam, _, sun, point, _, _ = q
    terms = np.array([ref.sky(cam[i], (point[i] - cam[i]) / np.linalg.norm(point[i] - cam[i]),
                              0.0, sun[i])[0] for i in range(len(cam))])
    _, _, _, _, normal, _ = q
    factor = 0.5 * (1.0 + np.sum(normal * point, axis=1) / np.linalg.norm(point, axis=1))
    compare(ref_out, pert_out, gpu_out, "seed %d" % seed, terms, factor)
    # Outside the domain: finite values.
    qo = make_queries(rng, 2000, atm.bottom_radius, domain=False)
    for v in gpu_outputs(torch, model_or_set, qo).values():
        assert np.all(np.isfinite(v))


def test_model_queries_combined_vs_oracle(atmo, oracle, torch):
    m = earth_model(atmo)
    m.Init(4)
    a = m.atmosphere_at()
    S = m.scattering()
    run_case(atmo, oracle, torch, m.lut_set(), a, atmo.DEFAULT_SHAPE, m.transmittance(), S, S,
             m.irradiance(), True, 11)


def test_model_queries_separate_textures_vs_oracle(atmo, oracle, torch):
    shape = oracle.MEDIUM_SHAPE
    m = earth_model(atmo, combined=False, shape=shape)
    m.Init(4)
    a = m.atmosphere_at()
    run_case(atmo, oracle, torch, m.lut_set(), a, shape, m.transmittance(), m.scattering(),
             m.single_mie_scattering(), m.irradiance(), False, 12)


def test_batch_instance_queries_vs_oracle(atmo, oracle, torch):
    from test_gpu_parity import random_atmosphere
    rng = np.random.default_rng(21)
    atms = [random_atmosphere(oracle, rng) for _ in range(2)]
    shape = oracle.MEDIUM_SHAPE
    b = atmo.Batch(atms, [shape] * 2, [3, 4])
    b.run()
    atmo.synchronize_stream()
    i = 1
    S = b.read(i, atmo.LUT_SCATTERING)
    run_case(atmo, oracle, torch, b.lut_set(i), atms[i], shape,
             b.read(i, atmo.LUT_TRANSMITTANCE), S, S, b.read(i, atmo.LUT_IRRADIANCE), True, 13,
             n=200)
    with pytest.raises(atmo.AtmoError):
        b.lut_set(i).solar_radiance(luminance=True)


def test_luminance_api_and_solar_radiance(atmo, torch):
    m = earth_model(atmo)
    m.Init(4)
    s = m.lut_set()
    sky_k, sun_k = m.luminance_factors()
    a = m.atmosphere_at()
    r = s.solar_radiance()
    for i in range(3):
        assert r[i] == pytest.approx(a.solar_irradiance[i] / (np.pi * a.sun_angular_radius ** 2),
                                     rel=1e-12)
    rl = s.solar_radiance(luminance=True)
    k6 = [float("%.6f" % k) for k in sun_k]
    for i in range(3):
        assert rl[i] == pytest.approx(r[i] * k6[i], rel=1e-6)
    rng = np.random.default_rng(3)
    cam, view, sun, point, normal, shadow = (
        torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
        for x in make_queries(rng, 256, 6360.0, 6420.0))
    rad, _ = s.sky_radiance(cam, view, sun)
    lum, _ = s.sky_radiance(cam, view, sun, luminance=True)
    ks = torch.tensor([float("%.6f" % k) for k in sky_k], device="cuda")
    torch.testing.assert_close(lum, rad * ks, rtol=1e-6, atol=0.0)
    a1, b1 = s.sun_and_sky_irradiance(point, normal, sun)
    a2, b2 = s.sun_and_sky_irradiance(point, normal, sun, luminance=True)
    ksun = torch.tensor(k6, device="cuda")
    torch.testing.assert_close(a2, a1 * ksun, rtol=1e-6, atol=0.0)
    torch.testing.assert_close(b2, b1 * ks, rtol=1e-6, atol=0.0)
    # One sun direction for every query equals the per-query form.
    one = sun[0].contiguous()
    r1, _ = s.sky_radiance(cam, view, one)
    r2, _ = s.sky_radiance(cam, view, one.expand_as(sun).contiguous())
    torch.testing.assert_close(r1, r2, rtol=0.0, atol=0.0)


def test_fifteen_wavelength_model_has_luminance_api_only(atmo, torch):
    m = earth_model(atmo, n_lambda=15)
    m.Init(2)
    s = m.lut_set()
    v = torch.tensor([[0.0, 0.0, 6361.0]], device="cuda")
    d = torch.tensor([[0.0, 0.6, 0.8]], device="cuda")
    sun = torch.tensor([0.0, 0.0, 1.0], device="cuda")
    lum, _ = s.sky_radiance(v, d, sun, luminance=True)
    assert torch.isfinite(lum).all() and (lum > 0).all()
    with pytest.raises(atmo.AtmoError):
        s.sky_radiance(v, d, sun, luminance=False)


def test_shade_view_equals_queries(atmo, torch):
    m = earth_model(atmo)
    m.Init(4)
    s = m.lut_set()
    W, H = 64, 48
    cam = np.array([0.0, 0.0, 6360.0 + 1.5])
    fwd = np.array([0.0, 0.9, 0.1]); fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, [0.0, 0.0, 1.0]); right /= np.linalg.norm(right)
    up = np.cross(right, fwd)
    sun = np.array([0.3, 0.5, 0.4]); sun /= np.linalg.norm(sun)
    view = atmo.PinholeView()
    for name, v in (("camera", cam), ("right", right), ("up", up), ("forward", fwd),
                    ("sun_direction", sun), ("albedo", [0.1, 0.2, 0.3])):
        setattr(view, name, (C.c_float * 3)(*v))
    view.fov_y = np.radians(50.0)
    view.width, view.height = W, H
    rng = np.random.default_rng(5)
    depth = rng.uniform(0.1, 100.0, size=(H, W)).astype(np.float32)
    dt = torch.from_numpy(depth).cuda()
    sky, shaded = s.shade_view(view, dt)
    # The same pixels through the query kernels, with the rays built here.
    f32 = lambda x: np.asarray(x, np.float32)  # noqa: E731
    t = np.float32(np.tan(np.float32(0.5 * np.float32(view.fov_y))))
    ii, jj = np.meshgrid(np.arange(W), np.arange(H))
    sx = ((2 * ii + 1) / np.float32(W) - 1) * t * (np.float32(W) / np.float32(H))
    sy = (1 - (2 * jj + 1) / np.float32(H)) * t
    rays = f32(fwd)[None, None] + sx[..., None] * f32(right) + sy[..., None] * f32(up)
    rays /= np.linalg.norm(rays, axis=-1, keepdims=True)
    rays = torch.from_numpy(f32(rays.reshape(-1, 3))).cuda()
    camt = torch.from_numpy(f32(np.tile(cam, (W * H, 1)))).cuda()
    sunt = torch.from_numpy(f32(sun)).cuda()
    r_sky, t_sky = s.sky_radiance(camt, rays, sunt)
    pts = camt + rays * dt.reshape(-1, 1)
    r_pt, t_pt = s.sky_radiance_to_point(camt, pts, sunt)
    su, sk = s.sun_and_sky_irradiance(pts, -rays, sunt)
    alb = torch.tensor([0.1, 0.2, 0.3], device="cuda") / np.pi
    expect = r_pt + t_pt * alb * (su + sk)
    torch.testing.assert_close(sky.reshape(-1, 4)[:, :3], r_sky, rtol=2e-4, atol=1e-7)
    torch.testing.assert_close(sky.reshape(-1, 4)[:, 3], t_sky[:, 1], rtol=2e-4, atol=1e-7)
    # The shading kernel integrates along the pixel's own ray; the query kernel
    # takes the direction of p - camera, with p = camera + depth x ray held in
    # FP32 at planet scale (~0.5 m spacing at 6,360 km), which turns that
    # direction by up to ~5e-4 km / depth radians.  Short segments, where
    # S(camera) - T S(p) cancels, magnify that: the two agree to the query
    # bound where the turn is small (depth >= 10 km: <= 5e-5 rad).
    got = shaded.reshape(-1, 4)[:, :3]
    far = dt.reshape(-1) >= 10.0
    assert far.sum() > 0.85 * far.numel()
    torch.testing.assert_close(got[far], expect[far], rtol=TOL_RENDER, atol=1e-6)
    torch.testing.assert_close(got[~far], expect[~far], rtol=5e-2, atol=1e-6)


@pytest.mark.parametrize("combined", [True, False], ids=["combined", "separate"])
def test_shade_view_vs_oracle(atmo, oracle, torch, combined):
    """shade_view against the oracle's FP64 render functions along each
    pixel's exact ray (point = camera + depth x ray in FP64), on the pixels
    where the oracle is well conditioned (the robustness mask of the query
    tests), with the query tests' bounds: sky radiance within TOL_RENDER, the
    shaded value (radiance to the point plus the lit albedo) within
    TOL_RENDER of itself plus TOL_TERMS of the sky radiance along the ray."""
    m = earth_model(atmo, combined=combined)
    m.Init(4)
    s = m.lut_set()
    W, H = 48, 32
    cam = np.array([0.0, 0.0, 6360.0 + 1.5])
    fwd = np.array([0.0, 0.9, 0.1]); fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, [0.0, 0.0, 1.0]); right /= np.linalg.norm(right)
    up = np.cross(right, fwd)
    sun = np.array([0.3, 0.5, 0.4]); sun /= np.linalg.norm(sun)
    albedo = np.array([0.1, 0.2, 0.3])
    view = atmo.PinholeView()
    for name, v in (("camera", cam), ("right", right), ("up", up), ("forward", fwd),
                    ("sun_direction", sun), ("albedo", albedo)):
        setattr(view, name, (C.c_float * 3)(*v))
    view.fov_y = np.radians(50.0)
    view.width, view.height = W, H
    rng = np.random.default_rng(6)
    depth = rng.uniform(0.1, 100.0, size=(H, W)).astype(np.float32)
    sky, shaded = s.shade_view(view, torch.from_numpy(depth).cuda())
    torch.cuda.synchronize()
    f32 = lambda x: np.asarray(x, np.float32)  # noqa: E731
    t = np.float32(np.tan(np.float32(0.5 * np.float32(view.fov_y))))
    ii, jj = np.meshgrid(np.arange(W), np.arange(H))
    sx = ((2 * ii + 1) / np.float32(W) - 1) * t * (np.float32(W) / np.float32(H))
    sy = (1 - (2 * jj + 1) / np.float32(H)) * t
    rays = f32(fwd)[None, None] + sx[..., None] * f32(right) + sy[..., None] * f32(up)
    rays = (rays / np.linalg.norm(rays, axis=-1, keepdims=True)).reshape(-1, 3)
    c64, s64 = f32(cam).astype(np.float64), f32(sun).astype(np.float64)
    d64 = depth.reshape(-1).astype(np.float64)
    T = m.transmittance()
    S = m.scattering()
    I = m.irradiance()
    M = S if combined else m.single_mie_scattering()
    ref = OracleRender(oracle, m.atmosphere_at(), atmo.DEFAULT_SHAPE, T, S, M, I, combined)
    alb = f32(albedo).astype(np.float64) / np.pi

    def evaluate(perturb):
        out = {"sky": np.zeros((W * H, 3)), "pt": np.zeros((W * H, 3))}
        for i in range(W * H):
            c, v, sn = c64, rays[i].astype(np.float64), s64
            if perturb:
                # ~0.5 m: FP32's own rounding of a coordinate at 6360 km.
                c = c + rng.normal(size=3) * 8e-8 * np.linalg.norm(c)
                v = v + rng.normal(size=3) * ROBUST_STEP
                v /= np.linalg.norm(v)
                sn = sn + rng.normal(size=3) * ROBUST_STEP
                sn /= np.linalg.norm(sn)
            p = c + v * d64[i]
            out["sky"][i] = ref.sky(c, v, 0.0, sn)[0]
            pt, pt_t = ref.to_point(c, p, 0.0, sn)
            su, sk = ref.sun_sky(p, -v, sn)
            out["pt"][i] = pt + pt_t * alb * (su + sk)
        return out

    ref_out, pert_out = evaluate(False), evaluate(True)
    gpu_out = {"sky": sky.reshape(-1, 4)[:, :3].cpu().numpy().astype(np.float64),
               "pt": shaded.reshape(-1, 4)[:, :3].cpu().numpy().astype(np.float64)}
    # The reference's domain: the point in the atmosphere shell and the
    # segment from the camera to it above the ground.
    a = m.atmosphere_at()
    q = (np.tile(c64, (W * H, 1)), rays.astype(np.float64), None,
         c64 + rays.astype(np.float64) * d64[:, None], None, None, d64)
    keep = in_domain(q, a.bottom_radius, a.top_radius)
    assert keep.mean() > 0.3
    sub = lambda d: {k: v[keep] for k, v in d.items()}  # noqa: E731
    compare(sub(ref_out), sub(pert_out), sub(gpu_out), "shade_view",
            terms=ref_out["sky"][keep])


def model_test_view_queries(rb, sun_theta_deg, width=64, height=36):
    """The view of atmosphere/reference/model_test.cc:436-477 (camera at
    (2000, -8000, 500) m above a planet centred at (0, 0, -Rb), pitch pi/30,
    50 degree vertical field of view, 640x360), sampled on a width x height
    grid of pixel centres, with the sun at (theta, phi = 90 deg) (the test
    cases' :812-1080).  Per pixel: the view ray; the point is the ground
    point 1 m above the surface where the ray hits the planet, else 10 km
    along the ray; the normal is the radial direction at the point."""
    pitch = np.pi / 30.0
    tan_fov = np.tan(np.radians(50.0) / 2.0)
    aspect = 640.0 / 360.0
    xs = (np.arange(width) + 0.5) / width * 2.0 - 1.0
    ys = (np.arange(height) + 0.5) / height * 2.0 - 1.0
    x, y = np.meshgrid(xs, ys)
    vx, vy, vz = tan_fov * aspect * x, tan_fov * y, -np.ones_like(x)
    # model_from_view rotation rows (1, 0, 0), (0, -sin p, -cos p), (0, cos p, -sin p).
    view = np.stack([vx, -np.sin(pitch) * vy - np.cos(pitch) * vz,
                     np.cos(pitch) * vy - np.sin(pitch) * vz], axis=-1).reshape(-1, 3)
    view /= np.linalg.norm(view, axis=1, keepdims=True)
    n = len(view)
    cam = np.tile([2.0, -8.0, 0.5 + rb], (n, 1))
    th = np.radians(sun_theta_deg)
    sun = np.tile([0.0, np.sin(th), np.cos(th)], (n, 1))
    rmu = np.sum(cam * view, axis=1)
    disc = rmu * rmu - (np.sum(cam * cam, axis=1) - rb * rb)
    t_ground = -rmu - np.sqrt(np.maximum(disc, 0.0))
    ground = (disc >= 0.0) & (t_ground > 0.0)
    point = cam + view * np.where(ground, t_ground, 10.0)[:, None]
    normal = point / np.linalg.norm(point, axis=1, keepdims=True)
    point = np.where(ground[:, None], normal * (rb + 1e-3), point)
    shadow = np.zeros(n)
    return as_f32((cam, view, sun, point, normal, shadow)), ground


@pytest.mark.parametrize("combined", [True, False], ids=["combined", "separate"])
@pytest.mark.parametrize("sun_theta", [65.0, 88.0])
def test_model_test_view_vs_oracle(atmo, oracle, torch, sun_theta, combined):
    """The render functions along the model_test view's pixel rays (sky
    pixels and ground pixels) on the reference's default LUTs, against the
    oracle's FP64 restatement of them, with the conditioning mask of
    run_case."""
    m = earth_model(atmo, combined=combined)
    m.Init(4)
    a = m.atmosphere_at()
    S = m.scattering()
    M = S if combined else m.single_mie_scattering()
    q, ground = model_test_view_queries(a.bottom_radius, sun_theta)
    assert 0.2 < ground.mean() < 0.8          # the horizon crosses the image
    ref = OracleRender(oracle, a, atmo.DEFAULT_SHAPE, m.transmittance(), S, M,
                       m.irradiance(), combined)
    rng = np.random.default_rng(int(sun_theta))
    ref_out = oracle_outputs(ref, q, rng, False)
    # Positions move by ~0.5 m, FP32's own rounding of a coordinate at
    # 6360 km (the random workload uses ~4x that).
    pert_out = oracle_outputs(ref, q, rng, True, position=8e-8)
    gpu_out = gpu_outputs(torch, m.lut_set(), q)
    cam, _, sun, point, normal, _ = q
    terms = np.array([ref.sky(cam[i], (point[i] - cam[i]) / np.linalg.norm(point[i] - cam[i]),
                              0.0, sun[i])[0] for i in range(len(cam))])
    factor = 0.5 * (1.0 + np.sum(normal * point, axis=1) / np.linalg.norm(point, axis=1))
    # The camera is 500 m above the ground, where FP32 positions (~0.5 m at
    # 6360 km) move the ground-side mu mapping of near-horizontal rays: fewer
    # queries pass the conditioning mask than for the random workload.
    compare(ref_out, pert_out, gpu_out, "model_test view, sun %g deg" % sun_theta, terms,
            factor, min_robust=0.25)
