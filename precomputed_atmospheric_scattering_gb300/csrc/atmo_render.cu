// atmo_render.cu -- render-time queries on the precomputed LUTs:
// GetSkyRadiance, GetSkyRadianceToPoint and GetSunAndSkyIrradiance
// (atmosphere/functions.glsl:1705-1896) with the radiance and luminance API of
// atmosphere/model.cc:221-281, one query per thread, in FP32 like the
// reference's shader.  The ray geometry uses the same cancellation-free
// (rho, r, r mu) forms as the precomputation kernels; the LUT lookups are the
// software GL-LINEAR fetches of atmo_device.cuh.
#include "atmo_passes.cuh"
#include "atmo_render.h"

namespace atmo {
namespace {

constexpr int kQueryThreads = 128;

__device__ __forceinline__ F3 Load3(const float* p, long long i) {
  return F3{p[3 * i], p[3 * i + 1], p[3 * i + 2]};
}
__device__ __forceinline__ void Store3(float* p, long long i, F3 v) {
  p[3 * i] = v.x;
  p[3 * i + 1] = v.y;
  p[3 * i + 2] = v.z;
}
__device__ __forceinline__ float Dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 Normalize(F3 a) { return a * rsqrtf(Dot(a, a)); }

// GetExtrapolatedSingleMieScattering (functions.glsl:1633-1645).
__device__ F3 ExtrapolatedSingleMie(const Consts& c, F3 rgb, float alpha) {
  if (rgb.x <= 0.0f) return f3(0.0f);
  const float k = alpha / rgb.x * (c.rayleigh.x / c.mie_sca.x);
  return F3{rgb.x * k * (c.mie_sca.x / c.rayleigh.x), rgb.y * k * (c.mie_sca.y / c.rayleigh.y),
            rgb.z * k * (c.mie_sca.z / c.rayleigh.z)};
}

// The 4D lookup of Scattering4 returning the alpha channel too; the weights
// of a node's taps formed once and the taps accumulated by FMA chains (2%
// less time per 1920x1080 shading request than pairwise products and adds).
__device__ float4 ScatteringRGBA(const float4* __restrict__ tex, const Shape& s,
                                 const Lookup4& L) {
  const int W = s.sw(), Hh = s.smu, D = s.sr;
  const float fy = floorf(L.y), fz = floorf(L.z);
  const float b = L.y - fy, c = L.z - fz;
  const int j0 = ClampIdx((int)fy, Hh), j1 = ClampIdx((int)fy + 1, Hh);
  const int k0 = ClampIdx((int)fz, D), k1 = ClampIdx((int)fz + 1, D);
  const int rows[4] = {(k0 * Hh + j0) * W, (k0 * Hh + j1) * W, (k1 * Hh + j0) * W,
                       (k1 * Hh + j1) * W};
  const float wr[4] = {(1.0f - b) * (1.0f - c), b * (1.0f - c), (1.0f - b) * c, b * c};
  float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const float fx = floorf(L.xl);
  const float a = L.xl - fx;
#pragma unroll
  for (int node = 0; node < 2; ++node) {
    const int base = node == 0 ? L.b0 : L.b1;
    const float wn = node == 0 ? 1.0f - L.lerp_nu : L.lerp_nu;
    const int i0 = ClampIdx(base + (int)fx, W), i1 = ClampIdx(base + (int)fx + 1, W);
    const float wa0 = (1.0f - a) * wn, wa1 = a * wn;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 t0 = __ldg(ATMO_CHECKED_PTR(kCheckLutTexel, tex, rows[q], i0, W * Hh * D));
      const float4 t1 = __ldg(ATMO_CHECKED_PTR(kCheckLutTexel, tex, rows[q], i1, W * Hh * D));
      const float w0 = wa0 * wr[q], w1 = wa1 * wr[q];
      acc.x = fmaf(t1.x, w1, fmaf(t0.x, w0, acc.x));
      acc.y = fmaf(t1.y, w1, fmaf(t0.y, w0, acc.y));
      acc.z = fmaf(t1.z, w1, fmaf(t0.z, w0, acc.z));
      acc.w = fmaf(t1.w, w1, fmaf(t0.w, w0, acc.w));
    }
  }
  return acc;
}

// GetCombinedScattering (functions.glsl:1658-1689) at the point p of a ray
// with r mu = rmu.
__device__ F3 CombinedScattering(const RenderLuts& q, const RadialPoint& p, float rmu, float mu_s,
                                 float nu, bool ground, F3* mie) {
  const Consts& c = q.c;
  const Shape& s = q.s;
  const float u_mu = UMuFromRMu(c, s, p, rmu, ground);
  const float u_mu_s = UMuSFromMuS(c, s, clampf(mu_s, -1.0f, 1.0f));
  const float u_r = TexCoord(s, kMapSR, p.rho / c.H);
  const Lookup4 L = MakeLookup(s, (nu + 1.0f) * 0.5f, u_mu_s, u_mu, u_r);
  if (q.combined) {
    const float4 v = ScatteringRGBA(q.S, s, L);
    const F3 rgb{v.x, v.y, v.z};
    *mie = ExtrapolatedSingleMie(c, rgb, v.w);
    return rgb;
  }
  *mie = Scattering4(q.M, s, L);
  return Scattering4(q.S, s, L);
}

// A ray from a point at radius r along r mu = rmu, in (rho, r, rmu) form.
struct RayStart {
  RadialPoint p;
  float rmu, delta;   // r mu and rho^2 - (r mu)^2
  bool ground;        // RayIntersectsGround (functions.glsl:240-246)
};
__device__ RayStart MakeRayStart(const Consts& c, float r, float rmu, bool at_top) {
  RayStart o;
  o.p.r = r;
  o.p.rho = at_top ? c.H : sqrtf(fmaxf((r - c.Rb) * (r + c.Rb), 0.0f));
  o.p.h = at_top ? c.Rt - c.Rb : o.p.rho * o.p.rho / (r + c.Rb);
  o.rmu = rmu;
  o.delta = (o.p.rho - rmu) * (o.p.rho + rmu);
  o.ground = rmu < 0.0f && o.delta <= 0.0f;
  return o;
}

// GetTransmittance (functions.glsl:493-515) over distance d from the start.
__device__ F3 RayTransmittance(const RenderLuts& q, const RayStart& o, float d) {
  const Consts& c = q.c;
  const RadialPoint pd = PointAlongRay(c, o.p.rho, o.rmu, d);
  const TStart st = MakeTStart(c, q.s, q.T, q.Tau, o.p.rho, o.p.r, o.ground ? -o.rmu : o.rmu,
                               o.delta);
  return SegmentTransmittance(c, q.s, q.T, q.Tau, o.rmu, o.delta, pd, d, o.ground, st);
}

// Moves a camera outside the atmosphere to the top boundary along the view
// ray (functions.glsl:1720-1731, :1799-1808).  Returns false when the ray
// misses the atmosphere.
__device__ bool EnterAtmosphere(const Consts& c, F3* camera, F3 view, float* r, float* rmu,
                                bool* at_top) {
  *r = sqrtf(Dot(*camera, *camera));
  *rmu = Dot(*camera, view);
  *at_top = false;
  const float disc = *rmu * *rmu - (*r - c.Rt) * (*r + c.Rt);
  const float sq = sqrtf(disc);   // NaN when the ray misses the sphere
  const float d_top = -*rmu - sq;
  if (d_top > 0.0f) {
    *camera = fma3(view, d_top, *camera);
    *r = c.Rt;
    *rmu = -sq;
    *at_top = true;
  }
  return !(*r > c.Rt);
}

__device__ F3 SkyRadiance(const RenderLuts& q, F3 camera, F3 view, float shadow_length, F3 sun,
                          F3* transmittance) {
  const Consts& c = q.c;
  float r, rmu;
  bool at_top;
  if (!EnterAtmosphere(c, &camera, view, &r, &rmu, &at_top)) {
    *transmittance = f3(1.0f);
    return f3(0.0f);
  }
  const RayStart o = MakeRayStart(c, r, rmu, at_top);
  const float mu_s = Dot(camera, sun) / r;
  const float nu = Dot(view, sun);
  *transmittance = o.ground ? f3(0.0f)
                            : TransmittanceLookup(c, q.s, q.T, o.p.rho, r, rmu, o.delta);
  F3 mie, scattering;
  if (shadow_length == 0.0f) {
    scattering = CombinedScattering(q, o.p, rmu, mu_s, nu, o.ground, &mie);
  } else {
    const float d = shadow_length;
    const RadialPoint pp = PointAlongRay(c, o.p.rho, rmu, d);
    const float mu_s_p = (r * mu_s + d * nu) / pp.r;
    scattering = CombinedScattering(q, pp, rmu + d, mu_s_p, nu, o.ground, &mie);
    const F3 st = RayTransmittance(q, o, d);
    scattering = scattering * st;
    mie = mie * st;
  }
  return scattering * RayleighPhase(c, nu) + mie * MiePhase(c, nu);
}

__device__ F3 SkyRadianceToPoint(const RenderLuts& q, F3 camera, F3 point, float shadow_length,
                                 F3 sun, F3* transmittance) {
  const Consts& c = q.c;
  const F3 view = Normalize(point - camera);
  float r, rmu;
  bool at_top;
  EnterAtmosphere(c, &camera, view, &r, &rmu, &at_top);
  const RayStart o = MakeRayStart(c, r, rmu, at_top);
  const float mu_s = Dot(camera, sun) / r;
  const float nu = Dot(view, sun);
  const F3 to_point = point - camera;
  float d = sqrtf(Dot(to_point, to_point));
  *transmittance = RayTransmittance(q, o, d);
  F3 mie;
  F3 scattering = CombinedScattering(q, o.p, rmu, mu_s, nu, o.ground, &mie);
  d = fmaxf(d - shadow_length, 0.0f);
  const RadialPoint pp = PointAlongRay(c, o.p.rho, rmu, d);
  const float mu_s_p = (r * mu_s + d * nu) / pp.r;
  F3 mie_p;
  const F3 scattering_p = CombinedScattering(q, pp, rmu + d, mu_s_p, nu, o.ground, &mie_p);
  const F3 shadow_t = shadow_length > 0.0f ? RayTransmittance(q, o, d) : *transmittance;
  scattering = scattering - shadow_t * scattering_p;
  if (q.combined) {
    mie = ExtrapolatedSingleMie(c, scattering, mie.x - shadow_t.x * mie_p.x);
  } else {
    mie = mie - shadow_t * mie_p;
  }
  mie = mie * smoothstepf(0.0f, 0.01f, mu_s);
  return scattering * RayleighPhase(c, nu) + mie * MiePhase(c, nu);
}

__device__ F3 SunAndSkyIrradiance(const RenderLuts& q, F3 point, F3 normal, F3 sun,
                                  F3* sky_irradiance) {
  const Consts& c = q.c;
  const float r = sqrtf(Dot(point, point));
  const float mu_s = Dot(point, sun) / r;
  *sky_irradiance =
      Irradiance(c, q.s, q.I, r - c.Rb, mu_s) * ((1.0f + Dot(normal, point) / r) * 0.5f);
  RadialPoint p;
  p.r = r;
  p.rho = sqrtf(fmaxf((r - c.Rb) * (r + c.Rb), 0.0f));
  p.h = r - c.Rb;
  return c.solar * TransmittanceToSun(c, q.s, q.T, p, Dot(point, sun)) *
         fmaxf(Dot(normal, sun), 0.0f);
}

// One pixel of a shading request: GetSkyRadiance along the view ray and
// GetSkyRadianceToPoint to p = camera + depth view.  Both start with the 4D
// lookup at the camera (or where the ray enters the atmosphere) along the
// ray; since p lies on the pixel's own ray, that lookup, the ray's set-up and
// the phase functions are made once for both (the query kernels take the
// direction of p - camera instead, which differs from the ray by rounding).
// A ray that misses the atmosphere takes the general forms.
__device__ void ShadePixel(const RenderLuts& q, F3 camera, F3 view, float depth, F3 sun, F3* sky,
                           F3* t_sky, F3* in_scatter, F3* t_point) {
  const Consts& c = q.c;
  const F3 point = fma3(view, depth, camera);
  F3 cam = camera;
  float r, rmu;
  bool at_top;
  if (!EnterAtmosphere(c, &cam, view, &r, &rmu, &at_top)) {
    *t_sky = f3(1.0f);
    *sky = f3(0.0f);
    *in_scatter = SkyRadianceToPoint(q, camera, point, 0.0f, sun, t_point);
    return;
  }
  const RayStart o = MakeRayStart(c, r, rmu, at_top);
  const float mu_s = Dot(cam, sun) / r;
  const float nu = Dot(view, sun);
  const float phase_r = RayleighPhase(c, nu), phase_m = MiePhase(c, nu);
  F3 mie;
  const F3 scattering = CombinedScattering(q, o.p, rmu, mu_s, nu, o.ground, &mie);
  *t_sky = o.ground ? f3(0.0f) : TransmittanceLookup(c, q.s, q.T, o.p.rho, r, rmu, o.delta);
  *sky = scattering * phase_r + mie * phase_m;
  const F3 to_point = point - cam;
  const float d = sqrtf(Dot(to_point, to_point));
  *t_point = RayTransmittance(q, o, d);
  const RadialPoint pp = PointAlongRay(c, o.p.rho, rmu, d);
  const float mu_s_p = (r * mu_s + d * nu) / pp.r;
  F3 mie_p;
  const F3 scattering_p = CombinedScattering(q, pp, rmu + d, mu_s_p, nu, o.ground, &mie_p);
  const F3 s2 = scattering - *t_point * scattering_p;
  F3 m2 = q.combined ? ExtrapolatedSingleMie(c, s2, mie.x - t_point->x * mie_p.x)
                     : mie - *t_point * mie_p;
  m2 = m2 * smoothstepf(0.0f, 0.01f, mu_s);
  *in_scatter = s2 * phase_r + m2 * phase_m;
}

__device__ F3 K(const float k[3]) { return F3{k[0], k[1], k[2]}; }

__global__ void __launch_bounds__(kQueryThreads)
k_query(const RenderLuts q, const QueryArrays x, int kind) {
  const long long i = (long long)blockIdx.x * kQueryThreads + threadIdx.x;
  if (i >= x.n) return;
  const F3 a = Load3(x.a, i), b = Load3(x.b, i);
  const F3 sun = Load3(x.sun, x.sun_stride == 0 ? 0 : i);
  const float shadow = x.shadow ? x.shadow[i] : 0.0f;
  F3 out0, out1;
  if (kind == (int)Query::kSkyRadiance) {
    out0 = SkyRadiance(q, a, b, shadow, sun, &out1);
    if (x.luminance) out0 = out0 * K(q.sky_k);
  } else if (kind == (int)Query::kSkyRadianceToPoint) {
    out0 = SkyRadianceToPoint(q, a, b, shadow, sun, &out1);
    if (x.luminance) out0 = out0 * K(q.sky_k);
  } else {
    out0 = SunAndSkyIrradiance(q, a, b, sun, &out1);
    if (x.luminance) {
      out0 = out0 * K(q.sun_k);
      out1 = out1 * K(q.sky_k);
    }
  }
  Store3(x.out0, i, out0);
  if (x.out1) Store3(x.out1, i, out1);
}

// One pixel of a shading request: the three queries of the reference's API
// along the pixel's view ray.
// 6 blocks per SM (80 registers, 76 bytes of spills) beat 8 at 64 registers
// (276 bytes of spills) by 3% and 7 at 72 registers by 1-3%, with the
// approximate division and square root of this file (with IEEE division, 8
// blocks had been 6% faster than 6).
__global__ void __launch_bounds__(kQueryThreads, 6)
k_shade_view(const RenderLuts q, const PinholeView v) {
  const long long pix = (long long)blockIdx.x * kQueryThreads + threadIdx.x;
  if (pix >= (long long)v.width * v.height) return;
  const int i = (int)(pix % v.width), j = (int)(pix / v.width);
  const float aspect = float(v.width) / float(v.height);
  const float sx = (float(2 * i + 1) / float(v.width) - 1.0f) * v.tan_half_fov_y * aspect;
  const float sy = (1.0f - float(2 * j + 1) / float(v.height)) * v.tan_half_fov_y;
  const F3 cam{v.camera[0], v.camera[1], v.camera[2]};
  const F3 right{v.right[0], v.right[1], v.right[2]};
  const F3 up{v.up[0], v.up[1], v.up[2]};
  const F3 fwd{v.forward[0], v.forward[1], v.forward[2]};
  const F3 sun{v.sun[0], v.sun[1], v.sun[2]};
  const F3 view = Normalize(fma3(right, sx, fma3(up, sy, fwd)));
  const float depth = v.depth[pix];
  const F3 point = fma3(view, depth, cam);
  F3 sky, t_sky, in_scatter, t_point, sky_irr;
  ShadePixel(q, cam, view, depth, sun, &sky, &t_sky, &in_scatter, &t_point);
  F3 sun_irr = SunAndSkyIrradiance(q, point, f3(0.0f) - view, sun, &sky_irr);
  if (v.luminance) {
    sky = sky * K(q.sky_k);
    in_scatter = in_scatter * K(q.sky_k);
    sun_irr = sun_irr * K(q.sun_k);
    sky_irr = sky_irr * K(q.sky_k);
  }
  const F3 albedo{v.albedo[0] * (1.0f / kPiF), v.albedo[1] * (1.0f / kPiF),
                  v.albedo[2] * (1.0f / kPiF)};
  const F3 shaded = fma3(t_point * albedo, sun_irr + sky_irr, in_scatter);
  v.sky[pix] = to4(sky, t_sky.y);
  v.shaded[pix] = to4(shaded, 1.0f);
}

}  // namespace

cudaError_t LaunchQuery(Query q, const RenderLuts& luts, const QueryArrays& x, cudaStream_t st) {
  if (x.n <= 0) return cudaSuccess;
  const long long blocks = (x.n + kQueryThreads - 1) / kQueryThreads;
  k_query<<<(unsigned)blocks, kQueryThreads, 0, st>>>(luts, x, (int)q);
  return cudaGetLastError();
}

cudaError_t LaunchShadeView(const RenderLuts& luts, const PinholeView& v, cudaStream_t st) {
  const long long n = (long long)v.width * v.height;
  if (n <= 0) return cudaSuccess;
  k_shade_view<<<(unsigned)((n + kQueryThreads - 1) / kQueryThreads), kQueryThreads, 0, st>>>(
      luts, v);
  return cudaGetLastError();
}

ATMO_CHECK_WORD_ACCESSOR(CheckWordRender)

}  // namespace atmo
