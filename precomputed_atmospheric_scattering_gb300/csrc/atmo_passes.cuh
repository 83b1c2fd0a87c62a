// atmo_passes.cuh -- per-texel bodies of the six precomputation passes
// (atmosphere/model.cc:125-208 shaders, functions.glsl:454-1586).  The kernels
// in atmo_kernels.cu map threads onto these; they also compile for the host.
#ifndef ATMO_PASSES_CUH_
#define ATMO_PASSES_CUH_

#include "atmo_instance.h"

#ifdef __CUDACC__
#define ATMO_PASS __device__ __forceinline__
#else
#define ATMO_PASS inline
#define __constant__
#endif
#include "atmo_trig.inc"

namespace atmo {

// ---------------------------------------------------------------------------
// Transmittance (functions.glsl:275-320, :454-463): the optical lengths of the
// three profiles over the samples q = first, first + stride, ... <= 500, as
// compensated (Kahan) FP32 sums.  The caller reduces over the stride lanes.
// ---------------------------------------------------------------------------
struct TransmittanceRay {
  float rho, rmu, dx;
  // The reference's own FP64 ray (functions.glsl:275-299 after :427-448) for
  // the horizon column, whose tangent ray can dip below the ground by FP64
  // rounding; zero elsewhere.
  double r64, rmu64_2, dx64;
  bool horizon;
};

// IEEE double operations that are never contracted into FMAs, so that the
// FP64 chain below rounds exactly like the reference's CPU model.
ATMO_PASS double dmul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
ATMO_PASS double dadd(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
ATMO_PASS double dsub(double a, double b) { return dadd(a, -b); }
ATMO_PASS double ddiv(double a, double b) {
#ifdef __CUDA_ARCH__
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}
ATMO_PASS double dsqrt(double a) {
#ifdef __CUDA_ARCH__
  return __dsqrt_rn(a);
#else
  return sqrt(a);
#endif
}

ATMO_PASS TransmittanceRay TransmittanceTexelRay(const Consts& c, const Shape& s, int texel) {
  int i = texel % s.tw, j = texel / s.tw;
  // GetRMuFromTransmittanceTextureUv at the texel centre: x = i / (n - 1).
  float x_mu = float(i) / float(s.tw - 1);
  float x_r = float(j) / float(s.th - 1);
  float rho = c.H * x_r;
  float r = sqrtf(rho * rho + c.Rb * c.Rb);
  float hm = (c.H - rho) * (c.H + rho);
  float d_min = hm / (c.Rt + r);
  float d_max = rho + c.H;
  float d = d_min + x_mu * (d_max - d_min);
  TransmittanceRay ray;
  ray.rho = rho;
  // r mu = (H^2 - rho^2 - d^2) / (2 d); mu = 1 when d = 0.
  ray.rmu = d == 0.0f ? r : clampf((hm - d * d) / (2.0f * d), -r, r);
  ray.dx = d / float(kOpticalLengthSamples);
  ray.horizon = i == s.tw - 1;
  ray.r64 = ray.rmu64_2 = ray.dx64 = 0.0;
  if (ray.horizon) {
    // functions.glsl:427-448, :207-214, :285-289 in the reference's order.
    const double Rb = c.dRb, Rt = c.dRt;
    double u = ddiv(double(i) + 0.5, double(s.tw)), v = ddiv(double(j) + 0.5, double(s.th));
    double xm = ddiv(dsub(u, ddiv(0.5, double(s.tw))), dsub(1.0, ddiv(1.0, double(s.tw))));
    double xr = ddiv(dsub(v, ddiv(0.5, double(s.th))), dsub(1.0, ddiv(1.0, double(s.th))));
    double H = dsqrt(dsub(dmul(Rt, Rt), dmul(Rb, Rb)));
    double rh = dmul(H, xr);
    double rr = dsqrt(dadd(dmul(rh, rh), dmul(Rb, Rb)));
    double dmn = dsub(Rt, rr), dmx = dadd(rh, H);
    double dd = dadd(dmn, dmul(xm, dsub(dmx, dmn)));
    double mu = dd == 0.0 ? 1.0
                          : ddiv(dsub(dsub(dmul(H, H), dmul(rh, rh)), dmul(dd, dd)),
                                 dmul(dmul(2.0, rr), dd));
    mu = fmin(fmax(mu, -1.0), 1.0);
    double disc = dadd(dmul(dmul(rr, rr), dsub(dmul(mu, mu), 1.0)), dmul(Rt, Rt));
    double dist = fmax(dadd(-dmul(rr, mu), dsqrt(fmax(disc, 0.0))), 0.0);
    ray.r64 = rr;
    ray.rmu64_2 = dmul(dmul(2.0, rr), mu);
    ray.dx64 = ddiv(dist, double(kOpticalLengthSamples));
  }
  return ray;
}

struct Kahan {
  float s = 0.0f, e = 0.0f;
  ATMO_PASS void add(float x) {
    float y = x - e;
    float t = s + y;
    e = (t - s) - y;
    s = t;
  }
};

// GetProfileDensity with the layer chosen by an FP64 altitude.
ATMO_PASS float ProfileDensity64(const ProfileF& p, double h) {
  return h < double(p.layer[0].width) ? LayerDensity(p.layer[0], (float)h)
                                      : LayerDensity(p.layer[1], (float)h);
}

// ProfileDensity for the optical-length samples: a layer without an
// exponential term (the ozone layers) skips its exp (its product with 0).
ATMO_PASS float SampleDensity(const ProfileF& p, float h) {
  const LayerF& l = h < p.layer[0].width ? p.layer[0] : p.layer[1];
  const float e = l.exp_term == 0.0f ? 0.0f : l.exp_term * expf(l.exp_scale * h);
  return clampf(e + l.linear_term * h + l.constant_term, 0.0f, 1.0f);
}

ATMO_PASS void OpticalLengthPartial(const Consts& c, const TransmittanceRay& ray, int first,
                                    int stride, float out[3]) {
  Kahan kr, km, ka;
  const float near_ground = 1e-5f * (c.Rt - c.Rb);
  for (int q = first; q <= kOpticalLengthSamples; q += stride) {
    float d = float(q) * ray.dx;
    RadialPoint p = PointAlongRay(c, ray.rho, ray.rmu, d);
    float w = (q == 0 || q == kOpticalLengthSamples) ? 0.5f : 1.0f;
    if (ray.horizon && p.h < near_ground) {
      // A sample at the tangent point of a horizon ray: the reference's
      // unclamped FP64 altitude decides between the layers (it can be
      // slightly negative, selecting layer 0).
      double di = dmul(double(q), ray.dx64);
      double ri = dsqrt(dadd(dadd(dmul(di, di), dmul(ray.rmu64_2, di)),
                             dmul(ray.r64, ray.r64)));
      double h = dsub(ri, c.dRb);
      kr.add(ProfileDensity64(c.prof_r, h) * w);
      km.add(ProfileDensity64(c.prof_m, h) * w);
      ka.add(ProfileDensity64(c.prof_a, h) * w);
      continue;
    }
    kr.add(SampleDensity(c.prof_r, p.h) * w);
    km.add(SampleDensity(c.prof_m, p.h) * w);
    ka.add(SampleDensity(c.prof_a, p.h) * w);
  }
  out[0] = kr.s;
  out[1] = km.s;
  out[2] = ka.s;
}

// Optical depth sum_i beta_i L_i of functions.glsl:306-320 (tau = -ln T).
ATMO_PASS F3 OpticalDepth(const Consts& c, const TransmittanceRay& ray, const float sums[3]) {
  return c.rayleigh * (sums[0] * ray.dx) + c.mie_ext * (sums[1] * ray.dx) +
         c.absorption * (sums[2] * ray.dx);
}

// ---------------------------------------------------------------------------
// Direct irradiance (functions.glsl:1443-1461, :1558-1567).
// ---------------------------------------------------------------------------
ATMO_PASS F3 DirectIrradianceTexel(const Instance& in, int texel) {
  const Consts& c = in.c;
  const Shape& s = in.s;
  int i = texel % s.iw, j = texel / s.iw;
  IrrRow row = in.tab.irows[j];
  float mu_s = in.tab.mus_i[i];
  float a = c.alpha_s;
  float f = mu_s < -a ? 0.0f : (mu_s > a ? mu_s : (mu_s + a) * (mu_s + a) / (4.0f * a));
  return c.solar * TransmittanceToTop(c, s, in.T, row.rho, row.r, row.r * mu_s) * f;
}

// Transmittance to the ground x albedo / pi of density row e = k * 16 + l:
// GetTransmittance(r, cos theta, distance_to_ground, true) with the end point
// exactly on the ground (rho = 0, r = Rb).
ATMO_PASS float4 GroundRowTransmittance(const Instance& in, int e) {
  const Consts& c = in.c;
  const Shape& s = in.s;
  DensityRow dr = in.tab.drows[e];
  if (!dr.ground) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  int k = e / kDensityThetaSamples;
  TexelRow row = in.tab.rows[k * s.smu];
  float rmu = row.r * dr.cos_t;
  float rmu_g = fminf(rmu + dr.dist_ground, 0.0f);
  TStart start = MakeTStart(c, s, in.T, in.Tau, row.rho, row.r, -rmu, dr.delta);
  RadialPoint ground_point;
  ground_point.rho = 0.0f;
  ground_point.r = c.Rb;
  ground_point.h = 0.0f;
  F3 t = SegmentTransmittance(c, s, in.T, in.Tau, rmu, dr.delta, ground_point,
                              rmu_g - rmu, true, start);
  return to4(t * c.albedo * (1.0f / kPiF), 0.0f);
}

// ---------------------------------------------------------------------------
// Single scattering (functions.glsl:650-730, :933-945; shader model.cc:142-157).
// ---------------------------------------------------------------------------
ATMO_PASS void SingleScatteringTexel(const Instance& in, long long texel, F3* rayleigh, F3* mie) {
  const Consts& c = in.c;
  const Shape& s = in.s;
  int k, j, col, n;
  SplitTexel(s, texel, &k, &j, &col, &n);
  TexelRow row = in.tab.rows[k * s.smu + j];
  TexelCol cc = in.tab.cols[col];
  TexelAngles ang = MakeAngles(s, row, cc, n);
  const bool ground = row.ground != 0;
  float dx = row.d / float(kSingleScatteringSamples);
  float rmu_s = row.r * ang.mu_s;
  TStart start = MakeTStart(c, s, in.T, in.Tau, row.rho, row.r,
                            ground ? -row.rmu : row.rmu, row.delta);
  F3 sum_r = f3(0.0f), sum_m = f3(0.0f);
  for (int i = 0; i <= kSingleScatteringSamples; ++i) {
    float d = float(i) * dx;
    float e = float(kSingleScatteringSamples - i) * dx;
    RadialPoint p = PointFromRho2(c, RayRho2(row, d, e));
    F3 t = SegmentTransmittance(c, s, in.T, in.Tau, row.rmu, row.delta, p, d, ground, start) *
           TransmittanceToSun(c, s, in.T, p, fmaf(d, ang.nu, rmu_s));
    float w = (i == 0 || i == kSingleScatteringSamples) ? 0.5f : 1.0f;
    sum_r = fma3(t, ProfileDensity(c.prof_r, p.h) * w, sum_r);
    sum_m = fma3(t, ProfileDensity(c.prof_m, p.h) * w, sum_m);
  }
  *rayleigh = sum_r * dx * c.solar * c.rayleigh;
  *mie = sum_m * dx * c.solar * c.mie_sca;
}

// Writes the single-scattering outputs of one texel (MRT of model.cc:143-156).
ATMO_PASS void StoreSingleScattering(const Instance& in, long long texel, F3 ray, F3 mie) {
  in.dR[texel] = to4(ray, 1.0f);
  in.dM[texel] = to4(mie, 1.0f);
  F3 lr = MatVec(in.c.lum, ray), lm = MatVec(in.c.lum, mie);
  float alpha = in.combined ? lm.x : 0.0f;
  if (in.blend) {
    float4 o = in.S[texel];
    in.S[texel] = make_float4(o.x + lr.x, o.y + lr.y, o.z + lr.z, o.w + alpha);
  } else {
    in.S[texel] = to4(lr, alpha);
  }
  if (!in.combined) {
    if (in.blend) {
      float4 o = in.M[texel];
      in.M[texel] = make_float4(o.x + lm.x, o.y + lm.y, o.z + lm.z, 0.0f);
    } else {
      in.M[texel] = to4(lm, 0.0f);
    }
  }
}

// ---------------------------------------------------------------------------
// Scattering density, plain per-texel form (functions.glsl:1163-1260, :1348-1367).
// ---------------------------------------------------------------------------
ATMO_PASS F3 ScatteringDensityTexel(const Instance& in, long long texel, int order) {
  const Consts& c = in.c;
  const Shape& s = in.s;
  int k, j, col, n;
  SplitTexel(s, texel, &k, &j, &col, &n);
  TexelRow row = in.tab.rows[k * s.smu + j];
  TexelCol cc = in.tab.cols[col];
  TexelAngles ang = MakeAngles(s, row, cc, n);
  F3 a_r = c.rayleigh * ProfileDensity(c.prof_r, row.h);
  F3 a_m = c.mie_sca * ProfileDensity(c.prof_m, row.h);
  const float u_r = (float(k) + 0.5f) / float(s.sr);
  const float dtdp = (kPiF / 16.0f) * (kPiF / 16.0f);
  F3 J = f3(0.0f);
  for (int l = 0; l < kDensityThetaSamples; ++l) {
    DensityRow dr = in.tab.drows[k * kDensityThetaSamples + l];
    F3 tg = f3(dr.t_ground);
    F3 row_sum = f3(0.0f);
    for (int m = 0; m < kDensityPhiSamples; ++m) {
      float2 cs = c_density_phi[m];
      float ox = cs.x * dr.sin_t, oy = cs.y * dr.sin_t;
      float nu1 = fmaf(ang.sx, ox, fmaf(ang.sy, oy, ang.mu_s * dr.cos_t));
      Lookup4 L = MakeLookup(s, (nu1 + 1.0f) * 0.5f, cc.u_mu_s, dr.u_mu, u_r);
      F3 radiance;
      if (order - 1 == 1) {
        radiance = Scattering4(in.dR, s, L) * RayleighPhase(c, nu1) +
                   Scattering4(in.dM, s, L) * MiePhase(c, nu1);
      } else {
        radiance = Scattering4(in.dR, s, L);
      }
      if (dr.ground) {
        // Ground point: |(0, 0, r) + omega_i * dist| = Rb, so the normal's
        // cosine with the sun is (r mu_s + dist nu1) / Rb.
        float mu_g = fmaf(dr.dist_ground, nu1, row.r * ang.mu_s) / c.Rb;
        radiance = fma3(tg, Irradiance(c, s, DeltaIrradiance(in, order - 2), 0.0f, mu_g),
                        radiance);
      }
      float nu2 = fmaf(ang.omega_x, ox, ang.mu * dr.cos_t);
      row_sum = fma3(radiance, a_r * RayleighPhase(c, nu2) + a_m * MiePhase(c, nu2), row_sum);
    }
    J = fma3(row_sum, dtdp * dr.sin_t, J);
  }
  return J;
}

// ---------------------------------------------------------------------------
// Indirect irradiance (functions.glsl:1477-1511, :1573-1586): the sum over the
// 64 phi samples m = first, first + stride, ... of every theta row.
// ---------------------------------------------------------------------------
ATMO_PASS F3 IndirectIrradiancePartial(const Instance& in, int texel, int order, int first,
                                     int stride) {
  const Consts& c = in.c;
  const Shape& s = in.s;
  int i = texel % s.iw, j = texel / s.iw;
  IrrRow ir = in.tab.irows[j];
  float mu_s = in.tab.mus_i[i];
  float sin_s = sqrtf(fmaxf((1.0f - mu_s) * (1.0f + mu_s), 0.0f));
  RadialPoint p;
  p.rho = ir.rho;
  p.r = ir.r;
  p.h = ir.h;
  const float u_r = TexCoord(s, kMapSR, ir.rho / c.H);
  const float u_mu_s = UMuSFromMuS(c, s, mu_s);
  const float dtdp = (kPiF / 32.0f) * (kPiF / 32.0f);
  F3 acc = f3(0.0f);
  for (int t = 0; t < kIndirectThetaSamples; ++t) {
    float2 th = c_indirect_theta[t];
    float u_mu = UMuFromRMu(c, s, p, ir.r * th.x, false);
    F3 row_sum = f3(0.0f);
    for (int m = first; m < kIndirectPhiSamples; m += stride) {
      float2 ph = c_indirect_phi[m];
      float nu = fmaf(ph.x * th.y, sin_s, th.x * mu_s);
      Lookup4 L = MakeLookup(s, (nu + 1.0f) * 0.5f, u_mu_s, u_mu, u_r);
      F3 radiance;
      if (order == 1) {
        radiance = Scattering4(in.dR, s, L) * RayleighPhase(c, nu) +
                   Scattering4(in.dM, s, L) * MiePhase(c, nu);
      } else {
        radiance = Scattering4(in.dR, s, L);
      }
      row_sum += radiance;
    }
    acc = fma3(row_sum, th.x * dtdp * th.y, acc);
  }
  return acc;
}

// ---------------------------------------------------------------------------
// Multiple scattering, plain per-texel form (functions.glsl:1285-1330,
// :1369-1383; shader model.cc:192-208).
// ---------------------------------------------------------------------------
ATMO_PASS F3 MultipleScatteringTexel(const Instance& in, long long texel, float* nu_out) {
  const Consts& c = in.c;
  const Shape& s = in.s;
  int k, j, col, n;
  SplitTexel(s, texel, &k, &j, &col, &n);
  TexelRow row = in.tab.rows[k * s.smu + j];
  TexelCol cc = in.tab.cols[col];
  TexelAngles ang = MakeAngles(s, row, cc, n);
  const bool ground = row.ground != 0;
  float dx = row.d / float(kMultipleScatteringSamples);
  float rmu_s = row.r * ang.mu_s;
  const float u_nu = (ang.nu + 1.0f) * 0.5f;
  TStart start = MakeTStart(c, s, in.T, in.Tau, row.rho, row.r,
                            ground ? -row.rmu : row.rmu, row.delta);
  F3 sum = f3(0.0f);
  for (int i = 0; i <= kMultipleScatteringSamples; ++i) {
    float d = float(i) * dx;
    float e = float(kMultipleScatteringSamples - i) * dx;
    RadialPoint p = PointFromRho2(c, RayRho2(row, d, e));
    float mu_s_i = clampf(fmaf(d, ang.nu, rmu_s) / p.r, -1.0f, 1.0f);
    // The distance from the sample to the ray's boundary is e (the
    // discriminant is invariant along the ray).
    float u_mu = UMuFromDistance(c, s, p, e, ground);
    Lookup4 L = MakeLookup(s, u_nu, UMuSFromMuS(c, s, mu_s_i), u_mu,
                           TexCoord(s, kMapSR, p.rho / c.H));
    F3 t = SegmentTransmittance(c, s, in.T, in.Tau, row.rmu, row.delta, p, d, ground, start);
    float w = (i == 0 || i == kMultipleScatteringSamples) ? 0.5f : 1.0f;
    sum = fma3(Scattering4(in.dJ, s, L) * t, dx * w, sum);
  }
  *nu_out = ang.nu;
  return sum;
}

}  // namespace atmo

#endif  // ATMO_PASSES_CUH_
