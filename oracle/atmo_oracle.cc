/*
 * CPU oracle for the atmosphere LUT precomputation -- TEST INFRASTRUCTURE ONLY.
 *
 * A double-precision restatement, in this project's own code, of the
 * reference's precomputation algorithm (ebruneton/precomputed_atmospheric_
 * scattering).  Each function cites the reference function it follows.  The
 * arithmetic is kept in the reference's order so that this restatement agrees
 * with the reference's own functions.glsl compiled as C++ (oracle/ref/) to
 * ~1e-12.  Textures use GL LINEAR filtering with CLAMP_TO_EDGE at texel
 * centres, as atmosphere/model.cc:427-430 and :444-448 configure them.
 *
 * Used only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline.
 */
#include "atmo_oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#if defined(__CUDACC__)
#define ORACLE_HD __host__ __device__
#else
#define ORACLE_HD
#endif

namespace {

constexpr double kPi = 3.14159265358979323846;

// The math of the texel evaluators, callable from host and (in the FP64 GPU
// build, atmo_oracle_gpu.cu) device code: the C library functions, and
// min / max with the std:: semantics.  The FLOP-counting build
// (atmo_oracle_count.cc) supplies its own, over its counting scalar type.
#ifndef ORACLE_COUNTING
namespace om {
ORACLE_HD inline double sqrt(double x) { return ::sqrt(x); }
ORACLE_HD inline double exp(double x) { return ::exp(x); }
ORACLE_HD inline double floor(double x) { return ::floor(x); }
ORACLE_HD inline double fmod(double x, double y) { return ::fmod(x, y); }
ORACLE_HD inline double pow(double x, double y) { return ::pow(x, y); }
ORACLE_HD inline double sin(double x) { return ::sin(x); }
ORACLE_HD inline double cos(double x) { return ::cos(x); }
template <class T>
ORACLE_HD inline T min(T a, T b) { return b < a ? b : a; }
template <class T>
ORACLE_HD inline T max(T a, T b) { return a < b ? b : a; }
}  // namespace om
#endif

// Hooks of the FLOP-counting build: the pass a texel evaluation belongs to,
// and the texture-filtering scope (GL filtering is done by the texture unit in
// the reference, so its arithmetic is counted apart).  Empty otherwise.
#ifndef ORACLE_COUNT_PASS
#define ORACLE_COUNT_PASS(kind)
#define ORACLE_COUNT_FILTER()
#endif

// ---------------------------------------------------------------------------
// Small vector types (the GLSL vec3 / spectrum of atmosphere/definitions.glsl)
// ---------------------------------------------------------------------------
struct Spec {
  double v[3];
  ORACLE_HD Spec() : v{0, 0, 0} {}
  ORACLE_HD explicit Spec(double a) : v{a, a, a} {}
  ORACLE_HD Spec(double a, double b, double c) : v{a, b, c} {}
  ORACLE_HD static Spec From(const double* p) { return Spec(p[0], p[1], p[2]); }
  ORACLE_HD double& operator[](int i) { return v[i]; }
  ORACLE_HD double operator[](int i) const { return v[i]; }
};
ORACLE_HD inline Spec operator+(const Spec& a, const Spec& b) {
  return Spec(a[0] + b[0], a[1] + b[1], a[2] + b[2]);
}
ORACLE_HD inline Spec operator-(const Spec& a, const Spec& b) {
  return Spec(a[0] - b[0], a[1] - b[1], a[2] - b[2]);
}
ORACLE_HD inline Spec operator*(const Spec& a, const Spec& b) {
  return Spec(a[0] * b[0], a[1] * b[1], a[2] * b[2]);
}
ORACLE_HD inline Spec operator/(const Spec& a, const Spec& b) {
  return Spec(a[0] / b[0], a[1] / b[1], a[2] / b[2]);
}
ORACLE_HD inline Spec operator*(const Spec& a, double s) {
  return Spec(a[0] * s, a[1] * s, a[2] * s);
}
ORACLE_HD inline Spec operator*(double s, const Spec& a) { return a * s; }
ORACLE_HD inline Spec operator/(const Spec& a, double s) {
  return Spec(a[0] / s, a[1] / s, a[2] / s);
}
ORACLE_HD inline Spec& operator+=(Spec& a, const Spec& b) { return a = a + b; }
ORACLE_HD inline Spec sexp(const Spec& a) {
  return Spec(om::exp(a[0]), om::exp(a[1]), om::exp(a[2]));
}
ORACLE_HD inline Spec smin(const Spec& a, const Spec& b) {
  return Spec(om::min(a[0], b[0]), om::min(a[1], b[1]), om::min(a[2], b[2]));
}

struct V3 {
  double x, y, z;
};
ORACLE_HD inline V3 operator+(const V3& a, const V3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
ORACLE_HD inline V3 operator-(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
ORACLE_HD inline V3 operator*(const V3& a, double s) { return {a.x * s, a.y * s, a.z * s}; }
ORACLE_HD inline double dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
ORACLE_HD inline double length(const V3& a) { return om::sqrt(dot(a, a)); }
ORACLE_HD inline V3 normalize(const V3& a) { return a * (1.0 / length(a)); }

ORACLE_HD inline double clampd(double x, double lo, double hi) { return om::min(om::max(x, lo), hi); }
// GLSL smoothstep; for the degenerate e0 == e1 (a point sun) it returns 0 at
// x <= e0 and 1 above, where the clamp formula would give 0/0.
ORACLE_HD inline double smoothstep(double e0, double e1, double x) {
  if (x <= e0) return 0.0;
  if (x >= e1) return 1.0;
  double t = (x - e0) / (e1 - e0);
  return t * t * (3.0 - 2.0 * t);
}

// ---------------------------------------------------------------------------
// Textures: GL LINEAR + CLAMP_TO_EDGE, texel centres at (i + 0.5) / n.
// ---------------------------------------------------------------------------
struct Tex2 {
  int w = 0, h = 0;
  const double* p = nullptr;  // RGBA
  ORACLE_HD Spec Get(int i, int j) const {
    i = om::min(om::max(i, 0), w - 1);
    j = om::min(om::max(j, 0), h - 1);
    return Spec::From(p + 4 * ((long long)j * w + i));
  }
};
struct Tex3 {
  int w = 0, h = 0, d = 0;
  const double* p = nullptr;  // RGBA
  ORACLE_HD Spec Get(int i, int j, int k) const {
    i = om::min(om::max(i, 0), w - 1);
    j = om::min(om::max(j, 0), h - 1);
    k = om::min(om::max(k, 0), d - 1);
    return Spec::From(p + 4 * (((long long)k * h + j) * w + i));
  }
};

ORACLE_HD Spec texture(const Tex2& t, double u, double v) {
  ORACLE_COUNT_FILTER();
  double x = u * t.w - 0.5, y = v * t.h - 0.5;
  double fi = om::floor(x), fj = om::floor(y);
  int i = (int)fi, j = (int)fj;
  double a = x - fi, b = y - fj;
  return t.Get(i, j) * ((1.0 - a) * (1.0 - b)) + t.Get(i + 1, j) * (a * (1.0 - b)) +
         t.Get(i, j + 1) * ((1.0 - a) * b) + t.Get(i + 1, j + 1) * (a * b);
}

ORACLE_HD Spec texture(const Tex3& t, double u, double v, double w) {
  ORACLE_COUNT_FILTER();
  double x = u * t.w - 0.5, y = v * t.h - 0.5, z = w * t.d - 0.5;
  double fi = om::floor(x), fj = om::floor(y), fk = om::floor(z);
  int i = (int)fi, j = (int)fj, k = (int)fk;
  double a = x - fi, b = y - fj, c = z - fk;
  Spec r;
  for (int dk = 0; dk < 2; ++dk)
    for (int dj = 0; dj < 2; ++dj)
      for (int di = 0; di < 2; ++di) {
        double wt = (di ? a : 1.0 - a) * (dj ? b : 1.0 - b) * (dk ? c : 1.0 - c);
        r += t.Get(i + di, j + dj, k + dk) * wt;
      }
  return r;
}

// Texel taps (clamped flat indices and weights) of the 3D lookup above.
ORACLE_HD void texture_taps(const Tex3& t, double u, double v, double w, int idx[8], double wt[8]) {
  ORACLE_COUNT_FILTER();
  double x = u * t.w - 0.5, y = v * t.h - 0.5, z = w * t.d - 0.5;
  double fi = om::floor(x), fj = om::floor(y), fk = om::floor(z);
  int i = (int)fi, j = (int)fj, k = (int)fk;
  double a = x - fi, b = y - fj, c = z - fk;
  int n = 0;
  for (int dk = 0; dk < 2; ++dk)
    for (int dj = 0; dj < 2; ++dj)
      for (int di = 0; di < 2; ++di) {
        int ii = om::min(om::max(i + di, 0), t.w - 1);
        int jj = om::min(om::max(j + dj, 0), t.h - 1);
        int kk = om::min(om::max(k + dk, 0), t.d - 1);
        idx[n] = (kk * t.h + jj) * t.w + ii;
        wt[n] = (di ? a : 1.0 - a) * (dj ? b : 1.0 - b) * (dk ? c : 1.0 - c);
        ++n;
      }
}

// ---------------------------------------------------------------------------
// Atmosphere model.
// ---------------------------------------------------------------------------
struct Layer {
  double width, exp_term, exp_scale, linear_term, constant_term;
};
struct Profile {
  Layer layers[2];
};
struct Atm {
  Spec solar_irradiance;
  double sun_angular_radius, bottom_radius, top_radius;
  Profile rayleigh_density;
  Spec rayleigh_scattering;
  Profile mie_density;
  Spec mie_scattering, mie_extinction;
  double mie_phase_function_g;
  Profile absorption_density;
  Spec absorption_extinction, ground_albedo;
  double mu_s_min;
  // Shape (atmosphere/constants.h:47-61 as run-time values).
  int T_W, T_H, S_R, S_MU, S_MU_S, S_NU, I_W, I_H;
};

ORACLE_HD Profile ToProfile(const oracle_profile& p) {
  Profile q;
  for (int i = 0; i < 2; ++i) {
    q.layers[i] = {p.layers[i].width, p.layers[i].exp_term, p.layers[i].exp_scale,
                   p.layers[i].linear_term, p.layers[i].constant_term};
  }
  return q;
}

ORACLE_HD Atm ToAtm(const oracle_atmosphere* a, const oracle_shape* s) {
  Atm t;
  t.solar_irradiance = Spec::From(a->solar_irradiance);
  t.sun_angular_radius = a->sun_angular_radius;
  t.bottom_radius = a->bottom_radius;
  t.top_radius = a->top_radius;
  t.rayleigh_density = ToProfile(a->rayleigh_density);
  t.rayleigh_scattering = Spec::From(a->rayleigh_scattering);
  t.mie_density = ToProfile(a->mie_density);
  t.mie_scattering = Spec::From(a->mie_scattering);
  t.mie_extinction = Spec::From(a->mie_extinction);
  t.mie_phase_function_g = a->mie_phase_function_g;
  t.absorption_density = ToProfile(a->absorption_density);
  t.absorption_extinction = Spec::From(a->absorption_extinction);
  t.ground_albedo = Spec::From(a->ground_albedo);
  t.mu_s_min = a->mu_s_min;
  if (s) {
    t.T_W = s->transmittance_width;
    t.T_H = s->transmittance_height;
    t.S_R = s->scattering_r;
    t.S_MU = s->scattering_mu;
    t.S_MU_S = s->scattering_mu_s;
    t.S_NU = s->scattering_nu;
    t.I_W = s->irradiance_width;
    t.I_H = s->irradiance_height;
  } else {
    t.T_W = 256; t.T_H = 64; t.S_R = 32; t.S_MU = 128; t.S_MU_S = 32; t.S_NU = 8;
    t.I_W = 64; t.I_H = 16;
  }
  return t;
}

ORACLE_HD Tex2 MakeT(const Atm& a, const double* p) { return Tex2{a.T_W, a.T_H, p}; }
ORACLE_HD Tex2 MakeI(const Atm& a, const double* p) { return Tex2{a.I_W, a.I_H, p}; }
ORACLE_HD Tex3 MakeS(const Atm& a, const double* p) {
  return Tex3{a.S_NU * a.S_MU_S, a.S_MU, a.S_R, p};
}

// functions.glsl:113-127
ORACLE_HD double ClampCosine(double mu) { return clampd(mu, -1.0, 1.0); }
ORACLE_HD double ClampDistance(double d) { return om::max(d, 0.0); }
ORACLE_HD double ClampRadius(const Atm& a, double r) { return clampd(r, a.bottom_radius, a.top_radius); }
ORACLE_HD double SafeSqrt(double x) { return om::sqrt(om::max(x, 0.0)); }

// functions.glsl:207-214
ORACLE_HD double DistanceToTopAtmosphereBoundary(const Atm& a, double r, double mu) {
  double discriminant = r * r * (mu * mu - 1.0) + a.top_radius * a.top_radius;
  return ClampDistance(-r * mu + SafeSqrt(discriminant));
}
// functions.glsl:222-229
ORACLE_HD double DistanceToBottomAtmosphereBoundary(const Atm& a, double r, double mu) {
  double discriminant = r * r * (mu * mu - 1.0) + a.bottom_radius * a.bottom_radius;
  return ClampDistance(-r * mu - SafeSqrt(discriminant));
}
// functions.glsl:240-246
ORACLE_HD bool RayIntersectsGround(const Atm& a, double r, double mu) {
  return mu < 0.0 && r * r * (mu * mu - 1.0) + a.bottom_radius * a.bottom_radius >= 0.0;
}
// functions.glsl:263-273
ORACLE_HD double GetLayerDensity(const Layer& l, double altitude) {
  double density = l.exp_term * om::exp(l.exp_scale * altitude) +
                   l.linear_term * altitude + l.constant_term;
  return clampd(density, 0.0, 1.0);
}
ORACLE_HD double GetProfileDensity(const Profile& p, double altitude) {
  return altitude < p.layers[0].width ? GetLayerDensity(p.layers[0], altitude)
                                      : GetLayerDensity(p.layers[1], altitude);
}
// functions.glsl:275-299 (500 intervals, trapezoidal rule)
ORACLE_HD double ComputeOpticalLengthToTopAtmosphereBoundary(const Atm& a, const Profile& p, double r,
                                                   double mu) {
  const int SAMPLE_COUNT = 500;
  double dx = DistanceToTopAtmosphereBoundary(a, r, mu) / double(SAMPLE_COUNT);
  double result = 0.0;
  for (int i = 0; i <= SAMPLE_COUNT; ++i) {
    double d_i = double(i) * dx;
    double r_i = om::sqrt(d_i * d_i + 2.0 * r * mu * d_i + r * r);
    double y_i = GetProfileDensity(p, r_i - a.bottom_radius);
    double weight_i = i == 0 || i == SAMPLE_COUNT ? 0.5 : 1.0;
    result += y_i * weight_i * dx;
  }
  return result;
}
// functions.glsl:306-320
ORACLE_HD Spec ComputeTransmittanceToTopAtmosphereBoundary(const Atm& a, double r, double mu) {
  return sexp(Spec(0.0) -
              (a.rayleigh_scattering *
                   ComputeOpticalLengthToTopAtmosphereBoundary(a, a.rayleigh_density, r, mu) +
               a.mie_extinction *
                   ComputeOpticalLengthToTopAtmosphereBoundary(a, a.mie_density, r, mu) +
               a.absorption_extinction * ComputeOpticalLengthToTopAtmosphereBoundary(
                                             a, a.absorption_density, r, mu)));
}
// functions.glsl:342-348
ORACLE_HD double GetTextureCoordFromUnitRange(double x, int n) {
  return 0.5 / double(n) + x * (1.0 - 1.0 / double(n));
}
ORACLE_HD double GetUnitRangeFromTextureCoord(double u, int n) {
  return (u - 0.5 / double(n)) / (1.0 - 1.0 / double(n));
}
// functions.glsl:402-421
ORACLE_HD void GetTransmittanceTextureUvFromRMu(const Atm& a, double r, double mu, double* u,
                                      double* v) {
  double H = om::sqrt(a.top_radius * a.top_radius - a.bottom_radius * a.bottom_radius);
  double rho = SafeSqrt(r * r - a.bottom_radius * a.bottom_radius);
  double d = DistanceToTopAtmosphereBoundary(a, r, mu);
  double d_min = a.top_radius - r;
  double d_max = rho + H;
  double x_mu = (d - d_min) / (d_max - d_min);
  double x_r = rho / H;
  *u = GetTextureCoordFromUnitRange(x_mu, a.T_W);
  *v = GetTextureCoordFromUnitRange(x_r, a.T_H);
}
// functions.glsl:427-448
ORACLE_HD void GetRMuFromTransmittanceTextureUv(const Atm& a, double u, double v, double* r,
                                      double* mu) {
  double x_mu = GetUnitRangeFromTextureCoord(u, a.T_W);
  double x_r = GetUnitRangeFromTextureCoord(v, a.T_H);
  double H = om::sqrt(a.top_radius * a.top_radius - a.bottom_radius * a.bottom_radius);
  double rho = H * x_r;
  *r = om::sqrt(rho * rho + a.bottom_radius * a.bottom_radius);
  double d_min = a.top_radius - *r;
  double d_max = rho + H;
  double d = d_min + x_mu * (d_max - d_min);
  double m = d == 0.0 ? 1.0 : (H * H - rho * rho - d * d) / (2.0 * *r * d);
  *mu = ClampCosine(m);
}
// functions.glsl:454-463
ORACLE_HD Spec ComputeTransmittanceToTopAtmosphereBoundaryTexture(const Atm& a, double fx, double fy) {
  double r, mu;
  GetRMuFromTransmittanceTextureUv(a, fx / a.T_W, fy / a.T_H, &r, &mu);
  return ComputeTransmittanceToTopAtmosphereBoundary(a, r, mu);
}
// functions.glsl:473-480
ORACLE_HD Spec GetTransmittanceToTopAtmosphereBoundary(const Atm& a, const Tex2& T, double r,
                                             double mu) {
  double u, v;
  GetTransmittanceTextureUvFromRMu(a, r, mu, &u, &v);
  return texture(T, u, v);
}
// functions.glsl:493-515
ORACLE_HD Spec GetTransmittance(const Atm& a, const Tex2& T, double r, double mu, double d,
                      bool ray_r_mu_intersects_ground) {
  double r_d = ClampRadius(a, om::sqrt(d * d + 2.0 * r * mu * d + r * r));
  double mu_d = ClampCosine((r * mu + d) / r_d);
  if (ray_r_mu_intersects_ground) {
    return smin(GetTransmittanceToTopAtmosphereBoundary(a, T, r_d, -mu_d) /
                    GetTransmittanceToTopAtmosphereBoundary(a, T, r, -mu),
                Spec(1.0));
  } else {
    return smin(GetTransmittanceToTopAtmosphereBoundary(a, T, r, mu) /
                    GetTransmittanceToTopAtmosphereBoundary(a, T, r_d, mu_d),
                Spec(1.0));
  }
}
// functions.glsl:552-563
ORACLE_HD Spec GetTransmittanceToSun(const Atm& a, const Tex2& T, double r, double mu_s) {
  double sin_theta_h = a.bottom_radius / r;
  double cos_theta_h = -om::sqrt(om::max(1.0 - sin_theta_h * sin_theta_h, 0.0));
  return GetTransmittanceToTopAtmosphereBoundary(a, T, r, mu_s) *
         smoothstep(-sin_theta_h * a.sun_angular_radius, sin_theta_h * a.sun_angular_radius,
                    mu_s - cos_theta_h);
}
// functions.glsl:650-667
ORACLE_HD void ComputeSingleScatteringIntegrand(const Atm& a, const Tex2& T, double r, double mu,
                                      double mu_s, double nu, double d,
                                      bool ray_r_mu_intersects_ground, Spec* rayleigh,
                                      Spec* mie) {
  double r_d = ClampRadius(a, om::sqrt(d * d + 2.0 * r * mu * d + r * r));
  double mu_s_d = ClampCosine((r * mu_s + d * nu) / r_d);
  Spec transmittance = GetTransmittance(a, T, r, mu, d, ray_r_mu_intersects_ground) *
                       GetTransmittanceToSun(a, T, r_d, mu_s_d);
  *rayleigh = transmittance * GetProfileDensity(a.rayleigh_density, r_d - a.bottom_radius);
  *mie = transmittance * GetProfileDensity(a.mie_density, r_d - a.bottom_radius);
}
// functions.glsl:680-687
ORACLE_HD double DistanceToNearestAtmosphereBoundary(const Atm& a, double r, double mu,
                                           bool ray_r_mu_intersects_ground) {
  return ray_r_mu_intersects_ground ? DistanceToBottomAtmosphereBoundary(a, r, mu)
                                    : DistanceToTopAtmosphereBoundary(a, r, mu);
}
// functions.glsl:695-730 (50 intervals)
ORACLE_HD void ComputeSingleScattering(const Atm& a, const Tex2& T, double r, double mu, double mu_s,
                             double nu, bool ray_r_mu_intersects_ground, Spec* rayleigh,
                             Spec* mie) {
  const int SAMPLE_COUNT = 50;
  double dx = DistanceToNearestAtmosphereBoundary(a, r, mu, ray_r_mu_intersects_ground) /
              double(SAMPLE_COUNT);
  Spec rayleigh_sum, mie_sum;
  for (int i = 0; i <= SAMPLE_COUNT; ++i) {
    double d_i = double(i) * dx;
    Spec rayleigh_i, mie_i;
    ComputeSingleScatteringIntegrand(a, T, r, mu, mu_s, nu, d_i, ray_r_mu_intersects_ground,
                                     &rayleigh_i, &mie_i);
    double weight_i = (i == 0 || i == SAMPLE_COUNT) ? 0.5 : 1.0;
    rayleigh_sum += rayleigh_i * weight_i;
    mie_sum += mie_i * weight_i;
  }
  *rayleigh = rayleigh_sum * dx * a.solar_irradiance * a.rayleigh_scattering;
  *mie = mie_sum * dx * a.solar_irradiance * a.mie_scattering;
}
// functions.glsl:739-747
ORACLE_HD double RayleighPhaseFunction(double nu) {
  double k = 3.0 / (16.0 * kPi);
  return k * (1.0 + nu * nu);
}
ORACLE_HD double MiePhaseFunction(double g, double nu) {
  double k = 3.0 / (8.0 * kPi) * (1.0 - g * g) / (2.0 + g * g);
  return k * (1.0 + nu * nu) / om::pow(1.0 + g * g - 2.0 * g * nu, 1.5);
}
// functions.glsl:773-831
ORACLE_HD void GetScatteringTextureUvwzFromRMuMuSNu(const Atm& a, double r, double mu, double mu_s,
                                          double nu, bool ray_r_mu_intersects_ground,
                                          double uvwz[4]) {
  double H = om::sqrt(a.top_radius * a.top_radius - a.bottom_radius * a.bottom_radius);
  double rho = SafeSqrt(r * r - a.bottom_radius * a.bottom_radius);
  double u_r = GetTextureCoordFromUnitRange(rho / H, a.S_R);
  double r_mu = r * mu;
  double discriminant = r_mu * r_mu - r * r + a.bottom_radius * a.bottom_radius;
  double u_mu;
  if (ray_r_mu_intersects_ground) {
    double d = -r_mu - SafeSqrt(discriminant);
    double d_min = r - a.bottom_radius;
    double d_max = rho;
    u_mu = 0.5 - 0.5 * GetTextureCoordFromUnitRange(
                           d_max == d_min ? 0.0 : (d - d_min) / (d_max - d_min), a.S_MU / 2);
  } else {
    double d = -r_mu + SafeSqrt(discriminant + H * H);
    double d_min = a.top_radius - r;
    double d_max = rho + H;
    u_mu = 0.5 + 0.5 * GetTextureCoordFromUnitRange((d - d_min) / (d_max - d_min), a.S_MU / 2);
  }
  double d = DistanceToTopAtmosphereBoundary(a, a.bottom_radius, mu_s);
  double d_min = a.top_radius - a.bottom_radius;
  double d_max = H;
  double aa = (d - d_min) / (d_max - d_min);
  double D = DistanceToTopAtmosphereBoundary(a, a.bottom_radius, a.mu_s_min);
  double A = (D - d_min) / (d_max - d_min);
  double u_mu_s =
      GetTextureCoordFromUnitRange(om::max(1.0 - aa / A, 0.0) / (1.0 + aa), a.S_MU_S);
  double u_nu = (nu + 1.0) / 2.0;
  uvwz[0] = u_nu;
  uvwz[1] = u_mu_s;
  uvwz[2] = u_mu;
  uvwz[3] = u_r;
}
// functions.glsl:837-890
ORACLE_HD void GetRMuMuSNuFromScatteringTextureUvwz(const Atm& a, const double uvwz[4], double* r,
                                          double* mu, double* mu_s, double* nu,
                                          bool* ray_r_mu_intersects_ground) {
  double H = om::sqrt(a.top_radius * a.top_radius - a.bottom_radius * a.bottom_radius);
  double rho = H * GetUnitRangeFromTextureCoord(uvwz[3], a.S_R);
  *r = om::sqrt(rho * rho + a.bottom_radius * a.bottom_radius);
  if (uvwz[2] < 0.5) {
    double d_min = *r - a.bottom_radius;
    double d_max = rho;
    double d = d_min + (d_max - d_min) *
                           GetUnitRangeFromTextureCoord(1.0 - 2.0 * uvwz[2], a.S_MU / 2);
    *mu = d == 0.0 ? -1.0 : ClampCosine(-(rho * rho + d * d) / (2.0 * *r * d));
    *ray_r_mu_intersects_ground = true;
  } else {
    double d_min = a.top_radius - *r;
    double d_max = rho + H;
    double d = d_min + (d_max - d_min) *
                           GetUnitRangeFromTextureCoord(2.0 * uvwz[2] - 1.0, a.S_MU / 2);
    *mu = d == 0.0 ? 1.0 : ClampCosine((H * H - rho * rho - d * d) / (2.0 * *r * d));
    *ray_r_mu_intersects_ground = false;
  }
  double x_mu_s = GetUnitRangeFromTextureCoord(uvwz[1], a.S_MU_S);
  double d_min = a.top_radius - a.bottom_radius;
  double d_max = H;
  double D = DistanceToTopAtmosphereBoundary(a, a.bottom_radius, a.mu_s_min);
  double A = (D - d_min) / (d_max - d_min);
  double aa = (A - x_mu_s * A) / (1.0 + x_mu_s * A);
  double d = d_min + om::min(aa, A) * (d_max - d_min);
  *mu_s = d == 0.0 ? 1.0 : ClampCosine((H * H - d * d) / (2.0 * a.bottom_radius * d));
  *nu = ClampCosine(uvwz[0] * 2.0 - 1.0);
}
// functions.glsl:905-926
ORACLE_HD void GetRMuMuSNuFromScatteringTextureFragCoord(const Atm& a, double fx, double fy,
                                               double fz, double* r, double* mu,
                                               double* mu_s, double* nu,
                                               bool* ray_r_mu_intersects_ground) {
  double frag_coord_nu = om::floor(fx / double(a.S_MU_S));
  double frag_coord_mu_s = om::fmod(fx, double(a.S_MU_S));
  double uvwz[4] = {frag_coord_nu / double(a.S_NU - 1), frag_coord_mu_s / double(a.S_MU_S),
                    fy / double(a.S_MU), fz / double(a.S_R)};
  GetRMuMuSNuFromScatteringTextureUvwz(a, uvwz, r, mu, mu_s, nu, ray_r_mu_intersects_ground);
  *nu = clampd(*nu, *mu * *mu_s - om::sqrt((1.0 - *mu * *mu) * (1.0 - *mu_s * *mu_s)),
               *mu * *mu_s + om::sqrt((1.0 - *mu * *mu) * (1.0 - *mu_s * *mu_s)));
}
// functions.glsl:958-976: two trilinear lookups lerped in nu.
ORACLE_HD void ScatteringLookupCoords(const Atm& a, double r, double mu, double mu_s, double nu,
                            bool ground, double uvw0[3], double uvw1[3], double* lerp) {
  double uvwz[4];
  GetScatteringTextureUvwzFromRMuMuSNu(a, r, mu, mu_s, nu, ground, uvwz);
  double tex_coord_x = uvwz[0] * double(a.S_NU - 1);
  double tex_x = om::floor(tex_coord_x);
  *lerp = tex_coord_x - tex_x;
  uvw0[0] = (tex_x + uvwz[1]) / double(a.S_NU);
  uvw0[1] = uvwz[2];
  uvw0[2] = uvwz[3];
  uvw1[0] = (tex_x + 1.0 + uvwz[1]) / double(a.S_NU);
  uvw1[1] = uvwz[2];
  uvw1[2] = uvwz[3];
}
ORACLE_HD Spec GetScattering(const Atm& a, const Tex3& S, double r, double mu, double mu_s, double nu,
                   bool ground) {
  double uvw0[3], uvw1[3], lerp;
  ScatteringLookupCoords(a, r, mu, mu_s, nu, ground, uvw0, uvw1, &lerp);
  return texture(S, uvw0[0], uvw0[1], uvw0[2]) * (1.0 - lerp) +
         texture(S, uvw1[0], uvw1[1], uvw1[2]) * lerp;
}
// functions.glsl:987-1009
ORACLE_HD Spec GetScattering(const Atm& a, const Tex3& SR, const Tex3& SM, const Tex3& SMulti, double r,
                   double mu, double mu_s, double nu, bool ground, int scattering_order) {
  if (scattering_order == 1) {
    Spec rayleigh = GetScattering(a, SR, r, mu, mu_s, nu, ground);
    Spec mie = GetScattering(a, SM, r, mu, mu_s, nu, ground);
    return rayleigh * RayleighPhaseFunction(nu) +
           mie * MiePhaseFunction(a.mie_phase_function_g, nu);
  }
  return GetScattering(a, SMulti, r, mu, mu_s, nu, ground);
}
// functions.glsl:1524-1533
ORACLE_HD void GetIrradianceTextureUvFromRMuS(const Atm& a, double r, double mu_s, double* u,
                                    double* v) {
  double x_r = (r - a.bottom_radius) / (a.top_radius - a.bottom_radius);
  double x_mu_s = mu_s * 0.5 + 0.5;
  *u = GetTextureCoordFromUnitRange(x_mu_s, a.I_W);
  *v = GetTextureCoordFromUnitRange(x_r, a.I_H);
}
// functions.glsl:1539-1548
ORACLE_HD void GetRMuSFromIrradianceTextureUv(const Atm& a, double u, double v, double* r,
                                    double* mu_s) {
  double x_mu_s = GetUnitRangeFromTextureCoord(u, a.I_W);
  double x_r = GetUnitRangeFromTextureCoord(v, a.I_H);
  *r = a.bottom_radius + x_r * (a.top_radius - a.bottom_radius);
  *mu_s = ClampCosine(2.0 * x_mu_s - 1.0);
}
// functions.glsl:1595-1601
ORACLE_HD Spec GetIrradiance(const Atm& a, const Tex2& I, double r, double mu_s) {
  double u, v;
  GetIrradianceTextureUvFromRMuS(a, r, mu_s, &u, &v);
  return texture(I, u, v);
}
// functions.glsl:1163-1260 (16 x 32 midpoint quadrature over the sphere)
ORACLE_HD Spec ComputeScatteringDensity(const Atm& a, const Tex2& T, const Tex3& SR, const Tex3& SM,
                              const Tex3& SMulti, const Tex2& I, double r, double mu,
                              double mu_s, double nu, int scattering_order) {
  V3 zenith_direction{0.0, 0.0, 1.0};
  V3 omega{om::sqrt(1.0 - mu * mu), 0.0, mu};
  double sun_dir_x = omega.x == 0.0 ? 0.0 : (nu - mu * mu_s) / omega.x;
  double sun_dir_y = om::sqrt(om::max(1.0 - sun_dir_x * sun_dir_x - mu_s * mu_s, 0.0));
  V3 omega_s{sun_dir_x, sun_dir_y, mu_s};
  const int SAMPLE_COUNT = 16;
  const double dphi = kPi / double(SAMPLE_COUNT);
  const double dtheta = kPi / double(SAMPLE_COUNT);
  Spec rayleigh_mie;
  for (int l = 0; l < SAMPLE_COUNT; ++l) {
    double theta = (double(l) + 0.5) * dtheta;
    double cos_theta = om::cos(theta);
    double sin_theta = om::sin(theta);
    bool ray_r_theta_intersects_ground = RayIntersectsGround(a, r, cos_theta);
    double distance_to_ground = 0.0;
    Spec transmittance_to_ground(0.0);
    Spec ground_albedo(0.0);
    if (ray_r_theta_intersects_ground) {
      distance_to_ground = DistanceToBottomAtmosphereBoundary(a, r, cos_theta);
      transmittance_to_ground = GetTransmittance(a, T, r, cos_theta, distance_to_ground, true);
      ground_albedo = a.ground_albedo;
    }
    for (int m = 0; m < 2 * SAMPLE_COUNT; ++m) {
      double phi = (double(m) + 0.5) * dphi;
      V3 omega_i{om::cos(phi) * sin_theta, om::sin(phi) * sin_theta, cos_theta};
      double domega_i = dtheta * dphi * om::sin(theta);
      double nu1 = dot(omega_s, omega_i);
      Spec incident_radiance = GetScattering(a, SR, SM, SMulti, r, omega_i.z, mu_s, nu1,
                                             ray_r_theta_intersects_ground,
                                             scattering_order - 1);
      V3 ground_normal = normalize(zenith_direction * r + omega_i * distance_to_ground);
      Spec ground_irradiance =
          GetIrradiance(a, I, a.bottom_radius, dot(ground_normal, omega_s));
      incident_radiance += transmittance_to_ground * ground_albedo * (1.0 / kPi) *
                           ground_irradiance;
      double nu2 = dot(omega, omega_i);
      double rayleigh_density =
          GetProfileDensity(a.rayleigh_density, r - a.bottom_radius);
      double mie_density = GetProfileDensity(a.mie_density, r - a.bottom_radius);
      rayleigh_mie += incident_radiance *
                      (a.rayleigh_scattering * rayleigh_density * RayleighPhaseFunction(nu2) +
                       a.mie_scattering * mie_density *
                           MiePhaseFunction(a.mie_phase_function_g, nu2)) *
                      domega_i;
    }
  }
  return rayleigh_mie;
}
// functions.glsl:1285-1330 (50 intervals)
ORACLE_HD Spec ComputeMultipleScattering(const Atm& a, const Tex2& T, const Tex3& J, double r,
                               double mu, double mu_s, double nu,
                               bool ray_r_mu_intersects_ground) {
  const int SAMPLE_COUNT = 50;
  double dx = DistanceToNearestAtmosphereBoundary(a, r, mu, ray_r_mu_intersects_ground) /
              double(SAMPLE_COUNT);
  Spec rayleigh_mie_sum;
  for (int i = 0; i <= SAMPLE_COUNT; ++i) {
    double d_i = double(i) * dx;
    double r_i = ClampRadius(a, om::sqrt(d_i * d_i + 2.0 * r * mu * d_i + r * r));
    double mu_i = ClampCosine((r * mu + d_i) / r_i);
    double mu_s_i = ClampCosine((r * mu_s + d_i * nu) / r_i);
    Spec rayleigh_mie_i =
        GetScattering(a, J, r_i, mu_i, mu_s_i, nu, ray_r_mu_intersects_ground) *
        GetTransmittance(a, T, r, mu, d_i, ray_r_mu_intersects_ground) * dx;
    double weight_i = (i == 0 || i == SAMPLE_COUNT) ? 0.5 : 1.0;
    rayleigh_mie_sum += rayleigh_mie_i * weight_i;
  }
  return rayleigh_mie_sum;
}
// functions.glsl:1443-1461
ORACLE_HD Spec ComputeDirectIrradiance(const Atm& a, const Tex2& T, double r, double mu_s) {
  double alpha_s = a.sun_angular_radius;
  double average_cosine_factor =
      mu_s < -alpha_s ? 0.0
                      : (mu_s > alpha_s ? mu_s
                                        : (mu_s + alpha_s) * (mu_s + alpha_s) / (4.0 * alpha_s));
  return a.solar_irradiance * GetTransmittanceToTopAtmosphereBoundary(a, T, r, mu_s) *
         average_cosine_factor;
}
// functions.glsl:1477-1511 (16 x 64 midpoint quadrature over the hemisphere)
ORACLE_HD Spec ComputeIndirectIrradiance(const Atm& a, const Tex3& SR, const Tex3& SM,
                               const Tex3& SMulti, double r, double mu_s,
                               int scattering_order) {
  const int SAMPLE_COUNT = 32;
  const double dphi = kPi / double(SAMPLE_COUNT);
  const double dtheta = kPi / double(SAMPLE_COUNT);
  Spec result;
  V3 omega_s{om::sqrt(1.0 - mu_s * mu_s), 0.0, mu_s};
  for (int j = 0; j < SAMPLE_COUNT / 2; ++j) {
    double theta = (double(j) + 0.5) * dtheta;
    for (int i = 0; i < 2 * SAMPLE_COUNT; ++i) {
      double phi = (double(i) + 0.5) * dphi;
      V3 omega{om::cos(phi) * om::sin(theta), om::sin(phi) * om::sin(theta),
               om::cos(theta)};
      double domega = dtheta * dphi * om::sin(theta);
      double nu = dot(omega, omega_s);
      result += GetScattering(a, SR, SM, SMulti, r, omega.z, mu_s, nu, false,
                              scattering_order) *
                omega.z * domega;
    }
  }
  return result;
}

// ---------------------------------------------------------------------------
// Rendering functions (functions.glsl:1633-1896).
// ---------------------------------------------------------------------------
// functions.glsl:1633-1645
ORACLE_HD Spec GetExtrapolatedSingleMieScattering(const Atm& a, const Spec& rgb, double alpha) {
  if (rgb[0] <= 0.0) return Spec(0.0);
  return rgb * alpha / rgb[0] * (a.rayleigh_scattering[0] / a.mie_scattering[0]) *
         (a.mie_scattering / a.rayleigh_scattering);
}
// functions.glsl:1658-1689; S/M are RGBA, combined selects alpha = Mie.r.
ORACLE_HD Spec GetCombinedScattering(const Atm& a, const Tex3& S, const double* Sraw, const Tex3& M,
                           bool combined, double r, double mu, double mu_s, double nu,
                           bool ground, Spec* single_mie) {
  double uvw0[3], uvw1[3], lerp;
  ScatteringLookupCoords(a, r, mu, mu_s, nu, ground, uvw0, uvw1, &lerp);
  Spec scattering = texture(S, uvw0[0], uvw0[1], uvw0[2]) * (1.0 - lerp) +
                    texture(S, uvw1[0], uvw1[1], uvw1[2]) * lerp;
  if (combined) {
    // Alpha channel: same trilinear weights on component 3.
    Tex3 alpha_view = S;
    (void)Sraw;
    auto alpha_lookup = [&](const double uvw[3]) {
      int idx[8];
      double w[8];
      texture_taps(alpha_view, uvw[0], uvw[1], uvw[2], idx, w);
      double s = 0.0;
      for (int t = 0; t < 8; ++t) s += w[t] * alpha_view.p[4LL * idx[t] + 3];
      return s;
    };
    double alpha = alpha_lookup(uvw0) * (1.0 - lerp) + alpha_lookup(uvw1) * lerp;
    *single_mie = GetExtrapolatedSingleMieScattering(a, scattering, alpha);
  } else {
    *single_mie = texture(M, uvw0[0], uvw0[1], uvw0[2]) * (1.0 - lerp) +
                  texture(M, uvw1[0], uvw1[1], uvw1[2]) * lerp;
  }
  return scattering;
}
// functions.glsl:1705-1769
ORACLE_HD Spec GetSkyRadiance(const Atm& a, const Tex2& T, const Tex3& S, const Tex3& M, bool combined,
                    V3 camera, const V3& view_ray, double shadow_length,
                    const V3& sun_direction, Spec* transmittance) {
  double r = length(camera);
  double rmu = dot(camera, view_ray);
  double distance_to_top_atmosphere_boundary =
      -rmu - om::sqrt(rmu * rmu - r * r + a.top_radius * a.top_radius);
  if (distance_to_top_atmosphere_boundary > 0.0) {
    camera = camera + view_ray * distance_to_top_atmosphere_boundary;
    r = a.top_radius;
    rmu += distance_to_top_atmosphere_boundary;
  } else if (r > a.top_radius) {
    *transmittance = Spec(1.0);
    return Spec(0.0);
  }
  double mu = rmu / r;
  double mu_s = dot(camera, sun_direction) / r;
  double nu = dot(view_ray, sun_direction);
  bool ray_r_mu_intersects_ground = RayIntersectsGround(a, r, mu);
  *transmittance = ray_r_mu_intersects_ground
                       ? Spec(0.0)
                       : GetTransmittanceToTopAtmosphereBoundary(a, T, r, mu);
  Spec single_mie_scattering, scattering;
  if (shadow_length == 0.0) {
    scattering = GetCombinedScattering(a, S, S.p, M, combined, r, mu, mu_s, nu,
                                       ray_r_mu_intersects_ground, &single_mie_scattering);
  } else {
    double d = shadow_length;
    double r_p = ClampRadius(a, om::sqrt(d * d + 2.0 * r * mu * d + r * r));
    double mu_p = (r * mu + d) / r_p;
    double mu_s_p = (r * mu_s + d * nu) / r_p;
    scattering = GetCombinedScattering(a, S, S.p, M, combined, r_p, mu_p, mu_s_p, nu,
                                       ray_r_mu_intersects_ground, &single_mie_scattering);
    Spec shadow_transmittance =
        GetTransmittance(a, T, r, mu, shadow_length, ray_r_mu_intersects_ground);
    scattering = scattering * shadow_transmittance;
    single_mie_scattering = single_mie_scattering * shadow_transmittance;
  }
  return scattering * RayleighPhaseFunction(nu) +
         single_mie_scattering * MiePhaseFunction(a.mie_phase_function_g, nu);
}
// functions.glsl:1787-1863
ORACLE_HD Spec GetSkyRadianceToPoint(const Atm& a, const Tex2& T, const Tex3& S, const Tex3& M,
                           bool combined, V3 camera, const V3& point, double shadow_length,
                           const V3& sun_direction, Spec* transmittance) {
  V3 view_ray = normalize(point - camera);
  double r = length(camera);
  double rmu = dot(camera, view_ray);
  double distance_to_top_atmosphere_boundary =
      -rmu - om::sqrt(rmu * rmu - r * r + a.top_radius * a.top_radius);
  if (distance_to_top_atmosphere_boundary > 0.0) {
    camera = camera + view_ray * distance_to_top_atmosphere_boundary;
    r = a.top_radius;
    rmu += distance_to_top_atmosphere_boundary;
  }
  double mu = rmu / r;
  double mu_s = dot(camera, sun_direction) / r;
  double nu = dot(view_ray, sun_direction);
  double d = length(point - camera);
  bool ray_r_mu_intersects_ground = RayIntersectsGround(a, r, mu);
  *transmittance = GetTransmittance(a, T, r, mu, d, ray_r_mu_intersects_ground);
  Spec single_mie_scattering;
  Spec scattering = GetCombinedScattering(a, S, S.p, M, combined, r, mu, mu_s, nu,
                                          ray_r_mu_intersects_ground, &single_mie_scattering);
  d = om::max(d - shadow_length, 0.0);
  double r_p = ClampRadius(a, om::sqrt(d * d + 2.0 * r * mu * d + r * r));
  double mu_p = (r * mu + d) / r_p;
  double mu_s_p = (r * mu_s + d * nu) / r_p;
  Spec single_mie_scattering_p;
  Spec scattering_p = GetCombinedScattering(a, S, S.p, M, combined, r_p, mu_p, mu_s_p, nu,
                                            ray_r_mu_intersects_ground,
                                            &single_mie_scattering_p);
  Spec shadow_transmittance = *transmittance;
  if (shadow_length > 0.0) {
    shadow_transmittance = GetTransmittance(a, T, r, mu, d, ray_r_mu_intersects_ground);
  }
  scattering = scattering - shadow_transmittance * scattering_p;
  if (combined) {
    // In the combined layout only the red component of single Mie survives the
    // subtraction; it is extrapolated again (functions.glsl:1852-1855).
    double mie_r = single_mie_scattering[0] -
                   shadow_transmittance[0] * single_mie_scattering_p[0];
    single_mie_scattering = GetExtrapolatedSingleMieScattering(a, scattering, mie_r);
  } else {
    single_mie_scattering =
        single_mie_scattering - shadow_transmittance * single_mie_scattering_p;
  }
  single_mie_scattering = single_mie_scattering * smoothstep(0.0, 0.01, mu_s);
  return scattering * RayleighPhaseFunction(nu) +
         single_mie_scattering * MiePhaseFunction(a.mie_phase_function_g, nu);
}
// functions.glsl:1878-1896
ORACLE_HD Spec GetSunAndSkyIrradiance(const Atm& a, const Tex2& T, const Tex2& I, const V3& point,
                            const V3& normal, const V3& sun_direction, Spec* sky_irradiance) {
  double r = length(point);
  double mu_s = dot(point, sun_direction) / r;
  *sky_irradiance = GetIrradiance(a, I, r, mu_s) * ((1.0 + dot(normal, point) / r) * 0.5);
  return a.solar_irradiance * GetTransmittanceToSun(a, T, r, mu_s) *
         om::max(dot(normal, sun_direction), 0.0);
}

// ---------------------------------------------------------------------------
// Threading: work stealing over blocks of `chunk` consecutive texels.  The
// default, 64, is finer than the reference's RunJobs jobs; a texture row
// (transmittance, irradiance) or an r-slice (scattering) per block is the
// reference's own partition (atmosphere/reference/model.cc:140-237).
// ---------------------------------------------------------------------------
template <typename F>
void ParallelFor(long long n, int threads, F&& fn, long long chunk = 64) {
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  if (chunk < 1) chunk = 1;
  std::atomic<long long> next(0);
  auto worker = [&]() {
    for (;;) {
      long long b = next.fetch_add(chunk);
      if (b >= n) break;
      long long e = std::min(n, b + chunk);
      for (long long i = b; i < e; ++i) fn(i);
    }
  };
  if (threads == 1 || n < chunk) {
    worker();
    return;
  }
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
  for (auto& th : pool) th.join();
}

ORACLE_HD inline void Store(double* p, const Spec& s, double alpha) {
  p[0] = s[0];
  p[1] = s[1];
  p[2] = s[2];
  p[3] = alpha;
}
ORACLE_HD inline Spec MatVec(const double m[9], const Spec& v) {
  return Spec(m[0] * v[0] + m[1] * v[1] + m[2] * v[2], m[3] * v[0] + m[4] * v[1] + m[5] * v[2],
              m[6] * v[0] + m[7] * v[1] + m[8] * v[2]);
}

ORACLE_HD void ScatteringTexelCoord(const Atm& a, long long idx, double* fx, double* fy, double* fz) {
  int W = a.S_NU * a.S_MU_S;
  *fx = double(idx % W) + 0.5;
  *fy = double((idx / W) % a.S_MU) + 0.5;
  *fz = double(idx / ((long long)W * a.S_MU)) + 0.5;
}

struct Buffers {
  std::vector<double> delta_irradiance, delta_rayleigh, delta_mie, delta_density,
      delta_multiple;
};

// Evaluates one texel of a pass (the *Texture functions of functions.glsl).
ORACLE_HD void EvalTexel(int kind, const Atm& a, const Tex2& T, const Tex3& SR, const Tex3& SM,
               const Tex3& SMulti, const Tex2& I, const Tex3& J, int order, long long idx,
               double* out, double* out2) {
  ORACLE_COUNT_PASS(kind);
  switch (kind) {
    case 0: {  // functions.glsl:454-463
      double fx = double(idx % a.T_W) + 0.5, fy = double(idx / a.T_W) + 0.5;
      Store(out, ComputeTransmittanceToTopAtmosphereBoundaryTexture(a, fx, fy), 1.0);
      break;
    }
    case 1: {  // functions.glsl:1558-1567
      double fx = double(idx % a.I_W) + 0.5, fy = double(idx / a.I_W) + 0.5;
      double r, mu_s;
      GetRMuSFromIrradianceTextureUv(a, fx / a.I_W, fy / a.I_H, &r, &mu_s);
      Store(out, ComputeDirectIrradiance(a, T, r, mu_s), 1.0);
      break;
    }
    case 2: {  // functions.glsl:933-945
      double fx, fy, fz, r, mu, mu_s, nu;
      bool g;
      ScatteringTexelCoord(a, idx, &fx, &fy, &fz);
      GetRMuMuSNuFromScatteringTextureFragCoord(a, fx, fy, fz, &r, &mu, &mu_s, &nu, &g);
      Spec ray, mie;
      ComputeSingleScattering(a, T, r, mu, mu_s, nu, g, &ray, &mie);
      Store(out, ray, 1.0);
      Store(out2, mie, 1.0);
      break;
    }
    case 3: {  // functions.glsl:1348-1367
      double fx, fy, fz, r, mu, mu_s, nu;
      bool g;
      ScatteringTexelCoord(a, idx, &fx, &fy, &fz);
      GetRMuMuSNuFromScatteringTextureFragCoord(a, fx, fy, fz, &r, &mu, &mu_s, &nu, &g);
      Store(out, ComputeScatteringDensity(a, T, SR, SM, SMulti, I, r, mu, mu_s, nu, order),
            1.0);
      break;
    }
    case 4: {  // functions.glsl:1573-1586
      double fx = double(idx % a.I_W) + 0.5, fy = double(idx / a.I_W) + 0.5;
      double r, mu_s;
      GetRMuSFromIrradianceTextureUv(a, fx / a.I_W, fy / a.I_H, &r, &mu_s);
      Store(out, ComputeIndirectIrradiance(a, SR, SM, SMulti, r, mu_s, order), 1.0);
      break;
    }
    case 5: {  // functions.glsl:1369-1383
      double fx, fy, fz, r, mu, mu_s, nu;
      bool g;
      ScatteringTexelCoord(a, idx, &fx, &fy, &fz);
      GetRMuMuSNuFromScatteringTextureFragCoord(a, fx, fy, fz, &r, &mu, &mu_s, &nu, &g);
      Store(out, ComputeMultipleScattering(a, T, J, r, mu, mu_s, nu, g), 1.0);
      if (out2) out2[0] = nu;
      break;
    }
  }
}

// atmosphere/model.cc:1048-1215 (pass order, blending) with the per-texel
// evaluation of atmosphere/reference/model.cc:133-237.
int Precompute(const Atm& a, unsigned num_scattering_orders, const double lum[9], bool blend,
               bool combined, int threads, double* transmittance, double* scattering,
               double* single_mie, double* irradiance, int density_stride,
               double seconds[6], bool by_rows = false) {
  using Clock = std::chrono::steady_clock;
  auto tick = Clock::now();
  auto lap = [&](int slot) {
    auto now = Clock::now();
    if (seconds)
      seconds[slot] +=
          1e-9 * (double)std::chrono::duration_cast<std::chrono::nanoseconds>(now - tick).count();
    tick = now;
  };
  const long long nT = (long long)a.T_W * a.T_H;
  const long long nI = (long long)a.I_W * a.I_H;
  const long long nS = (long long)a.S_NU * a.S_MU_S * a.S_MU * a.S_R;
  std::vector<double> dI(4 * nI), dR(4 * nS), dM(4 * nS), dJ(4 * nS), dMulti(4 * nS);
  Tex2 T = MakeT(a, transmittance);
  Tex2 DI = MakeI(a, dI.data());
  Tex3 DR = MakeS(a, dR.data()), DM = MakeS(a, dM.data()), DJ = MakeS(a, dJ.data()),
       DMulti = MakeS(a, dMulti.data());
  Tex3 none{1, 1, 1, nullptr};
  // Texels per work block: the reference's rows and r-slices, or 64.
  const long long slice = (long long)a.S_NU * a.S_MU_S * a.S_MU;
  const int stride = density_stride > 1 ? density_stride : 1;
  const long long chunk_T = by_rows ? a.T_W : 64, chunk_I = by_rows ? a.I_W : 64;
  const long long chunk_S = by_rows ? slice : 64;
  const long long chunk_sampled = by_rows ? std::max(1LL, slice / stride) : 64;

  // Transmittance (model.cc:1085-1091).
  ParallelFor(nT, threads, [&](long long i) {
    EvalTexel(0, a, T, none, none, none, DI, none, 0, i, transmittance + 4 * i, nullptr);
  }, chunk_T);
  lap(0);
  // Direct irradiance; irradiance is zeroed unless blending (model.cc:1093-1106).
  ParallelFor(nI, threads, [&](long long i) {
    EvalTexel(1, a, T, none, none, none, DI, none, 0, i, dI.data() + 4 * i, nullptr);
    if (!blend) Store(irradiance + 4 * i, Spec(0.0), 0.0);
  }, chunk_I);
  lap(1);
  // Single scattering (model.cc:1108-1134, shader model.cc:142-157).
  ParallelFor(nS, threads, [&](long long i) {
    EvalTexel(2, a, T, none, none, none, DI, none, 0, i, dR.data() + 4 * i, dM.data() + 4 * i);
    Spec ray = Spec::From(dR.data() + 4 * i), mie = Spec::From(dM.data() + 4 * i);
    Spec lray = MatVec(lum, ray), lmie = MatVec(lum, mie);
    double* s = scattering + 4 * i;
    double alpha = combined ? lmie[0] : 0.0;
    if (blend) {
      Store(s, Spec::From(s) + lray, s[3] + alpha);
    } else {
      Store(s, lray, alpha);
    }
    if (single_mie) {
      double* m = single_mie + 4 * i;
      if (blend) {
        Store(m, Spec::From(m) + lmie, 0.0);
      } else {
        Store(m, lmie, 0.0);
      }
    }
  }, chunk_S);
  lap(2);
  for (unsigned order = 2; order <= num_scattering_orders; ++order) {
    // Scattering density (model.cc:1140-1166).  The reference aliases
    // delta_multiple_scattering with delta_rayleigh (model.cc:897); the
    // separate buffer here holds the same values.
    const Tex3& multi_in = order == 2 ? DR : DMulti;
    if (density_stride <= 1) {
      ParallelFor(nS, threads, [&](long long i) {
        EvalTexel(3, a, T, DR, DM, multi_in, DI, none, (int)order, i, dJ.data() + 4 * i,
                  nullptr);
      }, chunk_S);
    } else {
      ParallelFor(nS / density_stride, threads, [&](long long i) {
        long long t = i * density_stride;
        EvalTexel(3, a, T, DR, DM, multi_in, DI, none, (int)order, t, dJ.data() + 4 * t,
                  nullptr);
      }, chunk_sampled);
    }
    lap(3);
    // Indirect irradiance with order - 1 (model.cc:1168-1189).
    std::vector<double> newI(4 * nI);
    ParallelFor(nI, threads, [&](long long i) {
      EvalTexel(4, a, T, DR, DM, multi_in, DI, none, (int)order - 1, i, newI.data() + 4 * i,
                nullptr);
    }, chunk_I);
    dI.swap(newI);
    DI.p = dI.data();
    ORACLE_COUNT_PASS(4);
    for (long long i = 0; i < nI; ++i) {
      Spec add = MatVec(lum, Spec::From(dI.data() + 4 * i));
      double* p = irradiance + 4 * i;
      Store(p, Spec::From(p) + add, p[3]);
    }
    lap(4);
    // Multiple scattering; scattering += lum * delta / RayleighPhase(nu)
    // (model.cc:1191-1210, shader model.cc:192-208).
    auto ms = [&](long long i) {
      double nu;
      EvalTexel(5, a, T, none, none, none, DI, DJ, 0, i, dMulti.data() + 4 * i, &nu);
      Spec add = MatVec(lum, Spec::From(dMulti.data() + 4 * i)) * (1.0 / RayleighPhaseFunction(nu));
      double* s = scattering + 4 * i;
      Store(s, Spec::From(s) + add, s[3]);
    };
    if (density_stride <= 1) {
      ParallelFor(nS, threads, ms, chunk_S);
    } else {
      ParallelFor(nS / density_stride, threads, [&](long long i) { ms(i * density_stride); },
                  chunk_sampled);
    }
    lap(5);
  }
  return 0;
}

constexpr double kLambdaMinCie = 360;
constexpr double kLambdaMaxCie = 830;

// The CIE 1931 2-degree colour matching functions, 5 nm steps from 360 nm
// (atmosphere/constants.h:69-165): columns lambda, x, y, z.
const double kCie[95][4] = {
#include "cie_1931_2deg.inc"
};
const double kXyzToSrgb[9] = {3.2406, -1.5372, -0.4986, -0.9689, 1.8758,
                              0.0415, 0.0557,  -0.2040, 1.0570};
constexpr double kMaxLuminousEfficacy = 683.0;

}  // namespace

// ===========================================================================
// C interface.
// ===========================================================================
extern "C" {

double oracle_distance_to_top(const oracle_atmosphere* a, double r, double mu) {
  return DistanceToTopAtmosphereBoundary(ToAtm(a, nullptr), r, mu);
}
double oracle_distance_to_bottom(const oracle_atmosphere* a, double r, double mu) {
  return DistanceToBottomAtmosphereBoundary(ToAtm(a, nullptr), r, mu);
}
int oracle_ray_intersects_ground(const oracle_atmosphere* a, double r, double mu) {
  return RayIntersectsGround(ToAtm(a, nullptr), r, mu) ? 1 : 0;
}
double oracle_distance_to_nearest(const oracle_atmosphere* a, double r, double mu, int g) {
  return DistanceToNearestAtmosphereBoundary(ToAtm(a, nullptr), r, mu, g != 0);
}
double oracle_profile_density(const oracle_profile* p, double altitude) {
  return GetProfileDensity(ToProfile(*p), altitude);
}
double oracle_optical_length(const oracle_atmosphere* a, const oracle_profile* p, double r,
                             double mu) {
  return ComputeOpticalLengthToTopAtmosphereBoundary(ToAtm(a, nullptr), ToProfile(*p), r, mu);
}
void oracle_transmittance_to_top(const oracle_atmosphere* a, double r, double mu,
                                 double out[3]) {
  Spec s = ComputeTransmittanceToTopAtmosphereBoundary(ToAtm(a, nullptr), r, mu);
  for (int i = 0; i < 3; ++i) out[i] = s[i];
}
double oracle_tex_coord_from_unit_range(double x, int n) {
  return GetTextureCoordFromUnitRange(x, n);
}
double oracle_unit_range_from_tex_coord(double u, int n) {
  return GetUnitRangeFromTextureCoord(u, n);
}
void oracle_transmittance_uv_from_rmu(const oracle_atmosphere* a, const oracle_shape* s,
                                      double r, double mu, double uv[2]) {
  GetTransmittanceTextureUvFromRMu(ToAtm(a, s), r, mu, &uv[0], &uv[1]);
}
void oracle_rmu_from_transmittance_uv(const oracle_atmosphere* a, const oracle_shape* s,
                                      double u, double v, double* r, double* mu) {
  GetRMuFromTransmittanceTextureUv(ToAtm(a, s), u, v, r, mu);
}
static void Out3(const Spec& s, double* o) {
  o[0] = s[0];
  o[1] = s[1];
  o[2] = s[2];
}
void oracle_lookup_transmittance_to_top(const oracle_atmosphere* a, const oracle_shape* s,
                                        const double* T, double r, double mu, double out[3]) {
  Atm at = ToAtm(a, s);
  Out3(GetTransmittanceToTopAtmosphereBoundary(at, MakeT(at, T), r, mu), out);
}
void oracle_lookup_transmittance(const oracle_atmosphere* a, const oracle_shape* s,
                                 const double* T, double r, double mu, double d, int g,
                                 double out[3]) {
  Atm at = ToAtm(a, s);
  Out3(GetTransmittance(at, MakeT(at, T), r, mu, d, g != 0), out);
}
void oracle_lookup_transmittance_to_sun(const oracle_atmosphere* a, const oracle_shape* s,
                                        const double* T, double r, double mu_s,
                                        double out[3]) {
  Atm at = ToAtm(a, s);
  Out3(GetTransmittanceToSun(at, MakeT(at, T), r, mu_s), out);
}
void oracle_single_scattering_integrand(const oracle_atmosphere* a, const oracle_shape* s,
                                        const double* T, double r, double mu, double mu_s,
                                        double nu, double d, int g, double rayleigh[3],
                                        double mie[3]) {
  Atm at = ToAtm(a, s);
  Spec ray, m;
  ComputeSingleScatteringIntegrand(at, MakeT(at, T), r, mu, mu_s, nu, d, g != 0, &ray, &m);
  Out3(ray, rayleigh);
  Out3(m, mie);
}
void oracle_single_scattering(const oracle_atmosphere* a, const oracle_shape* s,
                              const double* T, double r, double mu, double mu_s, double nu,
                              int g, double rayleigh[3], double mie[3]) {
  Atm at = ToAtm(a, s);
  Spec ray, m;
  ComputeSingleScattering(at, MakeT(at, T), r, mu, mu_s, nu, g != 0, &ray, &m);
  Out3(ray, rayleigh);
  Out3(m, mie);
}
double oracle_rayleigh_phase(double nu) { return RayleighPhaseFunction(nu); }
double oracle_mie_phase(double g, double nu) { return MiePhaseFunction(g, nu); }
void oracle_scattering_uvwz(const oracle_atmosphere* a, const oracle_shape* s, double r,
                            double mu, double mu_s, double nu, int g, double uvwz[4]) {
  GetScatteringTextureUvwzFromRMuMuSNu(ToAtm(a, s), r, mu, mu_s, nu, g != 0, uvwz);
}
void oracle_rmumusnu_from_uvwz(const oracle_atmosphere* a, const oracle_shape* s,
                               const double uvwz[4], double out[4], int* g) {
  bool gg;
  GetRMuMuSNuFromScatteringTextureUvwz(ToAtm(a, s), uvwz, &out[0], &out[1], &out[2], &out[3],
                                       &gg);
  *g = gg ? 1 : 0;
}
void oracle_rmumusnu_from_frag_coord(const oracle_atmosphere* a, const oracle_shape* s,
                                     const double frag[3], double out[4], int* g) {
  bool gg;
  GetRMuMuSNuFromScatteringTextureFragCoord(ToAtm(a, s), frag[0], frag[1], frag[2], &out[0],
                                            &out[1], &out[2], &out[3], &gg);
  *g = gg ? 1 : 0;
}
void oracle_lookup_scattering(const oracle_atmosphere* a, const oracle_shape* s,
                              const double* S, double r, double mu, double mu_s, double nu,
                              int g, double out[3]) {
  Atm at = ToAtm(a, s);
  Out3(GetScattering(at, MakeS(at, S), r, mu, mu_s, nu, g != 0), out);
}
void oracle_scattering_taps(const oracle_atmosphere* a, const oracle_shape* s, double r,
                            double mu, double mu_s, double nu, int g, int idx[16],
                            double w[16]) {
  Atm at = ToAtm(a, s);
  double uvw0[3], uvw1[3], lerp;
  ScatteringLookupCoords(at, r, mu, mu_s, nu, g != 0, uvw0, uvw1, &lerp);
  Tex3 shape_only = MakeS(at, nullptr);
  texture_taps(shape_only, uvw0[0], uvw0[1], uvw0[2], idx, w);
  texture_taps(shape_only, uvw1[0], uvw1[1], uvw1[2], idx + 8, w + 8);
  for (int i = 0; i < 8; ++i) {
    w[i] *= 1.0 - lerp;
    w[8 + i] *= lerp;
  }
}
void oracle_scattering_density(const oracle_atmosphere* a, const oracle_shape* s,
                               const double* T, const double* SR, const double* SM,
                               const double* SMulti, const double* I, double r, double mu,
                               double mu_s, double nu, int order, double out[3]) {
  Atm at = ToAtm(a, s);
  Out3(ComputeScatteringDensity(at, MakeT(at, T), MakeS(at, SR), MakeS(at, SM),
                                MakeS(at, SMulti), MakeI(at, I), r, mu, mu_s, nu, order),
       out);
}
void oracle_multiple_scattering(const oracle_atmosphere* a, const oracle_shape* s,
                                const double* T, const double* J, double r, double mu,
                                double mu_s, double nu, int g, double out[3]) {
  Atm at = ToAtm(a, s);
  Out3(ComputeMultipleScattering(at, MakeT(at, T), MakeS(at, J), r, mu, mu_s, nu, g != 0),
       out);
}
void oracle_direct_irradiance(const oracle_atmosphere* a, const oracle_shape* s,
                              const double* T, double r, double mu_s, double out[3]) {
  Atm at = ToAtm(a, s);
  Out3(ComputeDirectIrradiance(at, MakeT(at, T), r, mu_s), out);
}
void oracle_indirect_irradiance(const oracle_atmosphere* a, const oracle_shape* s,
                                const double* SR, const double* SM, const double* SMulti,
                                double r, double mu_s, int order, double out[3]) {
  Atm at = ToAtm(a, s);
  Out3(ComputeIndirectIrradiance(at, MakeS(at, SR), MakeS(at, SM), MakeS(at, SMulti), r,
                                 mu_s, order),
       out);
}
void oracle_irradiance_uv_from_rmus(const oracle_atmosphere* a, const oracle_shape* s,
                                    double r, double mu_s, double uv[2]) {
  GetIrradianceTextureUvFromRMuS(ToAtm(a, s), r, mu_s, &uv[0], &uv[1]);
}
void oracle_rmus_from_irradiance_uv(const oracle_atmosphere* a, const oracle_shape* s,
                                    double u, double v, double* r, double* mu_s) {
  GetRMuSFromIrradianceTextureUv(ToAtm(a, s), u, v, r, mu_s);
}
void oracle_lookup_irradiance(const oracle_atmosphere* a, const oracle_shape* s,
                              const double* I, double r, double mu_s, double out[3]) {
  Atm at = ToAtm(a, s);
  Out3(GetIrradiance(at, MakeI(at, I), r, mu_s), out);
}

void oracle_eval_texels(int kind, const oracle_atmosphere* a, const oracle_shape* s,
                        const double* T, const double* SR, const double* SM,
                        const double* SMulti, const double* I, const double* J, int order,
                        int n, const long long* idx, double* out, double* out2,
                        int threads) {
  Atm at = ToAtm(a, s);
  Tex2 t = MakeT(at, T), irr = MakeI(at, I);
  Tex3 sr = MakeS(at, SR), sm = MakeS(at, SM), smu = MakeS(at, SMulti), j = MakeS(at, J);
  ParallelFor(n, threads, [&](long long q) {
    double tmp2[4] = {0, 0, 0, 0};
    double* o2 = out2 ? out2 + 4 * q : tmp2;
    EvalTexel(kind, at, t, sr, sm, smu, irr, j, order, idx[q], out + 4 * q, o2);
  });
}

int oracle_precompute(const oracle_atmosphere* a, const oracle_shape* s,
                      unsigned num_scattering_orders, const double lum[9], int blend,
                      int combined, int threads, double* transmittance, double* scattering,
                      double* single_mie, double* irradiance) {
  if (!a || !s || !transmittance || !scattering || !irradiance) return -1;
  if (!combined && !single_mie) return -1;
  Atm at = ToAtm(a, s);
  return Precompute(at, num_scattering_orders, lum, blend != 0, combined != 0, threads,
                    transmittance, scattering, single_mie, irradiance, 1, nullptr);
}

int oracle_time_precompute_partitioned(const oracle_atmosphere* a, const oracle_shape* s,
                                       unsigned num_scattering_orders, int stride, int threads,
                                       int by_rows, double seconds[6]) {
  Atm at = ToAtm(a, s);
  const long long nT = (long long)at.T_W * at.T_H;
  const long long nI = (long long)at.I_W * at.I_H;
  const long long nS = (long long)at.S_NU * at.S_MU_S * at.S_MU * at.S_R;
  std::vector<double> T(4 * nT), S(4 * nS), M(4 * nS), I(4 * nI);
  const double id[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  for (int i = 0; i < 6; ++i) seconds[i] = 0.0;
  return Precompute(at, num_scattering_orders, id, false, false, threads, T.data(), S.data(),
                    M.data(), I.data(), stride, seconds, by_rows != 0);
}

int oracle_time_precompute_sample(const oracle_atmosphere* a, const oracle_shape* s,
                                  unsigned num_scattering_orders, int stride, int threads,
                                  double seconds[6]) {
  return oracle_time_precompute_partitioned(a, s, num_scattering_orders, stride, threads, 0,
                                            seconds);
}

double oracle_interpolate(const double* wavelengths, const double* values, int n,
                          double wavelength) {
  // atmosphere/model.cc:535-552
  if (wavelength < wavelengths[0]) return values[0];
  for (int i = 0; i < n - 1; ++i) {
    if (wavelength < wavelengths[i + 1]) {
      double u = (wavelength - wavelengths[i]) / (wavelengths[i + 1] - wavelengths[i]);
      return values[i] * (1.0 - u) + values[i + 1] * u;
    }
  }
  return values[n - 1];
}

double oracle_cie_table_value(double wavelength, int column) {
  // atmosphere/model.cc:521-533
  if (wavelength <= kLambdaMinCie || wavelength >= kLambdaMaxCie) return 0.0;
  double u = (wavelength - kLambdaMinCie) / 5.0;
  int row = (int)om::floor(u);
  u -= row;
  return kCie[row][column] * (1.0 - u) + kCie[row + 1][column] * u;
}

void oracle_radiance_to_luminance_factors(const double* wavelengths, const double* solar,
                                          int n, double lambda_power, double k[3]) {
  // atmosphere/model.cc:562-595
  const double lr = 680.0, lg = 550.0, lb = 440.0;
  k[0] = k[1] = k[2] = 0.0;
  double solar_r = oracle_interpolate(wavelengths, solar, n, lr);
  double solar_g = oracle_interpolate(wavelengths, solar, n, lg);
  double solar_b = oracle_interpolate(wavelengths, solar, n, lb);
  const int dlambda = 1;
  for (int lambda = (int)kLambdaMinCie; lambda < (int)kLambdaMaxCie; lambda += dlambda) {
    double x_bar = oracle_cie_table_value(lambda, 1);
    double y_bar = oracle_cie_table_value(lambda, 2);
    double z_bar = oracle_cie_table_value(lambda, 3);
    const double* m = kXyzToSrgb;
    double r_bar = m[0] * x_bar + m[1] * y_bar + m[2] * z_bar;
    double g_bar = m[3] * x_bar + m[4] * y_bar + m[5] * z_bar;
    double b_bar = m[6] * x_bar + m[7] * y_bar + m[8] * z_bar;
    double irradiance = oracle_interpolate(wavelengths, solar, n, lambda);
    k[0] += r_bar * irradiance / solar_r * om::pow(lambda / lr, lambda_power);
    k[1] += g_bar * irradiance / solar_g * om::pow(lambda / lg, lambda_power);
    k[2] += b_bar * irradiance / solar_b * om::pow(lambda / lb, lambda_power);
  }
  for (int i = 0; i < 3; ++i) k[i] *= kMaxLuminousEfficacy * dlambda;
}

void oracle_convert_spectrum_to_linear_srgb(const double* wavelengths, const double* spectrum,
                                            int n, double rgb[3]) {
  // atmosphere/model.cc:1020-1040
  double x = 0.0, y = 0.0, z = 0.0;
  const int dlambda = 1;
  for (int lambda = (int)kLambdaMinCie; lambda < (int)kLambdaMaxCie; lambda += dlambda) {
    double value = oracle_interpolate(wavelengths, spectrum, n, lambda);
    x += oracle_cie_table_value(lambda, 1) * value;
    y += oracle_cie_table_value(lambda, 2) * value;
    z += oracle_cie_table_value(lambda, 3) * value;
  }
  const double* m = kXyzToSrgb;
  rgb[0] = kMaxLuminousEfficacy * (m[0] * x + m[1] * y + m[2] * z) * dlambda;
  rgb[1] = kMaxLuminousEfficacy * (m[3] * x + m[4] * y + m[5] * z) * dlambda;
  rgb[2] = kMaxLuminousEfficacy * (m[6] * x + m[7] * y + m[8] * z) * dlambda;
}

static V3 ToV3(const double* p) { return V3{p[0], p[1], p[2]}; }

void oracle_sky_radiance(const oracle_atmosphere* a, const oracle_shape* s, const double* T,
                         const double* S, const double* M, int combined,
                         const double camera[3], const double view[3], double shadow_length,
                         const double sun[3], double out[3], double transmittance[3]) {
  Atm at = ToAtm(a, s);
  Spec tr;
  Spec r = GetSkyRadiance(at, MakeT(at, T), MakeS(at, S), MakeS(at, M), combined != 0,
                          ToV3(camera), ToV3(view), shadow_length, ToV3(sun), &tr);
  Out3(r, out);
  Out3(tr, transmittance);
}
void oracle_sky_radiance_to_point(const oracle_atmosphere* a, const oracle_shape* s,
                                  const double* T, const double* S, const double* M,
                                  int combined, const double camera[3], const double point[3],
                                  double shadow_length, const double sun[3], double out[3],
                                  double transmittance[3]) {
  Atm at = ToAtm(a, s);
  Spec tr;
  Spec r = GetSkyRadianceToPoint(at, MakeT(at, T), MakeS(at, S), MakeS(at, M), combined != 0,
                                 ToV3(camera), ToV3(point), shadow_length, ToV3(sun), &tr);
  Out3(r, out);
  Out3(tr, transmittance);
}
void oracle_sun_and_sky_irradiance(const oracle_atmosphere* a, const oracle_shape* s,
                                   const double* T, const double* I, const double point[3],
                                   const double normal[3], const double sun[3],
                                   double sun_irr[3], double sky_irr[3]) {
  Atm at = ToAtm(a, s);
  Spec sky;
  Spec sunv = GetSunAndSkyIrradiance(at, MakeT(at, T), MakeI(at, I), ToV3(point),
                                     ToV3(normal), ToV3(sun), &sky);
  Out3(sunv, sun_irr);
  Out3(sky, sky_irr);
}

}  // extern "C"
