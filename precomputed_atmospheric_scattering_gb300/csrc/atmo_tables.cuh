// atmo_tables.cuh -- FP64 set-up tables of one precomputation.
//
// The per-texel parameters (r, mu, mu_s) of the scattering, irradiance and
// density-quadrature rows are computed here in double precision with the
// reference's own formulas and operation order (atmosphere/functions.glsl:
// 207-246, :773-926, :1163-1200, :1539-1548), so that the FP32 kernels start
// every integral from the same (r, mu, mu_s, nu) as the reference's FP64 CPU
// model.  The translation unit is compiled without FMA contraction.
#ifndef ATMO_TABLES_CUH_
#define ATMO_TABLES_CUH_

#include "atmo_instance.h"

namespace atmo {
namespace dbl {

ATMO_HD double clampd(double x, double lo, double hi) { return fmin(fmax(x, lo), hi); }
ATMO_HD double SafeSqrt(double a) { return sqrt(fmax(a, 0.0)); }
ATMO_HD double ClampCosine(double mu) { return clampd(mu, -1.0, 1.0); }
ATMO_HD double DistanceToTop(double Rt, double r, double mu) {
  double disc = r * r * (mu * mu - 1.0) + Rt * Rt;
  return fmax(-r * mu + SafeSqrt(disc), 0.0);
}
ATMO_HD double DistanceToBottom(double Rb, double r, double mu) {
  double disc = r * r * (mu * mu - 1.0) + Rb * Rb;
  return fmax(-r * mu - SafeSqrt(disc), 0.0);
}
ATMO_HD bool RayIntersectsGround(double Rb, double r, double mu) {
  return mu < 0.0 && r * r * (mu * mu - 1.0) + Rb * Rb >= 0.0;
}
ATMO_HD double UnitRangeFromTexCoord(double u, int n) {
  return (u - 0.5 / double(n)) / (1.0 - 1.0 / double(n));
}
ATMO_HD double TexCoordFromUnitRange(double x, int n) {
  return 0.5 / double(n) + x * (1.0 - 1.0 / double(n));
}

// functions.glsl:842-876 for the row (k, j) of the scattering texture.
ATMO_HD TexelRow MakeTexelRow(const Consts& c, const Shape& s, int k, int j) {
  const double Rb = c.dRb, Rt = c.dRt, H = c.dH;
  double w = (double(k) + 0.5) / double(s.sr);
  double z = (double(j) + 0.5) / double(s.smu);
  double rho = H * UnitRangeFromTexCoord(w, s.sr);
  double r = sqrt(rho * rho + Rb * Rb);
  double mu;
  bool ground;
  if (z < 0.5) {
    double d_min = r - Rb, d_max = rho;
    double d = d_min + (d_max - d_min) * UnitRangeFromTexCoord(1.0 - 2.0 * z, s.smu / 2);
    mu = d == 0.0 ? -1.0 : ClampCosine(-(rho * rho + d * d) / (2.0 * r * d));
    ground = true;
  } else {
    double d_min = Rt - r, d_max = rho + H;
    double d = d_min + (d_max - d_min) * UnitRangeFromTexCoord(2.0 * z - 1.0, s.smu / 2);
    mu = d == 0.0 ? 1.0 : ClampCosine((H * H - rho * rho - d * d) / (2.0 * r * d));
    ground = false;
  }
  TexelRow row;
  row.r = (float)r;
  row.rho = (float)rho;
  row.h = (float)(r - Rb);
  row.mu = (float)mu;
  double rmu = r * mu;
  row.rmu = (float)rmu;
  // DistanceToNearestAtmosphereBoundary (functions.glsl:680-687).
  row.d = (float)(ground ? DistanceToBottom(Rb, r, mu) : DistanceToTop(Rt, r, mu));
  row.omega_x = (float)sqrt(fmax(1.0 - mu * mu, 0.0));
  double disc = rmu * rmu - rho * rho;   // r^2 (mu^2 - 1) + Rb^2
  row.q = (float)(ground ? SafeSqrt(disc) : 0.0);
  row.delta = (float)(-disc);
  row.ground = ground ? 1 : 0;
  row.pad[0] = row.pad[1] = 0;
  return row;
}

// functions.glsl:877-889 for column c.
ATMO_HD TexelCol MakeTexelCol(const Consts& c, const Shape& s, int col) {
  const double Rb = c.dRb, Rt = c.dRt, H = c.dH;
  double x_mu_s = UnitRangeFromTexCoord((double(col) + 0.5) / double(s.smus), s.smus);
  double d_min = Rt - Rb, d_max = H;
  double D = DistanceToTop(Rt, Rb, c.dmus_min);
  double A = (D - d_min) / (d_max - d_min);
  double a = (A - x_mu_s * A) / (1.0 + x_mu_s * A);
  double d = d_min + fmin(a, A) * (d_max - d_min);
  double mu_s = d == 0.0 ? 1.0 : ClampCosine((H * H - d * d) / (2.0 * Rb * d));
  TexelCol t;
  t.mu_s = (float)mu_s;
  t.sin_s = (float)sqrt(fmax(1.0 - mu_s * mu_s, 0.0));
  // Forward mapping of mu_s (functions.glsl:817-827).
  double dd = DistanceToTop(Rt, Rb, mu_s);
  double aa = (dd - d_min) / (d_max - d_min);
  t.u_mu_s = (float)TexCoordFromUnitRange(fmax(1.0 - aa / A, 0.0) / (1.0 + aa), s.smus);
  t.pad = 0.0f;
  return t;
}

// u_mu of (r, mu) (functions.glsl:787-813) in double precision.
ATMO_HD double UMu(const Consts& c, const Shape& s, double r, double mu, bool ground) {
  const double Rb = c.dRb, Rt = c.dRt, H = c.dH;
  double rho = SafeSqrt(r * r - Rb * Rb);
  double r_mu = r * mu;
  double disc = r_mu * r_mu - r * r + Rb * Rb;
  if (ground) {
    double d = -r_mu - SafeSqrt(disc);
    double d_min = r - Rb, d_max = rho;
    return 0.5 - 0.5 * TexCoordFromUnitRange(
                           d_max == d_min ? 0.0 : (d - d_min) / (d_max - d_min), s.smu / 2);
  }
  double d = -r_mu + SafeSqrt(disc + H * H);
  double d_min = Rt - r, d_max = rho + H;
  return 0.5 + 0.5 * TexCoordFromUnitRange((d - d_min) / (d_max - d_min), s.smu / 2);
}

// One theta sample l of ComputeScatteringDensity at r-slice k
// (functions.glsl:1194-1211).  t_ground is filled after the transmittance pass.
ATMO_HD DensityRow MakeDensityRow(const Consts& c, const Shape& s, int k, int l) {
  const double Rb = c.dRb, H = c.dH;
  double w = (double(k) + 0.5) / double(s.sr);
  double rho = H * UnitRangeFromTexCoord(w, s.sr);
  double r = sqrt(rho * rho + Rb * Rb);
  const double dtheta = kPiD / double(kDensityThetaSamples);
  double theta = (double(l) + 0.5) * dtheta;
  double ct = cos(theta), st = sin(theta);
  DensityRow d;
  d.cos_t = (float)ct;
  d.sin_t = (float)st;
  bool g = RayIntersectsGround(Rb, r, ct);
  d.ground = g ? 1 : 0;
  d.dist_ground = g ? (float)DistanceToBottom(Rb, r, ct) : 0.0f;
  d.u_mu = (float)UMu(c, s, r, ct, g);
  d.delta = (float)(rho * rho - (r * ct) * (r * ct));
  d.pad1 = d.pad2 = 0.0f;
  d.t_ground = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  return d;
}

// functions.glsl:1539-1548 for irradiance row j and column i.
ATMO_HD IrrRow MakeIrrRow(const Consts& c, const Shape& s, int j) {
  const double Rb = c.dRb, Rt = c.dRt;
  double x_r = UnitRangeFromTexCoord((double(j) + 0.5) / double(s.ih), s.ih);
  double r = Rb + x_r * (Rt - Rb);
  double h = x_r * (Rt - Rb);
  IrrRow row;
  row.r = (float)r;
  row.h = (float)h;
  row.rho = (float)sqrt(fmax(h * (r + Rb), 0.0));
  row.pad = 0.0f;
  return row;
}
ATMO_HD float IrrMuS(const Shape& s, int i) {
  double x = UnitRangeFromTexCoord((double(i) + 0.5) / double(s.iw), s.iw);
  return (float)ClampCosine(2.0 * x - 1.0);
}

// Number of table entries of one instance (the flat work of the table kernel).
ATMO_HD int TableEntries(const Shape& s) {
  return s.sr * s.smu + s.smus + s.sr * kDensityThetaSamples + s.ih + s.iw;
}

ATMO_HD void FillTableEntry(const Consts& c, const Shape& s, const Tables& t, int e) {
  if (e < s.sr * s.smu) {
    t.rows[e] = MakeTexelRow(c, s, e / s.smu, e % s.smu);
    return;
  }
  e -= s.sr * s.smu;
  if (e < s.smus) {
    t.cols[e] = MakeTexelCol(c, s, e);
    return;
  }
  e -= s.smus;
  if (e < s.sr * kDensityThetaSamples) {
    t.drows[e] = MakeDensityRow(c, s, e / kDensityThetaSamples, e % kDensityThetaSamples);
    return;
  }
  e -= s.sr * kDensityThetaSamples;
  if (e < s.ih) {
    t.irows[e] = MakeIrrRow(c, s, e);
    return;
  }
  e -= s.ih;
  if (e < s.iw) t.mus_i[e] = IrrMuS(s, e);
}

}  // namespace dbl
}  // namespace atmo

#endif  // ATMO_TABLES_CUH_
