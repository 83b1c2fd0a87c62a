// atmo_device.cuh -- device-side data layout and FP32 physics for the atmosphere
// LUT precomputation (GB300, sm_103a).
//
// The functions here compute what atmosphere/functions.glsl:113-1601 of
// ebruneton/precomputed_atmospheric_scattering computes, re-derived for FP32:
// every ray-sphere quantity is carried as (rho, r, r*mu) with rho^2 = r^2 - Rb^2,
// so that the cancellations of the reference's r^2(mu^2-1)+R^2 discriminants
// become products of well-conditioned factors ((H - rho)(H + rho), (a - b)(a + b)).
// Per-texel (r, mu, mu_s, nu) come from FP64 set-up tables (atmo_tables.cu), as
// the reference's FP64 CPU model computes them.
//
// Compiles with nvcc (device) and with a host C++ compiler, so the same FP32
// arithmetic can be exercised on the CPU.
#ifndef ATMO_DEVICE_CUH_
#define ATMO_DEVICE_CUH_

#include <math.h>
#include <stdint.h>

#include "atmo_check.cuh"

#ifdef __CUDACC__
#include <cuda_fp16.h>
#define ATMO_HD __host__ __device__ __forceinline__
#else
#define ATMO_HD inline
struct float4 { float x, y, z, w; };
struct float2 { float x, y; };
inline float4 make_float4(float a, float b, float c, float d) { return float4{a, b, c, d}; }
inline float2 make_float2(float a, float b) { return float2{a, b}; }
inline float rsqrtf(float x) { return 1.0f / sqrtf(x); }
#endif

namespace atmo {

constexpr float kPiF = 3.14159265358979323846f;
constexpr double kPiD = 3.14159265358979323846;
// Quadrature sizes of the reference (functions.glsl:285, :704, :1190, :1486).
constexpr int kOpticalLengthSamples = 500;
constexpr int kSingleScatteringSamples = 50;
constexpr int kMultipleScatteringSamples = 50;
constexpr int kDensityThetaSamples = 16;    // 16 theta x 32 phi over the sphere
constexpr int kDensityPhiSamples = 32;
constexpr int kIndirectThetaSamples = 16;   // 16 theta x 64 phi over the hemisphere
constexpr int kIndirectPhiSamples = 64;

// ---------------------------------------------------------------------------
// 3-wavelength spectra.
// ---------------------------------------------------------------------------
struct F3 {
  float x, y, z;
};
ATMO_HD F3 f3(float a) { return F3{a, a, a}; }
ATMO_HD F3 f3(float a, float b, float c) { return F3{a, b, c}; }
ATMO_HD F3 f3(const float4& v) { return F3{v.x, v.y, v.z}; }
ATMO_HD F3 operator+(F3 a, F3 b) { return F3{a.x + b.x, a.y + b.y, a.z + b.z}; }
ATMO_HD F3 operator-(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
ATMO_HD F3 operator*(F3 a, F3 b) { return F3{a.x * b.x, a.y * b.y, a.z * b.z}; }
ATMO_HD F3 operator/(F3 a, F3 b) { return F3{a.x / b.x, a.y / b.y, a.z / b.z}; }
ATMO_HD F3 operator*(F3 a, float s) { return F3{a.x * s, a.y * s, a.z * s}; }
ATMO_HD F3 operator*(float s, F3 a) { return F3{a.x * s, a.y * s, a.z * s}; }
ATMO_HD F3& operator+=(F3& a, F3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
ATMO_HD F3 fma3(F3 a, float s, F3 c) {
  return F3{fmaf(a.x, s, c.x), fmaf(a.y, s, c.y), fmaf(a.z, s, c.z)};
}
ATMO_HD F3 fma3(F3 a, F3 b, F3 c) {
  return F3{fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y), fmaf(a.z, b.z, c.z)};
}
ATMO_HD F3 min3(F3 a, float m) { return F3{fminf(a.x, m), fminf(a.y, m), fminf(a.z, m)}; }
// Quotient with <= 2 ulp error (__fdividef), for ratios of transmittances,
// which never sit on a LUT boundary.
ATMO_HD float div_approx(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdividef(a, b);
#else
  return a / b;
#endif
}
ATMO_HD F3 ratio3(F3 a, F3 b) {
  return F3{div_approx(a.x, b.x), div_approx(a.y, b.y), div_approx(a.z, b.z)};
}
ATMO_HD F3 exp3(F3 a) { return F3{expf(a.x), expf(a.y), expf(a.z)}; }
ATMO_HD float4 to4(F3 a, float w) { return make_float4(a.x, a.y, a.z, w); }

ATMO_HD float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
// GLSL smoothstep; for the degenerate e0 == e1 (a point sun) it returns 0 at
// x <= e0 and 1 above.
ATMO_HD float smoothstepf(float e0, float e1, float x) {
  if (x <= e0) return 0.0f;
  if (x >= e1) return 1.0f;
  float t = (x - e0) / (e1 - e0);
  return t * t * (3.0f - 2.0f * t);
}

// ---------------------------------------------------------------------------
// Per-instance constants (atmosphere/definitions.glsl:205-255 + derived).
// ---------------------------------------------------------------------------
struct LayerF {
  float width, exp_term, exp_scale, linear_term, constant_term;
};
struct ProfileF {
  LayerF layer[2];
};

// Texture sizes whose texel-centre mapping (functions.glsl:342-344) the
// kernels evaluate, with the mapping's constants 0.5 / n and 1 - 1 / n.
enum UnitMapIndex { kMapTW, kMapTH, kMapSR, kMapSMU2, kMapSMUS, kMapIW, kMapIH, kMapCount };

struct Shape {
  int tw, th;             // transmittance W x H
  int sr, smu, smus, snu; // scattering R, MU, MU_S, NU
  int iw, ih;             // irradiance W x H
  float map_c0[kMapCount];  // 0.5 / n (IEEE, as the kernels would compute it)
  float map_c1[kMapCount];  // 1 - 1 / n
  // Block shape of the row-restructured kernels (0: the built-in choice):
  // multiple-scattering rows per block and samples per line stage, then the
  // same for single scattering.  Set by the autotuner; results do not depend
  // on it.
  int tune[4];
  ATMO_HD int sw() const { return snu * smus; }
  ATMO_HD long long s_texels() const { return (long long)snu * smus * smu * sr; }
  ATMO_HD int t_texels() const { return tw * th; }
  ATMO_HD int i_texels() const { return iw * ih; }
};

struct Consts {
  F3 solar, rayleigh, mie_sca, mie_ext, absorption, albedo;
  ProfileF prof_r, prof_m, prof_a;
  float mie_g, alpha_s;       // Mie g, sun angular radius
  float Rb, Rt, H;            // bottom/top radius, H = sqrt(Rt^2 - Rb^2)
  float mus_A;                // A of the mu_s mapping (functions.glsl:823-824)
  float ray_k, mie_k;         // 3/(16 pi); 3/(8 pi)(1-g^2)/(2+g^2)
  float g2p1, m2g;            // 1+g^2, -2g
  float lum[9];               // luminance_from_radiance, row major
  // FP64 copies for the set-up tables.
  double dRb, dRt, dH, dmus_min, dA;
};

ATMO_HD float LayerDensity(const LayerF& l, float h) {
  // functions.glsl:263-267
  float d = l.exp_term * expf(l.exp_scale * h) + l.linear_term * h + l.constant_term;
  return clampf(d, 0.0f, 1.0f);
}
ATMO_HD float ProfileDensity(const ProfileF& p, float h) {
  // functions.glsl:269-273
  return h < p.layer[0].width ? LayerDensity(p.layer[0], h) : LayerDensity(p.layer[1], h);
}

ATMO_HD float TexCoordFromUnitRange(float x, int n) {
  // functions.glsl:342-344
  return 0.5f / float(n) + x * (1.0f - 1.0f / float(n));
}
// The same with the precomputed constants of the shape.
ATMO_HD float TexCoord(const Shape& s, int which, float x) {
  return fmaf(x, s.map_c1[which], s.map_c0[which]);
}

// A point on a ray: rho^2 = r^2 - Rb^2 kept separately from r so that the
// altitude r - Rb = rho^2 / (r + Rb) keeps its relative precision.
struct RadialPoint {
  float rho, r, h;
};
ATMO_HD RadialPoint PointFromRho2(const Consts& c, float rho2) {
  rho2 = clampf(rho2, 0.0f, c.H * c.H);
  RadialPoint p;
  p.rho = sqrtf(rho2);
  p.r = sqrtf(rho2 + c.Rb * c.Rb);
  p.h = rho2 / (p.r + c.Rb);
  return p;
}
// Point at distance d along the ray (rho, r*mu): rho_d^2 = d^2 + 2 r mu d + rho^2.
ATMO_HD RadialPoint PointAlongRay(const Consts& c, float rho, float rmu, float d) {
  return PointFromRho2(c, fmaf(d, d + 2.0f * rmu, rho * rho));
}

// ---------------------------------------------------------------------------
// Transmittance LUT (functions.glsl:402-421 mapping, :473-480 lookup).
// ---------------------------------------------------------------------------
// Distance to the top boundary from (rho, r) along r*mu:
// -r mu + sqrt(H^2 - rho^2 + (r mu)^2), in its cancellation-free form.
ATMO_HD float DistanceToTop(const Consts& c, float rho, float rmu) {
  float hm = (c.H - rho) * (c.H + rho);
  float sq = sqrtf(fmaxf(fmaf(rmu, rmu, hm), 0.0f));
  return rmu > 0.0f ? hm / (rmu + sq) : sq - rmu;
}

// GL LINEAR + CLAMP_TO_EDGE bilinear fetch of RGB from a float4 2D texture.
ATMO_HD F3 Bilinear(const float4* __restrict__ tex, int w, int h, float u, float v) {
  float x = u * float(w) - 0.5f, y = v * float(h) - 0.5f;
  float fx = floorf(x), fy = floorf(y);
  float a = x - fx, b = y - fy;
  int i0 = (int)fx, j0 = (int)fy;
  int i1 = i0 + 1, j1 = j0 + 1;
  i0 = i0 < 0 ? 0 : (i0 > w - 1 ? w - 1 : i0);
  i1 = i1 < 0 ? 0 : (i1 > w - 1 ? w - 1 : i1);
  j0 = j0 < 0 ? 0 : (j0 > h - 1 ? h - 1 : j0);
  j1 = j1 < 0 ? 0 : (j1 > h - 1 ? h - 1 : j1);
#ifdef __CUDA_ARCH__
  float4 t00 = __ldg(ATMO_CHECKED_PTR(kCheckLutTexel, tex, j0 * w, i0, w * h));
  float4 t10 = __ldg(ATMO_CHECKED_PTR(kCheckLutTexel, tex, j0 * w, i1, w * h));
  float4 t01 = __ldg(ATMO_CHECKED_PTR(kCheckLutTexel, tex, j1 * w, i0, w * h));
  float4 t11 = __ldg(ATMO_CHECKED_PTR(kCheckLutTexel, tex, j1 * w, i1, w * h));
#else
  float4 t00 = tex[j0 * w + i0], t10 = tex[j0 * w + i1];
  float4 t01 = tex[j1 * w + i0], t11 = tex[j1 * w + i1];
#endif
  float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b);
  float w01 = (1.0f - a) * b, w11 = a * b;
  return F3{t00.x * w00 + t10.x * w10 + t01.x * w01 + t11.x * w11,
            t00.y * w00 + t10.y * w10 + t01.y * w01 + t11.y * w11,
            t00.z * w00 + t10.z * w10 + t01.z * w01 + t11.z * w11};
}

// Transmittance LUT lookup (the mapping of functions.glsl:402-421 and the
// bilinear fetch of :473-480) for the ray from (rho, r) along r*mu = rmu.
// delta = rho^2 - rmu^2 = p^2 - Rb^2 (p the ray's impact parameter) is passed
// in because it is invariant along a ray and known accurately there; from it
// 1 - x_mu = (d_max - d) / (d_max - d_min) is formed without cancellation:
//   d_max - d = (rho + r mu) + (H - sqrt(H^2 - delta)),
//   rho + r mu = delta / (rho - r mu) when r mu < 0,
//   H - sqrt(H^2 - delta) = delta / (H + sqrt(H^2 - delta)),
// so that rays grazing the ground (delta ~ 0, x_mu ~ 1), where neighbouring
// texel columns can differ by orders of magnitude, keep their exact weights.
struct TCoords {
  int i00, i10, i01, i11;      // texel indices of the four taps
  float w00, w10, w01, w11;    // bilinear weights
};
ATMO_HD TCoords TransmittanceCoords(const Consts& c, const Shape& s, float rho, float r,
                                    float rmu, float delta) {
  const float a = -rmu;
  float sq = sqrtf(fmaxf(c.H * c.H - delta, 0.0f));
  float rho_minus_a = a > 0.0f ? (rho + a > 0.0f ? delta / (rho + a) : 0.0f) : rho - a;
  float dmax_minus_d = rho_minus_a + delta / (c.H + sq);
  float d_min = (c.H - rho) * (c.H + rho) / (c.Rt + r);
  float d_max = rho + c.H;
  float omx = clampf(dmax_minus_d / (d_max - d_min), 0.0f, 1.0f);
  // Texel coordinate X = x_mu (W - 1) = (W - 1) - Xc, fetched from the two
  // columns below W - 1 - floor(Xc) with weights computed from Xc itself.
  const int W = s.tw, Hh = s.th;
  float Xc = omx * float(W - 1);
  float f = floorf(Xc);
  float g = Xc - f;                       // weight of the lower column
  int i_hi = W - 1 - (int)f;
  int i_lo = i_hi - 1;
  i_hi = i_hi < 0 ? 0 : i_hi;
  i_lo = i_lo < 0 ? 0 : i_lo;
  float Y = rho / c.H * float(Hh - 1);
  float fy = floorf(Y);
  float b = Y - fy;
  int j0 = (int)fy, j1 = j0 + 1;
  j0 = j0 < 0 ? 0 : (j0 > Hh - 1 ? Hh - 1 : j0);
  j1 = j1 < 0 ? 0 : (j1 > Hh - 1 ? Hh - 1 : j1);
  TCoords t;
  t.i00 = (int)ATMO_CHECKED_INDEX(kCheckLutTexel, j0 * W + i_lo, W * Hh);
  t.i10 = (int)ATMO_CHECKED_INDEX(kCheckLutTexel, j0 * W + i_hi, W * Hh);
  t.i01 = (int)ATMO_CHECKED_INDEX(kCheckLutTexel, j1 * W + i_lo, W * Hh);
  t.i11 = (int)ATMO_CHECKED_INDEX(kCheckLutTexel, j1 * W + i_hi, W * Hh);
  t.w00 = g * (1.0f - b);
  t.w10 = (1.0f - g) * (1.0f - b);
  t.w01 = g * b;
  t.w11 = (1.0f - g) * b;
  return t;
}

ATMO_HD float4 LoadTexel(const float4* __restrict__ tex, int i) {
#ifdef __CUDA_ARCH__
  return __ldg(tex + i);
#else
  return tex[i];
#endif
}

ATMO_HD F3 FetchTransmittance(const float4* __restrict__ T, const TCoords& t) {
  float4 a = LoadTexel(T, t.i00), b = LoadTexel(T, t.i10);
  float4 c = LoadTexel(T, t.i01), d = LoadTexel(T, t.i11);
  return F3{a.x * t.w00 + b.x * t.w10 + c.x * t.w01 + d.x * t.w11,
            a.y * t.w00 + b.y * t.w10 + c.y * t.w01 + d.y * t.w11,
            a.z * t.w00 + b.z * t.w10 + c.z * t.w01 + d.z * t.w11};
}

ATMO_HD F3 TransmittanceLookup(const Consts& c, const Shape& s, const float4* __restrict__ T,
                               float rho, float r, float rmu, float delta) {
  return FetchTransmittance(T, TransmittanceCoords(c, s, rho, r, rmu, delta));
}

// A transmittance lookup kept as m * exp(-e) per channel, from the optical
// depth LUT (tau = -ln T): e = the smallest tau among the weighted taps and
// m = sum_k w_k exp(e - tau_k) in (0, 1].  Ratios of two such values stay
// accurate where the transmittance itself is below FP32's normal range.
struct TExp {
  F3 m, e;
};
ATMO_HD float MinTau(float a, float wa, float b, float wb, float c, float wc, float d,
                     float wd) {
  float m = 3.0e38f;
  if (wa > 0.0f) m = fminf(m, a);
  if (wb > 0.0f) m = fminf(m, b);
  if (wc > 0.0f) m = fminf(m, c);
  if (wd > 0.0f) m = fminf(m, d);
  return m;
}
ATMO_HD TExp FetchTau(const float4* __restrict__ Tau, const TCoords& t) {
  float4 a = LoadTexel(Tau, t.i00), b = LoadTexel(Tau, t.i10);
  float4 c = LoadTexel(Tau, t.i01), d = LoadTexel(Tau, t.i11);
  TExp r;
  r.e.x = MinTau(a.x, t.w00, b.x, t.w10, c.x, t.w01, d.x, t.w11);
  r.e.y = MinTau(a.y, t.w00, b.y, t.w10, c.y, t.w01, d.y, t.w11);
  r.e.z = MinTau(a.z, t.w00, b.z, t.w10, c.z, t.w01, d.z, t.w11);
  r.m.x = t.w00 * expf(r.e.x - a.x) + t.w10 * expf(r.e.x - b.x) + t.w01 * expf(r.e.x - c.x) +
          t.w11 * expf(r.e.x - d.x);
  r.m.y = t.w00 * expf(r.e.y - a.y) + t.w10 * expf(r.e.y - b.y) + t.w01 * expf(r.e.y - c.y) +
          t.w11 * expf(r.e.y - d.y);
  r.m.z = t.w00 * expf(r.e.z - a.z) + t.w10 * expf(r.e.z - b.z) + t.w01 * expf(r.e.z - c.z) +
          t.w11 * expf(r.e.z - d.z);
  return r;
}
// num / den for values in the m * exp(-e) form.
ATMO_HD F3 TExpRatio(const TExp& num, const TExp& den) {
  return F3{div_approx(num.m.x, den.m.x) * expf(den.e.x - num.e.x),
            div_approx(num.m.y, den.m.y) * expf(den.e.y - num.e.y),
            div_approx(num.m.z, den.m.z) * expf(den.e.z - num.e.z)};
}
// Below this the FP32 transmittance loses precision (subnormal range).
constexpr float kTinyTransmittance = 1e-30f;
ATMO_HD bool AnyTiny(F3 t) {
  return t.x < kTinyTransmittance || t.y < kTinyTransmittance || t.z < kTinyTransmittance;
}

// rho^2 - rmu^2 from FP32 inputs, as a product of two factors.
ATMO_HD float ImpactExcess(float rho, float rmu) { return (rho - rmu) * (rho + rmu); }

ATMO_HD F3 TransmittanceToTop(const Consts& c, const Shape& s, const float4* T, float rho,
                              float r, float rmu) {
  return TransmittanceLookup(c, s, T, rho, r, rmu, ImpactExcess(rho, rmu));
}

// GetTransmittance (functions.glsl:493-515) for the segment of length d from
// (rho, r, rmu) with invariant impact excess delta; `start` is the lookup at
// the start point in the direction the reference uses (-mu when the ray hits
// the ground).  When that is tiny the ratio is formed from optical depths.
// The start point's lookup, in both forms.
struct TStart {
  F3 t;        // linear
  TExp x;      // m * exp(-e), only filled when tiny
  bool tiny;   // t below kTinyTransmittance in some channel
};
ATMO_HD TStart MakeTStart(const Consts& c, const Shape& s, const float4* T, const float4* Tau,
                          float rho, float r, float rmu, float delta) {
  TCoords tc = TransmittanceCoords(c, s, rho, r, rmu, delta);
  TStart st;
  st.t = FetchTransmittance(T, tc);
  st.tiny = AnyTiny(st.t);
  st.x.m = f3(1.0f);
  st.x.e = f3(0.0f);
  if (st.tiny) st.x = FetchTau(Tau, tc);
  return st;
}

ATMO_HD F3 SegmentTransmittance(const Consts& c, const Shape& s, const float4* T,
                                const float4* Tau, float rmu, float delta,
                                const RadialPoint& pd, float d, bool ground,
                                const TStart& start) {
  float rmu_d = clampf(rmu + d, -pd.r, pd.r);
  TCoords tc = TransmittanceCoords(c, s, pd.rho, pd.r, ground ? -rmu_d : rmu_d, delta);
  if (start.tiny) {
    TExp x = FetchTau(Tau, tc);
    return min3(ground ? TExpRatio(x, start.x) : TExpRatio(start.x, x), 1.0f);
  }
  F3 t = FetchTransmittance(T, tc);
  return min3(ground ? ratio3(t, start.t) : ratio3(start.t, t), 1.0f);
}

// GetTransmittanceToSun (functions.glsl:552-563) at point p with r*mu_s = rmu_s.
ATMO_HD F3 TransmittanceToSun(const Consts& c, const Shape& s, const float4* T,
                              const RadialPoint& p, float rmu_s) {
  rmu_s = clampf(rmu_s, -p.r, p.r);
  float sin_theta_h = c.Rb / p.r;
  // mu_s - cos(theta_h) with cos(theta_h) = -rho / r.
  float x = (rmu_s + p.rho) / p.r;
  float e = sin_theta_h * c.alpha_s;
  return TransmittanceToTop(c, s, T, p.rho, p.r, rmu_s) * smoothstepf(-e, e, x);
}

// ---------------------------------------------------------------------------
// Scattering LUT mapping (functions.glsl:773-831) and 4D lookup (:958-976).
// ---------------------------------------------------------------------------
ATMO_HD float UMuSFromMuS(const Consts& c, const Shape& s, float mu_s) {
  // d = DistanceToTopAtmosphereBoundary(Rb, mu_s), cancellation-free.
  float rmus = c.Rb * mu_s;
  float sq = sqrtf(fmaf(rmus, rmus, c.H * c.H));
  float d = rmus > 0.0f ? (c.H * c.H) / (rmus + sq) : sq - rmus;
  float d_min = c.Rt - c.Rb, d_max = c.H;
  float a = (d - d_min) / (d_max - d_min);
  return TexCoord(s, kMapSMUS, fmaxf(1.0f - a / c.mus_A, 0.0f) / (1.0f + a));
}

// u_mu when the distance to the ray's boundary is known (d_ray).
ATMO_HD float UMuFromDistance(const Consts& c, const Shape& s, const RadialPoint& p,
                              float d_ray, bool ground) {
  if (ground) {
    float d_min = p.h, d_max = p.rho;
    float x = d_max == d_min ? 0.0f : clampf((d_ray - d_min) / (d_max - d_min), 0.0f, 1.0f);
    return 0.5f - 0.5f * TexCoord(s, kMapSMU2, x);
  }
  float d_min = (c.H - p.rho) * (c.H + p.rho) / (c.Rt + p.r);
  float d_max = p.rho + c.H;
  float x = clampf((d_ray - d_min) / (d_max - d_min), 0.0f, 1.0f);
  return 0.5f + 0.5f * TexCoord(s, kMapSMU2, x);
}

// u_mu from (rho, r*mu) alone (distance to the ground or to the top).
ATMO_HD float UMuFromRMu(const Consts& c, const Shape& s, const RadialPoint& p, float rmu,
                         bool ground) {
  float d;
  if (ground) {
    // -r mu - sqrt((r mu)^2 - rho^2) = rho^2 / (-r mu + sqrt(...)).
    float disc = fmaxf((rmu - p.rho) * (rmu + p.rho), 0.0f);
    float den = sqrtf(disc) - rmu;
    d = den > 0.0f ? p.rho * p.rho / den : 0.0f;
  } else {
    d = DistanceToTop(c, p.rho, rmu);
  }
  return UMuFromDistance(c, s, p, d, ground);
}

// Coordinates of one 4D lookup: the x texel column of the two nu nodes, the
// nu lerp, and the fractional (y, z) position.
struct Lookup4 {
  int b0, b1;       // first columns of the two nu nodes' blocks (node x MU_S)
  float xl;         // mu_s texel coordinate within a block (after -0.5)
  float lerp_nu;
  float y, z;       // y, z texel coordinates (after -0.5)
};
// The reference's x texel coordinate of a nu node n is (n + u_mu_s) / NU x W
// - 0.5 = n MU_S + (u_mu_s MU_S - 0.5).  It is kept as the block's first
// column plus the small within-block coordinate: formed as one float, its
// fraction would carry the rounding of n MU_S (growing with NU), and at a
// texel-centre lookup that rounding puts a weight on the neighbouring column,
// the previous node's brightest (highest-sun) texel.
ATMO_HD Lookup4 MakeLookup(const Shape& s, float u_nu, float u_mu_s, float u_mu, float u_r) {
  Lookup4 L;
  float tex_coord_x = u_nu * float(s.snu - 1);
  float tex_x = floorf(tex_coord_x);
  L.lerp_nu = tex_coord_x - tex_x;
  L.b0 = (int)tex_x * s.smus;
  L.b1 = L.b0 + s.smus;
  L.xl = fmaf(u_mu_s, float(s.smus), -0.5f);
  L.y = u_mu * float(s.smu) - 0.5f;
  L.z = u_r * float(s.sr) - 0.5f;
  return L;
}

ATMO_HD int ClampIdx(int i, int n) { return i < 0 ? 0 : (i > n - 1 ? n - 1 : i); }

// The 4D lookup of functions.glsl:958-976: two trilinear fetches (the nu
// nodes' blocks b0 and b1) that share their y (mu) and z (r) interpolation, with
// the nu lerp folded into the x weights.  32-bit indices (the scattering LUT
// has fewer than 2^31 texels).
ATMO_HD F3 Scattering4(const float4* __restrict__ tex, const Shape& s, const Lookup4& L) {
  const int W = s.sw(), Hh = s.smu, D = s.sr;
  const float fy = floorf(L.y), fz = floorf(L.z);
  const float b = L.y - fy, c = L.z - fz;
  const int j0 = ClampIdx((int)fy, Hh), j1 = ClampIdx((int)fy + 1, Hh);
  const int k0 = ClampIdx((int)fz, D), k1 = ClampIdx((int)fz + 1, D);
  const int r00 = (k0 * Hh + j0) * W, r01 = (k0 * Hh + j1) * W;
  const int r10 = (k1 * Hh + j0) * W, r11 = (k1 * Hh + j1) * W;
  const float w00 = (1.0f - b) * (1.0f - c), w01 = b * (1.0f - c);
  const float w10 = (1.0f - b) * c, w11 = b * c;
  F3 acc = f3(0.0f);
#pragma unroll
  for (int node = 0; node < 2; ++node) {
    const int base = node == 0 ? L.b0 : L.b1;
    const float wn = node == 0 ? 1.0f - L.lerp_nu : L.lerp_nu;
    const float fx = floorf(L.xl);
    const float a = L.xl - fx;
    const int i0 = ClampIdx(base + (int)fx, W), i1 = ClampIdx(base + (int)fx + 1, W);
    const float wa0 = (1.0f - a) * wn, wa1 = a * wn;
#ifdef __CUDA_ARCH__
#define ATMO_TAP(idx) __ldg(tex + ATMO_CHECKED_INDEX(kCheckLutTexel, (idx), W * Hh * D))
#else
#define ATMO_TAP(idx) tex[(idx)]
#endif
    const float4 t0 = ATMO_TAP(r00 + i0), t1 = ATMO_TAP(r00 + i1);
    const float4 t2 = ATMO_TAP(r01 + i0), t3 = ATMO_TAP(r01 + i1);
    const float4 t4 = ATMO_TAP(r10 + i0), t5 = ATMO_TAP(r10 + i1);
    const float4 t6 = ATMO_TAP(r11 + i0), t7 = ATMO_TAP(r11 + i1);
#undef ATMO_TAP
    const float v0 = wa0 * w00, v1 = wa1 * w00, v2 = wa0 * w01, v3 = wa1 * w01;
    const float v4 = wa0 * w10, v5 = wa1 * w10, v6 = wa0 * w11, v7 = wa1 * w11;
    acc.x += t0.x * v0 + t1.x * v1 + t2.x * v2 + t3.x * v3 + t4.x * v4 + t5.x * v5 +
             t6.x * v6 + t7.x * v7;
    acc.y += t0.y * v0 + t1.y * v1 + t2.y * v2 + t3.y * v3 + t4.y * v4 + t5.y * v5 +
             t6.y * v6 + t7.y * v7;
    acc.z += t0.z * v0 + t1.z * v1 + t2.z * v2 + t3.z * v3 + t4.z * v4 + t5.z * v5 +
             t6.z * v6 + t7.z * v7;
  }
  return acc;
}

// functions.glsl:739-747
ATMO_HD float RayleighPhase(const Consts& c, float nu) { return c.ray_k * (1.0f + nu * nu); }
ATMO_HD float MiePhase(const Consts& c, float nu) {
  float t = fmaf(c.m2g, nu, c.g2p1);
  float rs = rsqrtf(t);
  return c.mie_k * (1.0f + nu * nu) * (rs * rs * rs);
}

// ---------------------------------------------------------------------------
// Irradiance LUT (functions.glsl:1524-1533, :1595-1601).
// ---------------------------------------------------------------------------
ATMO_HD F3 Irradiance(const Consts& c, const Shape& s, const float4* I, float h, float mu_s) {
  float x_r = h / (c.Rt - c.Rb);
  float x_mu_s = mu_s * 0.5f + 0.5f;
  return Bilinear(I, s.iw, s.ih, TexCoord(s, kMapIW, x_mu_s), TexCoord(s, kMapIH, x_r));
}

ATMO_HD F3 MatVec(const float m[9], F3 v) {
  return F3{m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
            m[6] * v.x + m[7] * v.y + m[8] * v.z};
}

// ---------------------------------------------------------------------------
// FP64 set-up tables: per scattering texel row / column, computed once per
// precomputation by atmo_tables.cu with the reference's own double formulas.
// ---------------------------------------------------------------------------
struct TexelRow {        // one (r-slice k, mu-row j) of the scattering LUT
  float r, rho, h;       // r, sqrt(r^2 - Rb^2), r - Rb
  float mu, rmu;         // mu and r*mu of the row
  float d;               // distance to the ray's boundary (ground or top)
  float omega_x;         // sqrt(1 - mu^2)
  float q;               // ground: sqrt((r mu)^2 - rho^2); else 0
  float delta;           // rho^2 - (r mu)^2, invariant along the ray
  int ground;            // ray_r_mu_intersects_ground
  int pad[2];
};

// rho^2 at distance t along the texel row's ray, where e = row.d - t is the
// distance left to the ray's end (passed separately so that it is exactly 0
// at the last quadrature sample), written so that no form cancels: for a
// ground ray e (e + 2q) vanishes exactly at the ground point; for an upward
// ray t (t + 2 r mu) + rho^2 adds non-negative terms; for a downward ray that
// misses the ground (t + r mu)^2 + q adds non-negative terms.
ATMO_HD float RayRho2(const TexelRow& row, float t, float e) {
  if (row.ground) return e * (e + 2.0f * row.q);
  if (row.rmu >= 0.0f) return fmaf(t, t + 2.0f * row.rmu, row.rho * row.rho);
  float u = t + row.rmu;
  return fmaf(u, u, row.delta);
}
struct TexelCol {        // one mu_s column c
  float mu_s, sin_s;     // mu_s, sqrt(1 - mu_s^2)
  float u_mu_s;          // forward-mapped texture coordinate of mu_s
  float pad;
};
struct DensityRow {      // one (r-slice k, theta sample l) of the density integral
  float cos_t, sin_t;    // cos/sin of theta_l
  float dist_ground;     // distance to the ground (0 when the ray misses it)
  int ground;            // RayIntersectsGround(r, cos theta_l)
  float u_mu;            // texture coordinate of (r, cos theta_l)
  float delta;           // rho^2 - (r cos theta_l)^2, invariant along the row's ray
  float pad1, pad2;
  float4 t_ground;       // transmittance to the ground x albedo / pi
};

struct IrrRow {          // one r row of the irradiance LUT
  float r, rho, h, pad;
};

struct Tables {
  TexelRow* rows;        // [sr * smu]
  // [sr * smu] the order in which the multiple-scattering blocks take the
  // rows (by the invariant delta of their rays, so that the rows in flight
  // read the same delta-density rows), or nullptr: k-major order.  Any order
  // gives the same LUTs.
  int* row_order;
  TexelCol* cols;        // [smus]
  DensityRow* drows;     // [sr * 16]
  IrrRow* irows;         // [ih]
  float* mus_i;          // [iw] mu_s of the irradiance columns
};

// Texel (x, y, z) of the scattering LUT -> (row, column, nu node).
ATMO_HD void SplitTexel(const Shape& s, long long idx, int* k, int* j, int* c, int* n) {
  int W = s.sw();
  int x = (int)(idx % W);
  long long yz = idx / W;
  *j = (int)(yz % s.smu);
  *k = (int)(yz / s.smu);
  *n = x / s.smus;
  *c = x % s.smus;
}

// The texel's nu after the clamp of functions.glsl:924-925, and the sun
// direction of functions.glsl:1176-1180 (omega_s = (sx, sy, mu_s)).
struct TexelAngles {
  float mu, mu_s, nu, omega_x, sx, sy;
  bool on_node;   // nu not clamped: the texel's own nu node (functions.glsl:924-925)
};
ATMO_HD TexelAngles MakeAngles(const Shape& s, const TexelRow& row, const TexelCol& col,
                               int n) {
  TexelAngles a;
  a.mu = row.mu;
  a.mu_s = col.mu_s;
  a.omega_x = row.omega_x;
  float nu_g = clampf(float(n) / float(s.snu - 1) * 2.0f - 1.0f, -1.0f, 1.0f);
  float mm = row.mu * col.mu_s;
  float lim = row.omega_x * col.sin_s;   // sqrt((1 - mu^2)(1 - mu_s^2))
  float t = clampf(nu_g - mm, -lim, lim);
  a.on_node = t == nu_g - mm;
  a.nu = mm + t;
  a.sx = row.omega_x == 0.0f ? 0.0f : clampf(t / row.omega_x, -col.sin_s, col.sin_s);
  float ax = fabsf(a.sx);
  a.sy = sqrtf(fmaxf((col.sin_s - ax) * (col.sin_s + ax), 0.0f));
  return a;
}

}  // namespace atmo

#endif  // ATMO_DEVICE_CUH_
