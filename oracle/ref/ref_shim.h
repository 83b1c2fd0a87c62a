/*
 * Definitions shim that lets the reference's atmosphere/functions.glsl compile
 * as C++ in double precision, the way atmosphere/reference/functions.cc:43-54
 * compiles it over the (absent) dimensional_types library.
 *
 * This file is this project's own code.  It supplies what
 * atmosphere/reference/definitions.h would: scalar physical types (all double
 * here: no dimensional checking), 3-wavelength spectra, vec2/vec3/vec4 with
 * GLSL member syntax, GLSL built-ins, units, the AtmosphereParameters struct
 * (field names as in atmosphere/definitions.glsl:185-255) and textures with GL
 * LINEAR + CLAMP_TO_EDGE filtering at texel centres (atmosphere/model.cc:427-448).
 *
 * Test infrastructure: only the recipe in oracle/ref/Makefile builds it, into
 * oracle/_ref/, in a container where the reference sources are present.
 */
#ifndef ATMO_REF_SHIM_H_
#define ATMO_REF_SHIM_H_

#include <algorithm>
#include <cassert>
#include <cmath>
#include <vector>

namespace refshim {

typedef double Length, Wavelength, Angle, SolidAngle, Power, LuminousPower, Number,
    InverseLength, Area, Volume, NumberDensity, Irradiance, Radiance, SpectralPower,
    SpectralIrradiance, SpectralRadiance, SpectralRadianceDensity, ScatteringCoefficient,
    InverseSolidAngle, LuminousIntensity, Luminance, Illuminance;

struct vec2 {
  double x, y;
  vec2() : x(0), y(0) {}
  vec2(double a, double b) : x(a), y(b) {}
};
inline vec2 operator/(const vec2& a, const vec2& b) { return vec2(a.x / b.x, a.y / b.y); }

struct vec3 {
  double x, y, z;
  vec3() : x(0), y(0), z(0) {}
  vec3(double a, double b, double c) : x(a), y(b), z(c) {}
};
inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, double s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(double s, const vec3& a) { return a * s; }
inline double dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double length(const vec3& a) { return std::sqrt(dot(a, a)); }
inline vec3 normalize(const vec3& a) { return a * (1.0 / length(a)); }

struct vec4 {
  double x, y, z, w;
  vec4() : x(0), y(0), z(0), w(0) {}
  vec4(double a, double b, double c, double d) : x(a), y(b), z(c), w(d) {}
};
inline vec4 operator/(const vec4& a, const vec4& b) {
  return vec4(a.x / b.x, a.y / b.y, a.z / b.z, a.w / b.w);
}

// A spectrum sampled at the 3 wavelengths of one precomputation group.
struct Spectrum {
  double v[3];
  Spectrum() : v{0, 0, 0} {}
  explicit Spectrum(double a) : v{a, a, a} {}
  Spectrum(double a, double b, double c) : v{a, b, c} {}
  double& operator[](int i) { return v[i]; }
  double operator[](int i) const { return v[i]; }
};
inline Spectrum operator+(const Spectrum& a, const Spectrum& b) {
  return Spectrum(a[0] + b[0], a[1] + b[1], a[2] + b[2]);
}
inline Spectrum operator-(const Spectrum& a, const Spectrum& b) {
  return Spectrum(a[0] - b[0], a[1] - b[1], a[2] - b[2]);
}
inline Spectrum operator-(const Spectrum& a) { return Spectrum(-a[0], -a[1], -a[2]); }
inline Spectrum operator*(const Spectrum& a, const Spectrum& b) {
  return Spectrum(a[0] * b[0], a[1] * b[1], a[2] * b[2]);
}
inline Spectrum operator/(const Spectrum& a, const Spectrum& b) {
  return Spectrum(a[0] / b[0], a[1] / b[1], a[2] / b[2]);
}
inline Spectrum operator*(const Spectrum& a, double s) {
  return Spectrum(a[0] * s, a[1] * s, a[2] * s);
}
inline Spectrum operator*(double s, const Spectrum& a) { return a * s; }
inline Spectrum& operator+=(Spectrum& a, const Spectrum& b) { return a = a + b; }
inline Spectrum exp(const Spectrum& a) {
  return Spectrum(std::exp(a[0]), std::exp(a[1]), std::exp(a[2]));
}
inline Spectrum min(const Spectrum& a, const Spectrum& b) {
  return Spectrum(std::min(a[0], b[0]), std::min(a[1], b[1]), std::min(a[2], b[2]));
}

typedef Spectrum DimensionlessSpectrum, PowerSpectrum, IrradianceSpectrum, RadianceSpectrum,
    RadianceDensitySpectrum, ScatteringSpectrum;
typedef vec3 Position, Direction, Luminance3, Illuminance3;

// GLSL built-ins used by functions.glsl.
using std::cos;
using std::exp;
using std::floor;
using std::max;
using std::min;
using std::pow;
using std::sin;
using std::sqrt;
inline double clamp(double x, double lo, double hi) { return std::min(std::max(x, lo), hi); }
inline double mod(double x, double y) { return x - y * std::floor(x / y); }
// GLSL smoothstep; for the degenerate e0 == e1 (a point sun) it returns 0 at
// x <= e0 and 1 above, where the clamp formula would give 0/0.
inline double smoothstep(double e0, double e1, double x) {
  if (x <= e0) return 0.0;
  if (x >= e1) return 1.0;
  double t = (x - e0) / (e1 - e0);
  return t * t * (3.0 - 2.0 * t);
}

// Units (atmosphere/definitions.glsl:143-172): all base units are 1.
constexpr double PI = 3.14159265358979323846;
constexpr Length m = 1.0;
constexpr Wavelength nm = 1.0;
constexpr Angle rad = 1.0;
constexpr SolidAngle sr = 1.0;
constexpr Power watt = 1.0;
constexpr LuminousPower lm = 1.0;
constexpr Length km = 1000.0 * m;
constexpr Area m2 = m * m;
constexpr Volume m3 = m * m * m;
constexpr Angle pi = PI * rad;
constexpr Angle deg = pi / 180.0;
constexpr Irradiance watt_per_square_meter = watt / m2;
constexpr Radiance watt_per_square_meter_per_sr = watt / (m2 * sr);
constexpr SpectralIrradiance watt_per_square_meter_per_nm = watt / (m2 * nm);
constexpr SpectralRadiance watt_per_square_meter_per_sr_per_nm = watt / (m2 * sr * nm);
constexpr SpectralRadianceDensity watt_per_cubic_meter_per_sr_per_nm = watt / (m3 * sr * nm);
constexpr LuminousIntensity cd = lm / sr;
constexpr LuminousIntensity kcd = 1000.0 * cd;
constexpr Luminance cd_per_square_meter = cd / m2;
constexpr Luminance kcd_per_square_meter = kcd / m2;

struct DensityProfileLayer {
  Length width = 0;
  Number exp_term = 0;
  InverseLength exp_scale = 0;
  InverseLength linear_term = 0;
  Number constant_term = 0;
};
struct DensityProfile {
  DensityProfileLayer layers[2];
};
struct AtmosphereParameters {
  IrradianceSpectrum solar_irradiance;
  Angle sun_angular_radius = 0;
  Length bottom_radius = 0;
  Length top_radius = 0;
  DensityProfile rayleigh_density;
  ScatteringSpectrum rayleigh_scattering;
  DensityProfile mie_density;
  ScatteringSpectrum mie_scattering;
  ScatteringSpectrum mie_extinction;
  Number mie_phase_function_g = 0;
  DensityProfile absorption_density;
  ScatteringSpectrum absorption_extinction;
  DimensionlessSpectrum ground_albedo;
  Number mu_s_min = 0;
};

// Textures over double RGBA storage (x fastest), filtered like GL LINEAR with
// CLAMP_TO_EDGE.  Only the RGB components are read as a spectrum.
template <class T>
struct Texture2 {
  int w, h;
  const double* p;
  Spectrum Get(int i, int j) const {
    i = std::min(std::max(i, 0), w - 1);
    j = std::min(std::max(j, 0), h - 1);
    const double* q = p + 4 * ((long long)j * w + i);
    return Spectrum(q[0], q[1], q[2]);
  }
};
template <class T>
struct Texture3 {
  int w, h, d;
  const double* p;
  Spectrum Get(int i, int j, int k) const {
    i = std::min(std::max(i, 0), w - 1);
    j = std::min(std::max(j, 0), h - 1);
    k = std::min(std::max(k, 0), d - 1);
    const double* q = p + 4 * (((long long)k * h + j) * w + i);
    return Spectrum(q[0], q[1], q[2]);
  }
};
template <class T>
Spectrum texture(const Texture2<T>& t, const vec2& uv) {
  double x = uv.x * t.w - 0.5, y = uv.y * t.h - 0.5;
  double fi = std::floor(x), fj = std::floor(y);
  int i = (int)fi, j = (int)fj;
  double a = x - fi, b = y - fj;
  return t.Get(i, j) * ((1.0 - a) * (1.0 - b)) + t.Get(i + 1, j) * (a * (1.0 - b)) +
         t.Get(i, j + 1) * ((1.0 - a) * b) + t.Get(i + 1, j + 1) * (a * b);
}
template <class T>
Spectrum texture(const Texture3<T>& t, const vec3& uvw) {
  double x = uvw.x * t.w - 0.5, y = uvw.y * t.h - 0.5, z = uvw.z * t.d - 0.5;
  double fi = std::floor(x), fj = std::floor(y), fk = std::floor(z);
  int i = (int)fi, j = (int)fj, k = (int)fk;
  double a = x - fi, b = y - fj, c = z - fk;
  Spectrum r;
  for (int dk = 0; dk < 2; ++dk)
    for (int dj = 0; dj < 2; ++dj)
      for (int di = 0; di < 2; ++di)
        r += t.Get(i + di, j + dj, k + dk) *
             ((di ? a : 1.0 - a) * (dj ? b : 1.0 - b) * (dk ? c : 1.0 - c));
  return r;
}

struct Tag {};
typedef Texture2<Tag> TransmittanceTexture;
typedef Texture2<Tag> IrradianceTexture;
template <class T>
using AbstractScatteringTexture = Texture3<T>;
typedef Texture3<Spectrum> ReducedScatteringTexture;
typedef Texture3<Spectrum> ScatteringTexture;
typedef Texture3<Spectrum> ScatteringDensityTexture;

}  // namespace refshim

#define IN(x) const x&
#define OUT(x) x&
#define TEMPLATE(x) template <class x>
#define TEMPLATE_ARGUMENT(x) <x>

#endif  // ATMO_REF_SHIM_H_
