// atmo_consts.h -- host-side conversion of an atmo_atmosphere (the 3-wavelength
// AtmosphereParameters of atmosphere/definitions.glsl:205-255) into the
// per-instance kernel constants, with parameter validation.
#ifndef ATMO_CONSTS_H_
#define ATMO_CONSTS_H_

#include <cmath>
#include <string>

#include "../../include/atmo/atmo.h"
#include "atmo_device.cuh"

namespace atmo {

inline bool Finite(double x) { return std::isfinite(x); }

inline bool ValidShape(const atmo_lut_shape& s, std::string* why) {
  const int v[8] = {s.transmittance_width, s.transmittance_height, s.scattering_r,
                    s.scattering_mu,       s.scattering_mu_s,      s.scattering_nu,
                    s.irradiance_width,    s.irradiance_height};
  for (int x : v) {
    if (x < 2 || x > 65536) {
      *why = "LUT sizes must be in [2, 65536]";
      return false;
    }
  }
  if (s.scattering_mu % 2 != 0 || s.scattering_mu < 4) {
    *why = "scattering_mu must be even and >= 4";
    return false;
  }
  long long texels = (long long)s.scattering_r * s.scattering_mu * s.scattering_mu_s *
                     s.scattering_nu;
  if (texels > (1LL << 31) - 1) {
    *why = "scattering LUT too large";
    return false;
  }
  return true;
}

inline atmo_lut_shape DefaultShape() {
  // atmosphere/constants.h:47-61
  atmo_lut_shape s;
  s.transmittance_width = 256;
  s.transmittance_height = 64;
  s.scattering_r = 32;
  s.scattering_mu = 128;
  s.scattering_mu_s = 32;
  s.scattering_nu = 8;
  s.irradiance_width = 64;
  s.irradiance_height = 16;
  return s;
}

// Fills the tuned block shapes registered for these LUT sizes (atmo_program.cu).
void ApplyTuning(const atmo_lut_shape& sizes, Shape* s);

inline Shape ToShape(const atmo_lut_shape& s) {
  Shape t;
  t.tw = s.transmittance_width;
  t.th = s.transmittance_height;
  t.sr = s.scattering_r;
  t.smu = s.scattering_mu;
  t.smus = s.scattering_mu_s;
  t.snu = s.scattering_nu;
  t.iw = s.irradiance_width;
  t.ih = s.irradiance_height;
  const int n[kMapCount] = {t.tw, t.th, t.sr, t.smu / 2, t.smus, t.iw, t.ih};
  for (int i = 0; i < kMapCount; ++i) {
    volatile float fn = (float)n[i];   // the kernels' 0.5f / float(n), IEEE
    t.map_c0[i] = 0.5f / fn;
    t.map_c1[i] = 1.0f - 1.0f / fn;
  }
  for (int i = 0; i < 4; ++i) t.tune[i] = 0;
  ApplyTuning(s, &t);
  return t;
}

inline bool ValidAtmosphere(const atmo_atmosphere& a, std::string* why) {
  auto fin3 = [](const double* v) { return Finite(v[0]) && Finite(v[1]) && Finite(v[2]); };
  auto finp = [](const atmo_density_profile& p) {
    for (int i = 0; i < 2; ++i) {
      const atmo_density_layer& l = p.layers[i];
      if (!Finite(l.width) || !Finite(l.exp_term) || !Finite(l.exp_scale) ||
          !Finite(l.linear_term) || !Finite(l.constant_term))
        return false;
    }
    return true;
  };
  if (!fin3(a.solar_irradiance) || !fin3(a.rayleigh_scattering) || !fin3(a.mie_scattering) ||
      !fin3(a.mie_extinction) || !fin3(a.absorption_extinction) || !fin3(a.ground_albedo) ||
      !finp(a.rayleigh_density) || !finp(a.mie_density) || !finp(a.absorption_density) ||
      !Finite(a.sun_angular_radius) || !Finite(a.bottom_radius) || !Finite(a.top_radius) ||
      !Finite(a.mie_phase_function_g) || !Finite(a.mu_s_min)) {
    *why = "non-finite atmosphere parameter";
    return false;
  }
  if (!(a.bottom_radius > 0.0) || !(a.top_radius > a.bottom_radius)) {
    *why = "radii must satisfy 0 < bottom_radius < top_radius";
    return false;
  }
  if (!(a.mie_phase_function_g > -1.0 && a.mie_phase_function_g < 1.0)) {
    *why = "mie_phase_function_g must be in (-1, 1)";
    return false;
  }
  if (!(a.mu_s_min >= -1.0 && a.mu_s_min < 1.0)) {
    *why = "mu_s_min (cos of the maximum sun zenith angle) must be in [-1, 1)";
    return false;
  }
  if (!(a.sun_angular_radius >= 0.0 && a.sun_angular_radius < 0.5)) {
    *why = "sun_angular_radius must be in [0, 0.5)";
    return false;
  }
  return true;
}

inline LayerF ToLayer(const atmo_density_layer& l) {
  return LayerF{(float)l.width, (float)l.exp_term, (float)l.exp_scale, (float)l.linear_term,
                (float)l.constant_term};
}
inline ProfileF ToProfile(const atmo_density_profile& p) {
  return ProfileF{{ToLayer(p.layers[0]), ToLayer(p.layers[1])}};
}
inline F3 ToF3(const double* v) { return F3{(float)v[0], (float)v[1], (float)v[2]}; }

// Kernel constants of one atmosphere; lum is the row-major
// luminance_from_radiance matrix (NULL = identity).
inline Consts MakeConsts(const atmo_atmosphere& a, const float* lum) {
  Consts c;
  c.solar = ToF3(a.solar_irradiance);
  c.rayleigh = ToF3(a.rayleigh_scattering);
  c.mie_sca = ToF3(a.mie_scattering);
  c.mie_ext = ToF3(a.mie_extinction);
  c.absorption = ToF3(a.absorption_extinction);
  c.albedo = ToF3(a.ground_albedo);
  c.prof_r = ToProfile(a.rayleigh_density);
  c.prof_m = ToProfile(a.mie_density);
  c.prof_a = ToProfile(a.absorption_density);
  const double g = a.mie_phase_function_g;
  c.mie_g = (float)g;
  c.alpha_s = (float)a.sun_angular_radius;
  const double Rb = a.bottom_radius, Rt = a.top_radius;
  const double H = std::sqrt(Rt * Rt - Rb * Rb);
  c.Rb = (float)Rb;
  c.Rt = (float)Rt;
  c.H = (float)H;
  // functions.glsl:819-824: A from the distance to the top at mu_s_min.
  const double mu = a.mu_s_min;
  const double D =
      std::fmax(-Rb * mu + std::sqrt(std::fmax(Rb * Rb * (mu * mu - 1.0) + Rt * Rt, 0.0)), 0.0);
  const double A = (D - (Rt - Rb)) / (H - (Rt - Rb));
  c.mus_A = (float)A;
  c.ray_k = (float)(3.0 / (16.0 * kPiD));
  c.mie_k = (float)(3.0 / (8.0 * kPiD) * (1.0 - g * g) / (2.0 + g * g));
  c.g2p1 = (float)(1.0 + g * g);
  c.m2g = (float)(-2.0 * g);
  for (int i = 0; i < 9; ++i) c.lum[i] = lum ? lum[i] : ((i % 4 == 0) ? 1.0f : 0.0f);
  c.dRb = Rb;
  c.dRt = Rt;
  c.dH = H;
  c.dmus_min = mu;
  c.dA = A;
  return c;
}

}  // namespace atmo

#endif  // ATMO_CONSTS_H_
