/*
 * Builds the reference's own atmosphere/functions.glsl as C++ (double
 * precision) over the shim in ref_shim.h, once per LUT shape, and exports a
 * small C interface (ref_*) with the same argument conventions as the
 * oracle restatement (oracle/atmo_oracle.h).  Test infrastructure only: it
 * pins the restatement and generates the golden fixtures in tests/golden/.
 */
#include <atomic>
#include <cstring>
#include <thread>

#include "../atmo_oracle.h"
#include "ref_shim.h"

namespace {
template <typename F>
void ForEach(long long n, int threads, F&& fn) {
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::atomic<long long> next(0);
  auto worker = [&]() {
    for (;;) {
      long long b = next.fetch_add(32);
      if (b >= n) break;
      long long e = std::min(n, b + 32);
      for (long long i = b; i < e; ++i) fn(i);
    }
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
  for (auto& th : pool) th.join();
}
}  // namespace

#define ATMO_REF_SHAPE(NS, TW, TH, SR, SMU, SMUS, SNU, IW, IH)                  \
  namespace NS {                                                                \
  using namespace refshim;                                                      \
  constexpr int TRANSMITTANCE_TEXTURE_WIDTH = TW;                               \
  constexpr int TRANSMITTANCE_TEXTURE_HEIGHT = TH;                              \
  constexpr int SCATTERING_TEXTURE_R_SIZE = SR;                                 \
  constexpr int SCATTERING_TEXTURE_MU_SIZE = SMU;                               \
  constexpr int SCATTERING_TEXTURE_MU_S_SIZE = SMUS;                            \
  constexpr int SCATTERING_TEXTURE_NU_SIZE = SNU;                               \
  constexpr int SCATTERING_TEXTURE_WIDTH = SNU * SMUS;                          \
  constexpr int SCATTERING_TEXTURE_HEIGHT = SMU;                                \
  constexpr int SCATTERING_TEXTURE_DEPTH = SR;                                  \
  constexpr int IRRADIANCE_TEXTURE_WIDTH = IW;                                  \
  constexpr int IRRADIANCE_TEXTURE_HEIGHT = IH;

#define ATMO_REF_SHAPE_END }

ATMO_REF_SHAPE(shape_default, 256, 64, 32, 128, 32, 8, 64, 16)
#include "atmosphere/functions.glsl"
#include "ref_passes.inc"
ATMO_REF_SHAPE_END

ATMO_REF_SHAPE(shape_medium, 128, 32, 8, 32, 16, 8, 32, 8)
#include "atmosphere/functions.glsl"
#include "ref_passes.inc"
ATMO_REF_SHAPE_END

ATMO_REF_SHAPE(shape_small, 64, 16, 4, 16, 8, 4, 16, 4)
#include "atmosphere/functions.glsl"
#include "ref_passes.inc"
ATMO_REF_SHAPE_END

ATMO_REF_SHAPE(shape_small_nu128, 64, 16, 4, 16, 8, 128, 16, 4)
#include "atmosphere/functions.glsl"
#include "ref_passes.inc"
ATMO_REF_SHAPE_END

namespace {
using refshim::AtmosphereParameters;
using refshim::DensityProfile;
using refshim::Spectrum;

DensityProfile Prof(const oracle_profile& p) {
  DensityProfile q;
  for (int i = 0; i < 2; ++i) {
    q.layers[i].width = p.layers[i].width;
    q.layers[i].exp_term = p.layers[i].exp_term;
    q.layers[i].exp_scale = p.layers[i].exp_scale;
    q.layers[i].linear_term = p.layers[i].linear_term;
    q.layers[i].constant_term = p.layers[i].constant_term;
  }
  return q;
}
Spectrum Sp(const double* v) { return Spectrum(v[0], v[1], v[2]); }
AtmosphereParameters Atm(const oracle_atmosphere* a) {
  AtmosphereParameters p;
  p.solar_irradiance = Sp(a->solar_irradiance);
  p.sun_angular_radius = a->sun_angular_radius;
  p.bottom_radius = a->bottom_radius;
  p.top_radius = a->top_radius;
  p.rayleigh_density = Prof(a->rayleigh_density);
  p.rayleigh_scattering = Sp(a->rayleigh_scattering);
  p.mie_density = Prof(a->mie_density);
  p.mie_scattering = Sp(a->mie_scattering);
  p.mie_extinction = Sp(a->mie_extinction);
  p.mie_phase_function_g = a->mie_phase_function_g;
  p.absorption_density = Prof(a->absorption_density);
  p.absorption_extinction = Sp(a->absorption_extinction);
  p.ground_albedo = Sp(a->ground_albedo);
  p.mu_s_min = a->mu_s_min;
  return p;
}
int ShapeId(const oracle_shape* s) {
  auto is = [&](int a, int b, int c, int d, int e, int f, int g, int h) {
    return s->transmittance_width == a && s->transmittance_height == b &&
           s->scattering_r == c && s->scattering_mu == d && s->scattering_mu_s == e &&
           s->scattering_nu == f && s->irradiance_width == g && s->irradiance_height == h;
  };
  if (is(256, 64, 32, 128, 32, 8, 64, 16)) return 0;
  if (is(128, 32, 8, 32, 16, 8, 32, 8)) return 1;
  if (is(64, 16, 4, 16, 8, 4, 16, 4)) return 2;
  if (is(64, 16, 4, 16, 8, 128, 16, 4)) return 3;
  return -1;
}
void Out3(const Spectrum& s, double* o) { o[0] = s[0]; o[1] = s[1]; o[2] = s[2]; }
}  // namespace

#define ATMO_REF_DISPATCH(s, ...)                   \
  switch (ShapeId(s)) {                              \
    case 0: { using namespace shape_default; __VA_ARGS__; } break; \
    case 1: { using namespace shape_medium; __VA_ARGS__; } break;  \
    case 2: { using namespace shape_small; __VA_ARGS__; } break;   \
    case 3: { using namespace shape_small_nu128; __VA_ARGS__; } break; \
    default: return -1;                              \
  }

extern "C" {

int ref_has_shape(const oracle_shape* s) { return ShapeId(s) >= 0 ? 1 : 0; }

int ref_precompute(const oracle_atmosphere* a, const oracle_shape* s, unsigned orders,
                   const double lum[9], int blend, int combined, int threads, double* t_out,
                   double* s_out, double* m_out, double* i_out) {
  AtmosphereParameters atm = Atm(a);
  ATMO_REF_DISPATCH(s, return RunPrecompute(atm, orders, lum, blend != 0, combined != 0, threads,
                                            t_out, s_out, m_out, i_out));
  return 0;
}

/* Point functions on the default shape's instantiation (shape-independent
   ones) or on the given shape (texture-dependent ones). */
int ref_point_geometry(const oracle_atmosphere* a, double r, double mu, double out[5]) {
  using namespace shape_default;
  AtmosphereParameters atm = Atm(a);
  out[0] = DistanceToTopAtmosphereBoundary(atm, r, mu);
  out[1] = DistanceToBottomAtmosphereBoundary(atm, r, mu);
  out[2] = RayIntersectsGround(atm, r, mu) ? 1.0 : 0.0;
  out[3] = RayleighPhaseFunction(mu);
  out[4] = MiePhaseFunction(atm.mie_phase_function_g, mu);
  return 0;
}
int ref_transmittance_to_top(const oracle_atmosphere* a, double r, double mu, double out[3]) {
  using namespace shape_default;
  Out3(ComputeTransmittanceToTopAtmosphereBoundary(Atm(a), r, mu), out);
  return 0;
}
int ref_scattering_uvwz(const oracle_atmosphere* a, const oracle_shape* s, double r, double mu,
                        double mu_s, double nu, int ground, double out[4]) {
  AtmosphereParameters atm = Atm(a);
  ATMO_REF_DISPATCH(s, {
    vec4 u = GetScatteringTextureUvwzFromRMuMuSNu(atm, r, mu, mu_s, nu, ground != 0);
    out[0] = u.x; out[1] = u.y; out[2] = u.z; out[3] = u.w;
  });
  return 0;
}
int ref_frag_coord_to_rmumusnu(const oracle_atmosphere* a, const oracle_shape* s,
                               const double frag[3], double out[4], int* ground) {
  AtmosphereParameters atm = Atm(a);
  ATMO_REF_DISPATCH(s, {
    Length r; Number mu, mu_s, nu; bool g;
    GetRMuMuSNuFromScatteringTextureFragCoord(atm, vec3(frag[0], frag[1], frag[2]), r, mu, mu_s, nu, g);
    out[0] = r; out[1] = mu; out[2] = mu_s; out[3] = nu; *ground = g ? 1 : 0;
  });
  return 0;
}
/* Render-time functions (non-combined layout, as the C++ build compiles
   functions.glsl). */
int ref_sky_radiance(const oracle_atmosphere* a, const oracle_shape* s, const double* T,
                     const double* S, const double* M, const double camera[3],
                     const double view[3], double shadow, const double sun[3], double out[3],
                     double tr[3]) {
  AtmosphereParameters atm = Atm(a);
  ATMO_REF_DISPATCH(s, {
    TransmittanceTexture t{TRANSMITTANCE_TEXTURE_WIDTH, TRANSMITTANCE_TEXTURE_HEIGHT, T};
    ReducedScatteringTexture st{SCATTERING_TEXTURE_WIDTH, SCATTERING_TEXTURE_HEIGHT, SCATTERING_TEXTURE_DEPTH, S};
    ReducedScatteringTexture mt{SCATTERING_TEXTURE_WIDTH, SCATTERING_TEXTURE_HEIGHT, SCATTERING_TEXTURE_DEPTH, M};
    DimensionlessSpectrum trs;
    Out3(GetSkyRadiance(atm, t, st, mt, vec3(camera[0], camera[1], camera[2]),
                        vec3(view[0], view[1], view[2]), shadow, vec3(sun[0], sun[1], sun[2]), trs), out);
    Out3(trs, tr);
  });
  return 0;
}
int ref_sky_radiance_to_point(const oracle_atmosphere* a, const oracle_shape* s, const double* T,
                              const double* S, const double* M, const double camera[3],
                              const double point[3], double shadow, const double sun[3],
                              double out[3], double tr[3]) {
  AtmosphereParameters atm = Atm(a);
  ATMO_REF_DISPATCH(s, {
    TransmittanceTexture t{TRANSMITTANCE_TEXTURE_WIDTH, TRANSMITTANCE_TEXTURE_HEIGHT, T};
    ReducedScatteringTexture st{SCATTERING_TEXTURE_WIDTH, SCATTERING_TEXTURE_HEIGHT, SCATTERING_TEXTURE_DEPTH, S};
    ReducedScatteringTexture mt{SCATTERING_TEXTURE_WIDTH, SCATTERING_TEXTURE_HEIGHT, SCATTERING_TEXTURE_DEPTH, M};
    DimensionlessSpectrum trs;
    Out3(GetSkyRadianceToPoint(atm, t, st, mt, vec3(camera[0], camera[1], camera[2]),
                               vec3(point[0], point[1], point[2]), shadow, vec3(sun[0], sun[1], sun[2]), trs), out);
    Out3(trs, tr);
  });
  return 0;
}
int ref_sun_and_sky_irradiance(const oracle_atmosphere* a, const oracle_shape* s, const double* T,
                               const double* I, const double point[3], const double normal[3],
                               const double sun[3], double sun_irr[3], double sky_irr[3]) {
  AtmosphereParameters atm = Atm(a);
  ATMO_REF_DISPATCH(s, {
    TransmittanceTexture t{TRANSMITTANCE_TEXTURE_WIDTH, TRANSMITTANCE_TEXTURE_HEIGHT, T};
    IrradianceTexture it{IRRADIANCE_TEXTURE_WIDTH, IRRADIANCE_TEXTURE_HEIGHT, I};
    IrradianceSpectrum sky;
    Out3(GetSunAndSkyIrradiance(atm, t, it, vec3(point[0], point[1], point[2]),
                                vec3(normal[0], normal[1], normal[2]), vec3(sun[0], sun[1], sun[2]), sky), sun_irr);
    Out3(sky, sky_irr);
  });
  return 0;
}

}  // extern "C"
