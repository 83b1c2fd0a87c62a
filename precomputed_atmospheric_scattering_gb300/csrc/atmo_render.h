// atmo_render.h -- render-time queries on precomputed LUTs (host side).
#ifndef ATMO_RENDER_H_
#define ATMO_RENDER_H_

#include <cuda_runtime.h>

#include <cstring>

#include "atmo_instance.h"

namespace atmo {

// One resident LUT set and the atmosphere it was computed for, as the
// render kernels read it (the ATMOSPHERE constant and textures of the
// reference's shader, atmosphere/model.cc:691-744 and :221-281).
struct RenderLuts {
  Consts c;
  Shape s;
  const float4* T;      // transmittance
  const float4* Tau;    // optical depth of the same texels
  const float4* S;      // scattering (RGB + single-Mie red in alpha when combined)
  const float4* M;      // single Mie (nullptr when combined)
  const float4* I;      // irradiance
  int combined;
  float sky_k[3];       // SKY_SPECTRAL_RADIANCE_TO_LUMINANCE
  float sun_k[3];       // SUN_SPECTRAL_RADIANCE_TO_LUMINANCE
};

// Queries over device arrays of float triples.  `sun` holds one direction
// (sun_stride 0) or one per query (sun_stride 3); `shadow` may be null (0).
struct QueryArrays {
  const float* a;        // camera, or the point p of GetSunAndSkyIrradiance
  const float* b;        // view ray, point, or normal
  const float* shadow;   // shadow lengths
  const float* sun;
  int sun_stride;
  long long n;
  int luminance;         // apply the *_SPECTRAL_RADIANCE_TO_LUMINANCE factors
  float* out0;           // radiance, or sun irradiance
  float* out1;           // transmittance, or sky irradiance (may be null)
};

enum class Query { kSkyRadiance, kSkyRadianceToPoint, kSunAndSkyIrradiance };

cudaError_t LaunchQuery(Query q, const RenderLuts& luts, const QueryArrays& x, cudaStream_t st);

// A pinhole view: pixel (i, j) looks along
// normalize(forward + ((2 i + 1) / W - 1) tan(fov_y / 2) aspect right
//           + (1 - (2 j + 1) / H) tan(fov_y / 2) up).
struct PinholeView {
  float camera[3];
  float right[3], up[3], forward[3];
  float tan_half_fov_y;
  int width, height;
  float sun[3];
  const float* depth;    // per-pixel distance to the shaded point (length units)
  float albedo[3];       // of the shaded point, for the composite
  int luminance;
  float4* sky;           // GetSkyRadiance per pixel (alpha: transmittance green)
  float4* shaded;        // GetSkyRadianceToPoint + transmittance x albedo / pi x
                         // (sun + sky irradiance) at the point, normal = -view ray
};

cudaError_t LaunchShadeView(const RenderLuts& luts, const PinholeView& v, cudaStream_t st);

// The render view of one precomputed instance (luminance factors 1).
inline RenderLuts LutsOf(const Instance& in) {
  RenderLuts r;
  std::memset(&r, 0, sizeof(r));
  r.c = in.c;
  r.s = in.s;
  r.T = in.T;
  r.Tau = in.Tau;
  r.S = in.S;
  r.M = in.M;
  r.I = in.I;
  r.combined = in.combined;
  for (int i = 0; i < 3; ++i) r.sky_k[i] = r.sun_k[i] = 1.0f;
  return r;
}

}  // namespace atmo

// The C ABI's atmo_lut_set: a resident LUT set as the render-time queries
// read it, with the API switches of its owner.
struct atmo_lut_set {
  atmo::RenderLuts luts;
  bool radiance_api = true;    // RADIANCE_API_ENABLED (3 precomputed wavelengths)
  bool luminance_api = true;   // *_SPECTRAL_RADIANCE_TO_LUMINANCE factors known
  double solar[3] = {0, 0, 0};
  double sun_angular_radius = 0;
};

#endif  // ATMO_RENDER_H_
