// Exercises the atmosphere::Model C++ facade (include/atmosphere/model.h) the
// way the reference's callers use atmosphere::Model (atmosphere/demo/demo.cc,
// atmosphere/reference/model_test.cc): the Earth model of the demo, built with
// the reference's 19-argument constructor.
//
//   model_facade_test host   checks that need no GPU
//   model_facade_test gpu    Init(4) through the facade, compared texel for
//                            texel with the same model run through the C ABI
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "atmosphere/model.h"

namespace {

int failures = 0;

void Expect(bool ok, const char* what) {
  if (!ok) {
    std::printf("FAIL: %s\n", what);
    ++failures;
  }
}

// Ozone absorption cross sections (m^2) at 360, 370, ..., 830 nm.
const double kOzoneCrossSection[48] = {
    1.18e-27,  2.182e-28, 2.818e-28, 6.636e-28, 1.527e-27, 2.763e-27, 5.52e-27,  8.451e-27,
    1.582e-26, 2.316e-26, 3.669e-26, 4.924e-26, 7.752e-26, 9.016e-26, 1.48e-25,  1.602e-25,
    2.139e-25, 2.755e-25, 3.091e-25, 3.5e-25,   4.266e-25, 4.672e-25, 4.398e-25, 4.701e-25,
    5.019e-25, 4.305e-25, 3.74e-25,  3.215e-25, 2.662e-25, 2.238e-25, 1.852e-25, 1.473e-25,
    1.209e-25, 9.423e-26, 7.455e-26, 6.566e-26, 5.105e-26, 4.15e-26,  4.228e-26, 3.237e-26,
    2.451e-26, 2.801e-26, 2.534e-26, 1.624e-26, 1.465e-26, 2.078e-26, 1.383e-26, 7.105e-27};

struct EarthSpectra {
  std::vector<double> wavelengths, solar, rayleigh, mie_sca, mie_ext, ozone, albedo;
  EarthSpectra() {
    for (int i = 0; i < 48; ++i) {
      const double l = 360.0 + 10.0 * i;
      const double mie = 5.328e-3 / 1200.0;
      wavelengths.push_back(l);
      solar.push_back(1.5);
      rayleigh.push_back(1.24062e-6 * std::pow(l * 1e-3, -4.0));
      mie_sca.push_back(mie * 0.9);
      mie_ext.push_back(mie);
      ozone.push_back(300.0 * 2.687e20 / 15000.0 * kOzoneCrossSection[i]);
      albedo.push_back(0.1);
    }
  }
};

std::unique_ptr<atmosphere::Model> EarthModel(const EarthSpectra& e, unsigned n_lambda,
                                              bool combined) {
  using atmosphere::DensityProfileLayer;
  const double kPi = 3.14159265358979323846;
  return std::unique_ptr<atmosphere::Model>(new atmosphere::Model(
      e.wavelengths, e.solar, 0.00935 / 2.0, 6360000.0, 6420000.0,
      {DensityProfileLayer(0.0, 1.0, -1.0 / 8000.0, 0.0, 0.0)}, e.rayleigh,
      {DensityProfileLayer(0.0, 1.0, -1.0 / 1200.0, 0.0, 0.0)}, e.mie_sca, e.mie_ext, 0.8,
      {DensityProfileLayer(25000.0, 0.0, 0.0, 1.0 / 15000.0, -2.0 / 3.0),
       DensityProfileLayer(0.0, 0.0, 0.0, -1.0 / 15000.0, 8.0 / 3.0)},
      e.ozone, e.albedo, 102.0 / 180.0 * kPi, 1000.0, n_lambda, combined, false));
}

void HostChecks() {
  EarthSpectra e;
  std::unique_ptr<atmosphere::Model> m = EarthModel(e, 3, true);
  Expect(m->shader() == 0, "shader() has no GL object");
  const std::string src = m->shader_source();
  Expect(src.rfind("#version 330\n", 0) == 0, "shader source starts with #version 330");
  Expect(src.find("vec3(0.005802,0.013558,0.033100)") != std::string::npos,
         "Rayleigh coefficients printed with 6 decimals");
  Expect(src.find("GetSkyRadiance(") != std::string::npos, "API function in the shader");
  bool threw = false;
  try {
    m->SetProgramUniforms(1, 0, 1, 2);
  } catch (const std::runtime_error&) {
    threw = true;
  }
  Expect(threw, "SetProgramUniforms reports the missing OpenGL");

  double r = 0, g = 0, b = 0, rc = 0, gc = 0, bc = 0;
  atmosphere::Model::ConvertSpectrumToLinearSrgb(e.wavelengths, e.solar, &r, &g, &b);
  atmo_convert_spectrum_to_linear_srgb(e.wavelengths.data(), e.solar.data(),
                                       (unsigned)e.wavelengths.size(), &rc, &gc, &bc);
  Expect(r == rc && g == gc && b == bc, "ConvertSpectrumToLinearSrgb equals the C ABI");
  Expect(r > 0.0 && g > 0.0 && b > 0.0, "a flat solar spectrum has positive sRGB");
  Expect(atmosphere::Model::kLambdaR == 680.0 && atmosphere::Model::kLambdaG == 550.0 &&
             atmosphere::Model::kLambdaB == 440.0,
         "kLambdaR/G/B");

  threw = false;
  try {
    std::vector<double> short_albedo(3, 0.1);
    EarthSpectra bad;
    bad.albedo = short_albedo;
    EarthModel(bad, 3, true);
  } catch (const std::invalid_argument&) {
    threw = true;
  }
  Expect(threw, "a spectrum of the wrong size is rejected");
  threw = false;
  try {
    std::vector<double> w = {400.0, 500.0};
    std::vector<double> s = {1.0};
    atmosphere::Model::ConvertSpectrumToLinearSrgb(w, s, &r, &g, &b);
  } catch (const std::invalid_argument&) {
    threw = true;
  }
  Expect(threw, "ConvertSpectrumToLinearSrgb rejects mismatched sizes");
}

void GpuChecks() {
  EarthSpectra e;
  const atmo_lut_kind kinds[3] = {ATMO_LUT_TRANSMITTANCE, ATMO_LUT_SCATTERING,
                                  ATMO_LUT_IRRADIANCE};
  for (unsigned n_lambda : {3u, 15u}) {
    std::unique_ptr<atmosphere::Model> facade = EarthModel(e, n_lambda, true);
    facade->Init(4);
    // The same model through the C ABI directly.
    std::unique_ptr<atmosphere::Model> raw = EarthModel(e, n_lambda, true);
    if (atmo_model_init(raw->handle(), 4, nullptr) != ATMO_OK ||
        atmo_synchronize(nullptr) != ATMO_OK) {
      Expect(false, atmo_last_error());
      return;
    }
    for (atmo_lut_kind k : kinds) {
      const std::vector<float> a = facade->read_lut(k), b = raw->read_lut(k);
      Expect(a.size() == b.size() && std::memcmp(a.data(), b.data(), a.size() * 4) == 0,
             "facade LUT equals the C ABI's");
      bool finite = true, nonneg = true;
      for (float x : a) {
        finite = finite && std::isfinite(x);
        nonneg = nonneg && x >= 0.0f;
      }
      Expect(finite, "LUT texels are finite");
      // Radiance LUTs are non-negative; luminance LUTs (more than 3
      // wavelengths) hold linear sRGB, whose components can be negative.
      Expect(nonneg || n_lambda > 3, "radiance LUT texels are non-negative");
    }
    const atmo_lut_view s = facade->lut(ATMO_LUT_SCATTERING);
    Expect(s.width == 256 && s.height == 128 && s.depth == 32,
           "scattering LUT has the reference's default size");
  }
}

}  // namespace

int main(int argc, char** argv) {
  const std::string mode = argc > 1 ? argv[1] : "host";
  try {
    if (mode == "host") {
      HostChecks();
    } else if (mode == "gpu") {
      GpuChecks();
    } else {
      std::printf("usage: %s host|gpu\n", argv[0]);
      return 2;
    }
  } catch (const std::exception& ex) {
    std::printf("FAIL: exception %s\n", ex.what());
    return 1;
  }
  if (failures == 0) std::printf("ok\n");
  return failures == 0 ? 0 : 1;
}
