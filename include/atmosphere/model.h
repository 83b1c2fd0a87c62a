// atmosphere/model.h -- C++ facade with the signature of the reference's
// atmosphere::Model (ebruneton/precomputed_atmospheric_scattering,
// atmosphere/model.h:158-339), implemented over the C ABI of atmo/atmo.h.
//
// A program written against the reference compiles against this header
// unchanged (add -I<repo>/include and link libatmo_gb300.so):
//
//   reference                                  this facade
//   -----------------------------------------  ---------------------------------
//   DensityProfileLayer     model.h:165-178    same class, same members
//   Model(19 parameters)    model.h:182-281    same signature (+ optional LUT shape)
//   ~Model                  model.cc:801-811   atmo_model_destroy
//   Init(orders = 4)        model.h:285        atmo_model_init + synchronize
//   shader()                model.h:287        returns 0: no OpenGL here; the
//                                              shader text is shader_source()
//   SetProgramUniforms      model.h:289-294    throws: texture binding needs
//                                              OpenGL, unavailable on this machine;
//                                              the LUTs are device buffers
//                                              (lut(), read_lut())
//   ConvertSpectrumToLinearSrgb  model.h:301-304  same signature
//   kLambdaR/G/B            model.h:306-308    same values
//
// Error behaviour: the reference asserts on OpenGL errors; this facade throws
// std::runtime_error with the C ABI's message (atmo_last_error()).
#ifndef ATMOSPHERE_MODEL_H_
#define ATMOSPHERE_MODEL_H_

#include <stdexcept>
#include <string>
#include <vector>

#include "../atmo/atmo.h"

typedef unsigned int GLuint;

namespace atmosphere {

class DensityProfileLayer {
 public:
  DensityProfileLayer() : DensityProfileLayer(0.0, 0.0, 0.0, 0.0, 0.0) {}
  DensityProfileLayer(double width, double exp_term, double exp_scale, double linear_term,
                      double constant_term)
      : width(width),
        exp_term(exp_term),
        exp_scale(exp_scale),
        linear_term(linear_term),
        constant_term(constant_term) {}
  double width;
  double exp_term;
  double exp_scale;
  double linear_term;
  double constant_term;
};

class Model {
 public:
  Model(const std::vector<double>& wavelengths, const std::vector<double>& solar_irradiance,
        double sun_angular_radius, double bottom_radius, double top_radius,
        const std::vector<DensityProfileLayer>& rayleigh_density,
        const std::vector<double>& rayleigh_scattering,
        const std::vector<DensityProfileLayer>& mie_density,
        const std::vector<double>& mie_scattering, const std::vector<double>& mie_extinction,
        double mie_phase_function_g, const std::vector<DensityProfileLayer>& absorption_density,
        const std::vector<double>& absorption_extinction,
        const std::vector<double>& ground_albedo, double max_sun_zenith_angle,
        double length_unit_in_meters, unsigned int num_precomputed_wavelengths,
        bool combine_scattering_textures, bool half_precision,
        const atmo_lut_shape* lut_shape = nullptr)
      : combined_(combine_scattering_textures) {
    const size_t n = wavelengths.size();
    const std::vector<double>* spectra[] = {&solar_irradiance,      &rayleigh_scattering,
                                            &mie_scattering,        &mie_extinction,
                                            &absorption_extinction, &ground_albedo};
    for (const std::vector<double>* v : spectra) {
      if (v->size() != n) {
        throw std::invalid_argument(
            "atmosphere::Model: every spectrum must have one value per wavelength");
      }
    }
    const std::vector<atmo_density_layer> ray = Layers(rayleigh_density);
    const std::vector<atmo_density_layer> mie = Layers(mie_density);
    const std::vector<atmo_density_layer> abs = Layers(absorption_density);
    atmo_model_params p;
    p.wavelengths = wavelengths.data();
    p.num_wavelengths = (unsigned)n;
    p.solar_irradiance = solar_irradiance.data();
    p.sun_angular_radius = sun_angular_radius;
    p.bottom_radius = bottom_radius;
    p.top_radius = top_radius;
    p.rayleigh_density = ray.data();
    p.num_rayleigh_layers = (unsigned)ray.size();
    p.rayleigh_scattering = rayleigh_scattering.data();
    p.mie_density = mie.data();
    p.num_mie_layers = (unsigned)mie.size();
    p.mie_scattering = mie_scattering.data();
    p.mie_extinction = mie_extinction.data();
    p.mie_phase_function_g = mie_phase_function_g;
    p.absorption_density = abs.data();
    p.num_absorption_layers = (unsigned)abs.size();
    p.absorption_extinction = absorption_extinction.data();
    p.ground_albedo = ground_albedo.data();
    p.max_sun_zenith_angle = max_sun_zenith_angle;
    p.length_unit_in_meters = length_unit_in_meters;
    p.num_precomputed_wavelengths = num_precomputed_wavelengths;
    p.combine_scattering_textures = combine_scattering_textures ? 1 : 0;
    p.half_precision = half_precision ? 1 : 0;
    Check(atmo_model_create(&p, lut_shape, &model_), "atmo_model_create");
  }

  ~Model() {
    if (model_) atmo_model_destroy(model_);
  }
  Model(const Model&) = delete;
  Model& operator=(const Model&) = delete;

  // Precomputes the LUTs; returns when they are ready (the reference's Init
  // is synchronous from the caller's view).
  void Init(unsigned int num_scattering_orders = 4) {
    Check(atmo_model_init(model_, num_scattering_orders, nullptr), "atmo_model_init");
    Check(atmo_synchronize(nullptr), "atmo_synchronize");
  }

  // No OpenGL on this system: there is no shader object.
  GLuint shader() const { return 0; }

  // The GLSL source the reference compiles into shader() (its parameter
  // header and API functions; functions.glsl itself is not bundled).
  std::string shader_source() const {
    size_t needed = 0;
    Check(atmo_model_shader_source(model_, nullptr, 0, &needed), "atmo_model_shader_source");
    std::string s(needed, '\0');
    Check(atmo_model_shader_source(model_, &s[0], needed, &needed), "atmo_model_shader_source");
    s.resize(needed > 0 ? needed - 1 : 0);
    return s;
  }

  void SetProgramUniforms(GLuint program, GLuint transmittance_texture_unit,
                          GLuint scattering_texture_unit, GLuint irradiance_texture_unit,
                          GLuint optional_single_mie_scattering_texture_unit = 0) const {
    Check(atmo_model_set_program_uniforms(model_, program, transmittance_texture_unit,
                                          scattering_texture_unit, irradiance_texture_unit,
                                          optional_single_mie_scattering_texture_unit),
          "SetProgramUniforms");
  }

  static void ConvertSpectrumToLinearSrgb(const std::vector<double>& wavelengths,
                                          const std::vector<double>& spectrum, double* r,
                                          double* g, double* b) {
    if (wavelengths.size() != spectrum.size()) {
      throw std::invalid_argument("ConvertSpectrumToLinearSrgb: size mismatch");
    }
    Check(atmo_convert_spectrum_to_linear_srgb(wavelengths.data(), spectrum.data(),
                                               (unsigned)wavelengths.size(), r, g, b),
          "atmo_convert_spectrum_to_linear_srgb");
  }

  static constexpr double kLambdaR = ATMO_LAMBDA_R;
  static constexpr double kLambdaG = ATMO_LAMBDA_G;
  static constexpr double kLambdaB = ATMO_LAMBDA_B;

  // ---- device-buffer access (in place of the reference's GL textures) ----
  atmo_lut_view lut(atmo_lut_kind kind) const {
    atmo_lut_view v;
    Check(atmo_model_get_lut(model_, kind, &v), "atmo_model_get_lut");
    return v;
  }
  // float32 RGBA texels, x fastest (glGetTexImage order).
  std::vector<float> read_lut(atmo_lut_kind kind) const {
    const atmo_lut_view v = lut(kind);
    std::vector<float> out((size_t)v.width * v.height * v.depth * 4);
    Check(atmo_model_read_lut(model_, kind, out.data(), out.size() * sizeof(float)),
          "atmo_model_read_lut");
    return out;
  }
  bool combine_scattering_textures() const { return combined_; }
  atmo_model* handle() const { return model_; }

 private:
  static std::vector<atmo_density_layer> Layers(const std::vector<DensityProfileLayer>& in) {
    std::vector<atmo_density_layer> out;
    for (const DensityProfileLayer& l : in) {
      out.push_back(atmo_density_layer{l.width, l.exp_term, l.exp_scale, l.linear_term,
                                       l.constant_term});
    }
    return out;
  }
  static void Check(atmo_status s, const char* what) {
    if (s != ATMO_OK) {
      throw std::runtime_error(std::string(what) + ": " + atmo_last_error());
    }
  }

  atmo_model* model_ = nullptr;
  bool combined_;
};

}  // namespace atmosphere

#endif  // ATMOSPHERE_MODEL_H_
